"""ki_solve_device_noalloc: the solve for callers that cannot allocate device
memory while solving (an application that reserves all device memory for its
own allocator, or a latency-critical loop that cannot absorb cudaMalloc's
synchronization).  Its temporaries live in a fixed 32 MiB device array inside
the library.  It must give the same solution as the allocating entry point
ki_solve_device, call after call.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bind(lib):
    f = lib.ki_solve_device_noalloc
    V, I = ctypes.c_void_p, ctypes.c_int
    f.argtypes = [V, V, I, I, V, I, V, I, V]
    f.restype = I
    return f


def _case(pkg, holes):
    g = pkg.geometry
    if holes:
        prob = g.disc_with_ellipses(1 << 13, 4, seed=21)
    else:
        prob = g.star(256, 16)
    rng = np.random.default_rng(17)
    rhs = g.laplace_source_rhs(prob, g.random_sources(6, rng))
    kw = {}
    if holes:
        kw = dict(hole_centers=prob.hole_centers, hole_start=prob.hole_start,
                  hole_count=prob.hole_count)
    fac = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, id_tol=1e-10, **kw)
    return fac, rhs


@pytest.mark.parametrize("holes", [False, True])
def test_noalloc_matches_allocating_solve_twice(pkg, holes):
    torch = pytest.importorskip("torch")
    lib = pkg.load_library()
    noalloc = _bind(lib)
    fac, rhs = _case(pkg, holes)
    N, nrhs, nb = fac.n_dofs, rhs.shape[1], max(1, fac.n_border)
    d_b = torch.from_numpy(np.asfortranarray(rhs).T.copy()).cuda()   # column c = row c
    d_ref = torch.zeros_like(d_b)
    a_ref = torch.zeros((nrhs, nb), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    pkg._check(lib.ki_solve_device(fac._h, ctypes.c_void_p(d_b.data_ptr()), N, nrhs,
                                   ctypes.c_void_p(d_ref.data_ptr()), N,
                                   ctypes.c_void_p(a_ref.data_ptr()), nb, None))
    torch.cuda.synchronize()
    ref = d_ref.cpu().numpy()
    for call in range(2):
        d_x = torch.full_like(d_b, float("nan"))
        a_x = torch.full((nrhs, nb), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = noalloc(fac._h, ctypes.c_void_p(d_b.data_ptr()), N, nrhs,
                     ctypes.c_void_p(d_x.data_ptr()), N, ctypes.c_void_p(a_x.data_ptr()), nb, None)
        assert rc == pkg.KI_OK, lib.ki_last_error()
        torch.cuda.synchronize()
        x = d_x.cpu().numpy()
        # the tolerance of the parity tests: 10 x id_tol relative
        assert np.abs(x - ref).max() <= 10 * 1e-10 * np.abs(ref).max(), "call %d" % call
        if fac.n_border:
            a = a_x.cpu().numpy()
            assert np.abs(a - a_ref.cpu().numpy()).max() <= 10 * 1e-10 * np.abs(ref).max()


def test_noalloc_rejects_oversized_solve(pkg):
    torch = pytest.importorskip("torch")
    lib = pkg.load_library()
    noalloc = _bind(lib)
    fac, rhs = _case(pkg, False)
    N = fac.n_dofs
    d = torch.zeros(N, dtype=torch.float64, device="cuda")
    # 100,000 right-hand sides of 4,096 unknowns need ~3 GB of scratch: refused
    # before any device access, so the small buffers are never touched
    rc = noalloc(fac._h, ctypes.c_void_p(d.data_ptr()), N, 100000, ctypes.c_void_p(d.data_ptr()), N,
                 None, 1, None)
    assert rc == pkg.KI_ERR_ARG
    assert b"32 MiB" in lib.ki_last_error()
