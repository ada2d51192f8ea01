"""ki_solve_device_noalloc: the solve for callers that cannot allocate device
memory while solving (an application that reserves all device memory for its
own allocator, or a latency-critical loop that cannot absorb cudaMalloc's
synchronization).  Its temporaries live in a fixed 32 MiB device array inside
the library.  It runs the same launch sequence as the allocating entry point
ki_solve_device, so it must give bit-identical solutions, call after call:
FP64 and FP32 factorizations, simply and multiply connected boundaries, a
border wide enough for the split-K row reduction (n_border x nrhs > 4,096),
the handle's stream and a caller's stream.  This file is collected last on
purpose."""
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


def _case(pkg, kind, precision):
    g = pkg.geometry
    rng = np.random.default_rng(17)
    tol = 1e-10 if precision == "fp64" else 1e-6
    kw = dict(id_tol=tol, precision=pkg.PRECISION_FP64 if precision == "fp64" else pkg.PRECISION_FP32)
    if kind == "star":
        prob = g.star(256, 16)
        rhs = g.laplace_source_rhs(prob, g.random_sources(6, rng))
    elif kind == "holes":
        prob = g.disc_with_ellipses(1 << 13, 4, seed=21)
        rhs = g.laplace_source_rhs(prob, g.random_sources(6, rng))
    else:
        # 2D Stokes, 40 holes x 3 border columns = 120, times 40 right-hand
        # sides = 4,800 products: the wide (split-K) border reduction
        prob = g.disc_with_circles(1 << 13, 40, seed=5)
        src, frc = g.stokes_c3_sources(40)
        rhs = g.stokes_rhs(prob, src, frc)
        kw.update(solution_dimension=2, pde=pkg.PDE_STOKES)
    if prob.n_holes:
        kw.update(hole_centers=prob.hole_centers, hole_start=prob.hole_start,
                  hole_count=prob.hole_count)
    fac = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, **kw)
    return fac, rhs


@pytest.mark.parametrize("kind,precision,own_stream", [
    ("star", "fp64", False), ("holes", "fp64", False), ("holes", "fp32", True),
    ("stokes_wide", "fp64", True), ("stokes_wide", "fp32", False)])
def test_noalloc_matches_allocating_solve_twice(pkg, kind, precision, own_stream):
    torch = pytest.importorskip("torch")
    lib = pkg.load_library()
    noalloc = _bind(lib)
    fac, rhs = _case(pkg, kind, precision)
    N, nrhs, nb = fac.n_dofs, rhs.shape[1], max(1, fac.n_border)
    if kind == "stokes_wide":
        assert fac.n_border * nrhs > 4096
    stream = torch.cuda.Stream() if own_stream else None
    sptr = ctypes.c_void_p(stream.cuda_stream) if stream is not None else None
    d_b = torch.from_numpy(np.asfortranarray(rhs).T.copy()).cuda()   # column c = row c
    d_ref = torch.zeros_like(d_b)
    a_ref = torch.zeros((nrhs, nb), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    pkg._check(lib.ki_solve_device(fac._h, ctypes.c_void_p(d_b.data_ptr()), N, nrhs,
                                   ctypes.c_void_p(d_ref.data_ptr()), N,
                                   ctypes.c_void_p(a_ref.data_ptr()), nb, sptr))
    torch.cuda.synchronize()
    ref = d_ref.cpu().numpy()
    assert np.isfinite(ref).all()
    for call in range(2):
        d_x = torch.full_like(d_b, float("nan"))
        a_x = torch.full((nrhs, nb), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = noalloc(fac._h, ctypes.c_void_p(d_b.data_ptr()), N, nrhs,
                     ctypes.c_void_p(d_x.data_ptr()), N, ctypes.c_void_p(a_x.data_ptr()), nb, sptr)
        assert rc == pkg.KI_OK, lib.ki_last_error()
        torch.cuda.synchronize()
        # the same kernels in the same order on the same data: bit-identical
        assert np.array_equal(d_x.cpu().numpy(), ref), "call %d" % call
        if fac.n_border:
            assert np.array_equal(a_x.cpu().numpy(), a_ref.cpu().numpy()), "call %d" % call


def test_noalloc_rejects_oversized_solve(pkg):
    torch = pytest.importorskip("torch")
    lib = pkg.load_library()
    noalloc = _bind(lib)
    fac, rhs = _case(pkg, "star", "fp64")
    N = fac.n_dofs
    d = torch.zeros(N, dtype=torch.float64, device="cuda")
    # 100,000 right-hand sides of 4,096 unknowns need ~3 GB of scratch: refused
    # before any device access, so the small buffers are never touched
    rc = noalloc(fac._h, ctypes.c_void_p(d.data_ptr()), N, 100000, ctypes.c_void_p(d.data_ptr()), N,
                 None, 1, None)
    assert rc == pkg.KI_ERR_ARG
    assert b"32 MiB" in lib.ki_last_error()
