"""CPU oracle for the skeletonization solver: TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package, and only as the checker / the timed reference CPU path.  The product
path (the CUDA library behind include/ki_gpu.h) never imports it.

  * ``port``  -- oracle/port/ki_port.cpp, a C++ restatement of the
    reference's factor and solve (kern_interp/skel_factorization,
    kern_interp/kernel, kern_interp/quadtree), compiled by ``build_port``;
  * ``ref``   -- the reference's own sources compiled by oracle/build_ref.py
    (only where the reference tree is present).
"""
import ctypes
import glob
import hashlib
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SRC = os.path.join(HERE, "port", "ki_port.cpp")
PORT_LIB = os.path.join(HERE, "port", "libkiport.so")

_blas = None


def load_openblas():
    """Load scipy's bundled OpenBLAS into the process (RTLD_GLOBAL) so the
    port and the reference build can resolve LAPACK symbols."""
    global _blas
    if _blas is None:
        import scipy
        libs = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
        cands = sorted(glob.glob(os.path.join(libs, "libscipy_openblas*.so")))
        if not cands:
            raise RuntimeError("scipy's bundled OpenBLAS not found")
        _blas = ctypes.CDLL(cands[0], mode=ctypes.RTLD_GLOBAL)
    return _blas


def build_port(force=False):
    """Compile the C++ restatement (gcc, OpenMP) into oracle/port/libkiport.so."""
    src = open(PORT_SRC, "rb").read()
    stamp = hashlib.sha1(src).hexdigest()
    stamp_file = PORT_LIB + ".stamp"
    if (not force and os.path.exists(PORT_LIB) and os.path.exists(stamp_file)
            and open(stamp_file).read() == stamp):
        return PORT_LIB
    subprocess.run(["g++", "-O2", "-fopenmp", "-std=c++17", "-fPIC", "-shared",
                    PORT_SRC, "-o", PORT_LIB, "-ldl"], check=True)
    with open(stamp_file, "w") as f:
        f.write(stamp)
    return PORT_LIB


_P = ctypes.c_void_p


def _dp(a):
    return a.ctypes.data_as(_P)


class _Lib:
    def __init__(self, path, prefix, has_params):
        load_openblas()
        self.lib = ctypes.CDLL(path)
        self.prefix = prefix
        self.has_params = has_params
        f = getattr(self.lib, prefix + "_solve")
        base = [ctypes.c_int] * 4 + [_P] * 4 + [ctypes.c_int] + [_P] * 4 + \
               [ctypes.c_int, ctypes.c_double, ctypes.c_int]
        if has_params:
            base += [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int]
        f.argtypes = base + [_P] * 3
        f.restype = ctypes.c_int
        self.solve_fn = f


def ref_update_solve(frames, rhs, tol, threads=1, solution_dim=1, pde=0):
    """The reference's incremental re-factorization (compiled reference only,
    default tree/proxy parameters): frames[0] initialized and skeletonized,
    every later frame applied with QuadTree::perturb and skeletonized again
    (kiref_update_solve in ref_driver.cpp).  frames: problems of one size and
    hole layout; rhs: one (N,) right-hand side per frame.  Returns (mu
    (frames, N), alpha (frames, n_border), seconds (frames,), compressed
    boxes (frames,))."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("_ki_build_ref", os.path.join(HERE, "build_ref.py"))
    br = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(br)
    load_openblas()
    lib = ctypes.CDLL(br.build())
    fn = lib.kiref_update_solve
    fn.argtypes = [ctypes.c_int] * 5 + [_P] * 4 + [ctypes.c_int] + [_P] * 4 + \
                  [ctypes.c_double, ctypes.c_int] + [_P] * 3
    fn.restype = ctypes.c_int
    p0 = frames[0]
    dim = int(np.asarray(p0.points).shape[1])
    nf, n = len(frames), p0.n
    N = n * solution_dim
    c = 1 if solution_dim == 1 else (3 if dim == 2 else 6)
    nb = c * p0.n_holes
    cat = lambda k: np.ascontiguousarray(np.concatenate(
        [np.asarray(getattr(p, k), np.float64).reshape(-1) for p in frames]))
    pts, nrm, wts, cur, hc = (cat(k) for k in
                              ("points", "normals", "weights", "curvatures", "hole_centers"))
    hs = np.ascontiguousarray(p0.hole_start, np.int32)
    hn = np.ascontiguousarray(p0.hole_count, np.int32)
    b = np.ascontiguousarray(np.concatenate([np.asarray(r, np.float64).reshape(-1) for r in rhs]))
    mu = np.zeros(nf * N)
    alpha = np.zeros(max(1, nf * nb))
    st = np.zeros(2 * nf)
    rc = fn(n, dim, solution_dim, pde, nf, _dp(pts), _dp(nrm), _dp(wts), _dp(cur), p0.n_holes,
            _dp(hc), _dp(hs), _dp(hn), _dp(b), tol, threads, _dp(mu), _dp(alpha), _dp(st))
    if rc != 0:
        raise RuntimeError("reference update solve failed")
    return (mu.reshape(nf, N), alpha[:nf * nb].reshape(nf, nb), st[0::2].copy(),
            st[1::2].astype(int))


def solve(prob, rhs, tol, threads=1, leaf=64, proxy=None, ratio=2.0, min_compress=64,
          solution_dim=1, pde=0, impl="port"):
    """Factor + solve with the oracle.  rhs: (N, nrhs).  Returns (mu, alpha,
    stats) with mu (N, nrhs), alpha (n_border, nrhs), stats dict.  The
    boundary's dimension is prob.points.shape[1]; proxy None takes the
    reference default (128 in 2D, the fixed 32-point sphere in 3D)."""
    dim = int(np.asarray(prob.points).shape[1])
    if proxy is None:
        proxy = 128 if dim == 2 else 0
    if impl == "port":
        lib = _Lib(build_port(), "kiport", True)
    else:
        import importlib.util
        spec = importlib.util.spec_from_file_location("_ki_build_ref", os.path.join(HERE, "build_ref.py"))
        br = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(br)
        # the reference's 3D proxy sphere is fixed (kern_interp/kernel/kernel.h:44-62):
        # NUM_PROXY_POINTS only matters in 2D
        lib = _Lib(br.build(leaf=leaf, proxy=proxy if dim == 2 else 128, ratio=ratio,
                            min_compress=min_compress),
                   "kiref", False)
    rhs = np.asarray(rhs, dtype=np.float64)
    if rhs.ndim == 1:
        rhs = rhs[:, None]
    N = prob.n * solution_dim
    nrhs = rhs.shape[1]
    c = 1 if solution_dim == 1 else (3 if dim == 2 else 6)
    # the Neumann (1) and Gaussian (2) kernels have no border (empty U)
    nb = 0 if pde in (1, 2) else c * prob.n_holes
    pts = np.ascontiguousarray(prob.points, np.float64)
    nrm = np.ascontiguousarray(prob.normals, np.float64)
    wts = np.ascontiguousarray(prob.weights, np.float64)
    cur = np.ascontiguousarray(prob.curvatures, np.float64)
    hc = np.ascontiguousarray(prob.hole_centers, np.float64).reshape(-1)
    hs = np.ascontiguousarray(prob.hole_start, np.int32)
    hn = np.ascontiguousarray(prob.hole_count, np.int32)
    b = np.asfortranarray(rhs)
    mu = np.zeros((N, nrhs), order="F")
    alpha = np.zeros((max(nb, 1), nrhs), order="F")
    st = np.zeros(8)
    args = [prob.n, dim, solution_dim, pde, _dp(pts), _dp(nrm), _dp(wts), _dp(cur),
            prob.n_holes, _dp(hc), _dp(hs), _dp(hn), _dp(b), nrhs, tol, threads]
    if lib.has_params:
        args += [leaf, proxy, ratio, min_compress]
    args += [_dp(mu), _dp(alpha), _dp(st)]
    rc = lib.solve_fn(*args)
    if rc != 0:
        msg = ""
        if impl == "port":
            lib.lib.kiport_last_error.restype = ctypes.c_char_p
            msg = lib.lib.kiport_last_error().decode()
        raise RuntimeError("oracle solve failed: " + msg)
    stats = dict(factor_s=st[0], solve_s=st[1], levels=int(st[2]), root=int(st[3]),
                 compressed=int(st[4]), redundant=int(st[5]))
    return mu, alpha[:nb], stats


def dense_matrix(prob, solution_dim=1):
    """Dense Nystrom matrix of the reference kernel (Kernel::operator(); in
    3D with the row-sum diagonal of a surface without holes)."""
    lib = ctypes.CDLL(build_port())
    N = prob.n * solution_dim
    out = np.zeros((N, N), order="F")
    dim = int(np.asarray(prob.points).shape[1])
    lib.kiport_dense_dim.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int] + [_P] * 5
    curv = prob.curvatures if prob.curvatures is not None else np.zeros(prob.n)
    lib.kiport_dense_dim(prob.n, dim, solution_dim, _dp(np.ascontiguousarray(prob.points)),
                     _dp(np.ascontiguousarray(prob.normals)),
                         _dp(np.ascontiguousarray(prob.weights)),
                         _dp(np.ascontiguousarray(curv)), _dp(out))
    return out


def laplace_forward(prob, targets, mu):
    """u(x) = sum_s K(x, s) mu_s at domain points (Kernel::apply_forward with
    forward=true, kern_interp/kernel/kernel.cpp:809-825; the 2D Laplace
    forward entry equals the off-diagonal entry with target normal 0)."""
    d = targets[:, None, :] - prob.points[None, :, :]
    rn = (d * prob.normals[None]).sum(-1)
    r2 = (d ** 2).sum(-1)
    K = -prob.weights[None] / (2 * np.pi) * rn / r2
    return K @ mu


def residual_rows(prob, mu, alpha, rhs, rows, solution_dim=1, threads=None):
    """Rows of the bordered system's residual, computed with the port's FP64
    kernel entries: returns (res (len(rows), nrhs), res_border (n_border,
    nrhs)) with res = K[rows] mu + U[rows] alpha - f[rows] and res_border =
    Psi mu - alpha.  O(len(rows) * N) work (plus O(N^2) for a 3D diagonal)."""
    lib = ctypes.CDLL(build_port())
    dim = int(np.asarray(prob.points).shape[1])
    N = prob.n * solution_dim
    mu = np.asfortranarray(np.asarray(mu, np.float64).reshape(N, -1))
    nrhs = mu.shape[1]
    f = np.asfortranarray(np.asarray(rhs, np.float64).reshape(N, nrhs))
    c = 1 if solution_dim == 1 else (3 if dim == 2 else 6)
    nb = c * prob.n_holes
    al = np.zeros((max(nb, 1), nrhs), order="F")
    if nb:
        al[:] = np.asarray(alpha, np.float64).reshape(nb, nrhs)
    rows = np.ascontiguousarray(rows, np.int32)
    res = np.zeros((rows.size, nrhs), order="F")
    res_b = np.zeros((max(nb, 1), nrhs), order="F")
    curv = prob.curvatures if prob.curvatures is not None else np.zeros(prob.n)
    hc = np.ascontiguousarray(prob.hole_centers, np.float64).reshape(-1)
    hs = np.ascontiguousarray(prob.hole_start, np.int32)
    hn = np.ascontiguousarray(prob.hole_count, np.int32)
    fn = lib.kiport_residual_rows
    fn.argtypes = [ctypes.c_int] * 3 + [_P] * 4 + [ctypes.c_int] + [_P] * 6 + [ctypes.c_int, _P,
                                                                               ctypes.c_int,
                                                                               ctypes.c_int, _P, _P]
    fn.restype = ctypes.c_int
    rc = fn(prob.n, dim, solution_dim, _dp(np.ascontiguousarray(prob.points, np.float64)),
            _dp(np.ascontiguousarray(prob.normals, np.float64)),
            _dp(np.ascontiguousarray(prob.weights, np.float64)),
            _dp(np.ascontiguousarray(curv, np.float64)), prob.n_holes, _dp(hc), _dp(hs), _dp(hn),
            _dp(mu), _dp(al), _dp(f), nrhs, _dp(rows), rows.size, threads or os.cpu_count() or 1,
            _dp(res), _dp(res_b))
    if rc != 0:
        lib.kiport_last_error.restype = ctypes.c_char_p
        raise RuntimeError("oracle residual failed: " + lib.kiport_last_error().decode())
    return res, res_b[:nb]
