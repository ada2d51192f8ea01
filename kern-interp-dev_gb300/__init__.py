"""kern_interp_gb300 -- Python mirror of the reference's factor-and-solve
surface over the GB300 C-ABI library (include/ki_gpu.h, libki_gpu.so).

The classes keep the reference's names and argument meaning
(kern_interp, C++ namespace kern_interp):

  Boundary            kern_interp/boundaries/boundary.h:47-64 (public data)
  Kernel              kern_interp/kernel/kernel.h:18-66
  QuadTree            kern_interp/quadtree/quadtree.h:111-149 (initialize_tree)
  SkelFactorization   kern_interp/skel_factorization/skel_factorization.h:20-58
  linear_solve        kern_interp/linear_solve.h:29-31
  boundary_integral_solve   kern_interp/linear_solve.h:17-19

Matrices cross the boundary as column-major float64 arrays (the reference's
ki_Mat layout).  There is no CPU fallback: every call runs on the GPU, and
loading fails loudly when the library is missing.
"""
import ctypes
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libki_gpu.so")

KI_OK, KI_ERR_ARG, KI_ERR_CUDA, KI_ERR_NUMERIC, KI_ERR_TIMEOUT, KI_ERR_OOM, KI_ERR_STATE = range(7)
PDE_LAPLACE, PDE_LAPLACE_NEUMANN, PDE_GAUSS, PDE_STOKES = range(4)
PRECISION_FP64, PRECISION_FP32 = 0, 1

EXPORTED = ["ki_factor_create", "ki_factor_destroy", "ki_factor_get_info", "ki_solve",
            "ki_solve_device", "ki_apply", "ki_eval_targets", "ki_last_error", "ki_version",
            "ki_factor_get_profile", "ki_factor_set_profiling", "ki_apply_rows",
            "ki_measure_fma_peak", "ki_tensor_core_check", "ki_solve_refined", "ki_solve_refined_device",
            "ki_solve_device_noalloc", "ki_apply_fmm", "ki_apply_fmm_ex", "ki_trim_memory",
            "ki_launch_count", "ki_rank_model_floats",
            "ki_rank_model_train", "ki_rank_model_predict", "ki_rank_model_grad",
            "ki_factor_get_box_log", "ki_factor_update", "ki_autotune", "ki_tune_set",
            "ki_tune_get", "ki_rank_model_predict_bf16"]
RANK_MODEL_PATH = os.path.join(HERE, "rank_model.npy")
# the autotuner's table (ki_autotune's output), loaded with the library
TUNE_PATH = os.path.join(HERE, "tune_gb300.json")
BOX_LOG_COLUMNS = 15   # 12 features, n, k, level


class KiError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("ki error %d: %s" % (code, msg))
        self.code = code


class _Desc(ctypes.Structure):
    _fields_ = [("n_points", ctypes.c_int), ("domain_dimension", ctypes.c_int),
                ("solution_dimension", ctypes.c_int), ("pde", ctypes.c_int),
                ("points", ctypes.c_void_p), ("normals", ctypes.c_void_p),
                ("weights", ctypes.c_void_p), ("curvatures", ctypes.c_void_p),
                ("n_holes", ctypes.c_int), ("hole_centers", ctypes.c_void_p),
                ("hole_node_start", ctypes.c_void_p), ("hole_node_count", ctypes.c_void_p),
                ("max_leaf_dofs", ctypes.c_int), ("num_proxy_points", ctypes.c_int),
                ("radius_ratio", ctypes.c_double), ("min_dofs_to_compress", ctypes.c_int),
                ("id_tol", ctypes.c_double), ("precision", ctypes.c_int),
                ("rank_model", ctypes.c_void_p)]


class _RefineInfo(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_int), ("residual0", ctypes.c_double),
                ("residual", ctypes.c_double), ("updates", ctypes.c_int),
                ("drift_bound", ctypes.c_double)]


class _Info(ctypes.Structure):
    _fields_ = [("n_dofs", ctypes.c_int), ("n_levels", ctypes.c_int),
                ("n_compressed", ctypes.c_int), ("n_redundant", ctypes.c_long),
                ("n_root", ctypes.c_int), ("n_border", ctypes.c_int),
                ("factor_seconds", ctypes.c_double), ("device_bytes", ctypes.c_long),
                ("n_sketched", ctypes.c_int), ("n_fallback", ctypes.c_int),
                ("n_reused", ctypes.c_int)]


_lib = None


def load_library(path=None):
    """Load libki_gpu.so (raises OSError when it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise OSError("libki_gpu.so not found at %s: run __graft_entry__.build()" % p)
    lib = ctypes.CDLL(p)
    V = ctypes.c_void_p
    I = ctypes.c_int
    lib.ki_factor_create.argtypes = [ctypes.POINTER(_Desc), ctypes.POINTER(V)]
    lib.ki_factor_destroy.argtypes = [V]
    lib.ki_factor_update.argtypes = [V, ctypes.POINTER(_Desc)]
    lib.ki_autotune.argtypes = [ctypes.POINTER(_Desc), I, I, ctypes.c_char_p, I]
    lib.ki_tune_set.argtypes = [ctypes.c_char_p]
    lib.ki_tune_get.argtypes = [ctypes.c_char_p, I]
    lib.ki_factor_get_info.argtypes = [V, ctypes.POINTER(_Info)]
    lib.ki_solve.argtypes = [V, V, I, I, V, I, V, I]
    lib.ki_solve_device.argtypes = [V, V, I, I, V, I, V, I, V]
    lib.ki_apply.argtypes = [V, V, I, I, V, I, V, I]
    lib.ki_eval_targets.argtypes = [V, V, I, V, I, I, V, I, V, I]
    lib.ki_apply_fmm.argtypes = [V, V, I, I, V, I, V, I]
    lib.ki_apply_fmm_ex.argtypes = [V, V, I, I, V, I, V, I, I, I]
    lib.ki_launch_count.restype = ctypes.c_longlong
    lib.ki_launch_count.argtypes = []
    lib.ki_apply_rows.argtypes = [V, V, I, V, I, I, V, I, V, I]
    lib.ki_factor_get_profile.argtypes = [V, ctypes.c_char_p, I]
    lib.ki_factor_set_profiling.argtypes = [V, I]
    lib.ki_solve_refined.argtypes = [V, V, I, I, V, I, V, I, ctypes.c_double, I,
                                     ctypes.POINTER(_RefineInfo)]
    lib.ki_solve_refined_device.argtypes = [V, V, I, V, V, ctypes.c_double, I,
                                            ctypes.POINTER(_RefineInfo), V]
    F = ctypes.POINTER(ctypes.c_float)
    lib.ki_rank_model_train.argtypes = [V, V, I, I, ctypes.c_float, ctypes.c_uint, V, F]
    lib.ki_rank_model_predict.argtypes = [V, V, I, V]
    lib.ki_rank_model_predict_bf16.argtypes = [V, V, I, V]
    lib.ki_rank_model_grad.argtypes = [V, V, V, I, V, F]
    lib.ki_factor_get_box_log.argtypes = [V, V, I, ctypes.POINTER(I)]
    lib.ki_measure_fma_peak.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    lib.ki_tensor_core_check.argtypes = [ctypes.POINTER(ctypes.c_double)]
    lib.ki_last_error.restype = ctypes.c_char_p
    lib.ki_version.restype = ctypes.c_char_p
    for name in EXPORTED:
        getattr(lib, name)
    if path is None:
        _lib = lib
        # the autotuner's table for this GPU model, when one was recorded
        if os.path.exists(TUNE_PATH) and not os.environ.get("KI_NO_TUNE_TABLE"):
            with open(TUNE_PATH) as fh:
                table = json.load(fh)["table"]
            _check_lib(lib, lib.ki_tune_set(json.dumps(table).encode()))
    return lib


def _check(rc):
    if rc != KI_OK:
        raise KiError(rc, load_library().ki_last_error().decode())


def _check_lib(lib, rc):
    if rc != KI_OK:
        raise KiError(rc, lib.ki_last_error().decode())


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _make_desc(params, points, normals, weights, curvatures, hole_centers, hole_start,
               hole_count):
    """(ki_problem_desc, arrays it points to) for a boundary; params =
    (dim, solution_dimension, pde, max_leaf_dofs, num_proxy_points,
    radius_ratio, min_dofs_to_compress, id_tol, precision, rank model)."""
    dim, sd, pde, mld, npx, rr, mdc, tol, prec, rm = params
    # normals / weights may be None for the Gaussian kernel (read as zeros)
    keep = [np.ascontiguousarray(points, np.float64).reshape(-1),
            None if normals is None else np.ascontiguousarray(normals, np.float64).reshape(-1),
            None if weights is None else np.ascontiguousarray(weights, np.float64).reshape(-1)]
    keep.append(None if curvatures is None else
                np.ascontiguousarray(curvatures, np.float64).reshape(-1))
    nh = 0 if hole_centers is None else int(np.asarray(hole_centers).shape[0])
    hc = np.ascontiguousarray(hole_centers, np.float64).reshape(-1) if nh else None
    hs = np.ascontiguousarray(hole_start, np.int32) if nh else None
    hn = np.ascontiguousarray(hole_count, np.int32) if nh else None
    keep += [hc, hs, hn, rm]
    n = keep[0].shape[0] // dim
    return (_Desc(n, dim, sd, pde, _ptr(keep[0]), _ptr(keep[1]), _ptr(keep[2]), _ptr(keep[3]),
                  nh, _ptr(hc), _ptr(hs), _ptr(hn), mld, npx, rr, mdc, tol, prec, _ptr(rm)),
            keep)


def tune_set(table):
    """Replace the library's autotuning table ({"id:17": 2, ...}; {} restores
    the built-in heuristics)."""
    _check(load_library().ki_tune_set(json.dumps(table).encode()))


def tune_get():
    buf = ctypes.create_string_buffer(1 << 16)
    _check(load_library().ki_tune_get(buf, len(buf)))
    return json.loads(buf.value.decode())


def autotune(points, normals, weights, curvatures=None, nrhs=16, repeats=2, id_tol=1e-10,
             solution_dimension=1, pde=PDE_LAPLACE, hole_centers=None, hole_start=None,
             hole_count=None, max_leaf_dofs=64, num_proxy_points=0, radius_ratio=2.0,
             min_dofs_to_compress=64, precision=PRECISION_FP64, rank_model=None):
    """ki_autotune on this boundary (the Factor constructor's arguments):
    returns {"table": ..., "ms": ...}; the library keeps the table."""
    lib = load_library()
    dim = int(np.asarray(points).shape[-1])
    if isinstance(rank_model, str) and rank_model == "default":
        rank_model = load_rank_model()
    rm = None if rank_model is None else np.ascontiguousarray(rank_model, np.float32)
    params = (dim, solution_dimension, pde, max_leaf_dofs, num_proxy_points, radius_ratio,
              min_dofs_to_compress, id_tol, precision, rm)
    d, keep = _make_desc(params, points, normals, weights, curvatures, hole_centers, hole_start,
                         hole_count)
    buf = ctypes.create_string_buffer(1 << 18)
    _check(lib.ki_autotune(ctypes.byref(d), nrhs, repeats, buf, len(buf)))
    del keep
    return json.loads(buf.value.decode())


class Factor:
    """One factorization on the GPU (owns a ki_factor handle)."""

    def __init__(self, points, normals, weights, curvatures=None, id_tol=1e-10,
                 solution_dimension=1, pde=PDE_LAPLACE, hole_centers=None, hole_start=None,
                 hole_count=None, max_leaf_dofs=64, num_proxy_points=0, radius_ratio=2.0,
                 min_dofs_to_compress=64, precision=PRECISION_FP64, domain_dimension=None,
                 rank_model=None):
        """points/normals: (n, dim) arrays, dim 2 or 3 (inferred unless given).
        num_proxy_points 0 takes the reference default (128 on a circle in 2D,
        the 8 x 4 theta x phi sphere = 32 in 3D).  rank_model: a learned rank
        predictor blob (float32 array; "default" loads rank_model.npy) that
        FP32 factorizations use to size sketched IDs."""
        lib = load_library()
        dim = int(domain_dimension or np.asarray(points).shape[-1])
        if dim not in (2, 3):
            raise ValueError("points must be (n, 2) or (n, 3)")
        if isinstance(rank_model, str) and rank_model == "default":
            rank_model = load_rank_model()
        rm = None if rank_model is None else np.ascontiguousarray(rank_model, np.float32)
        self._params = (dim, solution_dimension, pde, max_leaf_dofs, num_proxy_points,
                        radius_ratio, min_dofs_to_compress, id_tol, precision, rm)
        d = self._desc(points, normals, weights, curvatures, hole_centers, hole_start, hole_count)
        h = ctypes.c_void_p()
        _check(lib.ki_factor_create(ctypes.byref(d), ctypes.byref(h)))
        self._h = h
        self._set_sizes()

    def _desc(self, points, normals, weights, curvatures, hole_centers, hole_start, hole_count):
        """The ki_problem_desc of a boundary with this factor's parameters (the
        arrays it points to are kept in self._keep)."""
        d, self._keep = _make_desc(self._params, points, normals, weights, curvatures,
                                   hole_centers, hole_start, hole_count)
        self._n_holes = d.n_holes
        return d

    def _set_sizes(self):
        dim, sd = self._params[0], self._params[1]
        n = self._keep[0].shape[0] // dim
        self.n_dofs = n * sd
        self.n_points = n
        self.solution_dimension = sd
        self.domain_dimension = dim
        # the library's count: the Neumann and Gaussian kernels have no border
        self.n_border = self.info()["n_border"]

    def update(self, points, normals, weights, curvatures=None, hole_centers=None, hole_start=None,
               hole_count=None):
        """Re-factorize for a perturbed boundary (ki_factor_update: the
        reference's QuadTree::perturb then skeletonize), keeping the factors of
        the boxes the perturbation left unchanged; the parameters are the
        constructor's.  Returns info()["n_reused"], the boxes kept."""
        d = self._desc(points, normals, weights, curvatures, hole_centers, hole_start, hole_count)
        _check(load_library().ki_factor_update(self._h, ctypes.byref(d)))
        self._set_sizes()
        return self.info()["n_reused"]

    def close(self):
        if getattr(self, "_h", None):
            load_library().ki_factor_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        i = _Info()
        _check(load_library().ki_factor_get_info(self._h, ctypes.byref(i)))
        return {f: getattr(i, f) for f, _ in _Info._fields_}

    def box_log(self):
        """(rows, 15) float32: per ID box the 12 predictor features, n, k, level."""
        lib = load_library()
        rows = ctypes.c_int()
        _check(lib.ki_factor_get_box_log(self._h, None, 0, ctypes.byref(rows)))
        out = np.zeros((rows.value, BOX_LOG_COLUMNS), np.float32)
        if rows.value:
            _check(lib.ki_factor_get_box_log(self._h, _ptr(out), rows.value, ctypes.byref(rows)))
        return out

    def profile(self):
        """Per-stage device times and algorithmic counts (dict)."""
        import json
        buf = ctypes.create_string_buffer(1 << 16)
        _check(load_library().ki_factor_get_profile(self._h, buf, len(buf)))
        return json.loads(buf.value.decode())

    def set_profiling(self, on=True):
        _check(load_library().ki_factor_set_profiling(self._h, 1 if on else 0))

    def solve(self, b):
        """x (and alpha for holes) with b: (n_dofs,) or (n_dofs, nrhs)."""
        b = np.asarray(b, np.float64)
        vec = b.ndim == 1
        B = np.asfortranarray(b.reshape(self.n_dofs, -1))
        nrhs = B.shape[1]
        X = np.zeros_like(B, order="F")
        A = np.zeros((max(1, self.n_border), nrhs), order="F")
        _check(load_library().ki_solve(self._h, _ptr(B), self.n_dofs, nrhs, _ptr(X), self.n_dofs,
                                       _ptr(A), max(1, self.n_border)))
        x = X[:, 0] if vec else X
        if self.n_border:
            return x, (A[:, 0] if vec else A)
        return x

    def solve_refined(self, b, tol=1e-8, max_steps=10):
        """Iterative refinement against the FP64 operator (ki_solve_refined):
        returns (x[, alpha], info dict with steps, residual0, residual)."""
        b = np.asarray(b, np.float64)
        vec = b.ndim == 1
        B = np.asfortranarray(b.reshape(self.n_dofs, -1))
        nrhs = B.shape[1]
        X = np.zeros_like(B, order="F")
        A = np.zeros((max(1, self.n_border), nrhs), order="F")
        info = _RefineInfo()
        _check(load_library().ki_solve_refined(self._h, _ptr(B), self.n_dofs, nrhs, _ptr(X),
                                               self.n_dofs, _ptr(A), max(1, self.n_border),
                                               tol, max_steps, ctypes.byref(info)))
        res = dict(steps=info.steps, residual0=info.residual0, residual=info.residual,
                   updates=info.updates, drift_bound=info.drift_bound)
        x = X[:, 0] if vec else X
        if self.n_border:
            return x, (A[:, 0] if vec else A), res
        return x, res

    def solve_refined_device(self, d_b, d_x, nrhs, d_alpha=0, tol=1e-8, max_steps=10, stream=0):
        """Device-pointer refined solve (column-major, ld = n_dofs / n_border)."""
        info = _RefineInfo()
        _check(load_library().ki_solve_refined_device(
            self._h, ctypes.c_void_p(d_b), nrhs, ctypes.c_void_p(d_x),
            ctypes.c_void_p(d_alpha) if d_alpha else None, tol, max_steps, ctypes.byref(info),
            ctypes.c_void_p(stream) if stream else None))
        return dict(steps=info.steps, residual0=info.residual0, residual=info.residual,
                   updates=info.updates, drift_bound=info.drift_bound)

    def solve_device(self, d_b, d_x, nrhs, d_alpha=0, stream=0):
        """Device-pointer solve (integers: cudaMalloc'd addresses, column-major)."""
        _check(load_library().ki_solve_device(self._h, ctypes.c_void_p(d_b), self.n_dofs, nrhs,
                                              ctypes.c_void_p(d_x), self.n_dofs,
                                              ctypes.c_void_p(d_alpha) if d_alpha else None,
                                              max(1, self.n_border),
                                              ctypes.c_void_p(stream) if stream else None))

    def apply(self, x, alpha=None):
        """Dense FP64 operator y = K x (+ U alpha) on the GPU."""
        x = np.asarray(x, np.float64)
        vec = x.ndim == 1
        X = np.asfortranarray(x.reshape(self.n_dofs, -1))
        Y = np.zeros_like(X, order="F")
        A = None
        if alpha is not None:
            A = np.asfortranarray(np.asarray(alpha, np.float64).reshape(self.n_border, -1))
        _check(load_library().ki_apply(self._h, _ptr(X), self.n_dofs, X.shape[1], _ptr(A),
                                       max(1, self.n_border), _ptr(Y), self.n_dofs))
        return Y[:, 0] if vec else Y

    def apply_fmm(self, x, alpha=None, order=0, fp32=False):
        """K x (+ U alpha) by the fast multipole method (2D Laplace); order:
        expansion terms (0: 24), fp32: FP32 expansion arithmetic."""
        x = np.asarray(x, np.float64)
        vec = x.ndim == 1
        X = np.asfortranarray(x.reshape(self.n_dofs, -1))
        Y = np.zeros_like(X, order="F")
        A = None
        if alpha is not None:
            A = np.asfortranarray(np.asarray(alpha, np.float64).reshape(self.n_border, -1))
        _check(load_library().ki_apply_fmm_ex(self._h, _ptr(X), self.n_dofs, X.shape[1], _ptr(A),
                                              max(1, self.n_border), _ptr(Y), self.n_dofs,
                                              int(order), int(bool(fp32))))
        return Y[:, 0] if vec else Y

    def apply_rows(self, rows, x, alpha=None):
        """Rows of the dense FP64 operator product K x (+ U alpha)."""
        rows = np.ascontiguousarray(rows, np.int32)
        x = np.asarray(x, np.float64)
        X = np.asfortranarray(x.reshape(self.n_dofs, -1))
        Y = np.zeros((rows.size, X.shape[1]), order="F")
        A = None
        if alpha is not None:
            A = np.asfortranarray(np.asarray(alpha, np.float64).reshape(self.n_border, -1))
        _check(load_library().ki_apply_rows(self._h, _ptr(rows), rows.size, _ptr(X), self.n_dofs,
                                            X.shape[1], _ptr(A), max(1, self.n_border), _ptr(Y),
                                            max(1, rows.size)))
        return Y

    def eval_targets(self, targets, mu, alpha=None):
        targets = np.ascontiguousarray(targets, np.float64).reshape(-1, self.domain_dimension)
        mu = np.asarray(mu, np.float64)
        vec = mu.ndim == 1
        M = np.asfortranarray(mu.reshape(self.n_dofs, -1))
        nt = targets.shape[0] * self.solution_dimension
        out = np.zeros((nt, M.shape[1]), order="F")
        A = None
        if alpha is not None:
            A = np.asfortranarray(np.asarray(alpha, np.float64).reshape(self.n_border, -1))
        _check(load_library().ki_eval_targets(self._h, _ptr(targets), targets.shape[0], _ptr(M),
                                              self.n_dofs, M.shape[1], _ptr(A),
                                              max(1, self.n_border), _ptr(out), nt))
        return out[:, 0] if vec else out


def rank_model_floats():
    return int(load_library().ki_rank_model_floats())


def load_rank_model(path=None):
    """The trained rank-predictor blob shipped with the package (or the one
    at `path`, or at $KI_RANK_MODEL)."""
    return np.load(path or os.environ.get("KI_RANK_MODEL") or RANK_MODEL_PATH).astype(np.float32)


def rank_model_train(features, ratios, epochs=2000, lr=3e-3, seed=0):
    """Train the rank MLP on the GPU; returns (model blob, final MSE)."""
    X = np.ascontiguousarray(features, np.float32)
    y = np.ascontiguousarray(ratios, np.float32)
    m = np.zeros(rank_model_floats(), np.float32)
    loss = ctypes.c_float()
    _check(load_library().ki_rank_model_train(_ptr(X), _ptr(y), X.shape[0], epochs, lr, seed,
                                              _ptr(m), ctypes.byref(loss)))
    return m, float(loss.value)


def rank_model_predict(model, features, bf16=False):
    """Predicted rank fractions: FP32 on the CUDA cores, or (bf16) BF16 on the
    tensor cores as the FP32 factorizations infer them."""
    X = np.ascontiguousarray(features, np.float32)
    out = np.zeros(X.shape[0], np.float32)
    lib = load_library()
    fn = lib.ki_rank_model_predict_bf16 if bf16 else lib.ki_rank_model_predict
    _check(fn(_ptr(np.ascontiguousarray(model, np.float32)), _ptr(X), X.shape[0], _ptr(out)))
    return out


def rank_model_grad(model, features, ratios):
    """(loss, gradient) of the mean squared error, from the GPU kernels."""
    X = np.ascontiguousarray(features, np.float32)
    y = np.ascontiguousarray(ratios, np.float32)
    g = np.zeros(rank_model_floats(), np.float32)
    loss = ctypes.c_float()
    _check(load_library().ki_rank_model_grad(_ptr(np.ascontiguousarray(model, np.float32)), _ptr(X),
                                             _ptr(y), X.shape[0], _ptr(g), ctypes.byref(loss)))
    return float(loss.value), g


def tensor_core_check():
    """Largest relative difference of the tensor-core sketch machinery
    (tcgen05 TF32 MMAs into TMEM) from the same product in FP64, on fixed
    data on the current GPU (ki_tensor_core_check)."""
    e = ctypes.c_double()
    _check(load_library().ki_tensor_core_check(ctypes.byref(e)))
    return e.value


def measure_fma_peak():
    """(FP64, FP32) CUDA-core FMA throughput of the current GPU, GFLOP/s."""
    a, b = ctypes.c_double(), ctypes.c_double()
    _check(load_library().ki_measure_fma_peak(ctypes.byref(a), ctypes.byref(b)))
    return a.value, b.value


# ----------------------------------------------------------- reference mirror

class Boundary:
    """Boundary data (kern_interp/boundaries/boundary.h:47-64).  points and
    normals are interleaved (x, y[, z]) per node; holes is a list of
    (center, node_start, node_count)."""

    def __init__(self, points, normals, weights, curvatures=None, holes=(), boundary_values=None):
        self.points = np.asarray(points, np.float64).reshape(-1)
        self.normals = np.asarray(normals, np.float64).reshape(-1)
        self.weights = np.asarray(weights, np.float64)
        self.curvatures = None if curvatures is None else np.asarray(curvatures, np.float64)
        self.holes = list(holes)
        self.boundary_values = boundary_values

    @classmethod
    def from_problem(cls, prob, boundary_values=None):
        holes = [(prob.hole_centers[h], int(prob.hole_start[h]), int(prob.hole_count[h]))
                 for h in range(prob.n_holes)]
        return cls(prob.points, prob.normals, prob.weights, prob.curvatures, holes, boundary_values)


class Kernel:
    """Kernel(solution_dimension, domain_dimension, pde, boundary, domain_points)
    (kern_interp/kernel/kernel.h:38-66)."""
    LAPLACE, LAPLACE_NEUMANN, GAUSS, STOKES = range(4)

    def __init__(self, solution_dimension, domain_dimension, pde, boundary, domain_points=()):
        self.solution_dimension = solution_dimension
        self.domain_dimension = domain_dimension
        self.pde = pde
        self.boundary = boundary
        self.domain_points = np.asarray(domain_points, np.float64).reshape(-1)


class QuadTree:
    """QuadTree::initialize_tree (kern_interp/quadtree/quadtree.h:122-123).
    The tree itself is built on the factorization path; this object carries
    the boundary, the parameters the reference fixes as macros, and (after
    skeletonize) the factorization -- the reference stores its factors in
    the tree too (quadtree.h:61-63, 118-119)."""

    def __init__(self, max_leaf_dofs=64):
        self.max_leaf_dofs = max_leaf_dofs
        self.boundary = None
        self.factor = None

    def initialize_tree(self, boundary, solution_dimension, domain_dimension):
        if domain_dimension not in (2, 3):
            raise KiError(KI_ERR_ARG, "domain_dimension must be 2 or 3")
        if self.factor is not None:
            self.factor.close()
            self.factor = None
        self.boundary = boundary
        self.solution_dimension = solution_dimension
        self.domain_dimension = domain_dimension

    def perturb(self, perturbed_boundary):
        """QuadTree::perturb (quadtree.cpp:581-890): the tree now describes
        perturbed_boundary (points identified by index), and the next
        skeletonize keeps the factors of the boxes the change left alone
        (ki_factor_update)."""
        if self.boundary is None:
            raise KiError(KI_ERR_STATE, "perturb: tree not initialized")
        self.boundary = perturbed_boundary


class SkelFactorization:
    """SkelFactorization(id_tol, fact_threads) (skel_factorization.h:27).
    fact_threads is accepted for signature parity and ignored (the GPU
    processes every box of a level in one launch)."""

    def __init__(self, id_tol, fact_threads=1, num_proxy_points=0, radius_ratio=2.0,
                 min_dofs_to_compress=64, precision=PRECISION_FP64):
        self.id_tol = id_tol
        self.fact_threads = fact_threads
        self.num_proxy_points = num_proxy_points
        self.radius_ratio = radius_ratio
        self.min_dofs_to_compress = min_dofs_to_compress
        self.precision = precision

    def skeletonize(self, kernel, quadtree):
        """Factor the tree's boundary.  A tree factorized before (and
        perturbed since) is re-factorized keeping the unchanged boxes' factors,
        as the reference's skeletonize skips boxes still compressed
        (skel_factorization.cpp:199-208); other parameters than the previous
        factorization's start afresh."""
        b = quadtree.boundary
        holes = b.holes
        hc = np.array([h[0] for h in holes]) if holes else None
        hs = np.array([h[1] for h in holes], np.int32) if holes else None
        hn = np.array([h[2] for h in holes], np.int32) if holes else None
        dim = quadtree.domain_dimension
        pts, nrm = b.points.reshape(-1, dim), b.normals.reshape(-1, dim)
        params = (dim, kernel.solution_dimension, kernel.pde, quadtree.max_leaf_dofs,
                  self.num_proxy_points, self.radius_ratio, self.min_dofs_to_compress,
                  self.id_tol, self.precision, None)
        fac = quadtree.factor
        if fac is not None and fac._params[:9] == params[:9] and fac._params[9] is None:
            fac.update(pts, nrm, b.weights, b.curvatures, hc, hs, hn)
            return
        if fac is not None:
            fac.close()
        quadtree.factor = Factor(pts, nrm, b.weights, b.curvatures, self.id_tol,
                                 kernel.solution_dimension, kernel.pde, hc, hs, hn,
                                 quadtree.max_leaf_dofs, self.num_proxy_points, self.radius_ratio,
                                 self.min_dofs_to_compress, self.precision, domain_dimension=dim)

    def solve(self, quadtree, b):
        return quadtree.factor.solve(b)

    def multiply_connected_solve(self, quadtree, b):
        return quadtree.factor.solve(b)


def linear_solve(skel_factorization, quadtree, f):
    """mu (and alpha when the boundary has holes) (linear_solve.cpp:202-227)."""
    return quadtree.factor.solve(f)


def boundary_integral_solve(kernel, boundary, quadtree, id_tol, fact_threads, domain_points,
                            **params):
    """Factor the tree (initialized with `boundary` here when it was not
    initialized before; a perturbed tree is re-factorized), solve with
    boundary.boundary_values and evaluate at the domain points
    (linear_solve.cpp:257-303; without the is_in_domain masking, which needs
    the reference's concrete Boundary classes)."""
    skel = SkelFactorization(id_tol, fact_threads, **params)
    if quadtree.boundary is None:
        quadtree.initialize_tree(boundary, kernel.solution_dimension, kernel.domain_dimension)
    skel.skeletonize(kernel, quadtree)
    res = linear_solve(skel, quadtree, boundary.boundary_values)
    targets = np.asarray(domain_points, np.float64).reshape(-1, kernel.domain_dimension)
    if isinstance(res, tuple):
        mu, alpha = res
        return quadtree.factor.eval_targets(targets, mu, alpha)
    return quadtree.factor.eval_targets(targets, res)


from . import geometry  # noqa: E402,F401
from . import replicas  # noqa: E402,F401


def launch_count():
    """Kernels the library has launched since it was loaded."""
    return int(load_library().ki_launch_count())
