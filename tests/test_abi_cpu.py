"""C-ABI library checks that need no GPU: it loads, exports every symbol
include/ki_gpu.h declares, and rejects bad arguments before touching CUDA."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "ki_gpu.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(ki_\w+)\s*\(", text, re.M)))


def test_header_declares_expected_entry_points():
    syms = declared_symbols()
    for s in ["ki_factor_create", "ki_factor_destroy", "ki_solve", "ki_solve_device",
              "ki_apply", "ki_eval_targets", "ki_last_error"]:
        assert s in syms


def test_library_exports_every_declared_symbol(lib):
    for s in declared_symbols():
        assert hasattr(lib, s), s


def test_version(lib):
    assert b"sm_103a" in lib.ki_version()


def _desc(pkg, prob, **kw):
    keep = [np.ascontiguousarray(prob.points).reshape(-1), np.ascontiguousarray(prob.normals).reshape(-1),
            np.ascontiguousarray(prob.weights), np.ascontiguousarray(prob.curvatures)]
    ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    args = dict(n_points=prob.n, domain_dimension=2, solution_dimension=1, pde=0,
                points=ptr(keep[0]), normals=ptr(keep[1]), weights=ptr(keep[2]),
                curvatures=ptr(keep[3]), n_holes=0, hole_centers=None, hole_node_start=None,
                hole_node_count=None, max_leaf_dofs=0, num_proxy_points=0, radius_ratio=0.0,
                min_dofs_to_compress=0, id_tol=1e-10, precision=0)
    args.update(kw)
    return pkg._Desc(**args), keep


@pytest.mark.parametrize("bad", [dict(domain_dimension=4), dict(domain_dimension=1),
                                 dict(domain_dimension=3, num_proxy_points=30),
                                 dict(domain_dimension=3, pde=3, solution_dimension=2),
                                 dict(n_points=0), dict(id_tol=0.0),
                                 dict(id_tol=float("nan")), dict(pde=5), dict(precision=7),
                                 dict(pde=1, solution_dimension=2),
                                 dict(pde=2, domain_dimension=3, num_proxy_points=32),
                                 dict(pde=1, normals=None), dict(pde=0, weights=None),
                                 dict(solution_dimension=2), dict(max_leaf_dofs=-1),
                                 dict(n_holes=1)])
def test_bad_arguments_rejected(pkg, lib, bad):
    prob = pkg.geometry.star(8, 16)
    d, keep = _desc(pkg, prob, **bad)
    h = ctypes.c_void_p()
    rc = lib.ki_factor_create(ctypes.byref(d), ctypes.byref(h))
    assert rc == pkg.KI_ERR_ARG
    assert lib.ki_last_error()
    assert not h.value


@pytest.mark.parametrize("pde", [1, 2])
def test_neumann_and_gauss_pass_validation(pkg, lib, have_gpu, pde):
    """The Neumann and Gaussian kernels (2D, scalar) pass argument checks;
    the Gaussian kernel reads neither normals nor weights, so NULL is
    accepted for both (the reference reads its empty arrays as zeros)."""
    if have_gpu:
        pytest.skip("a GPU would factorize; this checks validation only")
    prob = pkg.geometry.star(8, 16)
    kw = dict(pde=pde)
    if pde == 2:
        kw.update(normals=None, weights=None)
    d, keep = _desc(pkg, prob, **kw)
    h = ctypes.c_void_p()
    rc = lib.ki_factor_create(ctypes.byref(d), ctypes.byref(h))
    assert rc != pkg.KI_ERR_ARG, lib.ki_last_error()
    assert b"CUDA" in lib.ki_last_error()


def test_non_finite_input_rejected(pkg, lib):
    prob = pkg.geometry.star(8, 16)
    prob.points[5, 0] = np.nan
    d, keep = _desc(pkg, prob)
    h = ctypes.c_void_p()
    assert lib.ki_factor_create(ctypes.byref(d), ctypes.byref(h)) == pkg.KI_ERR_ARG
    assert b"non-finite" in lib.ki_last_error()


def test_hole_range_checked(pkg, lib):
    prob = pkg.geometry.star(8, 16)
    hc = np.zeros(2)
    hs = np.array([100], np.int32)
    hn = np.array([100], np.int32)
    ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    d, keep = _desc(pkg, prob, n_holes=1, hole_centers=ptr(hc), hole_node_start=ptr(hs),
                    hole_node_count=ptr(hn))
    h = ctypes.c_void_p()
    assert lib.ki_factor_create(ctypes.byref(d), ctypes.byref(h)) == pkg.KI_ERR_ARG


def test_null_handles(pkg, lib):
    assert lib.ki_solve(None, None, 1, 1, None, 1, None, 1) == pkg.KI_ERR_ARG
    assert lib.ki_factor_get_info(None, None) == pkg.KI_ERR_ARG
    assert lib.ki_factor_destroy(None) == pkg.KI_OK


def test_no_gpu_reports_cuda_error(pkg, lib, have_gpu):
    if have_gpu:
        pytest.skip("a GPU is present")
    prob = pkg.geometry.star(8, 16)
    d, keep = _desc(pkg, prob)
    h = ctypes.c_void_p()
    assert lib.ki_factor_create(ctypes.byref(d), ctypes.byref(h)) == pkg.KI_ERR_CUDA


def test_tune_table_round_trip_and_rejects(pkg, lib):
    """The autotuner's table (ki_tune_set / ki_tune_get) needs no GPU: a table
    set comes back as set, {} clears it, malformed or out-of-range input is
    rejected with KI_ERR_ARG and leaves the table as it was."""
    saved = pkg.tune_get()
    try:
        table = {"id:17": 3, "schur:42": 5, "sweep:3": 0, "id:300": 1}
        pkg.tune_set(table)
        assert pkg.tune_get() == table
        for bad in ['{"id:17": 4}', '{"nope:1": 0}', '{"id:999": 0}', '{"id:1" 0}', '[1]',
                    '{"schur:3": 1,}', '{"sweep:1": 0} x']:
            rc = lib.ki_tune_set(bad.encode())
            assert rc == pkg.KI_ERR_ARG, bad
            assert pkg.tune_get() == table, bad
        pkg.tune_set({})
        assert pkg.tune_get() == {}
    finally:
        pkg.tune_set(saved)
