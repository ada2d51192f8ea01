"""The tree built on the GPU (descent codes, their sort, boxes level by
level, neighbour lists, leaf DOF lists) against the host partition build
(KI_TREE_BUILD=host): the same boxes, numbering and lists give the same
factorization, so the solutions agree bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _solve(pkg, monkeypatch, mode, prob, f, **kw):
    if mode == "host":
        monkeypatch.setenv("KI_TREE_BUILD", "host")
    else:
        monkeypatch.delenv("KI_TREE_BUILD", raising=False)
    fac = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, **kw)
    out = fac.solve(f)
    info = fac.info()
    info["on_gpu"] = fac.profile()["host"]["tree_built_on_gpu"]
    fac.close()
    return out, info


@pytest.mark.parametrize("case", ["laplace_holes", "stokes", "laplace3d", "leaf33",
                                  "laplace_holes_262k", "laplace3d_65k"])
def test_gpu_tree_matches_host_tree(pkg, monkeypatch, case):
    g = pkg.geometry
    kw = dict(id_tol=1e-8)
    if case == "laplace_holes_262k":
        prob = g.disc_with_ellipses(1 << 18, 64, seed=1)
        f = g.laplace_source_rhs(prob, g.random_sources(2, np.random.default_rng(1)))
        kw.update(precision=pkg.PRECISION_FP32, id_tol=1e-6)
    elif case == "laplace3d_65k":
        prob = g.ellipsoid(1 << 16, (1.0, 0.7, 0.5))
        f = np.random.default_rng(6).standard_normal((prob.n, 1))
        kw.update(max_leaf_dofs=128, id_tol=1e-4, precision=pkg.PRECISION_FP32)
    elif case == "laplace_holes":
        prob = g.disc_with_ellipses(1 << 15, 12, seed=3)
        f = g.laplace_source_rhs(prob, g.random_sources(2, np.random.default_rng(1)))
    elif case == "leaf33":
        prob = g.star(1024, 16)
        f = g.laplace_source_rhs(prob, g.random_sources(2, np.random.default_rng(1)))
        kw.update(max_leaf_dofs=33)
    elif case == "stokes":
        prob = g.disc_with_circles(1 << 13, 10, seed=2)
        f = np.random.default_rng(4).standard_normal((2 * prob.n, 2))
        kw.update(solution_dimension=2, pde=pkg.PDE_STOKES)
    else:
        prob = g.ellipsoid(4096, (1.0, 0.7, 0.5))
        f = np.random.default_rng(5).standard_normal((prob.n, 2))
        kw.update(max_leaf_dofs=128, id_tol=1e-6)
    if prob.n_holes:
        kw.update(hole_centers=prob.hole_centers, hole_start=prob.hole_start,
                  hole_count=prob.hole_count)
    a, ia = _solve(pkg, monkeypatch, "gpu", prob, f, **kw)
    b, ib = _solve(pkg, monkeypatch, "host", prob, f, **kw)
    assert ia["on_gpu"] == 1 and ib["on_gpu"] == 0
    for k in ("n_levels", "n_compressed", "n_redundant", "n_root"):
        assert ia[k] == ib[k], (k, ia, ib)
    a = a if isinstance(a, tuple) else (a,)
    b = b if isinstance(b, tuple) else (b,)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
