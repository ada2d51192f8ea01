"""The tree built from GPU-sorted descent codes against the host partition
build (KI_TREE_BUILD=host): the same boxes give the same factorization, so
the solutions agree bit for bit."""
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
    fac.close()
    return out, info


@pytest.mark.parametrize("case", ["laplace_holes", "stokes", "laplace3d", "leaf33"])
def test_gpu_tree_matches_host_tree(pkg, monkeypatch, case):
    g = pkg.geometry
    kw = dict(id_tol=1e-8)
    if case == "laplace_holes":
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
    for k in ("n_levels", "n_compressed", "n_redundant", "n_root"):
        assert ia[k] == ib[k], (k, ia, ib)
    a = a if isinstance(a, tuple) else (a,)
    b = b if isinstance(b, tuple) else (b,)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
