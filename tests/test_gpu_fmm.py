"""The FP64 fast multipole apply of the 2D Laplace Nystrom operator
(ki_apply_fmm) against the dense FP64 product (ki_apply), and refined solves
whose residuals use it."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case,ncols", [("star", 3), ("holes", 40), ("ellipses_1m_sample", 2)])
def test_fmm_matches_dense_apply(pkg, case, ncols):
    g = pkg.geometry
    kw = {}
    if case == "star":
        prob = g.star(512, 16)
    elif case == "holes":
        prob = g.disc_with_ellipses(1 << 14, 12, seed=3)
    else:
        # the headline geometry family at 65,536 unknowns
        prob = g.disc_with_ellipses(1 << 16, 64, seed=1)
    if prob.n_holes:
        kw = dict(hole_centers=prob.hole_centers, hole_start=prob.hole_start,
                  hole_count=prob.hole_count)
    fac = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, id_tol=1e-6,
                     precision=pkg.PRECISION_FP32, **kw)
    rng = np.random.default_rng(0)
    x = rng.standard_normal((prob.n, ncols))
    al = rng.standard_normal((prob.n_holes, ncols)) if prob.n_holes else None
    yd = fac.apply(x, al)
    yf = fac.apply_fmm(x, al)
    err = np.abs(yf - yd).max() / np.abs(yd).max()
    # 24-term expansions: a few 1e-11 (the residuals of a 1e-8 target need 1e-10)
    assert err <= 1e-10, err


def test_refined_solve_fmm_equals_dense_residual(pkg, monkeypatch):
    g = pkg.geometry
    prob = g.disc_with_ellipses(1 << 13, 6, seed=5)
    f = g.laplace_source_rhs(prob, g.random_sources(4, np.random.default_rng(7)))
    kw = dict(hole_centers=prob.hole_centers, hole_start=prob.hole_start,
              hole_count=prob.hole_count)
    out = {}
    for mode in ("dense", "fmm"):
        monkeypatch.setenv("KI_RESIDUAL_APPLY", mode)
        fac = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, id_tol=1e-6,
                         precision=pkg.PRECISION_FP32, **kw)
        # the FMM's ~3e-11 relative error floors the residual it can certify
        out[mode] = fac.solve_refined(f, tol=1e-10, max_steps=20)
        assert out[mode][2]["residual"] <= 1e-10, out[mode][2]
    mu_d, mu_f = out["dense"][0], out["fmm"][0]
    assert np.abs(mu_d - mu_f).max() <= 1e-9 * np.abs(mu_d).max()


def test_fmm_rejects_other_kernels(pkg):
    g = pkg.geometry
    prob = g.ellipsoid(512)
    fac = pkg.Factor(prob.points, prob.normals, prob.weights, None, id_tol=1e-6)
    with pytest.raises(pkg.KiError) as e:
        fac.apply_fmm(np.ones(prob.n))
    assert e.value.code == pkg.KI_ERR_STATE
