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


def test_fp32_fmm_relative_error_within_its_credit(pkg):
    """The FP32 apply at 12 terms (the residual updates' operator) against
    the FP64 apply at 24 terms: per-column 2-norm relative error well below
    the 1e-5 the refinement credits it with, on random densities and on a
    refinement correction of the headline geometry family."""
    g = pkg.geometry
    prob = g.disc_with_ellipses(1 << 16, 64, seed=1)
    kw = dict(hole_centers=prob.hole_centers, hole_start=prob.hole_start,
              hole_count=prob.hole_count)
    fac = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, id_tol=1e-6,
                     precision=pkg.PRECISION_FP32, **kw)
    rng = np.random.default_rng(2)
    x = rng.standard_normal((prob.n, 33))          # two passes of 32 columns
    f = g.laplace_source_rhs(prob, g.random_sources(4, np.random.default_rng(3)))
    mu, al = fac.solve(f)
    x[:, 0] = mu[:, 0]                             # a smooth density
    y64 = fac.apply_fmm(x, order=24)
    y32 = fac.apply_fmm(x, order=12, fp32=True)
    err = np.linalg.norm(y32 - y64, axis=0) / np.linalg.norm(y64, axis=0)
    assert err.max() <= 3e-6, err.max()


def test_residual_updates_bound_the_true_residual(pkg, monkeypatch):
    """Refinement with residual updates (r -= A_low d): the FP64 residual of
    the returned solution, by the 24-term FP64 FMM, is at most the reported
    bound and within the drift bound of the updated residual."""
    g = pkg.geometry
    prob = g.star(4096, 16)                        # 65,536 unknowns, no holes
    B = g.laplace_source_rhs(prob, g.random_sources(3, np.random.default_rng(1)))
    # ID tolerance 1e-4: a first residual near 1e-4, so that reaching 1e-10
    # takes several corrections and the later ones are residual updates
    fac = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, id_tol=1e-4,
                     precision=pkg.PRECISION_FP32)
    tol = 1e-10
    mu, info = fac.solve_refined(B, tol=tol, max_steps=10)
    assert info["updates"] >= 1 and info["residual"] <= tol, info
    # the residual by the 32-term FP64 FMM (relative error ~2e-14); the
    # refinement's own FP64 products carry up to tol / 20 (their order is
    # chosen for that), which the drift bound does not include
    r = B - fac.apply_fmm(mu, order=32)
    true = (np.linalg.norm(r, axis=0) / np.linalg.norm(B, axis=0)).max()
    assert true <= info["residual"] + tol / 20, (true, info)
    raw = info["residual"] - info["drift_bound"]
    assert abs(true - raw) <= info["drift_bound"] + tol / 20, (true, info)
    # the same solve recomputing the FP64 residual after every correction
    monkeypatch.setenv("KI_REFINE_UPDATE", "0")
    mu2, info2 = fac.solve_refined(B, tol=1e-10, max_steps=10)
    assert info2["updates"] == 0 and info2["drift_bound"] == 0.0
    assert info2["steps"] == info["steps"], (info, info2)
    assert np.abs(mu2 - mu).max() <= 1e-9 * np.abs(mu).max()


def test_residual_updates_with_holes_match_recomputed_residuals(pkg, monkeypatch):
    """The bordered problem (holes): updates and FP64 recomputation give the
    same steps and solution, and the FP64 residual sits under the bound."""
    g = pkg.geometry
    prob = g.disc_with_ellipses(1 << 15, 16, seed=4)
    f = g.laplace_source_rhs(prob, g.random_sources(4, np.random.default_rng(5)))
    kw = dict(hole_centers=prob.hole_centers, hole_start=prob.hole_start,
              hole_count=prob.hole_count)
    # ID tolerance 1e-4: several corrections, the later ones residual updates
    fac = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, id_tol=1e-4,
                     precision=pkg.PRECISION_FP32, **kw)
    mu, al, info = fac.solve_refined(f, tol=1e-10, max_steps=10)
    monkeypatch.setenv("KI_REFINE_UPDATE", "0")
    mu2, al2, info2 = fac.solve_refined(f, tol=1e-10, max_steps=10)
    assert info["updates"] >= 1 and info2["updates"] == 0, (info, info2)
    assert info["steps"] == info2["steps"]
    assert info2["residual"] <= info["residual"] + 1e-10 / 20, (info, info2)
    assert np.abs(mu2 - mu).max() <= 1e-9 * np.abs(mu).max()
