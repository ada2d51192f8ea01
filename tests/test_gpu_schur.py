"""The FP32 Schur elimination of boxes with up to 128 redundant DOFs runs as
three launches: k_schur up to X = K_rr - T^T K_sr - K~_rs T, the register
Gauss-Jordan inverse k_gj, and k_schur's products with the inverse.  Against
the single kernel (KI_SCHUR_SPLIT=0, whose shared-memory Gauss-Jordan swaps
rows where k_gj records them, so the two round differently): the same tree
and accuracy of the same order, with the same number of refinement steps."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,holes", [(1 << 15, 8), (1 << 18, 64)])
def test_split_schur_matches_single_kernel(pkg, monkeypatch, n, holes):
    g = pkg.geometry
    prob = g.disc_with_ellipses(n, holes, seed=1)
    rng = np.random.default_rng(2)
    f = g.laplace_source_rhs(prob, g.random_sources(4, rng))
    kw = dict(id_tol=1e-6, precision=pkg.PRECISION_FP32, rank_model="default",
              hole_centers=prob.hole_centers, hole_start=prob.hole_start,
              hole_count=prob.hole_count)
    geo = (prob.points, prob.normals, prob.weights, prob.curvatures)
    out = {}
    for mode in ("1", "0"):
        monkeypatch.setenv("KI_SCHUR_SPLIT", mode)
        fac = pkg.Factor(*geo, **kw)
        mu, _ = fac.solve(f)
        _, _, rinfo = fac.solve_refined(f, tol=1e-8, max_steps=6)
        out[mode] = (fac.info(), mu, rinfo)
        fac.close()
    (i1, mu1, r1), (i0, mu0, r0) = out["1"], out["0"]
    assert i1["n_redundant"] == i0["n_redundant"] and i1["n_root"] == i0["n_root"]
    # plain FP32 solutions agree to the factorization's own accuracy (first
    # residuals ~1e-5 at ID tolerance 1e-6)
    assert (np.abs(mu1 - mu0).max(0) / np.abs(mu0).max(0)).max() <= 1e-3
    assert r1["residual0"] <= 5e-5 and r1["residual0"] <= 2 * r0["residual0"]
    assert r1["steps"] == r0["steps"] and r1["residual"] <= 1e-8
