"""The tensor-core ID sketch (tcgen05 TF32 MMAs, TMEM accumulators) of the
FP32 factorization: a self-check of the machinery on fixed data, and the
factor-and-solve with the sketches on the tensor cores (KI_TC_SKETCH=1)
against the same sketches folded on the CUDA cores (the default)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_tensor_core_selfcheck(pkg):
    # entries split hi + lo in TF32 (2^-22 relative each), exact +-1 signs,
    # FP32 accumulation over 64 rows in TMEM
    assert pkg.tensor_core_check() <= 5e-6


def _disc(pkg, n, holes, nrhs, seed=1):
    g = pkg.geometry
    prob = g.disc_with_ellipses(n, holes, seed=seed)
    rng = np.random.default_rng(2)
    f = g.laplace_source_rhs(prob, g.random_sources(nrhs, rng))
    kw = dict(id_tol=1e-6, precision=pkg.PRECISION_FP32, rank_model="default",
              hole_centers=prob.hole_centers, hole_start=prob.hole_start,
              hole_count=prob.hole_count)
    return prob, f, kw


@pytest.mark.parametrize("n,holes", [(1 << 16, 16), (1 << 18, 64)])
def test_tc_sketch_matches_cuda_core_fold(pkg, monkeypatch, n, holes):
    """Same boxes, same signs, ranks equal up to boxes whose rank sits on
    the tolerance; both forms refine to a 1e-8 residual in the same number
    of corrections, and refined further (1e-11) both reach the same
    solution."""
    prob, f, kw = _disc(pkg, n, holes, 8)
    geo = (prob.points, prob.normals, prob.weights, prob.curvatures)
    out = {}
    for mode in ("1", "0"):
        monkeypatch.setenv("KI_TC_SKETCH", mode)
        fac = pkg.Factor(*geo, **kw)
        info = fac.info()
        lv = fac.profile()["levels"]
        _, _, rinfo = fac.solve_refined(f, tol=1e-8, max_steps=6)
        mu, al, _ = fac.solve_refined(f, tol=1e-11, max_steps=8)
        fac.close()
        out[mode] = (info, lv, mu, al, rinfo)
    (i1, lv1, mu1, al1, r1), (i0, lv0, mu0, al0, r0) = out["1"], out["0"]
    # the tensor-core path ran (path 4) only when asked for
    assert sum(q["paths"][4] for q in lv1) > 0
    assert sum(q["paths"][4] for q in lv0) == 0
    assert i1["n_fallback"] <= max(2, i0["n_fallback"] + 2)
    assert abs(i1["n_redundant"] - i0["n_redundant"]) <= 1e-3 * i0["n_redundant"]
    assert r1["residual"] <= 1e-8 and r0["residual"] <= 1e-8
    assert r1["steps"] == r0["steps"]
    scale = np.abs(mu0).max(0)
    assert (np.abs(mu1 - mu0).max(0) / scale).max() <= 1e-8
