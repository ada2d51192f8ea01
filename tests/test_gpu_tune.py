"""The autotuner (ki_autotune): it times every candidate launch shape per
box-size bucket and keeps the fastest, and every candidate is a correct
factorization -- forcing any one of them on all buckets it saw gives the
same solution as the built-in heuristics: to 10 x the ID tolerance in FP64,
and, in FP32, after refinement against the FP64 operator."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CANDIDATES = {"id": 4, "schur": 6, "sweep": 3}


def _case(pkg, precision):
    g = pkg.geometry
    prob = g.disc_with_ellipses(1 << 15, 12, seed=3)
    rhs = g.laplace_source_rhs(prob, g.random_sources(3, np.random.default_rng(1)))
    kw = dict(hole_centers=prob.hole_centers, hole_start=prob.hole_start,
              hole_count=prob.hole_count, precision=precision)
    kw["id_tol"] = 1e-6 if precision == pkg.PRECISION_FP32 else 1e-10
    return prob, rhs, kw


def _solve(pkg, prob, rhs, kw):
    """FP64: the plain solve.  FP32: refined against the FP64 operator to
    1e-11, so that every correct factorization gives the same answer (two
    FP32 factorizations that differ only in rounding differ by about their
    own error, 1e-5 here, in a plain solve)."""
    fac = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, **kw)
    if kw["precision"] == pkg.PRECISION_FP32:
        mu, alpha, info = fac.solve_refined(rhs, tol=1e-11, max_steps=20)
        assert info["residual"] <= 1e-11
    else:
        mu, alpha = fac.solve(rhs)
    fac.close()
    return np.concatenate([mu.reshape(-1), alpha.reshape(-1)])


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_autotune_table_and_every_candidate_solves(pkg, prec):
    precision = pkg.PRECISION_FP32 if prec == "fp32" else pkg.PRECISION_FP64
    prob, rhs, kw = _case(pkg, precision)
    saved = pkg.tune_get()
    try:
        pkg.tune_set({})
        ref = _solve(pkg, prob, rhs, kw)
        res = pkg.autotune(prob.points, prob.normals, prob.weights, prob.curvatures, nrhs=8,
                           repeats=1, **kw)
        table, ms = res["table"], res["ms"]
        # every timed bucket got its fastest candidate
        assert ms and set(table) == set(ms)
        for key, times in ms.items():
            valid = [t for t in times if t >= 0]
            assert valid and times[table[key]] == min(valid), (key, times)
        buckets = {k: [b for b in ms if b.startswith(k + ":")] for k in CANDIDATES}
        assert buckets["id"] and buckets["schur"] and buckets["sweep"]
        # the tuned table, then each candidate of each knob forced on all its buckets
        tol = 1e-8 if precision == pkg.PRECISION_FP32 else 10 * kw["id_tol"]
        x = _solve(pkg, prob, rhs, kw)
        assert np.linalg.norm(x - ref) <= tol * np.linalg.norm(ref)
        for knob, n in CANDIDATES.items():
            if precision == pkg.PRECISION_FP64 and knob != "sweep":
                n = 2
            for c in range(n):
                pkg.tune_set({b: c for b in buckets[knob]})
                x = _solve(pkg, prob, rhs, kw)
                assert np.linalg.norm(x - ref) <= tol * np.linalg.norm(ref), (knob, c)
    finally:
        pkg.tune_set(saved)
