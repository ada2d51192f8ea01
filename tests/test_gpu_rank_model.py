"""Learned rank predictor: the MLP's GPU gradients against a NumPy
restatement of the same network (the CPU oracle), training, the box log,
and the FP32 factorization whose IDs are sketched to the predicted rank
(with the plain ID as fallback) inside the mixed-precision solve."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

F, H = 12, 64


def unpack(m):
    o = 0
    out = {}
    for name, size in (("mean", F), ("scale", F), ("W1", H * F), ("b1", H), ("W2", H * H),
                       ("b2", H), ("W3", H), ("b3", 1)):
        out[name] = m[o:o + size].astype(np.float64)
        o += size
    out["W1"] = out["W1"].reshape(H, F)
    out["W2"] = out["W2"].reshape(H, H)
    return out


def numpy_loss_grad(m, X, y):
    """Mean squared error of the logistic-output MLP and its gradient, FP64."""
    p = unpack(m)
    xn = (X.astype(np.float64) - p["mean"]) / p["scale"]
    z1 = xn @ p["W1"].T + p["b1"]
    a1 = np.maximum(z1, 0)
    z2 = a1 @ p["W2"].T + p["b2"]
    a2 = np.maximum(z2, 0)
    zo = a2 @ p["W3"] + p["b3"][0]
    o = 1 / (1 + np.exp(-zo))
    n = len(y)
    loss = np.mean((o - y) ** 2)
    d = 2 * (o - y) / n * o * (1 - o)
    g = {"b3": np.array([d.sum()]), "W3": a2.T @ d}
    gz2 = np.outer(d, p["W3"]) * (z2 > 0)
    g["W2"] = gz2.T @ a1
    g["b2"] = gz2.sum(0)
    gz1 = (gz2 @ p["W2"]) * (z1 > 0)
    g["W1"] = gz1.T @ xn
    g["b1"] = gz1.sum(0)
    flat = np.concatenate([np.zeros(2 * F), g["W1"].ravel(), g["b1"], g["W2"].ravel(), g["b2"],
                           g["W3"], g["b3"]])
    return loss, flat


def test_gpu_gradient_matches_numpy_oracle(pkg):
    rng = np.random.default_rng(0)
    X = rng.standard_normal((500, F)).astype(np.float32) * 2 + 1
    y = rng.uniform(0, 1, 500).astype(np.float32)
    model, _ = pkg.rank_model_train(X, y, epochs=0, seed=3)    # initialized, untrained
    loss_gpu, g_gpu = pkg.rank_model_grad(model, X, y)
    loss_np, g_np = numpy_loss_grad(model, X, y)
    assert abs(loss_gpu - loss_np) <= 1e-5 * max(1.0, loss_np)
    scale = np.abs(g_np).max()
    assert np.abs(g_gpu - g_np).max() <= 1e-4 * scale, np.abs(g_gpu - g_np).max() / scale


def test_gpu_training_fits_a_smooth_target(pkg):
    rng = np.random.default_rng(1)
    X = rng.standard_normal((4000, F)).astype(np.float32)
    w = rng.standard_normal(F)
    y = (1 / (1 + np.exp(-(X @ w) / 2))).astype(np.float32)
    m0, l0 = pkg.rank_model_train(X, y, epochs=0)
    m1, l1 = pkg.rank_model_train(X, y, epochs=800)
    assert l1 < 0.05 * l0, (l0, l1)
    pred = pkg.rank_model_predict(m1, X)
    assert np.mean((pred - y) ** 2) == pytest.approx(l1, rel=1e-3, abs=1e-7)


def _disc(pkg, n, holes, seed):
    g = pkg.geometry
    prob = g.disc_with_ellipses(n, holes, seed=seed)
    f = g.laplace_source_rhs(prob, g.random_sources(4, np.random.default_rng(seed)))
    kw = dict(hole_centers=prob.hole_centers, hole_start=prob.hole_start,
              hole_count=prob.hole_count)
    return prob, f, kw


def test_box_log_matches_factorization(pkg):
    prob, f, kw = _disc(pkg, 1 << 14, 8, 3)
    fac = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, id_tol=1e-6,
                     precision=pkg.PRECISION_FP32, **kw)
    log = fac.box_log()
    info = fac.info()
    assert log.shape[1] == 15 and log.shape[0] > 0
    assert int((log[:, 13] > 0).sum()) == info["n_compressed"]
    assert np.isfinite(log).all()
    assert ((log[:, 13] >= 0) & (log[:, 13] < log[:, 12])).all()
    assert info["n_sketched"] == 0 and info["n_fallback"] == 0


def test_learned_rank_sketched_factorization_in_mixed_solve(pkg):
    """FP32 factorization with IDs sketched to the shipped model's predicted
    ranks, refined against the FP64 operator: same solution as the plain
    FP32 factorization refined to the same residual, most boxes sketched,
    few fallbacks."""
    prob, f, kw = _disc(pkg, 1 << 16, 32, 12)
    common = dict(id_tol=1e-6, precision=pkg.PRECISION_FP32, **kw)
    plain = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, **common)
    learned = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures,
                         rank_model="default", **common)
    info = learned.info()
    n_id = learned.box_log().shape[0]
    assert info["n_sketched"] >= 0.5 * n_id, (info, n_id)
    assert info["n_fallback"] <= 0.2 * max(1, info["n_sketched"]), info
    mu_p, al_p, rp = plain.solve_refined(f, tol=1e-10, max_steps=20)
    mu_l, al_l, rl = learned.solve_refined(f, tol=1e-10, max_steps=20)
    assert rp["residual"] <= 1e-10 and rl["residual"] <= 1e-10, (rp, rl)
    # the sketched factorization is an approximate inverse of comparable quality
    assert rl["residual0"] <= 10 * rp["residual0"] + 1e-6, (rp, rl)
    assert np.abs(mu_l - mu_p).max() <= 1e-8 * np.abs(mu_p).max()


def test_underpredicting_model_falls_back_to_the_plain_id(pkg):
    """A model that predicts near-zero ranks (output bias shifted down) makes
    nearly every sketch too small: those boxes are recompressed by the plain
    ID and the factorization is the same approximate inverse."""
    prob, f, kw = _disc(pkg, 1 << 15, 16, 5)
    bad = pkg.load_rank_model().copy()
    bad[-1] -= 30.0
    common = dict(id_tol=1e-6, precision=pkg.PRECISION_FP32, **kw)
    plain = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, **common)
    fb = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, rank_model=bad,
                    **common)
    info = fb.info()
    assert info["n_sketched"] > 0 and info["n_fallback"] >= 0.9 * info["n_sketched"], info
    # the recompression runs the plain ID in the fallback's launch shape (32-row
    # folds), the plain factorization in the tuned shapes: rounding may move a
    # near-tie pivot, and the root skeleton by a DOF or two
    assert info["n_compressed"] == plain.info()["n_compressed"]
    assert abs(info["n_root"] - plain.info()["n_root"]) <= max(2, 0.01 * plain.info()["n_root"])
    mu_p = plain.solve(f)[0]
    mu_f = fb.solve(f)[0]
    # two FP32 approximate inverses (plain solves, no refinement) whose
    # skeletons may differ by a DOF
    assert np.abs(mu_f - mu_p).max() <= 3e-4 * np.abs(mu_p).max()


def bf16(a):
    """Round FP32 values to BF16 (nearest, ties to even), returned as FP32."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def test_tensor_core_bf16_inference(pkg):
    """The factorization's inference (BF16 operands, tcgen05 MMAs into FP32
    TMEM accumulators) against a NumPy restatement with the same BF16
    roundings, and within 0.01 of the FP32 network, on a trained model and a
    ragged sample count (not a multiple of the 128 samples of a CTA).  The
    restatement agrees to 1e-3, not exactly: an FP32 sum that lands on the
    other side of a BF16 rounding boundary moves one activation by one BF16
    step."""
    rng = np.random.default_rng(5)
    X = (rng.standard_normal((1000, F)) * 1.5 + 0.5).astype(np.float32)
    y = (1 / (1 + np.exp(-X[:, 0] + 0.5 * X[:, 3]))).astype(np.float32)
    model, _ = pkg.rank_model_train(X, y, epochs=200, seed=2)
    p = {k: v.astype(np.float32) for k, v in unpack(model).items()}
    Xr = X[:777]
    xn = bf16((Xr - p["mean"]) / p["scale"]).astype(np.float64)
    z1 = xn @ bf16(p["W1"]).astype(np.float64).T + p["b1"]
    h = bf16(np.maximum(z1, 0).astype(np.float32)).astype(np.float64)
    z2 = h @ bf16(p["W2"]).astype(np.float64).T + p["b2"]
    zo = np.maximum(z2, 0) @ p["W3"] + p["b3"][0]
    emul = 1 / (1 + np.exp(-zo))
    tc = pkg.rank_model_predict(model, Xr, bf16=True)
    fp32 = pkg.rank_model_predict(model, Xr)
    assert np.abs(tc - emul).max() <= 1e-3, np.abs(tc - emul).max()
    assert np.abs(tc - fp32).max() <= 1e-2, np.abs(tc - fp32).max()
    assert pkg.rank_model_predict(model, X[:0], bf16=True).size == 0
