"""Train the learned skeleton-rank predictor shipped as rank_model.npy.

Corpus: the box logs (features, n, rank) of plain FP32 factorizations --
no model, so every rank comes from the column-pivoted-QR ID -- of seeded
random boundaries: star curves r(theta) = 1 + sum_{k=2..8} a_k cos(k theta +
phi_k) with a_k ~ U(0, 0.3/k), phi_k ~ U(0, 2 pi) (seed 4), discs with
elliptical holes, Stokes discs with circular holes and ellipsoids with
random semi-axes in U(0.4, 1), each at several ID tolerances.  The target is
the rank fraction k / n (1 for a box the ID leaves uncompressed).  Training
runs on the GPU through the library's own forward/backward/Adam kernels
(ki_rank_model_train).  A held-out set (the disc with 64 ellipses of the
benchmark at 262,144 unknowns) reports the error and how often a sketch of
the predicted size would have been too small.

    python kern-interp-dev_gb300/train_rank_model.py [--stars 48] [--out PATH]
"""
import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def random_star(rng, nodes, q=16):
    """r(theta) = 1 + sum_{k=2..8} a_k cos(k theta + phi_k)."""
    import __graft_entry__ as g
    geo = g.load_package().geometry
    ks = np.arange(2, 9)
    a = rng.uniform(0, 0.3 / ks)
    ph = rng.uniform(0, 2 * np.pi, ks.size)

    def fun(t):
        t = np.asarray(t)
        r = 1 + (a[:, None] * np.cos(ks[:, None] * t[None] + ph[:, None])).sum(0)
        dr = (-a[:, None] * ks[:, None] * np.sin(ks[:, None] * t[None] + ph[:, None])).sum(0)
        d2r = (-a[:, None] * ks[:, None] ** 2 * np.cos(ks[:, None] * t[None] + ph[:, None])).sum(0)
        e = np.exp(1j * t)
        z = r * e
        dz = (dr + 1j * r) * e
        d2z = (d2r + 2j * dr - r) * e
        return z, dz, d2z
    panels = nodes // q
    br = geo._equal_arclength_breaks(fun, panels)
    z, n, w, k = geo._panel_curve(fun, br, q)
    return geo.Problem(np.stack([z.real, z.imag], 1), np.stack([n.real, n.imag], 1), w, k,
                       name="random_star")


def corpus(pkg, n_stars, seed=4):
    """(features, ratios) from plain FP32 factorizations."""
    g = pkg.geometry
    rng = np.random.default_rng(seed)
    cases = []
    for i in range(n_stars):
        cases.append(("laplace", random_star(rng, int(rng.choice([16384, 32768, 65536])))))
    for i in range(6):
        cases.append(("laplace", g.disc_with_ellipses(int(rng.choice([1 << 16, 1 << 17])),
                                                      int(rng.integers(8, 64)), seed=100 + i)))
    for i in range(3):
        cases.append(("stokes", g.disc_with_circles(1 << 14, int(rng.integers(10, 60)), seed=200 + i)))
    for i in range(3):
        ax = tuple(rng.uniform(0.4, 1.0, 3))
        cases.append(("laplace3", g.ellipsoid(8192, ax)))
    X, y = [], []
    import time
    t0 = time.time()
    for kind, prob in cases:
        # tolerances an FP32 factorization can resolve (the mixed form uses 1e-6)
        for tol in ((1e-3, 1e-4, 1e-5) if kind == "laplace3" else (1e-3, 1e-4, 1e-5, 1e-6)):
            kw = dict(id_tol=tol, precision=pkg.PRECISION_FP32)
            if kind == "stokes":
                kw.update(solution_dimension=2, pde=pkg.PDE_STOKES)
            if kind == "laplace3":
                kw.update(max_leaf_dofs=128)
            if prob.n_holes:
                kw.update(hole_centers=prob.hole_centers, hole_start=prob.hole_start,
                          hole_count=prob.hole_count)
            fac = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, **kw)
            log = fac.box_log()
            fac.close()
            n, k = log[:, 12], log[:, 13]
            X.append(log[:, :12])
            y.append(np.where(k > 0, k / n, 1.0))
    print("corpus: %d factorizations, %d boxes, %.1f s" % (len(X), sum(len(v) for v in y),
                                                          time.time() - t0))
    return np.concatenate(X).astype(np.float32), np.concatenate(y).astype(np.float32)


def sketch_report(pkg, model, X, y, n, margin=0.25, oversample=8):
    """MSE and the fraction of boxes whose sketch of the predicted size
    (min(n, ceil((1 + margin) k^) + oversample)) is smaller than or equal to
    the true rank (those would fall back to the plain ID)."""
    r = pkg.rank_model_predict(model, X)
    k_true = y * n
    l = np.minimum(n, np.ceil((1 + margin) * r * n) + oversample)
    fail = (l <= k_true) & (l < n)
    return dict(mse=float(np.mean((r - y) ** 2)), boxes=int(len(y)),
                sketch_too_small=float(fail.mean()),
                mean_sketch_over_n=float(np.mean(l / n)))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--stars", type=int, default=48)
    ap.add_argument("--epochs", type=int, default=3000)
    ap.add_argument("--out", default=os.path.join(HERE, "rank_model.npy"))
    a = ap.parse_args()
    import __graft_entry__ as g
    pkg = g.load_package()
    X, y = corpus(pkg, a.stars)
    model, loss = pkg.rank_model_train(X, y, epochs=a.epochs, lr=3e-3, seed=0)
    print("training set: %d boxes, final MSE %.3e" % (len(y), loss))
    held = pkg.geometry.disc_with_ellipses(1 << 18, 64, seed=11)
    fac = pkg.Factor(held.points, held.normals, held.weights, held.curvatures, id_tol=1e-6,
                     precision=pkg.PRECISION_FP32, hole_centers=held.hole_centers,
                     hole_start=held.hole_start, hole_count=held.hole_count)
    log = fac.box_log()
    fac.close()
    yh = np.where(log[:, 13] > 0, log[:, 13] / log[:, 12], 1.0).astype(np.float32)
    print("held out (disc minus 64 ellipses, 262,144 unknowns, tol 1e-6):",
          sketch_report(pkg, model, log[:, :12], yh, log[:, 12]))
    np.save(a.out, model)
    print("wrote", a.out)


if __name__ == "__main__":
    main()
