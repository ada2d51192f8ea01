"""Train the learned skeleton-rank predictor shipped as rank_model.npy, and
evaluate it on a held-out problem family.

Corpus (the learned-rank configuration): box logs (features, n, rank) of
plain FP64 factorizations -- no model, so every rank comes from the
column-pivoted-QR ID -- of seeded random boundaries (seed 4):
  - star curves r(theta) = 1 + sum_{k=2..8} a_k cos(k theta + phi_k),
    a_k ~ U(0, 0.3/k), phi_k ~ U(0, 2 pi), at 16,384, 32,768 or 65,536 nodes;
  - ellipsoids with semi-axes U(0.4, 1) at 32,768 nodes (3D Laplace);
each at an ID tolerance drawn from 1e-3 .. 1e-6 (1e-4 .. 1e-6 in 3D).  The
target is the rank fraction k / n (1 for a box the ID leaves uncompressed).
Training runs on the GPU through the library's own forward/backward/Adam
kernels (ki_rank_model_train); the factorizations infer in BF16 on the
tensor cores.

Held-out evaluation (families absent from the corpus): 3D Stokes on the
ellipsoid (1, 0.6, 0.4) (three unknowns per node: a solution dimension the
corpus never shows), and the disc minus 64 ellipses of the benchmark.  For
each: the network's error, how often a sketch of the predicted size is too
small (the box is then recompressed by the plain ID), and for 3D Stokes the
factor+solve time of the mixed form with the network against the plain FP64
form at the same residual.

    python kern-interp-dev_gb300/train_rank_model.py [--stars 2000] [--ellipsoids 200]
        [--eval-nodes 32768] [--out PATH] [--report PATH]
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


def corpus(pkg, n_stars, n_ellipsoids, seed=4, log=print):
    """(features, ratios) from plain FP64 factorizations."""
    import time
    g = pkg.geometry
    rng = np.random.default_rng(seed)
    X, y = [], []
    t0 = time.time()
    count = 0

    def add(prob, tol, **kw):
        nonlocal count
        fac = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, id_tol=tol,
                         precision=pkg.PRECISION_FP64, **kw)
        lg = fac.box_log()
        fac.close()
        n, k = lg[:, 12], lg[:, 13]
        X.append(lg[:, :12])
        y.append(np.where(k > 0, k / n, 1.0))
        count += 1

    for i in range(n_stars):
        prob = random_star(rng, int(rng.choice([16384, 32768, 65536])))
        add(prob, float(rng.choice([1e-3, 1e-4, 1e-5, 1e-6])))
        if (i + 1) % 250 == 0:
            log("  stars %d / %d, %.0f s" % (i + 1, n_stars, time.time() - t0))
    for i in range(n_ellipsoids):
        prob = g.ellipsoid(32768, tuple(rng.uniform(0.4, 1.0, 3)))
        add(prob, float(rng.choice([1e-4, 1e-5, 1e-6])), max_leaf_dofs=128)
        if (i + 1) % 25 == 0:
            log("  ellipsoids %d / %d, %.0f s" % (i + 1, n_ellipsoids, time.time() - t0))
    log("corpus: %d FP64 factorizations, %d boxes, %.1f s" % (count, sum(len(v) for v in y),
                                                             time.time() - t0))
    return np.concatenate(X).astype(np.float32), np.concatenate(y).astype(np.float32)


def sketch_report(pkg, model, X, y, n, margin=0.25, oversample=8):
    """Error of the network (BF16 tensor-core inference, as the
    factorizations run it) and the fraction of boxes whose sketch of the
    predicted size (min(n, ceil((1 + margin) k^) + oversample)) is smaller
    than or equal to the true rank (those would fall back to the plain ID)."""
    r = pkg.rank_model_predict(model, X, bf16=True)
    k_true = y * n
    l = np.minimum(n, np.ceil((1 + margin) * r * n) + oversample)
    fail = (l <= k_true) & (l < n)
    return dict(mse=float(np.mean((r - y) ** 2)), mean_abs_rank_error=float(np.mean(np.abs(r - y) * n)),
                boxes=int(len(y)), sketch_too_small=float(fail.mean()),
                mean_sketch_over_n=float(np.mean(l / n)))


def box_targets(fac):
    lg = fac.box_log()
    return lg[:, :12], np.where(lg[:, 13] > 0, lg[:, 13] / lg[:, 12], 1.0).astype(np.float32), lg[:, 12]


def evaluate_stokes3(pkg, model, nodes, tol=1e-6, log=print):
    """3D Stokes on the ellipsoid (1, 0.6, 0.4): the network against the
    plain FP64 ranks, and factor+solve times of the plain FP64 form and of
    the mixed form with and without the network (FP32 factorization refined
    against the FP64 operator to the plain form's residual)."""
    import time
    g = pkg.geometry
    prob = g.ellipsoid(nodes, (1.0, 0.6, 0.4))
    rhs = g.stokes3_rhs(prob, np.array([[2.0, 1.0, 1.0]]), np.array([[1.0, 0.5, -0.3]]))
    kw = dict(solution_dimension=3, pde=pkg.PDE_STOKES, max_leaf_dofs=128)
    out = {"problem": "3D Stokes, ellipsoid (1, 0.6, 0.4), %d nodes = %d unknowns, ID tol %g"
                      % (nodes, 3 * nodes, tol)}

    def timed(fn):
        import torch
        torch.cuda.synchronize()
        t = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return r, time.perf_counter() - t

    def plain():
        fac = pkg.Factor(prob.points, prob.normals, prob.weights, None, id_tol=tol,
                         precision=pkg.PRECISION_FP64, **kw)
        return fac, fac.solve(rhs)
    (fac64, x64), t64 = timed(plain)
    res64 = float(np.linalg.norm(fac64.apply(x64) - rhs) / np.linalg.norm(rhs))
    Xh, yh, nh = box_targets(fac64)
    fac64.close()
    out["plain_fp64"] = {"seconds": t64, "residual": res64}
    out["network_on_fp64_ranks"] = sketch_report(pkg, model, Xh, yh, nh)
    for name, m in (("mixed_with_network", model), ("mixed_without_network", None)):
        def mixed():
            fac = pkg.Factor(prob.points, prob.normals, prob.weights, None, id_tol=tol,
                             precision=pkg.PRECISION_FP32, rank_model=m, **kw)
            x, info = fac.solve_refined(rhs, tol=max(res64, 1e-12), max_steps=20)
            inf = fac.info()
            fac.close()
            return info, inf
        (info, inf), t = timed(mixed)
        out[name] = {"seconds": t, "residual": info["residual"], "corrections": info["steps"],
                     "boxes_sketched": inf["n_sketched"], "recompressions": inf["n_fallback"],
                     "boxes_compressed": inf["n_compressed"]}
        log(name, out[name])
    out["speedup_mixed_with_network_over_plain_fp64"] = t64 / out["mixed_with_network"]["seconds"]
    return out


def main():
    import json
    ap = argparse.ArgumentParser()
    ap.add_argument("--stars", type=int, default=2000)
    ap.add_argument("--ellipsoids", type=int, default=200)
    ap.add_argument("--epochs", type=int, default=3000)
    ap.add_argument("--eval-nodes", type=int, default=32768)
    ap.add_argument("--out", default=os.path.join(HERE, "rank_model.npy"))
    ap.add_argument("--report", default=None)
    ap.add_argument("--model", default=None,
                    help="evaluate this trained blob instead of building a corpus and training")
    a = ap.parse_args()
    import __graft_entry__ as g
    pkg = g.load_package()
    if a.model:
        model = pkg.load_rank_model(a.model)
        rep = {"corpus": {"model": os.path.basename(a.model)}}
    else:
        X, y = corpus(pkg, a.stars, a.ellipsoids, log=lambda *v: print(*v, flush=True))
        model, loss = pkg.rank_model_train(X, y, epochs=a.epochs, lr=3e-3, seed=0)
        rep = {"corpus": {"stars": a.stars, "ellipsoids": a.ellipsoids, "boxes": int(len(y)),
                          "train_mse": float(loss)}}
        print("training set: %d boxes, final MSE %.3e" % (len(y), loss), flush=True)
    held = pkg.geometry.disc_with_ellipses(1 << 18, 64, seed=1)
    fac = pkg.Factor(held.points, held.normals, held.weights, held.curvatures, id_tol=1e-6,
                     precision=pkg.PRECISION_FP64, hole_centers=held.hole_centers,
                     hole_start=held.hole_start, hole_count=held.hole_count)
    Xh, yh, nh = box_targets(fac)
    fac.close()
    rep["held_out_disc64_262k"] = sketch_report(pkg, model, Xh, yh, nh)
    print("held out (disc minus 64 ellipses, 262,144 unknowns, tol 1e-6):",
          rep["held_out_disc64_262k"], flush=True)
    rep["held_out_stokes3"] = evaluate_stokes3(pkg, model, a.eval_nodes,
                                               log=lambda *v: print(*v, flush=True))
    print(json.dumps(rep["held_out_stokes3"]), flush=True)
    if not a.model:
        np.save(a.out, model)
        print("wrote", a.out)
    if a.report:
        with open(a.report, "w") as fh:
            json.dump(rep, fh, indent=1)


if __name__ == "__main__":
    main()
