"""Benchmark: recursive-skeletonization factor + solve on one GB300.

Workload (default): 2D Laplace Dirichlet double-layer BIE on the disc of
radius 2 minus 64 ellipses (semi-axes U(0.02, 0.06), seed 1), 16-node
Gauss-Legendre panels, 1,048,576 unknowns, 32 right-hand sides from unit point
sources at |y| in [2.5, 4] (seed 2).  One step = one factorization (tree +
skeletonization + bordered system) and one solve of all 32 right-hand sides
to a 1e-8 relative residual.  Metric: DOF/s = unknowns x right-hand sides /
step time.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--precision mixed|fp64|fp32] [--unknowns N] [--nrhs R]

`value` is timed with the right-hand sides resident in HBM
(ki_solve_refined_device); `e2e` through the host-buffer C-ABI call
(ki_solve_refined), host<->device copies of the geometry, right-hand sides
and solutions inside the timed region.  --impl reference times the CPU
reference path (the oracle port: a C++ restatement of the reference's factor
and solve, linked to OpenBLAS) on all host cores, at the ID tolerance at
which its plain solve reaches the same residual (target / 10), and reports
the residual it reached.  The GPU arm also compares its solutions with that
CPU path on the same nodes and right-hand sides (`parity`).  With N > 1
(torchrun) every rank factors and solves its own copy of the problem
(replicas; the path has no exchange step), rank 0 prints the line.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64", "fp32"])
    ap.add_argument("--target", type=float, default=1e-8,
                    help="relative residual the refined forms reach")
    ap.add_argument("--mixed-tol", type=float, default=1e-6,
                    help="ID tolerance of the FP32 factorization of the mixed form")
    ap.add_argument("--max-steps", type=int, default=10)
    ap.add_argument("--no-refine", action="store_true",
                    help="fp64: one plain solve (the reference's arithmetic), no refinement")
    ap.add_argument("--no-compare", action="store_true",
                    help="mixed: do not also time the FP64 form at the same residual")
    ap.add_argument("--learned-rank", default="on", choices=["on", "off"],
                    help="mixed: size sketched IDs with the shipped rank predictor")
    ap.add_argument("--no-compare-learned", action="store_true",
                    help="mixed: do not also time the mixed form without the rank predictor")
    ap.add_argument("--workload", default="laplace2d_disc_ellipses",
                    choices=["laplace2d_disc_ellipses", "stokes2d_disc_circles", "laplace2d_star",
                             "laplace3d_ellipsoid"])
    ap.add_argument("--unknowns", dest="n", type=int, default=1 << 20)
    ap.add_argument("--holes", type=int, default=64)
    ap.add_argument("--nrhs", type=int, default=32)
    ap.add_argument("--tol", type=float, default=1e-8)
    ap.add_argument("--residual-rows", type=int, default=2048)
    ap.add_argument("--cpu-sample-n", type=int, default=1 << 20)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ref-tol", type=float, default=None,
                    help="ID tolerance of the CPU reference path (default: target / 10, the "
                         "decade at which its plain solve reaches the target residual)")
    ap.add_argument("--ref-residual-rows", type=int, default=256,
                    help="rows of the dense FP64 operator sampled to report the residual the "
                         "CPU reference path reaches")
    ap.add_argument("--no-update", action="store_true",
                    help="skip the incremental re-factorization measurement (workloads with holes)")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the solution comparison against the CPU reference path")
    return ap.parse_args()


def dist_env():
    import __graft_entry__ as g
    return g.load_package().replicas.env()


WORKLOAD_NOTES = {
    "laplace2d_disc_ellipses": "2D Laplace Dirichlet double layer, disc radius 2 minus ellipses "
                               "(semi-axes U(0.02,0.06), seed 1), 16-node GL panels, unit point "
                               "sources at |y| in [2.5,4] (seed 2)",
    "stokes2d_disc_circles": "2D Stokes Dirichlet completed double layer, unit disc minus circles "
                             "(radii U(0.005,0.02), gap 0.005, seed 3), 16-node GL panels, "
                             "Stokeslet at (2.5,0) force (1,0.5) plus seeded Stokeslets",
    "laplace2d_star": "2D Laplace star r=1+0.3cos(5t), 16-node GL panels, source (3,3)",
    "laplace3d_ellipsoid": "3D Laplace Dirichlet double layer on the ellipsoid (1,0.7,0.5), "
                           "Fibonacci nodes with area-Jacobian weights, row-sum diagonal, octree "
                           "leaf 128, 512-point proxy sphere, unit source at (2,1,1) plus seeded "
                           "sources at |y| in [2.5,4]",
}


class Workload:
    """Boundary, right-hand sides and the analytic interior field of one
    benchmark workload (seeded synthetic data)."""

    def __init__(self, pkg, name, n, holes, nrhs):
        g = pkg.geometry
        self.name = name
        self.sol_dim, self.pde = 1, pkg.PDE_LAPLACE
        self.dim, self.leaf, self.proxy = 2, 64, 0
        if name == "laplace3d_ellipsoid":
            self.dim, self.leaf, self.proxy = 3, 128, 512
            self.prob = g.ellipsoid(n, (1.0, 0.7, 0.5))
            rng = np.random.default_rng(2)
            extra = g.random_sources(max(0, nrhs - 1), rng)
            ang = rng.uniform(-1, 1, len(extra))
            extra3 = np.concatenate([extra * np.sqrt(1 - ang ** 2)[:, None],
                                     (np.hypot(*extra.T) * ang)[:, None]], 1)
            self.src = np.concatenate([[[2.0, 1.0, 1.0]], extra3])[:nrhs]
            self.rhs = g.laplace3_source_rhs(self.prob, self.src)
        elif name == "stokes2d_disc_circles":
            self.sol_dim, self.pde = 2, pkg.PDE_STOKES
            self.prob = g.disc_with_circles(n // 2, holes, seed=3)
            self.src, self.frc = g.stokes_c3_sources(nrhs)
            self.rhs = g.stokes_rhs(self.prob, self.src, self.frc)
            self.target_radius = 0.9
        elif name == "laplace2d_star":
            self.prob = g.star(n // 16, 16)
            rng = np.random.default_rng(2)
            self.src = np.concatenate([[[3.0, 3.0]], g.random_sources(nrhs - 1, rng)])[:nrhs]
            self.rhs = g.laplace_source_rhs(self.prob, self.src)
            self.target_radius = 0.5
        else:
            self.prob = g.disc_with_ellipses(n, holes, seed=1)
            rng = np.random.default_rng(2)
            self.src = g.random_sources(nrhs, rng)
            self.rhs = g.laplace_source_rhs(self.prob, self.src)
            self.target_radius = 1.9
        self.n = self.prob.n * self.sol_dim

    @property
    def n_border(self):
        c = 1 if self.sol_dim == 1 else (3 if self.dim == 2 else 6)
        return self.prob.n_holes * c

    def oracle_kw(self):
        return dict(solution_dim=self.sol_dim, pde=self.pde, leaf=self.leaf,
                    proxy=self.proxy or None)

    def factor_kw(self, tol, precision):
        p = self.prob
        kw = dict(id_tol=tol, solution_dimension=self.sol_dim, pde=self.pde, precision=precision,
                  max_leaf_dofs=self.leaf, num_proxy_points=self.proxy)
        if p.n_holes:
            kw.update(hole_centers=p.hole_centers, hole_start=p.hole_start, hole_count=p.hole_count)
        return kw

    def field(self, pkg, targets):
        g = pkg.geometry
        if self.dim == 3:
            return g.laplace3_source_field(targets, self.src)
        if self.sol_dim == 2:
            return np.stack([g.stokeslet_velocity(targets, y, f).reshape(-1)
                             for y, f in zip(self.src, self.frc)], 1)
        return g.laplace_source_field(targets, self.src)

    def targets(self, pkg, count, rng):
        g = pkg.geometry
        if self.dim == 3:
            return g.ellipsoid_targets(count, rng, (1.0, 0.7, 0.5))
        if self.prob.n_holes:
            return g.domain_targets(self.prob, count, rng, radius=self.target_radius)
        return g.disc_targets(count, rng, self.target_radius)


def make_problem(pkg, n, holes, nrhs, name="laplace2d_disc_ellipses"):
    w = Workload(pkg, name, n, holes, nrhs)
    return w.prob, w.src, w.rhs


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region:
    one `nvidia-smi -lms 200` process started before the region and stopped
    after it (a fork of this process while it drives the GPU would stall the
    launching thread), its lines drained by a reader thread."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.samples = []
        self._proc = None
        self._t = None

    def _read(self):
        for line in self._proc.stdout:
            row = [x.strip() for x in line.strip().split(",")]
            if len(row) >= 9:
                self.samples.append(row)

    def __enter__(self):
        try:
            self._proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
            time.sleep(0.3)   # the first sample precedes the timed work
        except Exception:
            self._proc = None
        return self

    def __exit__(self, *a):
        if self._proc is not None:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except Exception:
                self._proc.kill()
            self._t.join(timeout=5)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for nm, v in zip(names, s[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.samples)}


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def residual_sample(fac, prob, rhs, mu, alpha, nrows, seed=9):
    """Relative residual ||K mu + U alpha - f|| / ||f|| estimated from a
    uniform sample of rows with the dense FP64 operator."""
    N = rhs.shape[0]
    rng = np.random.default_rng(seed)
    rows = np.sort(rng.choice(N, size=min(nrows, N), replace=False)).astype(np.int32)
    y = fac.apply_rows(rows, mu, alpha)
    r = y - rhs[rows]
    est = np.sqrt(N / rows.size * (r ** 2).sum(0)) / np.linalg.norm(rhs, axis=0)
    return float(est.max()), float(np.median(est))


def cpu_oracle_run(prob, rhs, tol, threads, **kw):
    import oracle
    t0 = time.perf_counter()
    mu, alpha, st = oracle.solve(prob, rhs, tol, threads=threads, **kw)
    t1 = time.perf_counter()
    return t1 - t0, st, mu, alpha


def metric_name(target):
    """The metric string both arms print (the driver pairs them by it)."""
    return "factor+solve DOF/s (unknowns x rhs / s) at %g relative residual" % target


def ref_tol(args):
    return args.ref_tol if args.ref_tol is not None else args.target / 10


def oracle_residual(wl, mu, alpha, nrows, threads, seed=9):
    """Relative residual ||[K U; Psi -I][mu; alpha] - [f; 0]|| / ||f|| of a
    CPU solution, estimated from `nrows` uniformly sampled rows of the dense
    FP64 operator (the border rows are computed in full); max and median over
    the right-hand sides."""
    import oracle
    N = wl.n
    rng = np.random.default_rng(seed)
    rows = np.sort(rng.choice(N, size=min(nrows, N), replace=False))
    res, res_b = oracle.residual_rows(wl.prob, mu, alpha, wl.rhs, rows, solution_dim=wl.sol_dim,
                                      threads=threads)
    sq = N / rows.size * (res ** 2).sum(0) + (res_b ** 2).sum(0)
    est = np.sqrt(sq) / np.linalg.norm(wl.rhs, axis=0)
    return float(est.max()), float(np.median(est))


def run_reference(args, rank, world):
    """CPU arm: the reference's factor-and-solve restated in C++ (the oracle
    port: same tree, same LAPACK calls), on all host cores, at the ID
    tolerance at which its plain solve reaches the metric's residual."""
    import __graft_entry__ as g
    pkg = g.load_package()
    if rank != 0:
        return
    import oracle
    oracle.build_port()
    threads = os.cpu_count() or 1
    tol = ref_tol(args)
    n = min(args.n, args.cpu_sample_n)
    wl = Workload(pkg, args.workload, n, args.holes, args.nrhs)
    n = wl.n
    for _ in range(max(0, args.warmup)):
        cpu_oracle_run(wl.prob, wl.rhs, tol, threads, **wl.oracle_kw())
    times = []
    mu = alpha = None
    for _ in range(args.steps):
        dt, st, mu, alpha = cpu_oracle_run(wl.prob, wl.rhs, tol, threads, **wl.oracle_kw())
        times.append(dt)
    t = float(np.mean(times))
    value = n * args.nrhs / t
    # the residual the timed solutions reach (outside the timed region)
    rmax, rmed = oracle_residual(wl, mu, alpha, args.ref_residual_rows, threads)
    line = {
        "metric": metric_name(args.target),
        "value": value, "unit": "DOF/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "impl": "reference",
        "config": {"workload": args.workload, "holes": args.holes,
                   "unknowns": n, "nrhs": args.nrhs, "id_tol": tol,
                   "target_residual": args.target,
                   "residual_reached_max": rmax, "residual_reached_median": rmed,
                   "residual_rows_sampled": args.ref_residual_rows,
                   "id_tol_choice": "target / 10: the plain FP64 factor+solve at ID tol 1e-8 "
                                    "leaves a ~6e-8 residual on this workload, at 1e-9 ~3e-9",
                   "full_workload_unknowns": args.n, "ranks_launched": world,
                   "ranks_working": 1},
        "cpu_baseline": {"value": value, "unit": "DOF/s", "cores": threads, "kind": "port",
                         "sample": "%d unknowns (the full workload's geometry at this size), "
                                   "%d rhs, factor+solve per step, ID tol %g" % (n, args.nrhs, tol)},
        "e2e": {"value": value, "unit": "DOF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def max_rel_diff(a, b, scale=None):
    """max over columns of max|a - b| / max|scale| (column-wise relative
    max-norm; scale defaults to b)."""
    b = np.asarray(b, np.float64).reshape(b.shape[0], -1)
    a = np.asarray(a, np.float64).reshape(b.shape)
    sc = b if scale is None else np.asarray(scale, np.float64).reshape(-1, b.shape[1])
    den = np.abs(sc).max(0)
    den[den == 0] = 1.0
    return float((np.abs(a - b).max(0) / den).max())


def parity_check(pkg, args, wl, w2, kw, refine, mu, alpha, pmu, palpha, threads):
    """Solutions of the GPU forms against the CPU reference path on the same
    nodes and right-hand sides (w2, the CPU workload: the full workload unless
    --cpu-sample-n caps it).  Bar: 10 x the ID tolerance of the metric.
      main_form_vs_reference: the timed form's solution against the CPU path.
        A refined form meets a residual target, and a solution whose residual
        is near 1e-8 is up to cond(K) x 1e-8 from the exact discrete solution
        -- the CPU path at --ref-tol is itself ~1e-7 away at its ~3e-9
        residual -- so it passes when (a) its residual (dense FP64 rows on
        the CPU) meets the target and (b) its distance to the CPU path at
        --ref-tol / 10 (error well under the bar) is within the error the
        target allows: max(bar, target x error-per-residual of the CPU path
        at --ref-tol, measured against the same GPU factorization refined to
        1e-12);
      fp64_plain_vs_reference_same_tol: the plain FP64 GPU factor+solve (the
        reference's arithmetic) against the CPU path at the same ID tolerance,
        with both trees' statistics."""
    p = w2.prob
    geo = (p.points, p.normals, p.weights, p.curvatures)
    nb = w2.n_border
    bar = 10 * args.tol
    if w2.n != wl.n:
        fac = pkg.Factor(*geo, **w2.factor_kw(kw["id_tol"], kw["precision"]))
        if refine:
            out = fac.solve_refined(w2.rhs, tol=args.target, max_steps=args.max_steps)
            mu, alpha = out[0], (out[1] if len(out) == 3 else None)
        else:
            r = fac.solve(w2.rhs)
            mu, alpha = r if isinstance(r, tuple) else (r, None)
        fac.close()
    res = {"bar": bar, "unknowns": w2.n, "nrhs": w2.rhs.shape[1],
           "norm": "max over rhs of max|x_gpu - x_ref| / max|x_ref| (alpha: / max|mu_ref|)"}
    main = {"form": args.precision, "reference_id_tol": ref_tol(args)}
    if refine:
        fkw = w2.factor_kw(kw["id_tol"], kw["precision"])
        if "rank_model" in kw:
            fkw["rank_model"] = kw["rank_model"]
        fac = pkg.Factor(*geo, **fkw)
        out = fac.solve_refined(w2.rhs, tol=1e-12, max_steps=args.max_steps + 4)
        err_ref = max_rel_diff(pmu, out[0])
        fac.close()
        res_ref = oracle_residual(w2, pmu, palpha, 256, threads)[0]
        res_gpu = oracle_residual(w2, mu, alpha if alpha is not None else
                                  np.zeros((0, np.asarray(mu).reshape(w2.n * w2.sol_dim, -1).shape[1])),
                                  256, threads)[0]
        per = err_ref / max(res_ref, 1e-300)
        main.update({"residual": res_gpu, "target_residual": args.target,
                     "reference_residual_at_ref_tol": res_ref,
                     "reference_error_at_ref_tol": err_ref, "error_per_residual": per,
                     "error_bar": max(bar, args.target * per)})
        rt2 = ref_tol(args) / 10
        _, _, pmu, palpha = cpu_oracle_run(w2.prob, w2.rhs, rt2, threads, **w2.oracle_kw())
        main["reference_id_tol"] = rt2
    main["max_rel_diff_mu"] = max_rel_diff(mu, pmu)
    if nb:
        # the border unknowns of exterior-source data vanish analytically
        # (|alpha| ~ 1e-13): measured on the scale of the density
        main["max_rel_diff_alpha"] = max_rel_diff(alpha, palpha, scale=pmu)
    res["main_form_vs_reference"] = main
    fac = pkg.Factor(*geo, **w2.factor_kw(args.tol, pkg.PRECISION_FP64))
    r = fac.solve(w2.rhs)
    gmu, galpha = r if isinstance(r, tuple) else (r, None)
    gi = fac.info()
    fac.close()
    _, st, qmu, qalpha = cpu_oracle_run(w2.prob, w2.rhs, args.tol, threads, **w2.oracle_kw())
    plain = {"id_tol": args.tol, "max_rel_diff_mu": max_rel_diff(gmu, qmu),
             "tree_gpu": [gi["n_levels"], gi["n_root"], gi["n_compressed"], gi["n_redundant"]],
             "tree_reference": [st["levels"], st["root"], st["compressed"], st["redundant"]],
             "tree_fields": "levels, root skeleton, compressed boxes, redundant DOFs"}
    if nb:
        plain["max_rel_diff_alpha"] = max_rel_diff(galpha, qalpha, scale=qmu)
    res["fp64_plain_vs_reference_same_tol"] = plain
    plain_ok = (max(v for k, v in plain.items() if k.startswith("max_rel_diff")) <= bar and
                plain["tree_gpu"] == plain["tree_reference"])
    main_diffs = [v for k, v in main.items() if k.startswith("max_rel_diff")]
    if refine:
        main["pass"] = bool(main["residual"] <= args.target and
                            max(main_diffs) <= main["error_bar"])
    else:
        main["pass"] = bool(max(main_diffs) <= bar)
    plain["pass"] = bool(plain_ok)
    res["pass"] = bool(main["pass"] and plain_ok)
    return res


def measure_update(pkg, wl, kw, refine, args, frames=3):
    """Incremental re-factorization (ki_factor_update, the reference's
    QuadTree::perturb + skeletonize): frame after frame one hole is moved by
    a small step, the previous frame's factorization is updated, and a fresh
    factorization of the same frame is made; device-synchronized wall times
    of both, the boxes kept, and the two solutions of the frame's first
    right-hand side compared (refined to the target when the form refines)."""
    import torch
    g = pkg.geometry
    rng = np.random.default_rng(5)
    step = 0.004 if wl.sol_dim == 1 else 0.002

    def arrays(p):
        return (p.points, p.normals, p.weights, p.curvatures)

    def holes(p):
        return dict(hole_centers=p.hole_centers, hole_start=p.hole_start, hole_count=p.hole_count)

    def solve(fac, b):
        if refine:
            out = fac.solve_refined(b, tol=args.target, max_steps=args.max_steps)
            return np.concatenate([o.reshape(-1) for o in out[:-1]])
        out = fac.solve(b)
        return np.concatenate([o.reshape(-1) for o in (out if isinstance(out, tuple) else (out,))])

    base = {k: v for k, v in kw.items() if k not in ("hole_centers", "hole_start", "hole_count")}
    cur = wl.prob
    fac = pkg.Factor(*arrays(cur), **base, **holes(cur))
    n_comp = fac.info()["n_compressed"]
    upd, fresh, kept, diff = [], [], [], []
    for f in range(frames):
        h = int(rng.integers(0, cur.n_holes))
        d = np.zeros(wl.dim)
        d[f % wl.dim] = step if f % 2 == 0 else -step
        cur = g.move_hole(cur, h, d)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        kept.append(fac.update(*arrays(cur), **holes(cur)))
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        fr = pkg.Factor(*arrays(cur), **base, **holes(cur))
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        upd.append((t1 - t0) * 1e3)
        fresh.append((t2 - t1) * 1e3)
        b = wl.rhs[:, :1]
        xu, xf = solve(fac, b), solve(fr, b)
        diff.append(float(np.linalg.norm(xu - xf) / np.linalg.norm(xf)))
        fr.close()
    fac.close()
    return {"what": "one hole moved by %g per frame (geometry.move_hole), the previous frame's "
                    "factorization updated (ki_factor_update) vs a fresh factorization "
                    "(ki_factor_create) of the same frame; wall ms, device synchronized" % step,
            "frames": frames, "update_ms": upd, "fresh_ms": fresh,
            "speedup_median": float(np.median(np.array(fresh) / np.array(upd))),
            "boxes_kept": kept, "boxes_compressed": n_comp,
            "solution_rel_diff": diff}


def main():
    args = parse()
    import __graft_entry__ as g
    rep = g.load_package().replicas
    rank, world, local = rep.env()
    rep.init("nccl" if args.impl == "gb300" else "gloo")
    if args.impl == "reference":
        run_reference(args, rank, world)
        rep.finish()
        return
    import torch
    torch.cuda.set_device(local)
    import __graft_entry__ as g
    pkg = g.load_package()
    wl = Workload(pkg, args.workload, args.n, args.holes, args.nrhs)
    prob, src, rhs = wl.prob, wl.src, wl.rhs
    N = wl.n
    nrhs = args.nrhs
    # inputs resident in HBM for the `value` leg
    rhs_f = np.asfortranarray(rhs)
    d_b = torch.from_numpy(rhs_f.T.copy()).to("cuda")          # (nrhs, N): column c at row c
    d_x = torch.empty_like(d_b)
    nb = wl.n_border
    d_a = torch.empty((nrhs, max(1, nb)), dtype=torch.float64, device="cuda")
    pin_b = torch.from_numpy(rhs_f.T.copy()).pin_memory()
    pin_x = torch.empty_like(pin_b).pin_memory()
    pin_a = torch.empty((nrhs, max(1, nb)), dtype=torch.float64).pin_memory()

    def pinned(a):
        """A page-locked host copy of an array (made outside the timed region)."""
        if a is None:
            return None
        return torch.from_numpy(np.ascontiguousarray(a, np.float64)).pin_memory().numpy()

    # the geometry inputs, page-locked like the right-hand sides (the library
    # uploads them once per factorization; both legs time that copy)
    pin_geo = [pinned(prob.points), pinned(prob.normals), pinned(prob.weights),
               pinned(prob.curvatures)]
    barrier = rep.barrier

    def form(precision):
        """(factor kwargs, refine?) of a form: mixed = FP32 factorization at
        --mixed-tol refined against the FP64 operator to --target; fp64 =
        FP64 factorization at --tol, refined to --target unless --no-refine;
        fp32 = plain FP32 factorization and solve."""
        if precision in ("mixed", "mixed-plain"):
            kw = wl.factor_kw(args.mixed_tol, pkg.PRECISION_FP32)
            if precision == "mixed" and args.learned_rank == "on":
                kw["rank_model"] = "default"
            return kw, True
        if precision == "fp64":
            return wl.factor_kw(args.tol, pkg.PRECISION_FP64), not args.no_refine
        return wl.factor_kw(args.mixed_tol, pkg.PRECISION_FP32), False

    def run_form(precision, steps, warmup):
        kw, refine = form(precision)
        infos = []

        walls = []

        def step_device():
            t0 = time.perf_counter()
            fac = pkg.Factor(*pin_geo, **kw)
            t1 = time.perf_counter()
            fac.set_profiling(True)   # CUDA events around the solve's launch groups
            if refine:
                infos.append(fac.solve_refined_device(d_b.data_ptr(), d_x.data_ptr(), nrhs,
                                                      d_a.data_ptr(), tol=args.target,
                                                      max_steps=args.max_steps))
            else:
                fac.solve_device(d_b.data_ptr(), d_x.data_ptr(), nrhs, d_a.data_ptr())
            torch.cuda.synchronize()
            walls.append({"create_ms": (t1 - t0) * 1e3,
                          "solve_ms": (time.perf_counter() - t1) * 1e3})
            return fac

        def step_host():
            fac = pkg.Factor(*pin_geo, **kw)
            lib = pkg.load_library()
            if refine:
                info = pkg._RefineInfo()
                pkg._check(lib.ki_solve_refined(fac._h, pin_b.data_ptr(), N, nrhs,
                                                pin_x.data_ptr(), N, pin_a.data_ptr(), max(1, nb),
                                                args.target, args.max_steps,
                                                pkg.ctypes.byref(info)))
            else:
                pkg._check(lib.ki_solve(fac._h, pin_b.data_ptr(), N, nrhs, pin_x.data_ptr(), N,
                                        pin_a.data_ptr(), max(1, nb)))
            return fac

        for _ in range(warmup):
            step_device().close()
        infos.clear()
        walls.clear()
        hosts = []
        # ---- value: device-resident right-hand sides
        barrier()
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        stage_runs, level_stats, info = [], [], None
        with ClockSampler(local) as clk:
            n_launch0 = pkg.launch_count()
            ev0.record()
            for _ in range(steps):
                fac = step_device()
                prof = fac.profile()
                stage_runs.append(prof["factor"] + [dict(r, stage="refine:" + r["stage"])
                                                    for r in prof.get("refine", [])])
                level_stats = prof.get("levels", [])
                hosts.append(prof.get("host", {}))
                info = fac.info()
                fac.close()
            ev1.record()
            torch.cuda.synchronize()
            launches = (pkg.launch_count() - n_launch0) / steps
        barrier()
        t_dev = rep.max_over_ranks(ev0.elapsed_time(ev1) / 1e3 / steps, device="cuda")
        host = {}
        for rec in walls + hosts:
            for k, v in rec.items():
                host[k] = host.get(k, 0.0) + v / steps
        return dict(kw=kw, refine=refine, t_dev=t_dev, stage_runs=stage_runs,
                    level_stats=level_stats, info=info, infos=list(infos), clk=clk.summary(),
                    step_host=step_host, host=host, launches=launches)

    main_form = run_form(args.precision, args.steps, args.warmup)
    kw, refine = main_form["kw"], main_form["refine"]
    t_dev, stage_runs = main_form["t_dev"], main_form["stage_runs"]
    level_stats, info = main_form["level_stats"], main_form["info"]
    # ---- e2e: host buffers through the C ABI
    step_host = main_form["step_host"]
    barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        fac = step_host()
        fac.close()
    e1.record()
    torch.cuda.synchronize()
    barrier()
    t_e2e = rep.max_over_ranks(e0.elapsed_time(e1) / 1e3 / args.steps, device="cuda")

    # ---- the mixed form without the rank predictor (what the network gains)
    learned = None
    if args.precision == "mixed" and args.learned_rank == "on":
        learned = {"boxes_sketched": info.get("n_sketched"), "fallbacks": info.get("n_fallback")}
        if not args.no_compare_learned:
            c = run_form("mixed-plain", max(1, min(args.steps, 3)), 2)
            rw = c["infos"][-1] if c["infos"] else {}
            learned.update({"without_predictor_ms_per_step": c["t_dev"] * 1e3,
                            "with_predictor_ms_per_step": t_dev * 1e3,
                            "speedup_from_predictor": c["t_dev"] / t_dev,
                            "residual_without": rw.get("residual")})
    # ---- the FP64 form at the same target residual, for the comparison
    compare = None
    if args.precision == "mixed" and not args.no_compare:
        c = run_form("fp64", max(1, min(args.steps, 3)), 2)
        rc = c["infos"][-1] if c["infos"] else {}
        compare = {"form": "fp64 factorization at ID tol %g, refined to %g" % (args.tol, args.target),
                   "ms_per_step": c["t_dev"] * 1e3, "value": N * nrhs * world / c["t_dev"],
                   "unit": "DOF/s", "residual_first": rc.get("residual0"),
                   "residual": rc.get("residual"), "corrections": rc.get("steps"),
                   "speedup_of_mixed": c["t_dev"] / t_dev}

    # ---- accuracy of the last solution (sampled dense FP64 residual, analytic field)
    fac = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, **kw)
    fac.set_profiling(True)
    rinfo = None
    if refine:
        out = fac.solve_refined(rhs, tol=args.target, max_steps=args.max_steps)
        rinfo = out[-1]
        mu, alpha = out[0], (out[1] if len(out) == 3 else None)
    else:
        res = fac.solve(rhs)
        mu, alpha = res if isinstance(res, tuple) else (res, None)
    solve_prof = fac.profile()["solve"]
    rmax, rmed = residual_sample(fac, prob, rhs, mu, alpha, args.residual_rows)
    rng = np.random.default_rng(4)
    tg = wl.targets(pkg, 64, rng)
    u = fac.eval_targets(tg, mu, alpha)
    ue = wl.field(pkg, tg)
    pde_err = float(np.abs(u - ue).max() / np.abs(ue).max())
    fac.close()
    update = None
    if wl.prob.n_holes and not args.no_update:
        update = measure_update(pkg, wl, kw, refine, args)

    if rank != 0:
        rep.finish()
        return

    # ---- roofline of the dominant kernel (average over the timed steps)
    agg = {}
    for run in stage_runs:
        for s in run:
            a = agg.setdefault(s["stage"], {"ms": 0.0, "flops": 0.0, "bytes": 0.0, "launches": 0})
            for k in ("ms", "flops", "bytes", "launches"):
                a[k] += s[k]
    fam = {}
    for k, v in agg.items():
        f = fam.setdefault(k.split("@")[0], {"ms": 0.0, "flops": 0.0, "bytes": 0.0, "launches": 0})
        for q in ("ms", "flops", "bytes", "launches"):
            f[q] += v[q]
    # dominant stage family of the step (factorization stages and, for the
    # refined forms, the refinement's: FMM near field, M2L, ...), excluding
    # the correction solves (sweeps already listed as factor data) and groups
    # without an algorithmic flop count
    cand = {k: v for k, v in fam.items() if v["flops"] > 0}
    top = max(cand.items(), key=lambda kv: kv[1]["ms"])
    peaks, peak_src = load_peaks()
    fp64_gf, fp32_gf = pkg.measure_fma_peak()
    name, a = top
    sec = a["ms"] / 1e3
    ach_tflops = a["flops"] / sec / 1e12 if sec > 0 else 0.0
    if name.startswith("refine:fmm") or name == "refine:border_apply":
        # the FP32 FMM, and the FP64-accurate FMM and hole columns computed in
        # FP32-pair arithmetic: all on the FP32 pipes
        fp64_stage = False
    elif name.startswith("refine:"):
        fp64_stage = True
    else:
        fp64_stage = args.precision == "fp64"
    cc_peak = (fp64_gf if fp64_stage else fp32_gf) / 1e3
    describe = {
        "refine:fmm_near": ("k_leaf_eval (FMM leaf evaluation: local expansions at the targets "
                            "in FP64, near field over the 3x3 leaf neighbourhood with FP64 "
                            "entries and FP32-pair accumulation, 32 columns)",
                            "near-field point pairs x (4 x 32 + 12) + targets x p x (4 x 32 + 6) "
                            "flops / device time of the launches"),
        "refine:fmm_m2l": ("k_m2l (FMM multipole-to-local translations, rotated form)",
                           "interaction pairs x 32 columns x (4 p^2 + 14 p) flops (real p x p "
                           "core times complex multipoles, 2p phase rotations) / device time"),
        "schur": ("k_schur (schur stage: per box, the redundant block's LU or inverse and the "
                  "Schur updates of the skeleton and near-field blocks)",
                  "algorithmic Schur-complement flops summed over the level's boxes / device "
                  "time of the level's schur launches, summed over levels"),
        "id": ("k_id (id stage: fused ID-matrix assembly, TSQR or sketch, column-pivoted QR)",
               "algorithmic ID flops (4mnk - 2k^2(m+n) + 4/3 k^3 + k^2 r summed over the level's "
               "boxes) / device time of the level's ID launches, summed over levels"),
    }
    kname, kdef = describe.get(name, (name, "algorithmic flops of the stage / its device time"))
    share = a["ms"] / args.steps / (t_dev * 1e3)
    roofline = {"bound": "fp64" if fp64_stage else "fp32",
                "kernel": kname, "stage": name,
                "achieved": ach_tflops, "peak": cc_peak, "unit": "TFLOP/s",
                "frac": ach_tflops / cc_peak if cc_peak > 0 else None, "traffic": None,
                "share_of_step": share,
                "peak_source": "CUDA-core FMA peak measured on this GPU by ki_measure_fma_peak "
                               "(MEASURED_PEAKS.json lists only HBM copy and bf16 tensor peaks: "
                               "hbm %.0f GB/s, bf16 %.0f TFLOP/s, %s)" % (
                                   peaks.get("hbm_gbs", 0), peaks.get("bf16_tflops", 0), peak_src),
                "achieved_definition": kdef,
                "launches_per_step": a["launches"] / args.steps,
                "ms_per_step": a["ms"] / args.steps}
    # the solve's stages against the HBM roofline (algorithmic bytes: factor
    # matrices read once, right-hand-side rows read and written once)
    solve_roof = {}
    for rec in solve_prof:
        a2 = solve_roof.setdefault(rec["stage"], {"ms": 0.0, "bytes": 0.0, "flops": 0.0,
                                                  "launches": 0})
        for q in ("ms", "bytes", "flops", "launches"):
            a2[q] += rec[q]
    for k2, v2 in solve_roof.items():
        gbs = v2["bytes"] / (v2["ms"] / 1e3) / 1e9 if v2["ms"] > 0 and v2["bytes"] > 0 else None
        v2["achieved_gbs"] = gbs
        v2["frac_hbm"] = gbs / peaks["hbm_gbs"] if gbs else None
    stage_table = {k: {"ms_per_step": v["ms"] / args.steps, "launches_per_step": v["launches"] / args.steps,
                       "gflop_per_step": v["flops"] / args.steps / 1e9} for k, v in agg.items()}
    launches = int(round(main_form["launches"]))

    cpu = None
    parity = None
    if not args.no_cpu_baseline:
        try:
            n_cpu = min(args.n, args.cpu_sample_n)
            w2 = Workload(pkg, args.workload, n_cpu, args.holes, nrhs)
            n_cpu = w2.n
            thr = os.cpu_count() or 1
            rt = ref_tol(args)
            dt, st, pmu, palpha = cpu_oracle_run(w2.prob, w2.rhs, rt, thr, **w2.oracle_kw())
            cpu = {"value": n_cpu * nrhs / dt, "unit": "DOF/s", "cores": thr, "kind": "port",
                   "sample": "%d unknowns of the same geometry family, %d rhs, one factor+solve at "
                             "ID tol %g (%.1f s)" % (n_cpu, nrhs, rt, dt)}
            if not args.no_parity:
                parity = parity_check(pkg, args, wl, w2, kw, refine, mu, alpha, pmu, palpha, thr)
        except Exception as e:  # reported, not fatal
            cpu = {"value": None, "unit": "DOF/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": "failed: %s" % e}

    units = N * nrhs * world
    h2d = N * nrhs * 8 + prob.n * (2 * wl.dim + 2) * 8
    d2h = N * nrhs * 8 + max(1, nb) * nrhs * 8
    metric = (metric_name(args.target) if refine else
              "factor+solve DOF/s (unknowns x rhs / s) at ID tol %g" % args.tol)
    dtype = {"fp64": "f64", "fp32": "f32",
             "mixed": "f32 factorization and solves, f64 residuals (FMM)"}[args.precision]
    refines = main_form["infos"]
    config = {"workload": args.workload, "holes": args.holes, "unknowns": N,
              "description": WORKLOAD_NOTES[args.workload],
              "nrhs": nrhs, "precision": args.precision,
              "id_tol": args.mixed_tol if args.precision == "mixed" else args.tol,
              "target_residual": args.target if refine else None,
              "leaf": wl.leaf, "proxy": wl.proxy or (128 if wl.dim == 2 else 32),
              "l2": "factor working set >> 129 MB L2 (no flush needed)",
              "levels": info["n_levels"], "root_skeleton": info["n_root"],
              "compressed_boxes": info["n_compressed"]}
    if args.precision == "mixed":
        config["id_tol_note"] = ("the FP32 factorization runs at ID tol %g, not %g: FP32 rounding "
                                 "(2^-24 relative) bounds the tolerance an FP32 ID can honour, and "
                                 "ki_factor_create refuses FP32 id_tol < 5e-8; the %g residual is "
                                 "reached by FP64-residual refinement" % (args.mixed_tol, args.tol,
                                                                          args.target))
    line = {
        "metric": metric,
        "value": units / t_dev, "unit": "DOF/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_dev * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": dtype,
        "data": "synthetic (seeded boundary and sources)",
        "config": config,
        "gpu_launches": launches,
        "gpu_launches_note": "kernels the library launched per timed step (its launch counter, "
                             "ki_launch_count): tree sort, factorization levels, solves, FMM "
                             "applies, residual norms",
        "stages": stage_table,
        "solve_stages": solve_prof,
        "level_stats": level_stats,
        "host_wall_ms_per_step": main_form["host"],
        "refinement": {"steps_per_solve": [r["steps"] for r in refines],
                       "residual_first_solve": [r["residual0"] for r in refines],
                       "residual_final": [r["residual"] for r in refines],
                       "residual_updates": [r["updates"] for r in refines],
                       "drift_bound": [r["drift_bound"] for r in refines],
                       "residual_operator": "FMM (2D Laplace; FP64 at the target's order, "
                                            "updates by the FP32 12-term FMM)"
                       if (wl.dim == 2 and wl.sol_dim == 1 and N >= 4096) else "dense FP64"}
        if refine else None,
        "roofline": roofline,
        "solve_roofline": {"peak_gbs": peaks["hbm_gbs"], "peak_source": peak_src,
                           "solves": len([r for r in solve_prof if r["stage"] == "sweep_up"]),
                           "stages": solve_roof},
        "e2e": {"value": units / t_e2e, "unit": "DOF/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": t_e2e * 1e3},
        # compact summaries last: they stay in the tail of the line
        "learned_rank": learned,
        "fp64_form_same_residual": compare,
        "incremental_update": update,
        "accuracy": {"residual_est_max": rmax, "residual_est_median": rmed,
                     "residual_rows_sampled": args.residual_rows, "pde_rel_err": pde_err,
                     "refined_residual": rinfo["residual"] if rinfo else None},
        "parity": parity,
        "clocks": main_form["clk"],
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)
    rep.finish()


if __name__ == "__main__":
    main()
