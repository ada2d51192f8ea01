"""Generate the golden fixtures in this folder from the REFERENCE's own CPU
solver (kern_interp, compiled from its sources by oracle/build_ref.py).

Run in a container where the reference tree is available:
    python tests/golden/make_golden.py
Each fixture stores the reference's solution (mu, and alpha for holes) and
statistics (levels, root skeleton size, compressed boxes, redundant DOFs),
the input arrays themselves (boundary generators are not bit-reproducible
across CPU architectures: libm and numpy differ in the last bits), and a
SHA-1 of those inputs.  The inputs were made by
kern-interp-dev_gb300/geometry.py (seeded).

The update_* fixtures hold the reference's incremental re-factorization
(QuadTree::perturb then skeletonize, oracle.ref_update_solve) over frames
that each move one hole, beside a fresh reference factorization of every
frame: frame 0's arrays, the moves, one right-hand side, and per frame the
two solutions and the two skeletonize times.
"""
import hashlib
import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def load_geometry():
    spec = importlib.util.spec_from_file_location(
        "ki_geometry", os.path.join(ROOT, "kern-interp-dev_gb300", "geometry.py"))
    g = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(g)
    return g


def input_hash(prob, rhs):
    h = hashlib.sha1()
    for a in (prob.points, prob.normals, prob.weights, prob.curvatures, rhs):
        h.update(np.ascontiguousarray(a, np.float64).tobytes())
    return h.hexdigest()


def stokes_rhs(prob, src=(2.5, 0.0), force=(1.0, 0.5)):
    """Boundary velocity of a 2D Stokeslet (interleaved per node)."""
    d = prob.points - np.asarray(src)[None]
    r2 = (d ** 2).sum(1)
    f = np.asarray(force)
    u = (-0.5 * np.log(r2)[:, None] * f[None] + d * (d @ f)[:, None] / r2[:, None]) / (4 * np.pi)
    return u.reshape(-1, 1)


def cases():
    """(name, problem, rhs, params) for every fixture; shared with the tests."""
    g = load_geometry()
    out = []
    prob, src, _ = g.star_c1()
    out.append(("star_c1", prob, g.laplace_source_rhs(prob, src),
                dict(tol=1e-10, proxy=64, ratio=1.5 / np.sqrt(2), leaf=64, min_compress=64,
                     solution_dim=1, pde=0)))
    prob = g.star(64, 16)
    out.append(("star_1024_default", prob, g.laplace_source_rhs(prob, np.array([[3.0, 3.0]])),
                dict(tol=1e-10, proxy=128, ratio=2.0, leaf=64, min_compress=64, solution_dim=1, pde=0)))
    prob = g.circle(1000, 0.25)
    out.append(("circle_1000", prob, g.laplace_source_rhs(prob, np.array([[-3.0, -2.0]])),
                dict(tol=1e-10, proxy=128, ratio=2.0, leaf=64, min_compress=64, solution_dim=1, pde=0)))
    prob = g.star(128, 16)
    out.append(("star_2048_tol1e-4", prob, g.laplace_source_rhs(prob, np.array([[2.0, -2.5]])),
                dict(tol=1e-4, proxy=128, ratio=2.0, leaf=64, min_compress=64, solution_dim=1, pde=0)))
    prob = g.star(4, 16)
    out.append(("star_64_root_leaf", prob, g.laplace_source_rhs(prob, np.array([[3.0, 3.0]])),
                dict(tol=1e-10, proxy=128, ratio=2.0, leaf=64, min_compress=64, solution_dim=1, pde=0)))
    prob = g.disc_with_ellipses(1 << 13, 6, seed=1)
    rng = np.random.default_rng(2)
    out.append(("disc6_8k", prob, g.laplace_source_rhs(prob, g.random_sources(3, rng)),
                dict(tol=1e-10, proxy=128, ratio=2.0, leaf=64, min_compress=64, solution_dim=1, pde=0)))
    prob = g.star(64, 16, amp=0.2, k=3)
    out.append(("stokes_star_2048", prob, stokes_rhs(prob),
                dict(tol=1e-10, proxy=128, ratio=2.0, leaf=64, min_compress=64, solution_dim=2, pde=3)))
    # 3D (octree, row-sum diagonals, proxy sphere; reference default proxy)
    prob = g.ellipsoid(3000, (1.0, 0.7, 0.5))
    out.append(("laplace3_ellipsoid_3000", prob,
                g.laplace3_source_rhs(prob, np.array([[2.0, 1.0, 1.0], [-1.5, 2.0, 0.5]])),
                dict(tol=1e-8, proxy=0, ratio=2.0, leaf=64, min_compress=64, solution_dim=1, pde=0)))
    prob = g.ellipsoid(1500, (1.0, 0.6, 0.4))
    out.append(("stokes3_ellipsoid_1500", prob,
                g.stokes3_rhs(prob, np.array([[2.0, 1.0, 1.0]]), np.array([[1.0, 0.5, -0.3]])),
                dict(tol=1e-7, proxy=0, ratio=2.0, leaf=64, min_compress=64, solution_dim=3, pde=3)))
    prob = g.spheres_with_holes(2400, [((0.2, 0.1, -0.1), 0.3, 600)])
    out.append(("laplace3_sphere_hole", prob,
                g.laplace3_source_rhs(prob, np.array([[2.0, 1.0, 1.0]])),
                dict(tol=1e-8, proxy=0, ratio=2.0, leaf=64, min_compress=64, solution_dim=1, pde=0)))
    prob = g.spheres_with_holes(1200, [((0.1, -0.2, 0.1), 0.35, 400)])
    out.append(("stokes3_sphere_hole", prob,
                g.stokes3_rhs(prob, np.array([[2.0, 1.0, 1.0]]), np.array([[1.0, 0.5, -0.3]])),
                dict(tol=1e-7, proxy=0, ratio=2.0, leaf=64, min_compress=64, solution_dim=3, pde=3)))
    # the other scalar 2D kernels (Kernel::Pde LAPLACE_NEUMANN = 1, GAUSS = 2):
    # interior Neumann data of exterior sources (the holes of the second case
    # are ignored, as the reference gives these kernels no border), and the
    # Gaussian covariance matrix on the reference's UniformDist grid with a
    # seeded random right-hand side at the covariance experiment's tolerance
    # (kern_interp/experiments/covar.cpp:22-44)
    prob = g.star(128, 16)
    out.append(("neumann_star_2048", prob,
                g.laplace_neumann_rhs(prob, np.array([[3.0, 1.0], [-2.0, 2.5]])),
                dict(tol=1e-10, proxy=128, ratio=2.0, leaf=64, min_compress=64, solution_dim=1, pde=1)))
    prob = g.disc_with_circles(2048, 2, seed=5)
    out.append(("neumann_disc_circles_2048", prob,
                g.laplace_neumann_rhs(prob, np.array([[2.5, -1.0]])),
                dict(tol=1e-10, proxy=128, ratio=2.0, leaf=64, min_compress=64, solution_dim=1, pde=1)))
    prob = g.uniform_grid(4096)
    out.append(("gauss_uniform_4096", prob, np.random.default_rng(7).standard_normal((prob.n, 1)),
                dict(tol=1e-6, proxy=128, ratio=2.0, leaf=64, min_compress=64, solution_dim=1, pde=2)))
    return out


def update_cases():
    """(name, problem, rhs, params, moves) of the re-factorization fixtures:
    frame 0 is the problem, each later frame moves one hole by (hole, delta)
    from the frame before (geometry.move_hole: an exact translation, so the
    frames rebuild bit for bit from frame 0 on any machine); one right-hand
    side serves every frame."""
    g = load_geometry()
    out = []
    prob = g.disc_with_ellipses(1 << 13, 6, seed=1)
    rng = np.random.default_rng(2)
    out.append(("update_disc6_8k", prob, g.laplace_source_rhs(prob, g.random_sources(1, rng)),
                dict(tol=1e-8, solution_dim=1, pde=0),
                [(2, (0.01, 0.0)), (4, (0.0, -0.01))]))
    prob = g.disc_with_circles(1 << 12, 6, seed=4)
    out.append(("update_stokes_circles_4k", prob, stokes_rhs(prob),
                dict(tol=1e-8, solution_dim=2, pde=3),
                [(1, (0.003, 0.0)), (3, (0.0, 0.003))]))
    return out


def update_frames(g, prob, moves):
    frames = [prob]
    for h, d in moves:
        frames.append(g.move_hole(frames[-1], h, d))
    return frames


def main_update(only=None):
    """The reference's incremental re-factorization over the frames
    (oracle.ref_update_solve: QuadTree::perturb + skeletonize) and a fresh
    reference factorization of every frame."""
    import oracle
    g = load_geometry()
    for name, prob, rhs, p, moves in update_cases():
        if only and name not in only:
            continue
        frames = update_frames(g, prob, moves)
        mu_inc, al_inc, sec_inc, comp_inc = oracle.ref_update_solve(
            frames, [rhs[:, 0]] * len(frames), p["tol"], threads=8,
            solution_dim=p["solution_dim"], pde=p["pde"])
        mu_fr, al_fr, sec_fr = [], [], []
        for fr in frames:
            mu, al, st = oracle.solve(fr, rhs[:, :1], p["tol"], threads=8,
                                      solution_dim=p["solution_dim"], pde=p["pde"], impl="ref")
            mu_fr.append(mu[:, 0])
            al_fr.append(al[:, 0])
            sec_fr.append(st["factor_s"])
        np.savez_compressed(os.path.join(HERE, name + ".npz"),
                            points=prob.points, normals=prob.normals, weights=prob.weights,
                            curvatures=prob.curvatures, hole_centers=prob.hole_centers,
                            hole_start=prob.hole_start, hole_count=prob.hole_count,
                            rhs=rhs[:, :1], input_sha1=input_hash(prob, rhs[:, :1]),
                            move_hole=np.array([h for h, _ in moves], np.int32),
                            move_delta=np.array([d for _, d in moves], np.float64),
                            mu_update=mu_inc, alpha_update=al_inc, mu_fresh=np.stack(mu_fr),
                            alpha_fresh=np.stack(al_fr), seconds_update=sec_inc,
                            seconds_fresh=np.array(sec_fr), compressed_update=comp_inc)
        print(name, prob.n, "update s", sec_inc, "fresh s", sec_fr)


def main(only=None):
    import oracle
    for name, prob, rhs, p in cases():
        if only and name not in only:
            continue
        mu_cols, al_cols = [], []
        st = None
        for c in range(rhs.shape[1]):   # the reference's bordered solve handles one column
            mu, al, st = oracle.solve(prob, rhs[:, c:c + 1], p["tol"], threads=8, leaf=p["leaf"],
                                      proxy=p["proxy"], ratio=p["ratio"],
                                      min_compress=p["min_compress"],
                                      solution_dim=p["solution_dim"], pde=p["pde"], impl="ref")
            mu_cols.append(mu[:, 0])
            al_cols.append(al[:, 0] if al.size else np.zeros(0))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), mu=np.stack(mu_cols, 1),
                            alpha=np.stack(al_cols, 1), input_sha1=input_hash(prob, rhs),
                            points=prob.points, normals=prob.normals, weights=prob.weights,
                            curvatures=prob.curvatures, rhs=rhs, hole_centers=prob.hole_centers,
                            hole_start=prob.hole_start, hole_count=prob.hole_count,
                            levels=st["levels"], root=st["root"], compressed=st["compressed"],
                            redundant=st["redundant"])
        print(name, prob.n, st)


if __name__ == "__main__":
    names = sys.argv[1:]
    solve_names = [n for n in names if not n.startswith("update_")]
    update_names = [n for n in names if n.startswith("update_")]
    if not names or solve_names:
        main(solve_names or None)
    if not names or update_names:
        main_update(update_names or None)
