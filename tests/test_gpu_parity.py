"""GPU parity through the C ABI: the CUDA factor + solve against the
reference's own outputs (golden fixtures) and against the CPU oracle on
freshly generated boundaries.  Tolerance (FP64 form): solution difference
<= 10 x id_tol relative (max-norm), the bar the solver's documentation states."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = ["star_c1", "star_1024_default", "circle_1000", "star_2048_tol1e-4",
          "star_64_root_leaf", "disc6_8k", "stokes_star_2048", "laplace3_ellipsoid_3000",
          "stokes3_ellipsoid_1500", "laplace3_sphere_hole", "stokes3_sphere_hole"]


def factor_for(pkg, prob, p, precision=0):
    return pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, id_tol=p["tol"],
                      solution_dimension=p["solution_dim"], pde=p["pde"],
                      hole_centers=prob.hole_centers if prob.n_holes else None,
                      hole_start=prob.hole_start if prob.n_holes else None,
                      hole_count=prob.hole_count if prob.n_holes else None,
                      max_leaf_dofs=p["leaf"], num_proxy_points=p["proxy"],
                      radius_ratio=p["ratio"], min_dofs_to_compress=p["min_compress"],
                      precision=precision)


def rel_max(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("name", GOLDEN)
def test_gpu_matches_reference_fixture(pkg, golden_cases, name):
    prob, rhs, p, data, h = golden_cases[name]
    assert str(data["input_sha1"]) == h
    fac = factor_for(pkg, prob, p)
    res = fac.solve(rhs)
    mu, alpha = res if isinstance(res, tuple) else (res, None)
    assert rel_max(mu, data["mu"]) <= 10 * p["tol"]
    info = fac.info()
    assert info["n_levels"] == int(data["levels"])
    assert info["n_root"] == int(data["root"])
    assert info["n_compressed"] == int(data["compressed"])
    assert info["n_redundant"] == int(data["redundant"])
    if alpha is not None:
        # the border unknowns of an exterior-source field vanish analytically
        # (|alpha| ~ 1e-13): compare on the scale of the density
        assert np.abs(alpha - data["alpha"]).max() <= 10 * p["tol"] * np.abs(data["mu"]).max()


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_gpu_matches_oracle_random_stars(pkg, oracle_mod, seed):
    rng = np.random.default_rng(100 + seed)
    amp = rng.uniform(0.1, 0.35)
    k = int(rng.integers(2, 9))
    panels = int(rng.integers(40, 400))
    prob = pkg.geometry.star(panels, 16, amp=amp, k=k)
    src = pkg.geometry.random_sources(2, rng)
    f = pkg.geometry.laplace_source_rhs(prob, src)
    tol = float(10.0 ** rng.uniform(-11, -5))
    mu_ref, _, st = oracle_mod.solve(prob, f, tol, threads=4)
    fac = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, id_tol=tol)
    mu = fac.solve(f)
    assert rel_max(mu, mu_ref) <= 10 * tol
    assert fac.info()["n_root"] == st["root"]


def test_gpu_holes_against_oracle_and_field(pkg, oracle_mod):
    g = pkg.geometry
    prob = g.disc_with_ellipses(1 << 15, 16, seed=7)
    rng = np.random.default_rng(3)
    src = g.random_sources(4, rng)
    f = g.laplace_source_rhs(prob, src)
    tol = 1e-10
    mu_ref, al_ref, _ = oracle_mod.solve(prob, f, tol, threads=8)
    fac = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, id_tol=tol,
                     hole_centers=prob.hole_centers, hole_start=prob.hole_start,
                     hole_count=prob.hole_count)
    mu, al = fac.solve(f)
    assert rel_max(mu, mu_ref) <= 10 * tol
    assert np.abs(al - al_ref).max() <= 10 * tol * np.abs(mu_ref).max()
    tg = g.domain_targets(prob, 40, rng)
    u = fac.eval_targets(tg, mu, al)
    ue = g.laplace_source_field(tg, src)
    assert np.abs(u - ue).max() <= 1e-8 * np.abs(ue).max()


def test_gpu_matches_oracle_disc64_262k_32rhs(pkg, oracle_mod):
    """The headline workload's geometry family at a quarter of its size: the
    disc of radius 2 minus 64 ellipses (seed 1), 262,144 unknowns, 32
    right-hand sides (seed 2), ID tolerance 1e-8.  The plain FP64 GPU
    factor+solve (the reference's arithmetic) and the mixed form (FP32
    factorization at 1e-6, refined against the FP64 operator to a 1e-8
    residual) both stay within 10 x 1e-8 of the CPU reference path
    (kern_interp/linear_solve.cpp:202-227 restated by the oracle port): the
    plain form against the reference path at the same ID tolerance, the
    refined form against the reference path at the tolerance where it
    reaches the same residual (1e-9: at 1e-8 its plain solve leaves a ~6e-8
    residual, and its own error, ~4e-7, would dominate the difference)."""
    g = pkg.geometry
    prob = g.disc_with_ellipses(1 << 18, 64, seed=1)
    rng = np.random.default_rng(2)
    f = g.laplace_source_rhs(prob, g.random_sources(32, rng))
    tol = 1e-8
    mu_ref, al_ref, st = oracle_mod.solve(prob, f, tol, threads=16)
    holes = dict(hole_centers=prob.hole_centers, hole_start=prob.hole_start,
                 hole_count=prob.hole_count)
    geo = (prob.points, prob.normals, prob.weights, prob.curvatures)

    def col_rel(a, b):
        return (np.abs(a - b).max(0) / np.abs(b).max(0)).max()

    fac = pkg.Factor(*geo, id_tol=tol, **holes)
    mu, al = fac.solve(f)
    info = fac.info()
    fac.close()
    assert col_rel(mu, mu_ref) <= 10 * tol
    assert np.abs(al - al_ref).max() <= 10 * tol * np.abs(mu_ref).max()
    # same tree: levels and root skeleton; the compressed-box count may move
    # by a box where a rank sits on the tolerance
    assert info["n_levels"] == st["levels"]
    assert abs(info["n_root"] - st["root"]) <= 0.02 * st["root"]
    fac = pkg.Factor(*geo, id_tol=1e-6, precision=pkg.PRECISION_FP32, **holes)
    mu2, al2, rinfo = fac.solve_refined(f, tol=tol, max_steps=6)
    fac.close()
    assert rinfo["residual"] <= tol
    mu_ref9, al_ref9, _ = oracle_mod.solve(prob, f, tol / 10, threads=16)
    assert col_rel(mu2, mu_ref9) <= 10 * tol
    assert np.abs(al2 - al_ref9).max() <= 10 * tol * np.abs(mu_ref9).max()


@pytest.mark.parametrize("wide_rows,schur_cap,full_cap,schur_wide_n,coop_min",
                         [("0", "0", "230400", "0", "384"), ("400", "225000", "230400", "288", "384"),
                          ("100000", "0", "0", "100000", "384"), ("0", "225000", "230400", "288", "0")])
def test_gpu_wide_path_matches_oracle(pkg, oracle_mod, monkeypatch, wide_rows, schur_cap,
                                      full_cap, schur_wide_n, coop_min):
    """Boxes with tall ID matrices go through the explicit-matrix blocked QR
    (cooperative panels, tiled trailing updates) and large boxes through the
    multi-CTA Schur elimination; forcing the thresholds down drives (nearly)
    every box through them, and (coop_min 0) every wide box's pivoted QR
    through the cooperative multi-CTA kernel."""
    monkeypatch.setenv("KI_WIDE_ROWS", wide_rows)
    monkeypatch.setenv("KI_SCHUR_SMEM_CAP", schur_cap)
    monkeypatch.setenv("KI_ID_FULL_CAP", full_cap)            # 0: packed triangles
    monkeypatch.setenv("KI_SCHUR_WIDE_N", schur_wide_n)       # 0: device-wide Schur
    monkeypatch.setenv("KI_COOP_CPQR_MIN_N", coop_min)
    g = pkg.geometry
    prob = g.disc_with_ellipses(1 << 13, 6, seed=5)
    f = g.laplace_source_rhs(prob, np.array([[3.0, 1.0]]))
    tol = 1e-10
    ref, al_ref, st = oracle_mod.solve(prob, f, tol, threads=4)
    fac = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, id_tol=tol,
                     hole_centers=prob.hole_centers, hole_start=prob.hole_start,
                     hole_count=prob.hole_count)
    mu, al = fac.solve(f)
    assert rel_max(mu, ref) <= 10 * tol
    assert fac.info()["n_root"] == st["root"]
    paths = [lv["paths"] for lv in fac.profile()["levels"]]
    if wide_rows == "0":
        assert sum(p[2] + p[3] for p in paths) > 0
    if full_cap == "0":
        assert sum(p[1] for p in paths) > 0


def stokes_psi_times(prob, mu):
    """Psi mu of the 2D Stokes bordered system, Psi built as the reference
    builds it (kern_interp/linear_solve.cpp:164-177): per hole the weighted
    x- and y-sums and the weighted x2*mu_x - x1*mu_y moment (absolute
    coordinates, as the reference writes them)."""
    out = np.zeros((3 * prob.n_holes, mu.shape[1]))
    for h in range(prob.n_holes):
        s = slice(int(prob.hole_start[h]), int(prob.hole_start[h] + prob.hole_count[h]))
        w = prob.weights[s][:, None]
        x = prob.points[s]
        mx, my = mu[2 * s.start:2 * s.stop:2], mu[2 * s.start + 1:2 * s.stop:2]
        out[3 * h] = (w * mx).sum(0)
        out[3 * h + 1] = (w * my).sum(0)
        out[3 * h + 2] = (w * (x[:, 1:2] * mx - x[:, 0:1] * my)).sum(0)
    return out


@pytest.mark.parametrize("holes", [3, 70])
def test_gpu_stokes_holes_against_oracle_and_field(pkg, oracle_mod, holes):
    """2D Stokes with circular holes (3 border unknowns per hole: Stokeslet and
    rotlet columns, kern_interp/linear_solve.cpp:77-97, 164-177); 70 holes
    take the wide-border (split-K GEMM) reductions.

    The bordered Stokes system is ill-conditioned (2-norm condition number
    2.4e6 at 4,096 unknowns with 3 or 20 holes, computed by SVD), so at
    tol 1e-10 the compiled reference itself differs from a dense LU solve by
    1e-7; its C++ restatement, which repeats its box order and LAPACK calls,
    agrees with it to 3e-11, but any other box order or QR moves the
    solution by up to ~1e-8.  The bars are therefore: the reference's own
    backward-error invariant (<= 50 tol, kern_interp/kern_interp_test.cpp:29-32)
    on both block rows; a distance to the exact discrete solution (the same
    factorization refined against the FP64 operator to a 1e-13 residual) no
    larger than the oracle's own distance to it (x3, + 10 tol); identical
    tree statistics; and the interior velocity of the exterior Stokeslets."""
    g = pkg.geometry
    prob = g.disc_with_circles(1 << 13, holes, seed=3)
    src, frc = g.stokes_c3_sources(3)
    f = g.stokes_rhs(prob, src, frc)
    tol = 1e-10
    ref, al_ref, st = oracle_mod.solve(prob, f, tol, threads=8, solution_dim=2, pde=3)
    fac = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, id_tol=tol,
                     solution_dimension=2, pde=pkg.PDE_STOKES, hole_centers=prob.hole_centers,
                     hole_start=prob.hole_start, hole_count=prob.hole_count)
    mu, al = fac.solve(f)
    fmax = np.abs(f).max()
    res1 = np.abs(fac.apply(mu, al) - f).max() / fmax
    res2 = np.abs(stokes_psi_times(prob, mu) - al).max() / fmax
    assert res1 <= 50 * tol and res2 <= 50 * tol, (res1, res2)
    mu_x, al_x, rinfo = fac.solve_refined(f, tol=1e-13, max_steps=10)
    assert rinfo["residual"] <= 1e-13, rinfo
    e_gpu, e_ref = rel_max(mu, mu_x), rel_max(ref, mu_x)
    assert e_gpu <= 3 * e_ref + 10 * tol, (e_gpu, e_ref, rel_max(mu, ref))
    scale = np.abs(mu_x).max()
    a_gpu, a_ref = np.abs(al - al_x).max() / scale, np.abs(al_ref - al_x).max() / scale
    assert a_gpu <= 3 * a_ref + 10 * tol, (a_gpu, a_ref)
    info = fac.info()
    assert info["n_root"] == st["root"]
    assert info["n_levels"] == st["levels"] and info["n_compressed"] == st["compressed"]
    rng = np.random.default_rng(8)
    tg = g.domain_targets(prob, 20, rng, radius=0.9)
    u = fac.eval_targets(tg, mu, al)
    ue = np.stack([g.stokeslet_velocity(tg, y, fr).reshape(-1) for y, fr in zip(src, frc)], 1)
    u_ref = fac.eval_targets(tg, ref, al_ref)
    err, err_ref = np.abs(u - ue).max(), np.abs(u_ref - ue).max()
    assert err <= max(1e-8 * np.abs(ue).max(), 2 * err_ref), (err, err_ref)


def test_gpu_multi_rhs_equals_single_columns(pkg):
    g = pkg.geometry
    prob = g.star(256, 16)
    rng = np.random.default_rng(5)
    F = g.laplace_source_rhs(prob, g.random_sources(33, rng))
    fac = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, id_tol=1e-9)
    X = fac.solve(F)
    for c in (0, 17, 32):
        np.testing.assert_array_equal(X[:, c], fac.solve(F[:, c]))


def test_gpu_deterministic(pkg):
    g = pkg.geometry
    prob = g.disc_with_ellipses(1 << 13, 4, seed=11)
    f = g.laplace_source_rhs(prob, np.array([[3.0, 0.5], [-2.6, 1.0]]))
    kw = dict(id_tol=1e-9, hole_centers=prob.hole_centers, hole_start=prob.hole_start,
              hole_count=prob.hole_count)
    a = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, **kw).solve(f)
    b = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, **kw).solve(f)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


@pytest.mark.parametrize("tol", [1e-6, 1e-10])
def test_gpu_dense_residual(pkg, tol):
    """Backward error against the dense FP64 operator (solve_err,
    kern_interp/linear_solve.cpp:339-426) <= 50 id_tol
    (kern_interp/kern_interp_test.cpp:29-32)."""
    g = pkg.geometry
    prob = g.star(1024, 16, amp=0.3, k=5)
    f = g.laplace_source_rhs(prob, np.array([[3.0, 3.0], [0.0, -2.0]]))
    fac = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, id_tol=tol)
    mu = fac.solve(f)
    r = fac.apply(mu) - f
    assert np.linalg.norm(r) / np.linalg.norm(f) <= 50 * tol


def test_gpu_nothing_compresses(pkg, oracle_mod):
    """min_dofs_to_compress above every box: the root holds every DOF and the
    factorization is a dense LU."""
    g = pkg.geometry
    prob = g.star(32, 16)
    f = g.laplace_source_rhs(prob, np.array([[3.0, 3.0]]))
    fac = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, id_tol=1e-10,
                     min_dofs_to_compress=100000)
    mu = fac.solve(f)
    assert fac.info()["n_root"] == prob.n and fac.info()["n_compressed"] == 0
    K = oracle_mod.dense_matrix(prob)
    np.testing.assert_allclose(mu, np.linalg.solve(K, f), rtol=0, atol=1e-11 * np.abs(mu).max())


def test_gpu_fp32_factorization_accuracy(pkg, oracle_mod):
    """FP32 form: the factorization is a preconditioner-grade approximate
    inverse; its solution stays within 1e-3 of the FP64 oracle."""
    g = pkg.geometry
    prob = g.star(256, 16)
    f = g.laplace_source_rhs(prob, np.array([[3.0, 3.0]]))
    ref, _, _ = oracle_mod.solve(prob, f, 1e-10, threads=4)
    fac = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, id_tol=1e-5,
                     precision=pkg.PRECISION_FP32)
    mu = fac.solve(f)
    assert rel_max(mu, ref) <= 1e-3


def test_solve_device_pointer_path(pkg):
    torch = pytest.importorskip("torch")
    g = pkg.geometry
    prob = g.star(128, 16)
    F = g.laplace_source_rhs(prob, np.array([[3.0, 3.0], [-3.0, 2.5]]))
    fac = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, id_tol=1e-10)
    host = fac.solve(F)
    db = torch.tensor(np.asfortranarray(F).T.copy(), dtype=torch.float64, device="cuda")  # (nrhs, N) rows = columns
    dx = torch.empty_like(db)
    torch.cuda.synchronize()
    fac.solve_device(db.data_ptr(), dx.data_ptr(), F.shape[1])
    torch.cuda.synchronize()
    np.testing.assert_array_equal(dx.cpu().numpy().T, host)


@pytest.mark.parametrize("sd,n,leaf", [(1, 16384, 128), (3, 4096, 128)])
def test_gpu_3d_ellipsoid_against_oracle_and_field(pkg, oracle_mod, sd, n, leaf):
    """3D Laplace / Stokes on the ellipsoid (1, 0.7, 0.5): octree, row-sum
    diagonals (Kernel::compute_diag_entries_3dlaplace/_3dstokes,
    kern_interp/kernel/kernel.cpp:124-301), 32-point proxy sphere.  Bars: the
    solution within 10 tol of the oracle, identical tree statistics, the
    dense FP64 backward error within 50 tol, and the interior field as close
    to the exterior source's as the oracle's own solution gets (the 3D
    Nystrom discretization, not the solver, limits that error)."""
    g = pkg.geometry
    prob = g.ellipsoid(n)
    tol = 1e-6
    if sd == 1:
        src = np.array([[2.0, 1.0, 1.0], [-1.5, 2.0, 0.5]])
        f = g.laplace3_source_rhs(prob, src)
    else:
        src, frc = np.array([[2.0, 1.0, 1.0]]), np.array([[1.0, 0.5, -0.3]])
        f = g.stokes3_rhs(prob, src, frc)
    pde = pkg.PDE_LAPLACE if sd == 1 else pkg.PDE_STOKES
    ref, _, st = oracle_mod.solve(prob, f, tol, threads=16, leaf=leaf, solution_dim=sd, pde=pde)
    fac = pkg.Factor(prob.points, prob.normals, prob.weights, None, id_tol=tol,
                     solution_dimension=sd, pde=pde, max_leaf_dofs=leaf)
    mu = fac.solve(f)
    assert rel_max(mu, ref) <= 10 * tol
    info = fac.info()
    assert (info["n_levels"], info["n_root"], info["n_compressed"], info["n_redundant"]) == \
        (st["levels"], st["root"], st["compressed"], st["redundant"])
    res = np.abs(fac.apply(mu) - f).max() / np.abs(f).max()
    assert res <= 50 * tol, res
    rng = np.random.default_rng(5)
    tg = g.ellipsoid_targets(16, rng)
    if sd == 1:
        ue = g.laplace3_source_field(tg, src)
    else:
        ue = np.stack([g.stokeslet3_velocity(tg, y, fr).reshape(-1) for y, fr in zip(src, frc)], 1)
    err = np.abs(fac.eval_targets(tg, mu) - ue).max()
    err_ref = np.abs(fac.eval_targets(tg, ref) - ue).max()
    assert err <= 1.5 * err_ref + 10 * tol * np.abs(ue).max(), (err, err_ref)


def test_gpu_wide_path_many_boxes_matches_oracle(pkg, oracle_mod, monkeypatch):
    """Every box through the wide path on a tree with more wide boxes per
    level than the GPU holds resident CTAs: the cooperative panel QR then
    runs in several launches per panel (batches of boxes)."""
    monkeypatch.setenv("KI_WIDE_ROWS", "0")
    g = pkg.geometry
    prob = g.disc_with_ellipses(1 << 16, 16, seed=5)
    f = g.laplace_source_rhs(prob, np.array([[3.0, 1.0]]))
    tol = 1e-8
    ref, al_ref, st = oracle_mod.solve(prob, f, tol, threads=16)
    fac = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, id_tol=tol,
                     hole_centers=prob.hole_centers, hole_start=prob.hole_start,
                     hole_count=prob.hole_count)
    mu, al = fac.solve(f)
    paths = [lv["paths"] for lv in fac.profile()["levels"]]
    info = fac.info()
    fac.close()
    assert max(p[2] + p[3] for p in paths) > 350, paths   # GB300: 304 resident CTAs
    assert rel_max(mu, ref) <= 10 * tol
    assert abs(info["n_compressed"] - st["compressed"]) <= 0.01 * st["compressed"]
