"""The CPU oracle (C++ restatement of the reference factor/solve) pinned
against the golden fixtures produced by the reference itself."""
import os

import numpy as np
import pytest


def test_golden_inputs_intact(golden_cases):
    for name, (prob, rhs, p, data, h) in golden_cases.items():
        assert str(data["input_sha1"]) == h, "fixture inputs corrupted: " + name


def test_generators_reproduce_fixture_inputs(golden_cases, pkg):
    """The seeded generators still produce the fixtures' boundaries (to
    rounding: libm differs across CPU architectures)."""
    g = pkg.geometry
    prob, src, _ = g.star_c1()
    fp = golden_cases["star_c1"][0]
    np.testing.assert_allclose(prob.points, fp.points, rtol=0, atol=1e-13)
    np.testing.assert_allclose(prob.weights, fp.weights, rtol=1e-12)


@pytest.mark.parametrize("name", ["star_c1", "star_1024_default", "circle_1000",
                                  "star_2048_tol1e-4", "star_64_root_leaf", "disc6_8k",
                                  "stokes_star_2048", "laplace3_ellipsoid_3000",
                                  "stokes3_ellipsoid_1500", "laplace3_sphere_hole",
                                  "stokes3_sphere_hole", "neumann_star_2048",
                                  "neumann_disc_circles_2048", "gauss_uniform_4096"])
def test_port_matches_reference_fixture(golden_cases, oracle_mod, name):
    prob, rhs, p, data, _ = golden_cases[name]
    mu, alpha, st = oracle_mod.solve(prob, rhs, p["tol"], threads=4, leaf=p["leaf"],
                                     proxy=p["proxy"], ratio=p["ratio"],
                                     min_compress=p["min_compress"],
                                     solution_dim=p["solution_dim"], pde=p["pde"])
    ref = data["mu"]
    # same tree, same LAPACK calls on identically ordered matrices: agreement to
    # rounding, far inside the 10 x id_tol solution tolerance
    assert np.abs(mu - ref).max() <= 1e-9 * np.abs(ref).max()
    assert st["levels"] == int(data["levels"])
    assert st["root"] == int(data["root"])
    assert st["compressed"] == int(data["compressed"])
    assert st["redundant"] == int(data["redundant"])
    if alpha.size:
        assert np.abs(alpha - data["alpha"]).max() <= 1e-9 * max(1.0, np.abs(data["alpha"]).max())


def test_update_fixture_inputs_intact(golden_updates):
    import make_golden
    for name, (frames, rhs, p, data) in golden_updates.items():
        assert str(data["input_sha1"]) == make_golden.input_hash(frames[0], rhs), name
        # each frame moves exactly one hole's nodes
        for f in range(1, len(frames)):
            moved = np.any(frames[f].points != frames[f - 1].points, axis=1)
            h = int(data["move_hole"][f - 1])
            s, c = int(data["hole_start"][h]), int(data["hole_count"][h])
            assert moved[s:s + c].all() and moved.sum() == c


@pytest.mark.parametrize("name", ["update_disc6_8k", "update_stokes_circles_4k"])
def test_port_matches_reference_update_fixture(golden_updates, oracle_mod, name):
    """The oracle's fresh factorization of every perturbed frame against the
    reference's fresh one (to rounding), and the reference's own incremental
    re-factorization (QuadTree::perturb + skeletonize) within its updating
    test's bound of the fresh one (50 id_tol,
    kern_interp/kern_interp_test.cpp:459-463)."""
    frames, rhs, p, data = golden_updates[name]
    for f, prob in enumerate(frames):
        mu, alpha, _ = oracle_mod.solve(prob, rhs, p["tol"], threads=4,
                                        solution_dim=p["solution_dim"], pde=p["pde"])
        ref = data["mu_fresh"][f]
        assert np.abs(mu[:, 0] - ref).max() <= 1e-9 * np.abs(ref).max(), f
        assert np.abs(alpha[:, 0] - data["alpha_fresh"][f]).max() <= 1e-9 * np.abs(ref).max(), f
        inc = np.concatenate([data["mu_update"][f], data["alpha_update"][f]])
        fresh = np.concatenate([ref, data["alpha_fresh"][f]])
        assert np.linalg.norm(inc - fresh) / np.linalg.norm(fresh) <= 50 * p["tol"], f


def test_port_pde_error_star(golden_cases, oracle_mod, pkg):
    """Interior field of an exterior source recovered to ~1e-12 (the reference's
    analytic-agreement tests, kern_interp/kern_interp_test.cpp:171-190)."""
    prob, src, tg = pkg.geometry.star_c1()
    f = pkg.geometry.laplace_source_rhs(prob, src)
    mu, _, _ = oracle_mod.solve(prob, f, 1e-10, threads=4, proxy=64, ratio=1.5 / np.sqrt(2))
    u = oracle_mod.laplace_forward(prob, tg, mu)
    ue = pkg.geometry.laplace_source_field(tg, src)
    assert np.abs(u - ue).max() <= 1e-10 * np.abs(ue).max()


def test_port_dense_residual(oracle_mod, pkg):
    """Backward error of the compressed solve against the dense Nystrom matrix
    (solve_err, kern_interp/linear_solve.cpp:339-426): <= 50 id_tol."""
    prob = pkg.geometry.star(32, 16)
    f = pkg.geometry.laplace_source_rhs(prob, np.array([[3.0, 3.0]]))
    tol = 1e-6
    mu, _, _ = oracle_mod.solve(prob, f, tol, threads=2)
    K = oracle_mod.dense_matrix(prob)
    r = K @ mu - f
    assert np.linalg.norm(r) / np.linalg.norm(f) <= 50 * tol


def test_port_neumann_field_and_gauss_backward_error(oracle_mod, pkg):
    """The other scalar kernels in the port, pinned by the physics and by
    dense algebra rather than by the reference alone.  Neumann
    (Kernel::one_d_kern, kernel.cpp:44-54): the single-layer field of the
    density solves the interior Neumann problem of an exterior source, so
    differences of the field at interior points match the source's field.
    Gauss (:55-60, three proxy rings :661-672): the compressed solve's
    backward error against the dense covariance matrix (exp(-r^2), 5 on the
    diagonal) <= 50 id_tol."""
    g = pkg.geometry
    prob = g.star(64, 16)
    src = np.array([[3.0, 1.0]])
    f = g.laplace_neumann_rhs(prob, src)
    mu, alpha, _ = oracle_mod.solve(prob, f, 1e-10, threads=2, pde=1)
    assert alpha.size == 0
    tg = g.disc_targets(40, np.random.default_rng(4), radius=0.45)
    d = tg[:, None, :] - prob.points[None]
    u = (prob.weights[None] / (2 * np.pi) * np.log(np.sqrt((d ** 2).sum(-1)))) @ mu[:, 0]
    ue = g.laplace_source_field(tg, src)[:, 0]
    err = np.abs((u - u[0]) - (ue - ue[0])).max() / np.abs(ue - ue[0]).max()
    assert err <= 1e-8, err

    grid = g.uniform_grid(1024)
    b = np.random.default_rng(7).standard_normal((grid.n, 1))
    tol = 1e-6
    x, _, _ = oracle_mod.solve(grid, b, tol, threads=2, pde=2)
    r2 = ((grid.points[:, None, :] - grid.points[None, :, :]) ** 2).sum(-1)
    K = np.exp(-r2)
    np.fill_diagonal(K, 5.0)
    assert np.linalg.norm(K @ x - b) / np.linalg.norm(b) <= 50 * tol


def test_reference_matches_port_random_star(oracle_mod, pkg):
    """Where the reference tree is present, the compiled reference and the port
    agree on a freshly generated boundary (not a stored fixture)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "_ki_build_ref", os.path.join(os.path.dirname(oracle_mod.__file__), "build_ref.py"))
    br = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(br)
    if not br.reference_present():
        pytest.skip("reference sources not present")
    prob = pkg.geometry.star(96, 16, amp=0.25, k=4)
    f = pkg.geometry.laplace_source_rhs(prob, np.array([[-2.5, 1.5]]))
    a, _, sa = oracle_mod.solve(prob, f, 1e-9, threads=4, impl="ref")
    b, _, sb = oracle_mod.solve(prob, f, 1e-9, threads=4, impl="port")
    assert np.abs(a - b).max() <= 1e-10 * np.abs(a).max()
    assert sa["root"] == sb["root"]



def _border_dense(prob, sd):
    """U (N x n_border) and Psi (n_border x N) of a 2D multiply connected
    boundary, restated in numpy from initialize_U_mat / initialize_Psi_mat
    (kern_interp/linear_solve.cpp:37-45, 77-97, 131-143, 164-177)."""
    n, H = prob.n, prob.n_holes
    N = n * sd
    c = 1 if sd == 1 else 3
    U = np.zeros((N, c * H))
    Psi = np.zeros((c * H, N))
    for h in range(H):
        rx = prob.points[:, 0] - prob.hole_centers[h, 0]
        ry = prob.points[:, 1] - prob.hole_centers[h, 1]
        r2 = rx * rx + ry * ry
        s0, n0 = prob.hole_start[h], prob.hole_count[h]
        w = prob.weights[s0:s0 + n0]
        if sd == 1:
            U[:, h] = 0.5 * np.log(r2)
            Psi[h, s0:s0 + n0] = w
            continue
        sc = 1.0 / (4 * np.pi)
        lg = -0.5 * np.log(r2)
        U[0::2, 3 * h] = sc * (lg + rx * rx / r2)
        U[1::2, 3 * h] = sc * (rx * ry / r2)
        U[0::2, 3 * h + 1] = sc * (rx * ry / r2)
        U[1::2, 3 * h + 1] = sc * (lg + ry * ry / r2)
        U[0::2, 3 * h + 2] = ry * sc / r2
        U[1::2, 3 * h + 2] = -rx * sc / r2
        Psi[3 * h, 2 * s0:2 * (s0 + n0):2] = w
        Psi[3 * h + 1, 2 * s0 + 1:2 * (s0 + n0):2] = w
        Psi[3 * h + 2, 2 * s0:2 * (s0 + n0):2] = w * prob.points[s0:s0 + n0, 1]
        Psi[3 * h + 2, 2 * s0 + 1:2 * (s0 + n0):2] = -w * prob.points[s0:s0 + n0, 0]
    return U, Psi


@pytest.mark.parametrize("kind", ["laplace2d_holes", "stokes2d_holes", "laplace3d"])
def test_port_residual_rows_match_dense(oracle_mod, pkg, kind):
    """kiport_residual_rows (the residual check used at sizes where the dense
    operator does not fit) equals the dense bordered residual
    [K U; Psi -I][mu; alpha] - [f; 0] on the rows asked for."""
    g = pkg.geometry
    rng = np.random.default_rng(5)
    sd = 1
    if kind == "laplace2d_holes":
        prob = g.disc_with_ellipses(1024, 3, seed=7)
    elif kind == "stokes2d_holes":
        prob, sd = g.disc_with_circles(512, 3, seed=7), 2
    else:
        prob = g.ellipsoid(800)
    N = prob.n * sd
    K = oracle_mod.dense_matrix(prob, solution_dim=sd)
    if kind == "laplace3d":
        U, Psi = np.zeros((N, 0)), np.zeros((0, N))
    else:
        U, Psi = _border_dense(prob, sd)
    nb = U.shape[1]
    mu = rng.standard_normal((N, 3))
    alpha = rng.standard_normal((nb, 3))
    f = rng.standard_normal((N, 3))
    rows = np.sort(rng.choice(N, 40, replace=False))
    res, res_b = oracle_mod.residual_rows(prob, mu, alpha, f, rows, solution_dim=sd, threads=4)
    full = K @ mu + U @ alpha - f
    np.testing.assert_allclose(res, full[rows], rtol=0, atol=1e-12 * np.abs(full).max())
    if nb:
        np.testing.assert_allclose(res_b, Psi @ mu - alpha, rtol=0, atol=1e-12 * np.abs(alpha).max())
