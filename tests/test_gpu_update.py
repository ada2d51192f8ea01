"""Re-factorization after a boundary perturbation (ki_factor_update: the
reference's QuadTree::perturb, kern_interp/quadtree/quadtree.cpp:581-890,
then skeletonize over the boxes still compressed,
kern_interp/skel_factorization/skel_factorization.cpp:199-208).

Checked the way the reference's updating test checks it
(SphereUpdateLosesNoAcc, kern_interp/kern_interp_test.cpp:424-465: the
updated factorization's solution against a fresh factorization's of the same
boundary, relative difference <= 50 id_tol), on frames that move one hole as
the reference's updating experiments do.  Besides: an update that changes
nothing copies every box below the top levels and reproduces the original
solution bit for bit; a boundary of another size is factorized from scratch;
a failed update leaves the handle's factorization in place."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _holes(prob):
    if not prob.n_holes:
        return {}
    return dict(hole_centers=prob.hole_centers, hole_start=prob.hole_start,
                hole_count=prob.hole_count)


def _arrays(prob):
    return (prob.points, prob.normals, prob.weights, prob.curvatures)


def _stack(sol):
    if isinstance(sol, tuple):
        return np.concatenate([sol[0].reshape(-1), sol[1].reshape(-1)])
    return sol.reshape(-1)


def _case(pkg, name):
    g = pkg.geometry
    if name == "laplace_holes":
        prob = g.disc_with_ellipses(1 << 15, 12, seed=3)
        kw = dict(id_tol=1e-8)
        rhs = g.laplace_source_rhs(prob, g.random_sources(2, np.random.default_rng(1)))
        move = (0, (0.004, -0.003))
    elif name == "stokes_holes":
        prob = g.disc_with_circles(1 << 13, 10, seed=2)
        kw = dict(id_tol=1e-8, solution_dimension=2, pde=pkg.PDE_STOKES)
        rhs = np.random.default_rng(4).standard_normal((2 * prob.n, 2))
        move = (3, (0.002, 0.001))
    else:   # laplace3d_holes
        prob = g.spheres_with_holes(8192, [((0.3, 0.0, 0.0), 0.15, 2048),
                                           ((-0.45, 0.1, 0.0), 0.1, 1024)])
        kw = dict(id_tol=1e-6, max_leaf_dofs=128)
        rhs = np.random.default_rng(5).standard_normal((prob.n, 2))
        move = (1, (0.0, 0.02, 0.0))
    return prob, kw, rhs, move


@pytest.mark.parametrize("name", ["laplace_holes", "stokes_holes", "laplace3d_holes"])
def test_update_matches_fresh_factorization(pkg, name):
    prob, kw, rhs, (h, delta) = _case(pkg, name)
    moved = pkg.geometry.move_hole(prob, h, delta)
    fac = pkg.Factor(*_arrays(prob), **kw, **_holes(prob))
    n_comp0 = fac.info()["n_compressed"]
    kept = fac.update(*_arrays(moved), **_holes(moved))
    upd = _stack(fac.solve(rhs))
    info = fac.info()
    fac.close()
    fresh_f = pkg.Factor(*_arrays(moved), **kw, **_holes(moved))
    fresh = _stack(fresh_f.solve(rhs))
    finfo = fresh_f.info()
    fresh_f.close()
    # the perturbation is local: most boxes keep their factors, some do not
    assert 0 < kept < n_comp0, (kept, n_comp0)
    assert info["n_reused"] == kept and finfo["n_reused"] == 0
    assert info["n_dofs"] == finfo["n_dofs"] and info["n_levels"] == finfo["n_levels"]
    # the reference's criterion (kern_interp_test.cpp:459-463)
    rel = np.linalg.norm(upd - fresh) / np.linalg.norm(fresh)
    assert rel <= 50 * kw["id_tol"], rel


@pytest.mark.parametrize("name", ["laplace_holes", "laplace3d_holes"])
def test_update_without_change_is_bitwise(pkg, name):
    prob, kw, rhs, _ = _case(pkg, name)
    fac = pkg.Factor(*_arrays(prob), **kw, **_holes(prob))
    before = _stack(fac.solve(rhs))
    n_comp = fac.info()["n_compressed"]
    kept = fac.update(*_arrays(prob), **_holes(prob))
    after = _stack(fac.solve(rhs))
    info = fac.info()
    fac.close()
    # every compressed box below the levels whose ID reads the whole level
    assert kept > 0.8 * n_comp, (kept, n_comp)
    assert info["n_compressed"] == n_comp
    np.testing.assert_array_equal(after, before)


def test_update_of_another_size_starts_afresh(pkg):
    g = pkg.geometry
    a = g.star(512, 16)
    b = g.star(640, 16)
    rhs = g.laplace_source_rhs(b, g.random_sources(2, np.random.default_rng(2)))
    fac = pkg.Factor(*_arrays(a), id_tol=1e-10)
    assert fac.update(*_arrays(b)) == 0
    x = fac.solve(rhs)
    assert fac.n_dofs == b.n
    fac.close()
    ref = pkg.Factor(*_arrays(b), id_tol=1e-10)
    y = ref.solve(rhs)
    ref.close()
    np.testing.assert_array_equal(x, y)


def test_failed_update_keeps_the_factorization(pkg):
    g = pkg.geometry
    prob = g.disc_with_ellipses(1 << 13, 4, seed=5)
    rhs = g.laplace_source_rhs(prob, g.random_sources(1, np.random.default_rng(3)))
    fac = pkg.Factor(*_arrays(prob), id_tol=1e-8, **_holes(prob))
    before = _stack(fac.solve(rhs))
    bad = prob.points.copy()
    bad[7, 0] = np.nan
    with pytest.raises(pkg.KiError):
        fac.update(bad, prob.normals, prob.weights, prob.curvatures, **_holes(prob))
    after = _stack(fac.solve(rhs))
    fac.close()
    np.testing.assert_array_equal(after, before)


def test_update_fp32_refined_at_headline_size(pkg):
    """The 262,144-node disc with 64 holes in the mixed-precision form (FP32
    factorization with the learned rank model, refinement to 1e-8): one hole
    moved, the updated factorization's refined solution against a fresh one's."""
    g = pkg.geometry
    prob = g.disc_with_ellipses(1 << 18, 64, seed=1)
    moved = g.move_hole(prob, 17, (0.005, 0.0))
    rhs = g.laplace_source_rhs(moved, g.random_sources(4, np.random.default_rng(7)))
    kw = dict(id_tol=1e-6, precision=pkg.PRECISION_FP32, rank_model="default")
    fac = pkg.Factor(*_arrays(prob), **kw, **_holes(prob))
    n_comp0 = fac.info()["n_compressed"]
    kept = fac.update(*_arrays(moved), **_holes(moved))
    mu, al, ri = fac.solve_refined(rhs, tol=1e-8)
    fac.close()
    fresh_f = pkg.Factor(*_arrays(moved), **kw, **_holes(moved))
    mu2, al2, ri2 = fresh_f.solve_refined(rhs, tol=1e-8)
    fresh_f.close()
    assert kept > 0.5 * n_comp0, (kept, n_comp0)
    assert ri["residual"] <= 1e-8 and ri2["residual"] <= 1e-8
    a = np.concatenate([mu.reshape(-1), al.reshape(-1)])
    b = np.concatenate([mu2.reshape(-1), al2.reshape(-1)])
    assert np.linalg.norm(a - b) / np.linalg.norm(b) <= 1e-6


@pytest.mark.parametrize("name", ["update_disc6_8k", "update_stokes_circles_4k"])
def test_update_matches_reference_update_fixture(pkg, golden_updates, name):
    """Frame after frame through ki_factor_update against the reference's
    own runs on the same frames: its fresh factorization of each frame to the
    fixtures' usual 10 id_tol, and its incremental one (QuadTree::perturb +
    skeletonize) within its updating test's 50 id_tol."""
    frames, rhs, p, data = golden_updates[name]
    kw = dict(id_tol=p["tol"], solution_dimension=p["solution_dim"], pde=p["pde"])
    fac = pkg.Factor(*_arrays(frames[0]), **kw, **_holes(frames[0]))
    for f, prob in enumerate(frames):
        if f > 0:
            assert fac.update(*_arrays(prob), **_holes(prob)) > 0
        mu, alpha = fac.solve(rhs)
        ref = data["mu_fresh"][f]
        scale = np.abs(ref).max()
        assert np.abs(mu[:, 0] - ref).max() <= 10 * p["tol"] * scale, f
        assert np.abs(alpha[:, 0] - data["alpha_fresh"][f]).max() <= 10 * p["tol"] * scale, f
        ours = np.concatenate([mu[:, 0], alpha[:, 0]])
        inc = np.concatenate([data["mu_update"][f], data["alpha_update"][f]])
        assert np.linalg.norm(ours - inc) / np.linalg.norm(inc) <= 50 * p["tol"], f
    fac.close()
