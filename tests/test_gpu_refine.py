"""Mixed precision: the FP32 factorization as the approximate inverse of an
iterative refinement whose residual is the FP64 operator (ki_solve_refined).
The refined solution is checked against a dense FP64 LU solve of the same
(bordered) Nystrom system -- the exact discrete solution, which the FP64
skeletonization itself only reaches to within its ID tolerance."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bordered_dense(oracle_mod, pkg, prob, sd):
    """[K U; Psi -I] with K from the oracle and U / Psi as the reference
    builds them (kern_interp/linear_solve.cpp:19-199), 2D."""
    K = oracle_mod.dense_matrix(prob, sd)
    if not prob.n_holes:
        return K
    N = K.shape[0]
    c = 1 if sd == 1 else 3
    nb = c * prob.n_holes
    U = np.zeros((N, nb))
    Psi = np.zeros((nb, N))
    for h in range(prob.n_holes):
        r = prob.points - prob.hole_centers[h]
        rn = np.hypot(r[:, 0], r[:, 1])
        s = slice(int(prob.hole_start[h]), int(prob.hole_start[h] + prob.hole_count[h]))
        w = prob.weights[s]
        if sd == 1:
            U[:, h] = np.log(rn)
            Psi[h, s] = w
        else:
            sc = 1 / (4 * np.pi)
            U[0::2, 3 * h] = sc * (np.log(1 / rn) + r[:, 0] ** 2 / rn ** 2)
            U[1::2, 3 * h] = sc * r[:, 1] * r[:, 0] / rn ** 2
            U[0::2, 3 * h + 1] = sc * r[:, 0] * r[:, 1] / rn ** 2
            U[1::2, 3 * h + 1] = sc * (np.log(1 / rn) + r[:, 1] ** 2 / rn ** 2)
            U[0::2, 3 * h + 2] = r[:, 1] * sc / rn ** 2
            U[1::2, 3 * h + 2] = -r[:, 0] * sc / rn ** 2
            idx = np.arange(s.start, s.stop)
            Psi[3 * h, 2 * idx] = w
            Psi[3 * h + 1, 2 * idx + 1] = w
            Psi[3 * h + 2, 2 * idx] = w * prob.points[s, 1]
            Psi[3 * h + 2, 2 * idx + 1] = -w * prob.points[s, 0]
    return np.block([[K, U], [Psi, -np.eye(nb)]])


@pytest.mark.parametrize("case", ["star", "holes", "stokes_holes"])
def test_fp32_factor_refined_to_fp64_solution(pkg, oracle_mod, case):
    g = pkg.geometry
    sd, pde, kw = 1, pkg.PDE_LAPLACE, {}
    if case == "star":
        prob = g.star(256, 16)
        f = g.laplace_source_rhs(prob, np.array([[3.0, 3.0], [-2.0, 3.5]]))
    elif case == "holes":
        prob = g.disc_with_ellipses(1 << 13, 6, seed=5)
        f = g.laplace_source_rhs(prob, g.random_sources(3, np.random.default_rng(1)))
    else:
        sd, pde = 2, pkg.PDE_STOKES
        prob = g.disc_with_circles(1 << 11, 3, seed=3)
        src, frc = g.stokes_c3_sources(2)
        f = g.stokes_rhs(prob, src, frc)
    if prob.n_holes:
        kw = dict(hole_centers=prob.hole_centers, hole_start=prob.hole_start,
                  hole_count=prob.hole_count)
    fac = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, id_tol=1e-6,
                     solution_dimension=sd, pde=pde, precision=pkg.PRECISION_FP32, **kw)
    out = fac.solve_refined(f, tol=1e-12, max_steps=20)
    info = out[-1]
    mu = out[0]
    # the FP32 factorization alone is an approximate inverse to ~1e-5
    assert info["residual0"] < 1e-3, info
    assert info["residual"] <= 1e-12, info
    A = bordered_dense(oracle_mod, pkg, prob, sd)
    nb = A.shape[0] - f.shape[0]
    xd = np.linalg.solve(A, np.vstack([f, np.zeros((nb, f.shape[1]))]))
    x = np.vstack([mu, out[1]]) if nb else mu
    err = np.abs(x - xd).max() / np.abs(xd).max()
    cond_bound = 1e-12 * (1e7 if sd == 2 else 1e3)     # Stokes bordered: cond ~ 2.4e6
    assert err <= cond_bound, (err, info)


def test_fp64_factor_one_refinement_step(pkg):
    """The plain FP64 factorization at ID tolerance 1e-8 leaves a residual of
    a few 1e-8; one refinement step takes it below 1e-12."""
    g = pkg.geometry
    prob = g.star(256, 16)
    f = g.laplace_source_rhs(prob, np.array([[3.0, 3.0]]))
    fac = pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, id_tol=1e-8)
    mu, info = fac.solve_refined(f, tol=1e-12, max_steps=3)
    assert 1e-11 < info["residual0"] < 1e-6, info
    assert info["residual"] <= 1e-12 and info["steps"] <= 2, info


def test_refined_3d_and_device_entry(pkg):
    import torch
    g = pkg.geometry
    prob = g.ellipsoid(4096)
    f = g.laplace3_source_rhs(prob, np.array([[2.0, 1.0, 1.0], [-1.5, 2.0, 0.5]]))
    fac = pkg.Factor(prob.points, prob.normals, prob.weights, None, id_tol=1e-5,
                     precision=pkg.PRECISION_FP32, max_leaf_dofs=128)
    mu, info = fac.solve_refined(f, tol=1e-11, max_steps=20)
    assert info["residual"] <= 1e-11, info
    d_b = torch.from_numpy(np.asfortranarray(f).T.copy()).cuda()
    d_x = torch.zeros_like(d_b)
    info2 = fac.solve_refined_device(d_b.data_ptr(), d_x.data_ptr(), 2, tol=1e-11, max_steps=20)
    torch.cuda.synchronize()
    x2 = d_x.cpu().numpy().T
    assert info2["steps"] == info["steps"]
    assert np.abs(x2 - mu).max() <= 1e-14 * np.abs(mu).max()
    res = np.abs(fac.apply(mu) - f).max() / np.abs(f).max()
    assert res <= 1e-10


def test_3d_laplace_apply_in_pair_arithmetic_matches_the_fp64_matrix(pkg, oracle_mod):
    """The 3D Laplace residual operator runs in FP32-pair arithmetic (the FP32
    pipes, ~1e-13 per entry): against the FP64 dense matrix of the oracle
    (the same row-sum diagonal), on several right-hand sides."""
    g = pkg.geometry
    prob = g.ellipsoid(3000, (1.0, 0.7, 0.5))
    K = oracle_mod.dense_matrix(prob)
    fac = pkg.Factor(prob.points, prob.normals, prob.weights, None, id_tol=1e-6)
    x = np.random.default_rng(2).standard_normal((prob.n, 5))
    y = fac.apply(x)
    ref = K @ x
    assert np.abs(y - ref).max() <= 1e-11 * np.abs(ref).max(), np.abs(y - ref).max()
