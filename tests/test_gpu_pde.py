"""The other scalar 2D kernels of the reference (Kernel::Pde LAPLACE_NEUMANN
and GAUSS, kern_interp/kernel/kernel.cpp:44-60) through the C ABI: the CUDA
factor + solve against the reference's own outputs (golden fixtures), the
Neumann density's single-layer field against the analytic one, the
Gaussian kernel's proxy rings, FP32 factorizations refined against the FP64
operator, and the reference's handling of holes (none: no border)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NEUMANN, GAUSS = 1, 2


def _factor(pkg, prob, p, precision=0, **kw):
    return pkg.Factor(prob.points, prob.normals, prob.weights, prob.curvatures, id_tol=p["tol"],
                      pde=p["pde"], hole_centers=prob.hole_centers if prob.n_holes else None,
                      hole_start=prob.hole_start if prob.n_holes else None,
                      hole_count=prob.hole_count if prob.n_holes else None,
                      precision=precision, **kw)


def _dense(prob, pde):
    """The reference's dense matrix (Kernel::operator(), not forward)."""
    d = prob.points[:, None, :] - prob.points[None, :, :]
    r2 = (d ** 2).sum(-1)
    np.fill_diagonal(r2, 1.0)
    if pde == NEUMANN:
        w = prob.weights
        K = w[None, :] + w[None, :] / (2 * np.pi) * (d * prob.normals[:, None, :]).sum(-1) / r2
        np.fill_diagonal(K, w - 0.5 + 0.5 * prob.curvatures * w / (2 * np.pi))
    else:
        K = np.exp(-r2)
        np.fill_diagonal(K, 5.0)
    return K


@pytest.mark.parametrize("name", ["neumann_star_2048", "neumann_disc_circles_2048",
                                  "gauss_uniform_4096"])
def test_matches_reference_fixture(pkg, golden_cases, name):
    prob, rhs, p, data, h = golden_cases[name]
    assert str(data["input_sha1"]) == h
    fac = _factor(pkg, prob, p)
    mu = fac.solve(rhs)
    # no border for these kernels, whatever holes the boundary has
    assert not isinstance(mu, tuple) and fac.n_border == 0
    ref = data["mu"]
    assert np.abs(mu - ref).max() <= 10 * p["tol"] * np.abs(ref).max()
    info = fac.info()
    assert info["n_levels"] == int(data["levels"])
    assert info["n_root"] == int(data["root"])
    assert info["n_compressed"] == int(data["compressed"])
    assert info["n_redundant"] == int(data["redundant"])


def test_neumann_field_matches_the_analytic_one(pkg, golden_cases):
    """Interior Neumann problem on the star with the normal derivative of
    log|x - y| / (2 pi) (sources outside): the single-layer potential of the
    density (the forward kernel, w/(2 pi) log|r|) equals the field up to a
    constant, so differences between interior points agree."""
    prob, rhs, p, data, _ = golden_cases["neumann_star_2048"]
    g = pkg.geometry
    fac = _factor(pkg, prob, p)
    mu = fac.solve(rhs[:, 0])
    rng = np.random.default_rng(4)
    tg = g.disc_targets(60, rng, radius=0.45)
    u = fac.eval_targets(tg, mu)
    exact = g.laplace_source_field(tg, np.array([[3.0, 1.0]]))[:, 0]   # column 0's source
    err = np.abs((u - u[0]) - (exact - exact[0])).max() / np.abs(exact - exact[0]).max()
    assert err <= 1e-8, err


@pytest.mark.parametrize("pde", [NEUMANN, GAUSS])
def test_fp32_factorization_refined_to_the_fp64_operator(pkg, golden_cases, pde):
    """FP32 factorization at ID tol 1e-6 as the preconditioner, refined
    against the dense FP64 operator (these kernels have no FMM) to 1e-11:
    the FP64 reference solution to 1e-9."""
    name = "neumann_star_2048" if pde == NEUMANN else "gauss_uniform_4096"
    prob, rhs, p, data, _ = golden_cases[name]
    fac = _factor(pkg, prob, dict(p, tol=1e-6), precision=pkg.PRECISION_FP32)
    mu, info = fac.solve_refined(rhs, tol=1e-11, max_steps=20)
    assert info["residual"] <= 1e-11, info
    K = _dense(prob, pde)
    x = np.linalg.solve(K, rhs)
    assert np.abs(mu - x).max() <= 1e-9 * np.abs(x).max()


def test_operator_apply_matches_the_dense_matrix(pkg, golden_cases):
    """ki_apply (the refinement's residual operator) for both kernels against
    the reference's dense matrix."""
    for name, pde in (("neumann_disc_circles_2048", NEUMANN), ("gauss_uniform_4096", GAUSS)):
        prob, rhs, p, data, _ = golden_cases[name]
        fac = _factor(pkg, prob, p)
        x = np.random.default_rng(1).standard_normal((prob.n, 2))
        y = fac.apply(x)
        ref = _dense(prob, pde) @ x
        assert np.abs(y - ref).max() <= 1e-12 * np.abs(ref).max(), name


def test_gauss_accepts_absent_normals_and_weights(pkg, golden_cases):
    """The Gaussian kernel reads neither: NULL normals and weights factor to
    the same solution as the reference's zero arrays."""
    prob, rhs, p, data, _ = golden_cases["gauss_uniform_4096"]
    fac = pkg.Factor(prob.points, None, None, None, id_tol=p["tol"], pde=GAUSS)
    mu = fac.solve(rhs)
    assert np.abs(mu - data["mu"]).max() <= 10 * p["tol"] * np.abs(data["mu"]).max()
