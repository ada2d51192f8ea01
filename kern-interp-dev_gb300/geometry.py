"""Boundary discretizations and right-hand sides for the solver's workloads.

Every workload is a seeded synthetic boundary: Gauss-Legendre panel
quadrature on closed curves (the reference ships no panel boundary; its
Boundary subclasses fill the same public arrays, kern_interp/boundaries/
boundary.h:47-64: points and normals interleaved per node, weights,
curvatures, hole descriptors, boundary values).

Conventions follow the reference's circle/annulus boundaries
(kern_interp/boundaries/circle.cpp:8-32, annulus.cpp:8-58): the outer curve
has outward normals and positive curvature; each hole carries normals
pointing into the hole and negative curvature.
"""
from dataclasses import dataclass, field
import numpy as np


@dataclass
class Problem:
    points: np.ndarray            # (n, 2) node coordinates
    normals: np.ndarray           # (n, 2) unit normals
    weights: np.ndarray           # (n,) quadrature weights (arc length)
    curvatures: np.ndarray        # (n,) signed curvature
    hole_centers: np.ndarray = field(default_factory=lambda: np.zeros((0, 2)))
    hole_start: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    hole_count: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    name: str = ""

    @property
    def n(self):
        return self.points.shape[0]

    @property
    def n_holes(self):
        return self.hole_centers.shape[0]


def gauss_legendre(q):
    x, w = np.polynomial.legendre.leggauss(q)
    return x, w


def _panel_curve(fun, t_breaks, q):
    """Discretize a closed parametric curve z(t) with q-node GL panels whose
    parameter breakpoints are t_breaks (len = panels + 1).  fun(t) returns
    (z, dz, d2z) as complex arrays."""
    x, w = gauss_legendre(q)
    a, b = t_breaks[:-1], t_breaks[1:]
    half = 0.5 * (b - a)
    t = (0.5 * (a + b))[:, None] + half[:, None] * x[None, :]
    t = t.ravel()
    wt = (half[:, None] * w[None, :]).ravel()
    z, dz, d2z = fun(t)
    speed = np.abs(dz)
    tangent = dz / speed
    normal = -1j * tangent                  # outward for counter-clockwise curves
    kappa = np.imag(np.conj(dz) * d2z) / speed ** 3
    return z, normal, wt * speed, kappa


def _equal_arclength_breaks(fun, panels, oversample=64):
    """Parameter breakpoints on [0, 2pi] that split the curve into panels of
    equal arc length (monotone interpolation of a fine arc-length table)."""
    m = panels * oversample
    t = np.linspace(0.0, 2 * np.pi, m + 1)
    mid = 0.5 * (t[:-1] + t[1:])
    _, dz, _ = fun(mid)
    s = np.concatenate([[0.0], np.cumsum(np.abs(dz) * (t[1] - t[0]))])
    targets = np.linspace(0.0, s[-1], panels + 1)
    br = np.interp(targets, s, t)
    br[0], br[-1] = 0.0, 2 * np.pi
    return br


def star(panels=256, q=16, amp=0.3, k=5):
    """Star curve r(theta) = 1 + amp cos(k theta), equal-theta panels."""
    def fun(t):
        r = 1 + amp * np.cos(k * t)
        dr = -amp * k * np.sin(k * t)
        d2r = -amp * k * k * np.cos(k * t)
        e = np.exp(1j * t)
        z = r * e
        dz = (dr + 1j * r) * e
        d2z = (d2r + 2j * dr - r) * e
        return z, dz, d2z
    z, nrm, w, kap = _panel_curve(fun, np.linspace(0, 2 * np.pi, panels + 1), q)
    return Problem(np.stack([z.real, z.imag], 1), np.stack([nrm.real, nrm.imag], 1),
                   w, kap, name="star")


def circle(n, radius=0.25):
    """The reference's circle test boundary (kern_interp/boundaries/circle.cpp:8-32):
    n equispaced nodes, trapezoid weights."""
    ang = np.arange(n) * 2.0 * np.pi / n
    pts = np.stack([radius * np.cos(ang), radius * np.sin(ang)], 1)
    nrm = np.stack([np.cos(ang), np.sin(ang)], 1)
    return Problem(pts, nrm, np.full(n, 2 * np.pi * radius / n), np.full(n, 1.0 / radius),
                   name="circle")


def _ellipse_fun(c, a, b, phi):
    rot = np.exp(1j * phi)

    def fun(t):
        z = c + rot * (a * np.cos(t) + 1j * b * np.sin(t))
        dz = rot * (-a * np.sin(t) + 1j * b * np.cos(t))
        d2z = rot * (-a * np.cos(t) - 1j * b * np.sin(t))
        return z, dz, d2z
    return fun


def _ellipse_perimeter(a, b):
    h = ((a - b) / (a + b)) ** 2
    return np.pi * (a + b) * (1 + 3 * h / (10 + np.sqrt(4 - 3 * h)))


def sample_ellipses(n_holes, rng, axis_lo=0.02, axis_hi=0.06, r_max=1.8, gap=0.01,
                    max_tries=200000):
    """Non-overlapping ellipses: semi-axes U(axis_lo, axis_hi), uniform
    orientation, centres rejection-sampled in |x| < r_max with the bounding
    circles (major semi-axis) at least `gap` apart."""
    cs, ax, ph = [], [], []
    tries = 0
    while len(cs) < n_holes:
        tries += 1
        if tries > max_tries:
            raise RuntimeError("could not place %d holes" % n_holes)
        c = rng.uniform(-r_max, r_max, 2)
        if np.hypot(*c) >= r_max:
            continue
        a, b = rng.uniform(axis_lo, axis_hi, 2)
        phi = rng.uniform(0, 2 * np.pi)
        rad = max(a, b)
        ok = all(np.hypot(*(c - c2)) >= rad + max(a2) + gap for c2, a2 in zip(cs, ax))
        if ok:
            cs.append(c)
            ax.append((a, b))
            ph.append(phi)
    return np.array(cs), np.array(ax), np.array(ph)


def disc_with_ellipses(n_unknowns=1 << 20, n_holes=64, radius=2.0, seed=1, q=16):
    """Disc of radius `radius` minus `n_holes` ellipses, q-node GL panels with
    equal node density per unit arc length; n_unknowns must be a multiple of q."""
    rng = np.random.default_rng(seed)
    cs, ax, ph = sample_ellipses(n_holes, rng)
    lens = [2 * np.pi * radius] + [_ellipse_perimeter(a, b) for a, b in ax]
    lens = np.array(lens)
    total_panels = n_unknowns // q
    if total_panels * q != n_unknowns:
        raise ValueError("n_unknowns must be a multiple of q")
    raw = total_panels * lens / lens.sum()
    panels = np.maximum(np.floor(raw).astype(int), 2)
    rem = total_panels - panels.sum()
    order = np.argsort(-(raw - np.floor(raw)))
    i = 0
    while rem != 0:
        j = order[i % len(order)]
        if rem > 0:
            panels[j] += 1
            rem -= 1
        elif panels[j] > 2:
            panels[j] -= 1
            rem += 1
        i += 1

    def outer(t):
        e = np.exp(1j * t)
        return radius * e, 1j * radius * e, -radius * e
    pts, nrm, wts, kap = [], [], [], []
    z, n_, w, k = _panel_curve(outer, np.linspace(0, 2 * np.pi, panels[0] + 1), q)
    pts.append(z); nrm.append(n_); wts.append(w); kap.append(k)
    starts, counts = [], []
    off = z.size
    for h in range(n_holes):
        fun = _ellipse_fun(cs[h, 0] + 1j * cs[h, 1], ax[h, 0], ax[h, 1], ph[h])
        br = _equal_arclength_breaks(fun, panels[h + 1])
        z, n_, w, k = _panel_curve(fun, br, q)
        # holes: normals into the hole, negative curvature
        pts.append(z); nrm.append(-n_); wts.append(w); kap.append(-k)
        starts.append(off); counts.append(z.size)
        off += z.size
    z = np.concatenate(pts); n_ = np.concatenate(nrm)
    return Problem(np.stack([z.real, z.imag], 1), np.stack([n_.real, n_.imag], 1),
                   np.concatenate(wts), np.concatenate(kap),
                   hole_centers=cs.copy(), hole_start=np.array(starts, np.int32),
                   hole_count=np.array(counts, np.int32), name="disc_with_ellipses")


def move_hole(prob, h, delta):
    """The boundary with hole h translated by `delta` (its nodes and centre;
    normals, weights and curvatures unchanged), every other node bitwise as
    before and at the same index: a perturbation frame of the reference's
    updating experiments, which move one hole's centre per frame
    (kern_interp/boundaries/ex2boundary.cpp:39-56,
    kern_interp/experiments/experiment_two.cpp:54-60)."""
    s, c = int(prob.hole_start[h]), int(prob.hole_count[h])
    d = np.asarray(delta, np.float64)
    pts = prob.points.copy()
    pts[s:s + c] += d[None]
    cs = prob.hole_centers.copy()
    cs[h] += d
    return Problem(pts, prob.normals.copy(), prob.weights.copy(), prob.curvatures.copy(),
                   hole_centers=cs, hole_start=prob.hole_start.copy(),
                   hole_count=prob.hole_count.copy(), name=prob.name + "_moved")


def sample_circles(n_holes, rng, r_lo=0.005, r_hi=0.02, domain_radius=1.0, gap=0.005,
                   max_tries=2000000):
    """Non-overlapping circles with radii U(r_lo, r_hi), centres rejection-
    sampled inside the disc, pairwise and boundary gaps at least `gap`."""
    cs, rs = [], []
    tries = 0
    while len(cs) < n_holes:
        tries += 1
        if tries > max_tries:
            raise RuntimeError("could not place %d circles" % n_holes)
        r = rng.uniform(r_lo, r_hi)
        c = rng.uniform(-domain_radius, domain_radius, 2)
        if np.hypot(*c) + r + gap > domain_radius:
            continue
        if all(np.hypot(*(c - c2)) >= r + r2 + gap for c2, r2 in zip(cs, rs)):
            cs.append(c)
            rs.append(r)
    return np.array(cs), np.array(rs)


def disc_with_circles(n_points=1 << 18, n_holes=200, radius=1.0, seed=3, q=16):
    """Disc minus `n_holes` circular holes (radii U(0.005, 0.02), gap 0.005),
    q-node GL panels with equal node density per unit arc length."""
    rng = np.random.default_rng(seed)
    cs, rs = sample_circles(n_holes, rng, domain_radius=radius)
    lens = np.concatenate([[2 * np.pi * radius], 2 * np.pi * rs])
    total_panels = n_points // q
    if total_panels * q != n_points:
        raise ValueError("n_points must be a multiple of q")
    raw = total_panels * lens / lens.sum()
    panels = np.maximum(np.floor(raw).astype(int), 2)
    rem = total_panels - panels.sum()
    order = np.argsort(-(raw - np.floor(raw)))
    i = 0
    while rem != 0:
        j = order[i % len(order)]
        if rem > 0:
            panels[j] += 1
            rem -= 1
        elif panels[j] > 2:
            panels[j] -= 1
            rem += 1
        i += 1

    def circ(c, r):
        def fun(t):
            e = np.exp(1j * t)
            return c + r * e, 1j * r * e, -r * e
        return fun
    pts, nrm, wts, kap, starts, counts = [], [], [], [], [], []
    z, n_, w, k = _panel_curve(circ(0j, radius), np.linspace(0, 2 * np.pi, panels[0] + 1), q)
    pts.append(z); nrm.append(n_); wts.append(w); kap.append(k)
    off = z.size
    for h in range(n_holes):
        z, n_, w, k = _panel_curve(circ(cs[h, 0] + 1j * cs[h, 1], rs[h]),
                                   np.linspace(0, 2 * np.pi, panels[h + 1] + 1), q)
        pts.append(z); nrm.append(-n_); wts.append(w); kap.append(-k)
        starts.append(off); counts.append(z.size)
        off += z.size
    z = np.concatenate(pts); n_ = np.concatenate(nrm)
    prob = Problem(np.stack([z.real, z.imag], 1), np.stack([n_.real, n_.imag], 1),
                   np.concatenate(wts), np.concatenate(kap), hole_centers=cs.copy(),
                   hole_start=np.array(starts, np.int32), hole_count=np.array(counts, np.int32),
                   name="disc_with_circles")
    prob.hole_radii = rs
    return prob


def stokeslet_velocity(x, y0, force):
    """Velocity at points x of a 2D Stokeslet at y0 with force f (unit
    viscosity): (1/4pi) (-log|r| f + (r.f) r / |r|^2), r = x - y0 -- the
    kernel the reference's border matrix uses (kern_interp/linear_solve.cpp:77-97)."""
    r = x - np.asarray(y0)[None]
    r2 = (r ** 2).sum(1)
    f = np.asarray(force, np.float64)
    return (-0.5 * np.log(r2)[:, None] * f[None] + r * (r @ f)[:, None] / r2[:, None]) / (4 * np.pi)


def stokes_rhs(prob, sources, forces):
    """Boundary velocity (interleaved per node, one column per Stokeslet)."""
    cols = [stokeslet_velocity(prob.points, y, f).reshape(-1) for y, f in zip(sources, forces)]
    return np.stack(cols, 1)


def stokes_c3_sources(nrhs, seed=3):
    """The Stokeslet at (2.5, 0) with force (1, 0.5), then nrhs-1 seeded random
    ones at |y| in [2.5, 4] with unit forces."""
    rng = np.random.default_rng(seed + 1000)
    src = [np.array([2.5, 0.0])]
    frc = [np.array([1.0, 0.5])]
    for _ in range(nrhs - 1):
        src.append(random_sources(1, rng)[0])
        a = rng.uniform(0, 2 * np.pi)
        frc.append(np.array([np.cos(a), np.sin(a)]))
    return np.array(src), np.array(frc)


def laplace_source_rhs(prob, sources):
    """Boundary values of u(x) = log|x - y| / (2 pi) for each source y (one
    column per source), the field the reference's SINGLE_ELECTRON condition
    uses (kern_interp/boundaries/boundary.cpp:69-74)."""
    sources = np.atleast_2d(sources)
    d = prob.points[:, None, :] - sources[None, :, :]
    return np.log(np.hypot(d[..., 0], d[..., 1])) / (2 * np.pi)


def laplace_neumann_rhs(prob, sources):
    """Normal derivatives (along the boundary's normals) of u(x) = log|x - y|
    / (2 pi) for each source y (one column per source): the data of an
    interior Neumann problem whose solution is that field, up to a constant."""
    sources = np.atleast_2d(sources)
    d = prob.points[:, None, :] - sources[None, :, :]
    r2 = (d ** 2).sum(-1)
    return (d * prob.normals[:, None, :]).sum(-1) / r2 / (2 * np.pi)


def uniform_grid(n):
    """The reference's UniformDist point set (kern_interp/boundaries/
    uniformdist.cpp:8-19): ceil(sqrt(n))^2 points 0.00123 + (i, j)/sqrt(n),
    i outer; no normals, weights or curvatures (zeros), no holes.  The
    Gaussian covariance kernel's test set."""
    s = np.sqrt(n)
    m = int(np.ceil(s))
    i, j = np.meshgrid(np.arange(m), np.arange(m), indexing="ij")
    pts = np.stack([0.00123 + i.reshape(-1) / s, 0.00123 + j.reshape(-1) / s], 1)
    z = np.zeros(pts.shape[0])
    return Problem(pts, np.zeros_like(pts), z, z.copy(), name="uniform_grid")


def laplace_source_field(targets, sources):
    sources = np.atleast_2d(sources)
    d = targets[:, None, :] - sources[None, :, :]
    return np.log(np.hypot(d[..., 0], d[..., 1])) / (2 * np.pi)


def random_sources(n, rng, r_lo=2.5, r_hi=4.0):
    r = rng.uniform(r_lo, r_hi, n)
    t = rng.uniform(0, 2 * np.pi, n)
    return np.stack([r * np.cos(t), r * np.sin(t)], 1)


def disc_targets(n, rng, radius=0.5):
    """n points uniform in the disc of the given radius."""
    r = radius * np.sqrt(rng.uniform(0, 1, n))
    t = rng.uniform(0, 2 * np.pi, n)
    return np.stack([r * np.cos(t), r * np.sin(t)], 1)


def domain_targets(prob, n, rng, radius=1.9, margin=0.02):
    """n points inside the disc of the given radius and outside every hole's
    bounding circle (its radius when known, else the largest ellipse axis)."""
    radii = getattr(prob, "hole_radii", None)
    out = []
    while len(out) < n:
        p = disc_targets(1, rng, radius)[0]
        ok = True
        for h, c in enumerate(prob.hole_centers):
            rh = radii[h] if radii is not None else 0.06
            if np.hypot(*(p - c)) < rh + margin:
                ok = False
                break
        if ok:
            out.append(p)
    return np.array(out)


def star_c1():
    """4,096-unknown star r = 1 + 0.3 cos 5 theta: 256 panels x 16 nodes,
    source y0 = (3, 3), 100 interior targets uniform in r < 0.5 (seed 0)."""
    prob = star(256, 16)
    src = np.array([[3.0, 3.0]])
    rng = np.random.default_rng(0)
    tg = disc_targets(100, rng, 0.5)
    return prob, src, tg


# ------------------------------------------------------------------- 3D --

def fibonacci_sphere(n):
    """n quasi-uniform unit vectors: z_i = 1 - (2i+1)/n, azimuth i times the
    golden angle."""
    i = np.arange(n, dtype=np.float64)
    z = 1.0 - (2.0 * i + 1.0) / n
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    phi = i * np.pi * (3.0 - np.sqrt(5.0))
    return np.stack([r * np.cos(phi), r * np.sin(phi), z], 1)


def ellipsoid(n, axes=(1.0, 0.7, 0.5), center=(0.0, 0.0, 0.0), inward=False):
    """Ellipsoid surface with semi-axes `axes`: Fibonacci-sphere nodes u_i
    mapped by x = D u (D = diag(axes)), area weights (4 pi / n) times the
    mapping's area Jacobian abc |D^-1 u|, unit normals D^-1 u / |D^-1 u|
    (outward; `inward` flips them, for a hole).  Curvatures are not used by
    the 3D kernels (the diagonal comes from row sums) and are zero."""
    u = fibonacci_sphere(n)
    D = np.asarray(axes, np.float64)
    g = u / D[None]
    gn = np.linalg.norm(g, axis=1)
    pts = u * D[None] + np.asarray(center, np.float64)[None]
    nrm = g / gn[:, None]
    if inward:
        nrm = -nrm
    w = (4 * np.pi / n) * np.prod(D) * gn
    return Problem(pts, nrm, w, np.zeros(n), hole_centers=np.zeros((0, 3)), name="ellipsoid")


def spheres_with_holes(n_outer, hole_specs, outer_axes=(1.0, 1.0, 1.0)):
    """Outer ellipsoid (outward normals) with interior spherical holes given as
    (center, radius, n_nodes) (normals pointing into each hole, the
    reference's convention for hole boundaries), the nodes of every hole after
    the outer surface's."""
    parts = [ellipsoid(n_outer, outer_axes)]
    starts, counts, centers = [], [], []
    off = n_outer
    for c, r, m in hole_specs:
        parts.append(ellipsoid(m, (r, r, r), center=c, inward=True))
        starts.append(off)
        counts.append(m)
        centers.append(c)
        off += m
    return Problem(np.concatenate([p.points for p in parts]),
                   np.concatenate([p.normals for p in parts]),
                   np.concatenate([p.weights for p in parts]),
                   np.zeros(off), hole_centers=np.array(centers, np.float64).reshape(-1, 3),
                   hole_start=np.array(starts, np.int32), hole_count=np.array(counts, np.int32),
                   name="spheres_with_holes")


def laplace3_source_field(x, sources):
    """u(x) = 1 / (4 pi |x - y|) for each source y (one column per source)."""
    d = x[:, None, :] - np.asarray(sources, np.float64)[None]
    return 1.0 / (4 * np.pi * np.linalg.norm(d, axis=2))


def laplace3_source_rhs(prob, sources):
    return laplace3_source_field(prob.points, sources)


def stokeslet3_velocity(x, y0, force):
    """Velocity of a 3D Stokeslet at y0 with force f (unit viscosity):
    (1/8pi) (f/|r| + (r.f) r/|r|^3), r = x - y0 (the kernel of the
    reference's 3D Stokes border columns, kern_interp/linear_solve.cpp:49-63)."""
    r = x - np.asarray(y0)[None]
    rn = np.linalg.norm(r, axis=1)
    f = np.asarray(force, np.float64)
    return (f[None] / rn[:, None] + r * (r @ f)[:, None] / rn[:, None] ** 3) / (8 * np.pi)


def stokes3_rhs(prob, sources, forces):
    """Boundary velocity (interleaved per node, one column per Stokeslet)."""
    return np.stack([stokeslet3_velocity(prob.points, y, f).reshape(-1)
                     for y, f in zip(sources, forces)], 1)


def ellipsoid_targets(n, rng, axes=(1.0, 0.7, 0.5), scale=0.5):
    """n points uniform in the ellipsoid scaled by `scale`."""
    out = []
    while len(out) < n:
        p = rng.uniform(-1, 1, 3)
        if (p ** 2).sum() < 1:
            out.append(p * scale * np.asarray(axes))
    return np.array(out)
