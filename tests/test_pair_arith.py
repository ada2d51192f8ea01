"""CPU restatements of the FP32-pair algorithms the GPU kernels use, checked
against FP64: the pair multiply-add of the FP64-accurate FMM and border apply
(ki_common.cuh pair_fma), the table-driven pair logarithm of the 2D Laplace
hole columns (pair_log), and the implicit-pivoting Gauss-Jordan inverse of the
Schur kernel (cta_gj_inverse_reg).  FP32 fused multiply-adds are emulated
through FP64 (the FP32 product is exact there), which rounds twice; the bounds
below leave room for that."""
import numpy as np

f32 = np.float32


def fma(a, b, c):
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def two_sum(a, b):
    s = f32(a + b)
    bb = f32(s - a)
    return s, f32(f32(a - f32(s - bb)) + f32(b - bb))


def split(v):
    h = f32(v)
    return h, f32(v - np.float64(h))


def pair_fma(h, l, e, d):
    p = f32(e[0] * d[0])
    q = fma(e[0], d[0], -p)
    q = fma(e[0], d[1], q)
    q = fma(e[1], d[0], q)
    s, err = two_sum(h, p)
    return s, f32(l + f32(err + q))


LN2 = 0.69314718055994530942
LN2_H = f32(0.693145751953125)
LN2_M = f32(LN2 - 0.693145751953125)
LN2_L = f32(LN2 - 0.693145751953125 - np.float64(LN2_M))
LOGC = [split(np.log(1 + (j + 0.5) / 256)) for j in range(256)]


def pair_log(xh, xl):
    bits = int(np.array([xh], np.float32).view(np.int32)[0])
    e = ((bits >> 23) & 0xFF) - 127
    m = np.array([(bits & 0x7FFFFF) | 0x3F800000], np.int32).view(np.float32)[0]
    j = (bits >> 15) & 0xFF
    c = f32(1 + (j + 0.5) / 256)
    p2 = np.array([(127 - e) << 23], np.int32).view(np.float32)[0]
    dl, dh = f32(xl * p2), f32(m - c)
    rc = f32(1.0 / np.float64(c))
    th = f32(dh * rc)
    tl = f32(f32(fma(-th, c, dh) + dl) * rc)
    q = f32(th * th)
    qe = fma(th, th, -q)
    rest = f32(f32(th * q) * fma(-th, fma(-th, f32(0.2), f32(0.25)), f32(1 / 3)))
    sh, sl = two_sum(th, f32(-0.5 * q))
    sl = f32(sl + f32(f32(tl - fma(f32(0.5), qe, f32(th * tl))) + rest))
    fe = f32(e)
    pm = f32(fe * LN2_M)
    s1, e1 = two_sum(f32(fe * LN2_H), LOGC[j][0])
    s2, e2 = two_sum(s1, pm)
    s3, e3 = two_sum(s2, sh)
    lo = f32(f32(f32(e1 + e2) + f32(e3 + fma(fe, LN2_M, -pm))) + f32(fma(fe, LN2_L, LOGC[j][1]) + sl))
    rh, rl = two_sum(s3, lo)
    return np.float64(rh) + np.float64(rl)


def test_pair_fma_sum_matches_fp64():
    rng = np.random.default_rng(1)
    e = rng.standard_normal(400) * 10.0 ** rng.uniform(-3, 3, 400)
    d = rng.standard_normal(400)
    h = l = f32(0)
    for a, b in zip(e, d):
        h, l = pair_fma(h, l, split(a), split(b))
    exact = float(np.sum(e.astype(np.longdouble) * d.astype(np.longdouble)))
    scale = float(np.sum(np.abs(e * d)))
    assert abs(np.float64(h) + np.float64(l) - exact) <= 1e-12 * scale


def test_pair_log_absolute_error():
    rng = np.random.default_rng(0)
    xs = np.concatenate([10 ** rng.uniform(-6, 2, 3000), 1 + rng.uniform(-1e-3, 1e-3, 500)])
    worst = 0.0
    for x in xs:
        xh, xl = split(x)
        xx = np.float64(xh) + np.float64(xl)
        worst = max(worst, abs(pair_log(xh, xl) - np.log(xx)))
    # squared distances of boundary points from hole centres lie in this range;
    # the refinement needs entries to ~1e-11
    assert worst <= 3e-13, worst


def test_implicit_pivot_gauss_jordan_inverse():
    rng = np.random.default_rng(2)
    for n in (1, 2, 7, 33, 64):
        A0 = rng.standard_normal((n, n))
        A = A0.copy()
        used = np.zeros(n, bool)
        piv, pinv = np.zeros(n, int), np.zeros(n, int)
        for j in range(n):
            col = A[:, j].copy()
            p = int(np.argmax(np.where(used, -1.0, np.abs(col))))
            used[p], piv[j], pinv[p] = True, p, j
            inv = 1.0 / col[p]
            row = A[p, :] * inv
            row[j] = inv
            A[p, :] = row
            f = np.where(np.arange(n) == p, 0.0, col)
            A -= np.outer(f, row)
            A[np.arange(n) != p, j] = -f[np.arange(n) != p] * inv
        X = np.empty_like(A)
        X[np.ix_(pinv, piv)] = A
        assert np.abs(X @ A0 - np.eye(n)).max() <= 1e-10 * max(1.0, np.abs(np.linalg.inv(A0)).max())
