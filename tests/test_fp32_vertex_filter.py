"""Soundness of the fp32-vertex orient3d filter, the cascade's first stage.

The device keeps one fp32 copy of every vertex (each coordinate rounded to
nearest; a coordinate that is neither zero nor of magnitude in
[2^-100, 2^40) is stored as NaN, which sends every test touching it to the
next stage). For a test it forms the nine coordinate differences in fp32
from those copies, evaluates Shewchuk's orient3d expression in fp32, and
decides the sign only when |det| exceeds a bound that covers

  * the rounding of each coordinate to fp32 and of each fp32 difference:
    per difference s = fl(P~ - D~) of the true difference t = P - D,
        |s - t| <= E := c (|s| + |P~| + |D~|),  c = 2^-24 (1 + 2^-20)
    (|P~ - P| <= u|P| <= u|P~| / (1 - u) for round to nearest in the normal
    range, and |fl(x) - x| <= u|x|, u = 2^-24);
  * the effect of those input errors on the determinant: with M = |s| + E,
    each monomial obeys |t_a t_b t_c - s_a s_b s_c| <= E_a M_b M_c
    + M_a E_b M_c + M_a M_b E_c, summed over the six monomials (delta);
  * the rounding of the fp32 evaluation: Shewchuk's stage-A bound
    (7u + 56u^2) times the permanent, covered by 8u times the permanent of
    the M values (permM >= the permanent of the s values);
  * the rounding of the bound's own evaluation (all its terms are products
    and sums of non-negative fp32 values: a factor 1 + 2^-20) and underflow
    (2^-140 absolute, far above the few 2^-149 ulps underflow can lose).

bound = (8u permM + delta)(1 + 2^-20) + 2^-140. Coordinates of magnitude
below 2^40 keep every product below 2^128 (no overflow).

This module restates that arithmetic operation for operation in numpy float32
(IEEE round to nearest, no fused multiply-add, as the device build with
--fmad=false computes it) and drives it with adversarial inputs: near-coplanar
points at every scale, large offsets with small differences (where the
coordinate rounding dominates), lattice points with exact zeros, mixed-scale
axes, points swept across the decision threshold, and coordinates outside
the admitted range. Every sign it decides must equal the exact sign.
"""
import numpy as np

import oracle

F = np.float32
U8 = F(4.76837158203125e-07)            # 8 * 2^-24
C = F(2.0 ** -24 * (1.0 + 2.0 ** -20))  # coordinate and difference rounding
GROW = F(1.0 + 2.0 ** -20)
TINY = F(2.0 ** -140)
LO, HI = 2.0 ** -100, 2.0 ** 40


def to_f32(x):
    """The device's fp32 vertex copy: nearest, NaN outside the admitted range."""
    x = np.asarray(x, np.float64)
    m = np.abs(x)
    ok = (x == 0) | ((m >= LO) & (m < HI))
    with np.errstate(over="ignore"):
        return np.where(ok, x.astype(np.float32), F(np.nan))


def filter_sign(a, b, c, d):
    """(decided, sign) per row, the device's fp32-vertex stage on rows of points."""
    A, B, Cc, D = (to_f32(p) for p in (a, b, c, d))
    with np.errstate(over="ignore", invalid="ignore", under="ignore"):
        s = [[P[:, j] - D[:, j] for j in range(3)] for P in (A, B, Cc)]
        (ax, ay, az), (bx, by, bz), (cx, cy, cz) = s
        det = az * (bx * cy - cx * by) + bz * (cx * ay - ax * cy) + cz * (ax * by - bx * ay)
        E = [[C * ((np.abs(s[i][j]) + np.abs(P[:, j])) + np.abs(D[:, j])) for j in range(3)]
             for i, P in enumerate((A, B, Cc))]
        M = [[np.abs(s[i][j]) + E[i][j] for j in range(3)] for i in range(3)]
        (Eax, Eay, Eaz), (Ebx, Eby, Ebz), (Ecx, Ecy, Ecz) = E
        (Max, May, Maz), (Mbx, Mby, Mbz), (Mcx, Mcy, Mcz) = M
        P1 = Mbx * Mcy + Mcx * Mby
        Q1 = (Ebx * Mcy + Mbx * Ecy) + (Ecx * Mby + Mcx * Eby)
        P2 = Mcx * May + Max * Mcy
        Q2 = (Ecx * May + Mcx * Eay) + (Eax * Mcy + Max * Ecy)
        P3 = Max * Mby + Mbx * May
        Q3 = (Eax * Mby + Max * Eby) + (Ebx * May + Mbx * Eay)
        permM = Maz * P1 + Mbz * P2 + Mcz * P3
        delta = (Eaz * P1 + Maz * Q1) + (Ebz * P2 + Mbz * Q2) + (Ecz * P3 + Mcz * Q3)
        bound = (U8 * permM + delta) * GROW + TINY
        pos, neg = det > bound, -det > bound
    return pos | neg, np.where(pos, 1, -1)


def _check(a, b, c, d):
    decided, sign = filter_sign(a, b, c, d)
    rows = np.nonzero(decided)[0]
    ex = np.array([oracle.port_orient3d_sign(a[i], b[i], c[i], d[i]) for i in rows], dtype=np.int64)
    bad = rows[ex != sign[rows]]
    assert len(bad) == 0, (a[bad[0]], b[bad[0]], c[bad[0]], d[bad[0]])
    return decided


def _near_coplanar(rng, n, scale, offset=0.0):
    a, b, c = (offset + scale * rng.standard_normal((n, 3)) for _ in range(3))
    u, v = rng.random((n, 1)), rng.random((n, 1))
    d = a + u * (b - a) + v * (c - a)
    nudge = rng.integers(-2, 3, size=(n, 3)).astype(np.float64)
    d = d + nudge * np.spacing(np.abs(d)) * (rng.random((n, 1)) < 0.5)
    return a, b, c, d


def _off_plane(rng, n, scale, offset=0.0):
    a, b, c = (offset + scale * rng.standard_normal((n, 3)) for _ in range(3))
    nrm = np.cross(b - a, c - a)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    u, v = rng.random((n, 1)), rng.random((n, 1))
    t = 10.0 ** rng.uniform(-12, -1, size=(n, 1)) * rng.choice([-1.0, 1.0], size=(n, 1))
    d = a + u * (b - a) + v * (c - a) + t * scale * nrm
    return a, b, c, d


def test_threshold_sweeps_across_scales():
    rng = np.random.default_rng(7)
    decided = 0
    total = 0
    for e in range(-30, 36, 5):
        for off in (0.0, 2.0 ** (e + 8), 2.0 ** (e + 20)):
            a, b, c, d = _off_plane(rng, 1500, 2.0 ** e, off)
            decided += _check(a, b, c, d).sum()
            total += len(a)
    assert 0.1 * total < decided < total  # decides many, escalates near the plane


def test_points_on_the_plane_up_to_rounding():
    rng = np.random.default_rng(8)
    for e in (-20, -3, 0, 4, 12, 30):
        for off in (0.0, 2.0 ** (e + 6), 2.0 ** (e + 18)):
            _check(*_near_coplanar(rng, 2000, 2.0 ** e, off))


def test_large_offsets_small_differences():
    """Coordinates far from the origin, differences tiny: the coordinate
    rounding, not the arithmetic, dominates the error."""
    rng = np.random.default_rng(9)
    for off in (1.0, 1e3, 1e6, 2.0 ** 39):
        for rel in (1e-3, 1e-5, 1e-7, 1e-9):
            a, b, c = (off + off * rel * rng.standard_normal((1500, 3)) for _ in range(3))
            d = off + off * rel * rng.standard_normal((1500, 3))
            _check(a, b, c, d)


def test_lattice_and_exact_zeros():
    rng = np.random.default_rng(10)
    for s in (2.0 ** -9, 1.0, 16.0, 2.0 ** 20):
        pts = [rng.integers(-6, 7, size=(3000, 3)).astype(np.float64) * s for _ in range(4)]
        pts[3][:1000, 2] = pts[0][:1000, 2]  # coplanar in z for a third of the rows
        pts[1][:1000, 2] = pts[0][:1000, 2]
        pts[2][:1000, 2] = pts[0][:1000, 2]
        decided = _check(*pts)
        # an exactly coplanar lattice test has det = 0 and must escalate
        assert not decided[:1000].any()


def test_mixed_scale_axes():
    rng = np.random.default_rng(11)
    scl = np.array([2.0 ** -30, 1.0, 2.0 ** 30])
    for k in range(6):
        s = scl[np.array([(k + j) % 3 for j in range(3)])]
        a, b, c, d = (rng.standard_normal((2000, 3)) * s for _ in range(4))
        _check(a, b, c, d)


def test_coordinates_outside_the_range_escalate():
    rng = np.random.default_rng(12)
    a, b, c, d = (rng.standard_normal((500, 3)) for _ in range(4))
    for bad in (2.0 ** 40, 2.0 ** 41, 2.0 ** -110, np.inf, np.nan):
        a2 = a.copy()
        a2[:, 1] = bad
        decided, _ = filter_sign(a2, b, c, d)
        assert not decided.any()


def test_workload_like_inputs_mostly_decided():
    """Recentred, x16-scaled meshes (coordinates ~ 20, edges ~ 0.05): the
    coordinate rounding costs the filter few decisions."""
    rng = np.random.default_rng(13)
    a = 20.0 + rng.standard_normal((4000, 3))
    b, c = a + 0.05 * rng.standard_normal((4000, 3)), a + 0.05 * rng.standard_normal((4000, 3))
    d = a + 0.05 * rng.standard_normal((4000, 3))
    decided = _check(a, b, c, d)
    assert decided.mean() > 0.97


def test_rounding_crosses_the_plane():
    """fp32 copies just on one side of the plane (or on it) while the true
    points, within half an fp32 ulp, lie on the other side: the filter must
    never decide the copies' sign."""
    rng = np.random.default_rng(14)
    n = 6000
    for scale, off in ((1.0, 0.0), (1.0, 100.0), (0.01, 20.0), (2.0 ** 10, 2.0 ** 20)):
        a, b, c = (np.float32(off + scale * rng.standard_normal((n, 3))).astype(np.float64) for _ in range(3))
        u, v = rng.random((n, 1)), rng.random((n, 1))
        d = np.float32(a + u * (b - a) + v * (c - a)).astype(np.float64)  # fp32 point near the plane
        step = np.spacing(np.abs(d).astype(np.float32)).astype(np.float64)
        # move every true coordinate by up to 0.45 fp32 ulp: the fp32 copies are unchanged
        jitter = (rng.random((n, 3)) - 0.5) * 0.9 * step
        d_true = d + jitter
        a_true = a + (rng.random((n, 3)) - 0.5) * 0.9 * np.spacing(np.abs(a).astype(np.float32)).astype(np.float64)
        assert np.array_equal(to_f32(d_true), to_f32(d)) and np.array_equal(to_f32(a_true), to_f32(a))
        _check(a_true, b, c, d_true)
