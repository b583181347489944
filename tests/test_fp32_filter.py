"""Soundness of the fp32 orient3d filter, the first stage of the cascade.

The device decides most orient3d signs in fp32 (orient3d_sign_filtered in
mcut_gb300/csrc/fe_common.cuh). The nine coordinate differences are formed
in fp64 and rounded once to fp32, to nearest. The filter runs only when every
nonzero difference lies in [2^-40, 2^41). It decides when |det| > 8u *
permanent (u = 2^-24), and otherwise escalates to the fp64 stage.

This module restates that arithmetic operation for operation in numpy
float32, which is IEEE round to nearest with no fused multiply-add, as the
device build (--fmad=false) is. It drives the filter with adversarial inputs:
- points swept across the decision threshold, and points on the plane up to
  rounding, at scales across the whole admitted range;
- large offsets with small differences;
- lattice points (exact zeros);
- mixed-scale axes;
- differences outside the range.
Every sign the filter decides must equal the exact sign (the oracle's
orient3d, pinned to the reference's). A wrong sign here would mean the bound
is not a bound.
"""
import numpy as np

import oracle

U8 = np.float32(4.76837158203125e-07)  # 8 * 2^-24
LO, HI = 2.0 ** -40, 2.0 ** 41


def filter_sign(a, b, c, d):
    """(decided, sign) per row, as the device's fp32 stage computes them."""
    ad, bd, cd = a - d, b - d, c - d  # fp64, one rounding each
    diffs = np.stack([ad, bd, cd], 1)  # (N, 3 points, 3 axes)
    mag = np.abs(diffs)
    ok = np.all((diffs == 0) | ((mag >= LO) & (mag < HI)), axis=(1, 2))
    f = diffs.astype(np.float32)  # to nearest, ties to even
    ax, ay, az = f[:, 0, 0], f[:, 0, 1], f[:, 0, 2]
    bx, by, bz = f[:, 1, 0], f[:, 1, 1], f[:, 1, 2]
    cx, cy, cz = f[:, 2, 0], f[:, 2, 1], f[:, 2, 2]
    with np.errstate(over="ignore", invalid="ignore", under="ignore"):
        bxcy, cxby, cxay, axcy, axby, bxay = bx * cy, cx * by, cx * ay, ax * cy, ax * by, bx * ay
        det = az * (bxcy - cxby) + bz * (cxay - axcy) + cz * (axby - bxay)
        perm = (np.abs(bxcy) + np.abs(cxby)) * np.abs(az) + (np.abs(cxay) + np.abs(axcy)) * np.abs(bz) \
            + (np.abs(axby) + np.abs(bxay)) * np.abs(cz)
        eb = U8 * perm
        pos, neg = det > eb, -det > eb
    decided = ok & (pos | neg)
    return decided, np.where(pos, 1, -1), ok


def exact_signs(a, b, c, d, rows):
    return np.array([oracle.port_orient3d_sign(a[i], b[i], c[i], d[i]) for i in rows], dtype=np.int64)


def _check(a, b, c, d):
    decided, sign, ok = filter_sign(a, b, c, d)
    rows = np.nonzero(decided)[0]
    ex = exact_signs(a, b, c, d, rows)
    bad = rows[ex != sign[rows]]
    assert len(bad) == 0, (a[bad[0]], b[bad[0]], c[bad[0]], d[bad[0]])
    return decided, ok


def _near_coplanar(rng, n, scale, offset=0.0):
    a, b, c = (offset + scale * rng.standard_normal((n, 3)) for _ in range(3))
    u, v = rng.random((n, 1)), rng.random((n, 1))
    d = a + u * (b - a) + v * (c - a)  # on the plane up to fp64 rounding
    nudge = rng.integers(-2, 3, size=(n, 3)).astype(np.float64)
    d = d + nudge * np.spacing(np.abs(d)) * (rng.random((n, 1)) < 0.5)
    return a, b, c, d


def _off_plane(rng, n, scale):
    """Points at a relative distance t from the plane of a, b, c, with t
    log-uniform over [1e-10, 1e-2]: the determinant relative to the permanent
    sweeps across the filter's threshold 8u = 4.8e-7."""
    a, b, c = (scale * rng.standard_normal((n, 3)) for _ in range(3))
    nrm = np.cross(b - a, c - a)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    u, v = rng.random((n, 1)), rng.random((n, 1))
    t = 10.0 ** rng.uniform(-10, -2, size=(n, 1)) * rng.choice([-1.0, 1.0], size=(n, 1))
    d = a + u * (b - a) + v * (c - a) + t * scale * nrm
    return a, b, c, d


def test_near_the_threshold_across_scales():
    rng = np.random.default_rng(11)
    tot_dec = tot = 0
    for k in range(-34, 36, 3):
        decided, ok = _check(*_off_plane(rng, 6000, 2.0 ** k))
        tot_dec += int(decided.sum())
        tot += int(ok.sum())
    # the filter decides the clear cases and escalates those near the threshold
    assert 0.3 * tot < tot_dec < 0.9 * tot


def test_on_the_plane_up_to_rounding():
    rng = np.random.default_rng(16)
    for k in range(-34, 36, 5):
        _check(*_near_coplanar(rng, 3000, 2.0 ** k))


def test_large_offsets_small_differences():
    rng = np.random.default_rng(12)
    for off in (1.0, 1e3, 1e6, 3e9):
        for scale in (1e-3, 1.0, 1e2):
            _check(*_near_coplanar(rng, 3000, scale, offset=off))
            a, b, c, d = (off + scale * rng.standard_normal((3000, 3)) for _ in range(4))
            _check(a, b, c, d)


def test_lattice_points_never_decide_a_zero():
    rng = np.random.default_rng(13)
    for step in (2.0 ** -20, 1.0, 2.0 ** 20):
        a, b, c, d = (step * rng.integers(-3, 4, size=(20000, 3)).astype(np.float64) for _ in range(4))
        decided, _ = _check(a, b, c, d)  # a decided row has the exact nonzero sign
        assert (~decided).any()  # the exact zeros escalate


def test_mixed_scale_axes():
    rng = np.random.default_rng(14)
    for sx, sy, sz in ((2.0 ** 39, 2.0 ** -38, 1.0), (2.0 ** -39, 2.0 ** -39, 2.0 ** 40), (1e-9, 1e9, 1.0)):
        s = np.array([sx, sy, sz])
        a, b, c = (s * rng.standard_normal((5000, 3)) for _ in range(3))
        u, v = rng.random((5000, 1)), rng.random((5000, 1))
        d = a + u * (b - a) + v * (c - a)
        _check(a, b, c, d)
        d2 = s * rng.standard_normal((5000, 3))
        _check(a, b, c, d2)


def test_differences_outside_the_range_escalate():
    rng = np.random.default_rng(15)
    for scale in (2.0 ** -45, 2.0 ** 43):
        a, b, c, d = (scale * rng.standard_normal((2000, 3)) for _ in range(4))
        decided, _, ok = filter_sign(a, b, c, d)
        assert not ok.any() and not decided.any()


def _f32_input_bits(d):
    """f32_filter_input's integer rounding of one fp64 difference (the device
    forms the fp32 bits from the fp64 bits), restated on Python integers:
    (in range, fp32 bits)."""
    b = int(np.float64(d).view(np.uint64))
    if (b << 1) & ((1 << 64) - 1) == 0:
        return True, 0
    e = (b >> 52) & 0x7FF
    if e < 1023 - 40 or e > 1023 + 40:
        return False, None
    m = b & 0xFFFFFFFFFFFFF
    fb = ((b >> 63) << 31) | ((e - 1023 + 127) << 23) | (m >> 29)
    r = m & 0x1FFFFFFF
    if r > 0x10000000 or (r == 0x10000000 and (fb & 1)):
        fb += 1
    return True, fb


def test_input_rounding_is_ieee_to_nearest_even():
    """The device's bitwise fp64 -> fp32 rounding equals the IEEE conversion
    the numpy restatement uses, ties and mantissa carries included."""
    rng = np.random.default_rng(17)
    e = rng.integers(1023 - 40, 1023 + 41, size=20000).astype(np.uint64)
    m = rng.integers(0, 1 << 52, size=20000, dtype=np.uint64)
    m[:4000] = (m[:4000] & ~np.uint64(0x1FFFFFFF)) | np.uint64(0x10000000)  # exact ties
    m[4000:6000] = np.uint64((1 << 52) - 1)  # rounds up into the exponent
    sgn = rng.integers(0, 2, size=20000).astype(np.uint64)
    d = ((sgn << np.uint64(63)) | (e << np.uint64(52)) | m).view(np.float64)
    want = d.astype(np.float32).view(np.uint32)
    for x, w in zip(d, want):
        ok, bits = _f32_input_bits(x)
        assert ok and bits == int(w), x
    for x in (0.0, -0.0):
        assert _f32_input_bits(x) == (True, 0)
    for x in (2.0 ** -41, -(2.0 ** 41), 2.0 ** 60, 5e-324):
        assert _f32_input_bits(x)[0] is False
