"""The device's integer-pipe replacements for fp64 compares and conversions.

GB300 runs fp64 at a small fraction of its integer rate, so the box code
compares doubles as integers and rounds fp64 to fp32 with bit operations
(fe_common.cuh):
- dlt_int / dkey: the IEEE order of non-NaN doubles, with -0 == +0;
- dmin_ref / dmax_ref: std::min / std::max on that order;
- f32_round: fp64 -> fp32 toward -inf / +inf (the tree's outward boxes).

Each is restated here on Python integers, operation for operation. It is
checked against the IEEE semantics it replaces on random doubles of every
class: normal, subnormal, +-0, +-inf, the fp32 overflow and underflow
boundaries, and values exactly representable in fp32. The candidate pair set
is complete only if the fp32 boxes never shrink: rd(x) <= x <= ru(x), each
the nearest float on its side.
"""
import math

import numpy as np

M64 = (1 << 64) - 1


def _bits(x):
    return int(np.float64(x).view(np.uint64))


def _signed(u):
    return u - (1 << 64) if u >> 63 else u


def dkey(a):
    ia = _signed(_bits(a))
    return _signed((0x8000000000000000 - (ia & M64)) & M64) if ia < 0 else ia


def dlt_int(a, b):
    return dkey(a) < dkey(b)


def dmax_ref(a, b):
    return b if dlt_int(a, b) else a


def dmin_ref(a, b):
    return b if dlt_int(b, a) else a


def f32_round(x, up):
    b = _bits(x)
    e = (b >> 52) & 0x7FF
    sign = b >> 63
    m = b & 0xFFFFFFFFFFFFF
    away = (sign != 0) != up
    if e == 0x7FF:
        fb = (sign << 31) | 0x7F800000 | (0x00400000 if m else 0)
    elif e > 1023 + 127:
        fb = (sign << 31) | (0x7F800000 if away else 0x7F7FFFFF)
    elif e >= 1023 - 126:
        fb = (sign << 31) | ((e - 1023 + 127) << 23) | (m >> 29)
        if away and (m & 0x1FFFFFFF) != 0:
            fb += 1
    else:
        sig = (m | (1 << 52)) if e else m
        sh = 926 - (e if e else 1)
        q = 0 if sh >= 64 else sig >> sh
        inexact = (sig != 0) if sh >= 64 else (sig & ((1 << sh) - 1)) != 0
        fb = (sign << 31) | q
        if away and inexact:
            fb += 1
    return float(np.uint32(fb & 0xFFFFFFFF).view(np.float32))


def _samples(rng, n):
    """Doubles of every class, with exact fp32 values and the boundaries."""
    out = [0.0, -0.0, math.inf, -math.inf, 5e-324, -5e-324, 2.0 ** -149, 2.0 ** -150, 2.0 ** -126,
           float(np.finfo(np.float32).max), float(np.finfo(np.float32).max) * (1 + 2.0 ** -30),
           2.0 ** 128, -(2.0 ** 128), 1.0, -1.0, 1.5, 2.0 ** -1022, 1e308]
    bits = rng.integers(0, 1 << 63, size=n, dtype=np.uint64) | (rng.integers(0, 2, size=n, dtype=np.uint64) << 63)
    out += [float(x) for x in bits.view(np.float64) if not math.isnan(x)]
    # exponents near fp32's range, where the rounding branches change
    e = rng.integers(1023 - 160, 1023 + 130, size=n).astype(np.uint64)
    m = rng.integers(0, 1 << 52, size=n, dtype=np.uint64)
    m[: n // 4] &= ~np.uint64((1 << 29) - 1)  # fp32-exact mantissas
    s = rng.integers(0, 2, size=n, dtype=np.uint64) << np.uint64(63)
    out += [float(x) for x in (s | (e << np.uint64(52)) | m).view(np.float64)]
    out += [float(x) for x in rng.standard_normal(n).astype(np.float32)]  # fp32-exact values
    return out


def test_integer_order_is_the_ieee_order():
    rng = np.random.default_rng(21)
    xs = _samples(rng, 3000)
    ys = list(xs)
    rng.shuffle(ys)
    for a, b in zip(xs + [0.0, -0.0, 0.0], ys + [-0.0, 0.0, 0.0]):
        assert dlt_int(a, b) == (a < b), (a, b)
        assert (dkey(a) <= dkey(b)) == (a <= b), (a, b)
        # std::max / std::min: the first argument unless the second is strictly beyond it
        assert _bits(dmax_ref(a, b)) == _bits(b if a < b else a), (a, b)
        assert _bits(dmin_ref(a, b)) == _bits(b if b < a else a), (a, b)


def _f32_below(x):
    """The largest fp32 value <= x (or -inf / the most negative float)."""
    f = np.float32(x)  # to nearest
    if math.isinf(x):
        return float(f)
    if float(f) > x:
        f = np.nextafter(f, np.float32(-np.inf))
    return float(f)


def _f32_above(x):
    f = np.float32(x)
    if math.isinf(x):
        return float(f)
    if float(f) < x:
        f = np.nextafter(f, np.float32(np.inf))
    return float(f)


def test_directed_rounding_is_the_nearest_float_on_each_side():
    rng = np.random.default_rng(22)
    with np.errstate(over="ignore"):
        for x in _samples(rng, 4000):
            rd, ru = f32_round(x, False), f32_round(x, True)
            assert rd <= x <= ru, x
            want_rd, want_ru = _f32_below(x), _f32_above(x)
            if abs(x) > float(np.finfo(np.float32).max) and not math.isinf(x):
                # beyond fp32's range: the finite extreme on the near side, infinity on the far side
                assert (rd, ru) == ((float(np.finfo(np.float32).max), math.inf) if x > 0
                                    else (-math.inf, -float(np.finfo(np.float32).max))), x
            else:
                assert rd == want_rd and ru == want_ru, (x, rd, want_rd, ru, want_ru)


def f32_vertex_coord(x):
    """f32_vertex_coord (fe_common.cuh) on the double's two 32-bit halves:
    zero stays zero, a magnitude in [2^-100, 2^40) rounds to nearest (ties to
    even), anything else is NaN."""
    u = _bits(x)
    hi, lo = u >> 32, u & 0xFFFFFFFF
    if ((hi << 1) & 0xFFFFFFFF) | lo == 0:
        return 0.0
    e = (hi >> 20) & 0x7FF
    if e < 1023 - 100 or e > 1023 + 39:
        return float("nan")
    fb = (hi & 0x80000000) | ((e - 1023 + 127) << 23) | ((hi & 0xFFFFF) << 3) | (lo >> 29)
    r = lo & 0x1FFFFFFF
    if r > 0x10000000 or (r == 0x10000000 and (fb & 1)):
        fb += 1
    return float(np.frombuffer(np.uint32(fb).tobytes(), np.float32)[0])


def test_vertex_copy_rounding_is_ieee_nearest():
    rng = np.random.default_rng(21)
    xs = list(_samples(rng, 20000))
    # exact ties, carries into the exponent, the range edges
    for e in (-100, -99, -1, 0, 1, 20, 39):
        b = 2.0 ** e
        xs += [b, -b, b * (1 + 2.0 ** -24), b * (1 + 3 * 2.0 ** -24), b * (2 - 2.0 ** -30), b * (1 - 2.0 ** -40)]
    xs += [2.0 ** 40, 2.0 ** -101, 0.0, -0.0, math.inf, -math.inf, math.nan]
    for x in xs:
        got = f32_vertex_coord(x)
        m = abs(x)
        if x == 0:
            assert got == 0.0
        elif not (2.0 ** -100 <= m < 2.0 ** 40):
            assert math.isnan(got), x
        else:
            want = float(np.float32(x))
            assert got == want, (x, got, want)
