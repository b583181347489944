"""Shewchuk's error-free primitives as the device writes them
(mcut_gb300/csrc/fe_common.cuh), restated operation for operation on Python
doubles (IEEE, round to nearest, no fused multiply-add): Two-Sum, Fast-Two-
Sum, Two-Diff, Veltkamp split, Two-Product, Two-Two-Diff and the
zero-eliminating expansion sum and scaling (Shewchuk, DCG 18:305-363, 1997).
Shared by the tests that check the device's predicates."""

SPLITTER = 134217729.0  # 2^27 + 1


def two_sum(a, b):
    s = a + b
    bv = s - a
    av = s - bv
    return s, (a - av) + (b - bv)


def fast_two_sum(a, b):
    s = a + b
    return s, b - (s - a)


def two_diff(a, b):
    s = a - b
    bv = a - s
    av = s + bv
    return s, (a - av) + (bv - b)


def split(a):
    c = SPLITTER * a
    big = c - a
    hi = c - big
    return hi, a - hi


def two_product(a, b):
    p = a * b
    ah, al = split(a)
    bh, bl = split(b)
    e1 = p - ah * bh
    e2 = e1 - al * bh
    e3 = e2 - ah * bl
    return p, al * bl - e3


def two_two_diff(a1, a0, b1, b0):
    x = [0.0] * 4
    i, x[0] = two_diff(a0, b0)
    j, k0 = two_sum(a1, i)
    i, x[1] = two_diff(k0, b1)
    x[3], x[2] = two_sum(j, i)
    return x


def fast_expansion_sum_zeroelim(e, f):
    h = []
    ei = fi = 0
    en, fn = e[0], f[0]

    def nxt(arr, k):
        return arr[k] if k < len(arr) else 0.0
    if (fn > en) == (fn > -en):
        q = en
        ei += 1
        en = nxt(e, ei)
    else:
        q = fn
        fi += 1
        fn = nxt(f, fi)
    if ei < len(e) and fi < len(f):
        if (fn > en) == (fn > -en):
            q, hh = fast_two_sum(en, q)
            ei += 1
            en = nxt(e, ei)
        else:
            q, hh = fast_two_sum(fn, q)
            fi += 1
            fn = nxt(f, fi)
        if hh != 0.0:
            h.append(hh)
        while ei < len(e) and fi < len(f):
            if (fn > en) == (fn > -en):
                q, hh = two_sum(q, en)
                ei += 1
                en = nxt(e, ei)
            else:
                q, hh = two_sum(q, fn)
                fi += 1
                fn = nxt(f, fi)
            if hh != 0.0:
                h.append(hh)
    while ei < len(e):
        q, hh = two_sum(q, en)
        ei += 1
        en = nxt(e, ei)
        if hh != 0.0:
            h.append(hh)
    while fi < len(f):
        q, hh = two_sum(q, fn)
        fi += 1
        fn = nxt(f, fi)
        if hh != 0.0:
            h.append(hh)
    if q != 0.0 or not h:
        h.append(q)
    return h


def scale_expansion_zeroelim(e, b):
    h = []
    bh, bl = split(b)
    p = e[0] * b
    ah, al = split(e[0])
    e1 = p - ah * bh
    e2 = e1 - al * bh
    e3 = e2 - ah * bl
    q, hh = p, al * bl - e3
    if hh != 0.0:
        h.append(hh)
    for i in range(1, len(e)):
        p = e[i] * b
        ah, al = split(e[i])
        e1 = p - ah * bh
        e2 = e1 - al * bh
        e3 = e2 - ah * bl
        p0 = al * bl - e3
        s, hh = two_sum(q, p0)
        if hh != 0.0:
            h.append(hh)
        q, hh = fast_two_sum(p, s)
        if hh != 0.0:
            h.append(hh)
    if q != 0.0 or not h:
        h.append(q)
    return h
