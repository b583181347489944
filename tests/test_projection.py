"""The device's projection matrix equals the reference's, bit for bit.

The reference projects a face and a point to 2-D with P = K R
(calculate_projection_matrix, math.cpp:710-793): a = n / |n|,
b = sign(n[mc]) e_mc, R = 2 (a+b)(a+b)^T / (a.b) - diag(1, -1, 1) (R = that
diagonal when a == b), and K keeps the two rows other than mc through a full
3 x 3 product. The device (projection_matrix in fe_common.cuh) takes two
exact shortcuts:
- it reads the selected entries of R directly, writing -0 as +0 as the
  product's 0.0 + ... sums do;
- it shares the quotient of the symmetric entry (apb_i apb_j == apb_j apb_i).
Both are restated here on Python doubles and compared entry by entry, as raw
bits, over random normals of every orientation, axis-aligned and
near-axis normals, and normals with signed zeros.
"""
import math

import numpy as np

I3 = [[1.0, 0.0, 0.0], [0.0, -1.0, 0.0], [0.0, 0.0, 1.0]]


def dot3(a, b):
    o = 0.0
    o = o + a[0] * b[0]
    o = o + a[1] * b[1]
    o = o + a[2] * b[2]
    return o


def largest_component(n):
    big, mc = 0.0, 0
    for i in range(3):
        t = abs(n[i])
        if t > big:
            big, mc = t, i
    return mc


def reference(n, mc):
    length = math.sqrt(dot3(n, n))
    a = [n[0] / length, n[1] / length, n[2] / length]
    b = [0.0, 0.0, 0.0]
    s = (0.0 < n[mc]) - (n[mc] < 0.0)
    b[mc] = 1.0 * float(s)
    R = [row[:] for row in I3]
    if a != b:
        apb = [a[0] + b[0], a[1] + b[1], a[2] + b[2]]
        adb = dot3(a, b)
        R = [[((apb[i] * apb[j]) / adb) * 2.0 - I3[i][j] for j in range(3)] for i in range(3)]
    K = [[0.0] * 3 for _ in range(2)]
    if mc == 0:
        K[0][1] = K[1][2] = 1.0
    elif mc == 1:
        K[0][0] = K[1][2] = 1.0
    else:
        K[0][0] = K[1][1] = 1.0
    P = []
    for i in range(2):
        for j in range(3):
            acc = 0.0
            for k in range(3):
                acc = acc + K[i][k] * R[k][j]
            P.append(acc)
    return P


def device(n, mc):
    length = math.sqrt(dot3(n, n))
    a = [n[0] / length, n[1] / length, n[2] / length]
    b = [0.0, 0.0, 0.0]
    s = (0.0 < n[mc]) - (n[mc] < 0.0)
    b[mc] = 1.0 * float(s)
    r0, r1 = (1 if mc == 0 else 0), (1 if mc == 2 else 2)
    P = [0.0] * 6
    if a[0] != b[0] or a[1] != b[1] or a[2] != b[2]:
        apb = [a[0] + b[0], a[1] + b[1], a[2] + b[2]]
        adb = dot3(a, b)
        q0 = [(apb[r0] * apb[j]) / adb for j in range(3)]
        q1 = [q0[r1] if j == r0 else (apb[r1] * apb[j]) / adb for j in range(3)]
        for j in range(3):
            e0 = (q0[j] * 2.0) - ((-1.0 if r0 == 1 else 1.0) if r0 == j else 0.0)
            e1 = (q1[j] * 2.0) - ((-1.0 if r1 == 1 else 1.0) if r1 == j else 0.0)
            P[j] = 0.0 if e0 == 0.0 else e0
            P[3 + j] = 0.0 if e1 == 0.0 else e1
    else:
        for j in range(3):
            P[j] = (-1.0 if r0 == 1 else 1.0) if r0 == j else 0.0
            P[3 + j] = (-1.0 if r1 == 1 else 1.0) if r1 == j else 0.0
    return P


def _bits(x):
    return int(np.float64(x).view(np.uint64))


def _normals(rng):
    out = [tuple(float(v) for v in rng.standard_normal(3)) for _ in range(20000)]
    for ax in range(3):
        for sg in (1.0, -1.0):
            e = [0.0, 0.0, 0.0]
            e[ax] = sg
            out.append(tuple(e))
            for eps in (1e-300, 1e-17, 1e-9, 1e-3):
                for other in range(3):
                    if other != ax:
                        f = list(e)
                        f[other] = eps * rng.choice([-1.0, 1.0])
                        out.append(tuple(f))
            g = list(e)
            g[(ax + 1) % 3] = -0.0
            out.append(tuple(g))
    # Newell normals of random triangles (the inputs the device sees)
    for _ in range(5000):
        v = rng.standard_normal((3, 3)) * 2.0 ** rng.integers(-20, 20)
        n = [0.0, 0.0, 0.0]
        for i in range(3):
            c, x = v[i], v[(i + 1) % 3]
            n[0] = n[0] + (c[1] - x[1]) * (c[2] + x[2])
            n[1] = n[1] + (c[2] - x[2]) * (c[0] + x[0])
            n[2] = n[2] + (c[0] - x[0]) * (c[1] + x[1])
        if dot3(n, n) > 0.0:
            out.append(tuple(n))
    return [tuple(float(x) for x in n) for n in out]


def test_device_projection_is_the_reference_product():
    rng = np.random.default_rng(51)
    for n in _normals(rng):
        mc = largest_component(n)
        ref, dev = reference(n, mc), device(n, mc)
        assert [_bits(x) for x in dev] == [_bits(x) for x in ref], (n, ref, dev)
