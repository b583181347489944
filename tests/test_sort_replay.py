"""The device's replay of libstdc++'s std::sort orders ties as std::sort does.

A polygon's plane-defining triplet is the first entry after the reference
sorts all vertex triplets by |orient2d| descending with std::sort
(determine_three_noncollinear_vertices, math.cpp:289-389). std::sort is not
stable, so equal values keep the order its introsort schedule leaves them
in, and the device replays that schedule (t_std_sort in fe_kernels.cu):
median-of-three pivot, unguarded partition, heap sort at the depth limit,
and the final insertion sorts. This module restates the replay operation for
operation and compares the resulting order with g++'s own std::sort (a
small C++ program built here). The inputs are tie-heavy arrays of every size
up to 400, all-equal, sorted and reversed arrays, and an adversarial input
(McIlroy's "killer adversary for quicksort") that drives the introsort to
its heap-sort fallback.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BUILD = os.path.join(ROOT, "tests", "_build")

CPP = r"""
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>
struct T { double v; int i; };
int main() {
    int n;
    while (std::scanf("%d", &n) == 1) {
        std::vector<T> a(n);
        for (int k = 0; k < n; ++k) { std::scanf("%lf", &a[k].v); a[k].i = k; }
        std::sort(a.begin(), a.end(), [](const T& x, const T& y) { return std::fabs(x.v) > std::fabs(y.v); });
        for (int k = 0; k < n; ++k) std::printf("%d ", a[k].i);
        std::printf("\n");
    }
    return 0;
}
"""


def std_sort_orders(arrays):
    os.makedirs(BUILD, exist_ok=True)
    src, exe = os.path.join(BUILD, "stdsort.cpp"), os.path.join(BUILD, "stdsort")
    with open(src, "w") as fh:
        fh.write(CPP)
    subprocess.run(["g++", "-O2", "-std=c++17", "-o", exe, src], check=True)
    text = "".join(f"{len(a)} " + " ".join(repr(float(x)) for x in a) + "\n" for a in arrays)
    out = subprocess.run([exe], input=text, check=True, capture_output=True, text=True).stdout
    return [[int(t) for t in ln.split()] for ln in out.splitlines()]


# ---- the device's replay (t_std_sort and its helpers), on [value, index] lists ----

def by_magnitude(a, b):
    """The device's tless: larger |value| first."""
    return abs(a[0]) > abs(b[0])


def ins_sort(f, lo, n, tless):
    for i in range(lo + 1, lo + n):
        v = f[i]
        if tless(v, f[lo]):
            f[lo + 1:i + 1] = f[lo:i]
            f[lo] = v
        else:
            j = i
            while tless(v, f[j - 1]):
                f[j] = f[j - 1]
                j -= 1
            f[j] = v


def unguarded_ins(f, frm, n, tless):
    for i in range(frm, n):
        v = f[i]
        j = i
        while tless(v, f[j - 1]):
            f[j] = f[j - 1]
            j -= 1
        f[j] = v


def median(f, r, a, b, c, tless):
    def sw(x, y):
        f[x], f[y] = f[y], f[x]
    if tless(f[a], f[b]):
        if tless(f[b], f[c]):
            sw(r, b)
        elif tless(f[a], f[c]):
            sw(r, c)
        else:
            sw(r, a)
    elif tless(f[a], f[c]):
        sw(r, a)
    elif tless(f[b], f[c]):
        sw(r, c)
    else:
        sw(r, b)


def sift(f, base, hole, length, v, tless):
    top = hole
    child = hole
    while child < (length - 1) // 2:
        child = 2 * (child + 1)
        if tless(f[base + child], f[base + child - 1]):
            child -= 1
        f[base + hole] = f[base + child]
        hole = child
    if (length & 1) == 0 and child == (length - 2) // 2:
        child = 2 * (child + 1)
        f[base + hole] = f[base + child - 1]
        hole = child - 1
    par = (hole - 1) // 2
    while hole > top and tless(f[base + par], v):
        f[base + hole] = f[base + par]
        hole = par
        par = (hole - 1) // 2
    f[base + hole] = v


def heap_sort(f, base, n, log, tless):
    log.append("heap")
    if n < 2:
        return
    par = (n - 2) // 2
    while True:
        sift(f, base, par, n, f[base + par], tless)
        if par == 0:
            break
        par -= 1
    for last in range(n - 1, 0, -1):
        v = f[base + last]
        f[base + last] = f[base]
        sift(f, base, 0, last, v, tless)


def device_sort(values, log=None, tless=by_magnitude):
    log = [] if log is None else log
    f = [[float(v), i] for i, v in enumerate(values)]
    n = len(f)
    if n < 2:
        return [x[1] for x in f]
    stack = []
    off, length, depth = 0, n, 2 * (n.bit_length() - 1)
    while True:
        while length > 16:
            if depth == 0:
                heap_sort(f, off, length, log, tless)
                length = 0
                break
            depth -= 1
            mid = length // 2
            median(f, off, off + 1, off + mid, off + length - 1, tless)
            lo, hi = 1, length
            while True:
                while tless(f[off + lo], f[off]):
                    lo += 1
                hi -= 1
                while tless(f[off], f[off + hi]):
                    hi -= 1
                if not lo < hi:
                    break
                f[off + lo], f[off + hi] = f[off + hi], f[off + lo]
                lo += 1
            assert len(stack) < 64
            stack.append((off + lo, length - lo, depth))
            length = lo
        if not stack:
            break
        off, length, depth = stack.pop()
    if n > 16:
        ins_sort(f, 0, 16, tless)
        unguarded_ins(f, 16, n, tless)
    else:
        ins_sort(f, 0, n, tless)
    return [x[1] for x in f]


def killer(n):
    """McIlroy's adversary (Software: Practice and Experience 29(4), 1999):
    values are fixed lazily, the pivot candidate becoming 'gas' -> solid, so
    that every partition is as uneven as the comparisons allow. Run against
    the replay, it yields a concrete input that exhausts the depth limit."""
    gas = n
    val = [gas] * n
    state = {"nsolid": 0, "candidate": 0}

    def freeze(x):
        val[x] = state["nsolid"]
        state["nsolid"] += 1

    def cmp_less(a, b):  # is item a < item b under the adversary
        x, y = a[1], b[1]
        if val[x] == gas and val[y] == gas:
            if x == state["candidate"]:
                freeze(x)
            else:
                freeze(y)
        if val[x] == gas:
            state["candidate"] = x
        elif val[y] == gas:
            state["candidate"] = y
        return val[x] < val[y]

    # descending by |v| sorts larger first: "a before b" == a has the larger key
    device_sort(list(range(n)), tless=lambda a, b: cmp_less(b, a))
    for i in range(n):
        if val[i] == gas:
            freeze(i)
    return [float(v) for v in val]


@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_replay_orders_as_std_sort():
    rng = np.random.default_rng(61)
    arrays = []
    for n in list(range(2, 70)) + list(rng.integers(70, 400, size=60)):
        k = int(rng.integers(1, 6))
        arrays.append(rng.choice([0.0, 1.0, 2.0, 3.0, 5.0, 8.0][:k + 1], size=n) * rng.choice([-1.0, 1.0], size=n))
        arrays.append(rng.standard_normal(n).round(1))
    arrays += [np.ones(300), np.arange(300.0), -np.arange(300.0), np.arange(300.0) % 7]
    kill = killer(220)
    arrays.append(np.array(kill))
    log = []
    device_sort(kill, log)
    assert "heap" in log  # the adversarial input reaches the heap-sort fallback
    want = std_sort_orders(arrays)
    for a, w in zip(arrays, want):
        assert device_sort(a) == w, len(a)
