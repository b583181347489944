"""CPU model of the traversal's query packets (k_src_packets in fe_kernels.cu).

The sorted source faces are split into packets: maximal subtrees of the
Karras hierarchy over their keys holding at most `pmax` faces. Every internal
node whose range is larger than pmax emits each child range that fits. The
model restates the kernel's per-node computation (direction, range end by
exponential then binary search, split position) and requires two things for
random keys, duplicate runs included, and every pmax in 1..32. First, the
packets partition the faces: each face is queried exactly once, which makes
the candidate pair set complete and free of duplicates. Second, each packet
is a whole subtree of the independent Karras construction whose parent holds
more than pmax faces.
"""
import random

import pytest

from test_tree_model import clz32, karras


def delta(keys, i, j):
    if j < 0 or j >= len(keys):
        return -1
    if keys[i] == keys[j]:
        return 32 + clz32(i ^ j)
    return clz32(keys[i] ^ keys[j])


def packets(keys, pmax):
    """The kernel's emission, node by node."""
    n = len(keys)
    if n <= pmax:
        return [(0, n - 1)] if n else []
    out = []
    for i in range(n - 1):
        d = 1 if delta(keys, i, i + 1) - delta(keys, i, i - 1) >= 0 else -1
        dmin = delta(keys, i, i - d)
        lmax = 2
        while delta(keys, i, i + lmax * d) > dmin:
            lmax <<= 1
        length, t = 0, lmax >> 1
        while t >= 1:
            if delta(keys, i, i + (length + t) * d) > dmin:
                length += t
            t >>= 1
        j = i + length * d
        lo, hi = min(i, j), max(i, j)
        if hi - lo + 1 > pmax:
            dnode = delta(keys, i, j)
            s, t = 0, (length + 1) >> 1
            while True:
                if delta(keys, i, i + (s + t) * d) > dnode:
                    s += t
                if t == 1:
                    break
                t = (t + 1) >> 1
            gamma = i + s * d + min(d, 0)
            if gamma - lo + 1 <= pmax:
                out.append((lo, gamma))
            if hi - gamma <= pmax:
                out.append((gamma + 1, hi))
    return out


def _subtrees(keys):
    """Every node's leaf range in the independent construction, with its parent's size."""
    nodes = karras(keys)
    ranges = {}
    for i, (lc, rc, lo, hi) in nodes.items():
        for c in (lc, rc):
            if c < 0:
                ranges[(~c, ~c)] = hi - lo + 1
            else:
                clo, chi = nodes[c][2], nodes[c][3]
                ranges[(clo, chi)] = hi - lo + 1
    return ranges


@pytest.mark.parametrize("seed", range(8))
def test_packets_partition_the_faces_into_maximal_subtrees(seed):
    rng = random.Random(seed)
    for _ in range(30):
        n = rng.choice([1, 2, 5, 31, 32, 33, 64, 100, 257, 600])
        mode = rng.randrange(3)
        if mode == 0:
            keys = sorted(rng.randrange(2 ** 30) for _ in range(n))
        elif mode == 1:
            keys = sorted(rng.randrange(8) for _ in range(n))
        else:
            keys = sorted(rng.randrange(2 ** 12) << rng.randrange(18) for _ in range(n))
        pmax = rng.randint(1, 32)
        got = packets(keys, pmax)
        cover = [0] * n
        for lo, hi in got:
            assert 0 <= lo <= hi < n and hi - lo + 1 <= pmax
            for f in range(lo, hi + 1):
                cover[f] += 1
        assert cover == [1] * n, (n, pmax)
        if n > pmax:
            sub = _subtrees(keys)
            for lo, hi in got:
                assert (lo, hi) in sub, (lo, hi)
                assert sub[(lo, hi)] > pmax
