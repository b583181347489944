"""CPU model of the cut tree's bottom-up build (k_build in fe_kernels.cu).

Every leaf climbs; the first child to reach a split deposits its far end and
stops, the second builds the parent. Splits whose node lies inside the
leaf's window (a larger boundary delta on each side within the window,
found from prefix / suffix maxima) exchange there, the rest through a
global table. Under random thread interleavings the model must give the
Karras construction's tree node for node (children and leaf ranges, Karras
numbering), with every node built exactly once.
"""
import random

import pytest

TOP = (2 ** 64 - 1, 2 ** 32 - 1)  # boundary delta beyond either mesh end


def clz32(v):
    return 32 - v.bit_length()


def karras(keys):
    """Karras (HPG 2012) over sorted keys, duplicates ordered by position:
    node i -> (left child, right child, first leaf, last leaf); ~j is leaf j."""
    n = len(keys)

    def delta(i, j):
        if j < 0 or j >= n:
            return -1
        if keys[i] == keys[j]:
            return 32 + clz32(i ^ j)
        return clz32(keys[i] ^ keys[j])

    nodes = {}
    for i in range(n - 1):
        d = 1 if delta(i, i + 1) - delta(i, i - 1) >= 0 else -1
        dmin = delta(i, i - d)
        lmax = 2
        while delta(i, i + lmax * d) > dmin:
            lmax <<= 1
        length, t = 0, lmax >> 1
        while t >= 1:
            if delta(i, i + (length + t) * d) > dmin:
                length += t
            t >>= 1
        j = i + length * d
        dnode = delta(i, j)
        split, t = 0, (length + 1) >> 1
        while True:
            if delta(i, i + (split + t) * d) > dnode:
                split += t
            if t == 1:
                break
            t = (t + 1) >> 1
        gamma = i + split * d + min(d, 0)
        lo, hi = min(i, j), max(i, j)
        nodes[i] = (~gamma if lo == gamma else gamma, ~(gamma + 1) if hi == gamma + 1 else gamma + 1, lo, hi)
    return nodes


def boundary(keys, j):
    """D(j): key XOR above position XOR of sorted leaves j and j+1."""
    if j < 0 or j >= len(keys) - 1:
        return TOP
    return (keys[j] ^ keys[j + 1], j ^ (j + 1))


def bottom_up(keys, window, rng):
    """The kernel's algorithm, one generator per leaf thread, interleaved at
    random at every exchange."""
    n = len(keys)
    inside = {}
    for b in range((n + window - 1) // window):
        w0, w1 = b * window, min(n, (b + 1) * window) - 1
        for i in range(w0, w1 + 1):
            d = boundary(keys, i)
            left = max(boundary(keys, j) for j in range(w0 - 1, i))
            right = max((boundary(keys, j) for j in range(i + 1, w1 + 1)), default=(0, 0))
            inside[(b, i - w0)] = i < w1 and d < left and d < right
    nodes, far_local, far_global, box_local, box_global = {}, {}, {}, {}, {}

    def thread(i):
        b = i // window
        w0, w1 = b * window, min(n, (b + 1) * window) - 1
        lo, hi, box = i, i, (i, i)  # the leaf range stands in for the box
        dl, dr = boundary(keys, i - 1), boundary(keys, i)
        while True:
            right = dr < dl  # the parent extends right: this node is its left child
            s = hi if right else lo - 1
            slot, far = (0, lo) if right else (1, hi)
            assert 0 <= s < n - 1
            yield
            if 0 <= s - w0 < window and inside[(b, s - w0)]:
                assert lo >= w0 and hi <= w1, "a window exchange from a node outside the window"
                key, fars, boxes = (b, s - w0), far_local, box_local
            else:
                key, fars, boxes = s, far_global, box_global
            boxes[(key, slot)] = box
            prev, fars[key] = fars.get(key), far
            if prev is None:
                return
            other = boxes[(key, slot ^ 1)]
            pl, pr = (lo, prev) if right else (prev, hi)
            pdl, pdr = boundary(keys, pl - 1), boundary(keys, pr)
            root = pl == 0 and pr == n - 1
            pidx = 0 if root else (pr if pdr < pdl else pl)
            assert pidx not in nodes, "a node built twice"
            lb, rb = (box, other) if right else (other, box)
            assert lb[1] + 1 == rb[0] and lb[0] == pl and rb[1] == pr
            nodes[pidx] = (~s if pl == s else s, ~(s + 1) if s + 1 == pr else s + 1, pl, pr)
            box = (pl, pr)
            if root:
                return
            lo, hi, dl, dr = pl, pr, pdl, pdr

    threads = [thread(i) for i in range(n)]
    live = list(range(n))
    while live:
        k = rng.randrange(len(live))
        try:
            next(threads[live[k]])
        except StopIteration:
            live.pop(k)
    return nodes


@pytest.mark.parametrize("seed", range(6))
def test_bottom_up_build_gives_the_karras_tree(seed):
    rng = random.Random(seed)
    for _ in range(12):
        n = rng.choice([2, 3, 5, 17, 64, 127, 128, 129, 300, 700])
        window = rng.choice([4, 8, 32, 128])
        mode = rng.randrange(4)
        if mode == 0:
            keys = sorted(rng.randrange(2 ** 30) for _ in range(n))
        elif mode == 1:
            keys = sorted(rng.randrange(16) for _ in range(n))  # many duplicates
        elif mode == 2:
            keys = [7] * n
        else:
            keys = sorted(rng.randrange(2 ** 10) << rng.randrange(20) for _ in range(n))
        expect = karras(keys)
        got = bottom_up(keys, window, rng)
        assert len(got) == n - 1
        for i in range(n - 1):
            assert expect[i] == got[i], (n, window, i)


@pytest.mark.parametrize("seed", range(4))
def test_every_pair_of_a_batch_has_its_own_subtree(seed):
    """A batch's cut keys carry the pair above the Morton code (pair << 23 |
    code), so each pair with two or more leaf clusters owns exactly one node
    whose leaf range is the pair's clusters: the node k_build records as the
    pair's root, where a one-pair query packet starts its walk (the nodes
    above it hold other pairs' clusters only)."""
    rng = random.Random(100 + seed)
    for _ in range(10):
        npairs = rng.choice([2, 3, 7, 40])
        keys, ranges = [], []
        for p in range(npairs):
            cnt = rng.choice([0, 1, 2, 3, 9, 33, 150])
            codes = sorted(rng.randrange(16 if rng.random() < 0.3 else 2 ** 23) for _ in range(cnt))
            ranges.append((len(keys), len(keys) + cnt - 1))
            keys += [(p << 23) | c for c in codes]
        if len(keys) < 2:
            continue
        nodes = karras(keys)
        for lo, hi in ranges:
            if hi - lo + 1 < 2:
                continue
            owners = [i for i, (_, _, a, b) in nodes.items() if (a, b) == (lo, hi)]
            assert len(owners) == 1, (lo, hi, owners)
            # the same node from the bottom-up build's merge rule
            built = bottom_up(keys, 32, rng)
            assert built[owners[0]][2:] == (lo, hi)
