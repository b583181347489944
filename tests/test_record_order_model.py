"""CPU model of the device's record ordering (k_sort_slices + k_rank_records
+ k_scatter_records in fe_kernels.cu): each 512-key slice is sorted in place
by a bitonic network in which thread t of 256 compares element
a = 2t - (t & (stride - 1)) with a + stride; every record's rank is the sum
over slices of the slice's keys below it (a lower bound in the sorted
slice); the scatter puts record i at its rank. The model runs the same
index arithmetic and checks that the ranks are a permutation giving the
keys in ascending order, for full, partial and single slices."""
import numpy as np
import pytest

CHUNK, THREADS = 512, 256


def sort_slice(keys, vals):
    m = len(keys)
    sk = np.full(CHUNK, np.iinfo(np.uint64).max, np.uint64)
    sv = np.zeros(CHUNK, np.uint32)
    sk[:m], sv[:m] = keys, vals
    size = 2
    while size <= CHUNK:
        stride = size >> 1
        while stride > 0:
            t = np.arange(THREADS)
            a = 2 * t - (t & (stride - 1))
            b = a + stride
            assert a.max() < CHUNK and b.max() < CHUNK and len(np.unique(np.concatenate([a, b]))) == CHUNK
            up = (a & size) == 0
            ka, kb = sk[a].copy(), sk[b].copy()
            sw = (ka > kb) == up
            sk[a[sw]], sk[b[sw]] = kb[sw], ka[sw]
            va, vb = sv[a].copy(), sv[b].copy()
            sv[a[sw]], sv[b[sw]] = vb[sw], va[sw]
            stride >>= 1
        size <<= 1
    return sk[:m], sv[:m]


@pytest.mark.parametrize("n", [1, 7, 511, 512, 513, 4000, 11000])
def test_slices_then_ranks_sort_every_key(n):
    rng = np.random.default_rng(n)
    keys = rng.choice(np.uint64(1) << np.uint64(40), size=n, replace=False).astype(np.uint64)
    vals = np.arange(n, dtype=np.uint32)
    for lo in range(0, n, CHUNK):
        keys[lo:lo + CHUNK], vals[lo:lo + CHUNK] = sort_slice(keys[lo:lo + CHUNK], vals[lo:lo + CHUNK])
        assert np.all(np.diff(keys[lo:lo + CHUNK].astype(np.float64)) > 0)
    rank = np.zeros(n, np.int64)
    for lo in range(0, n, CHUNK):
        rank += np.searchsorted(keys[lo:lo + CHUNK], keys, side="left")
    assert np.array_equal(np.sort(rank), np.arange(n))
    out = np.empty(n, np.uint64)
    out[rank] = keys
    assert np.all(np.diff(out.astype(np.float64)) > 0)
    back = np.empty(n, np.uint32)
    back[rank] = vals
    assert sorted(back.tolist()) == list(range(n))
