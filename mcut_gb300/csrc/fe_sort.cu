// LSD radix sort of (key, uint32 value) pairs, kSortDigitBits-bit digits,
// stable.
//
// One pass = three launches:
//   upsweep  : per-tile digit histogram (shared-memory atomics)
//   scan     : exclusive scan of the digit-major [digits x tiles] table, one
//              CTA per digit
//   downsweep: each warp ranks its keys in input order (lanes of equal digit
//              found by one ballot per digit bit), warps are combined per
//              digit in shared memory, the tile is reordered by digit in
//              shared memory and written out so that consecutive threads
//              store consecutive slots of a digit's run.
// A tile is 256 threads x 16 keys. Keys and values stream through HBM once
// per launch; the histogram table stays in L2.
#include <algorithm>
#include <atomic>
#include "fe_sort.cuh"

namespace mcgpu {

thread_local unsigned long long g_launches = 0;

void set_smem_once(const void* func, int bytes, std::atomic<unsigned long long>& done)
{
    int dev = 0;
    cudaGetDevice(&dev);
    const unsigned long long bit = 1ull << (dev & 63);
    if (done.load(std::memory_order_acquire) & bit) return;
    cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    done.fetch_or(bit, std::memory_order_acq_rel);
}

namespace {
constexpr int kThreads = 256;
constexpr int kItems = 16;
constexpr int kTile = kThreads * kItems;
constexpr int kWarps = kThreads / 32;
constexpr int kBits = kSortDigitBits;
constexpr int kDigits = (int)kSortDigits;
constexpr uint32_t kMask = kSortDigits - 1u;
constexpr int kPer = kDigits / kThreads; // consecutive digits a thread owns in the block-wide scans
static_assert(kTile == (int)kSortTile, "tile size");
static_assert(kDigits >= kThreads && kDigits % kThreads == 0, "digits per thread");
// the per-warp digit counts alias the tile's key area
static_assert((size_t)kWarps * kDigits * 4 <= (size_t)kTile * 8, "per-warp counts fit the tile buffer");

template <typename K>
__global__ void __launch_bounds__(kThreads) k_upsweep(const K* __restrict__ keys, uint32_t n, int shift,
    uint32_t* __restrict__ hist, uint32_t tiles)
{
    __shared__ uint32_t h[kDigits];
    for (int i = threadIdx.x; i < kDigits; i += kThreads) h[i] = 0;
    // all loads first: they are independent and overlap; the shared-memory
    // atomics below would otherwise serialise them
    K k[kItems];
    const size_t base = (size_t)blockIdx.x * kTile;
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        const size_t idx = base + (size_t)i * kThreads + threadIdx.x;
        k[i] = idx < n ? keys[idx] : (K)0;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        const size_t idx = base + (size_t)i * kThreads + threadIdx.x;
        if (idx < n) atomicAdd(&h[(uint32_t)(k[i] >> shift) & kMask], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kDigits; i += kThreads) hist[(size_t)i * tiles + blockIdx.x] = h[i];
}

// exclusive scan of m entries by one CTA of 1024 threads
__global__ void __launch_bounds__(1024) k_scan(uint32_t* __restrict__ a, uint32_t m)
{
    __shared__ uint32_t part[1024];
    const uint32_t per = (m + 1023) / 1024;
    const uint32_t lo = threadIdx.x * per, hi = min(m, lo + per);
    uint32_t s = 0;
    for (uint32_t i = lo; i < hi; ++i) s += a[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        uint32_t v = threadIdx.x >= off ? part[threadIdx.x - off] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t run = part[threadIdx.x] - s;
    for (uint32_t i = lo; i < hi; ++i) {
        const uint32_t v = a[i];
        a[i] = run;
        run += v;
    }
}

// one CTA per digit: exclusive scan of that digit's per-tile counts (in
// place) and the digit's total
__global__ void __launch_bounds__(kThreads) k_digit_scan(uint32_t* __restrict__ hist, uint32_t tiles,
    uint32_t* __restrict__ totals)
{
    __shared__ uint32_t ws[kWarps];
    uint32_t* row = hist + (size_t)blockIdx.x * tiles;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t carry = 0;
    for (uint32_t base = 0; base < tiles; base += kThreads) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t v = i < tiles ? row[i] : 0u;
        uint32_t inc = v;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, inc, o);
            if (lane >= o) inc += t;
        }
        if (lane == 31) ws[w] = inc;
        __syncthreads();
        uint32_t wpre = 0, tot = 0;
        for (int k = 0; k < kWarps; ++k) {
            if (k < w) wpre += ws[k];
            tot += ws[k];
        }
        if (i < tiles) row[i] = carry + wpre + inc - v;
        carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) totals[blockIdx.x] = carry;
}

// block-wide exclusive scan of one value per thread (wsum: kWarps words;
// every thread must call it)
__device__ __forceinline__ uint32_t block_exclusive(uint32_t x, uint32_t* wsum)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t inc = x;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, inc, o);
        if (lane >= o) inc += t;
    }
    __syncthreads();
    if (lane == 31) wsum[warp] = inc;
    __syncthreads();
    uint32_t wpre = 0;
    for (int w = 0; w < warp; ++w) wpre += wsum[w];
    return wpre + inc - x;
}

// Shared memory of the downsweep: the tile's keys and values in local
// sorted order (the per-warp digit counts before that), then the digits'
// global and tile-local run starts.
template <typename K>
constexpr size_t downsweep_smem()
{
    return (size_t)kTile * (sizeof(K) + sizeof(uint32_t)) + 2 * kDigits * sizeof(uint32_t) + kWarps * 4;
}

// four blocks per SM (<= 64 registers): the pass is bandwidth-bound and needs the occupancy
#ifndef MCGPU_DS_MINB
#define MCGPU_DS_MINB 4
#endif
template <typename K>
__global__ void __launch_bounds__(kThreads, MCGPU_DS_MINB) k_downsweep(const K* __restrict__ keys, const uint32_t* __restrict__ vals,
    K* __restrict__ okeys, uint32_t* __restrict__ ovals, uint32_t n, int shift, const uint32_t* __restrict__ hist,
    uint32_t tiles, const uint32_t* __restrict__ totals)
{
    extern __shared__ __align__(16) unsigned char ds_smem[];
    K* skeys = reinterpret_cast<K*>(ds_smem);                                // [kTile], after ranking
    uint32_t* svals = reinterpret_cast<uint32_t*>(skeys + kTile);            // [kTile], after ranking
    uint32_t (*wh)[kDigits] = reinterpret_cast<uint32_t (*)[kDigits]>(ds_smem); // [kWarps][kDigits], ranking only
    uint32_t* goff = reinterpret_cast<uint32_t*>(svals + kTile);             // global offset of digit d's run
    uint32_t* tstart = goff + kDigits;                                       // tile-local start of digit d
    uint32_t* wsum = tstart + kDigits;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int d0 = threadIdx.x * kPer; // the digits this thread owns in the scans
    for (int i = threadIdx.x; i < kWarps * kDigits; i += kThreads) (&wh[0][0])[i] = 0;
    {
        // digit bases: exclusive scan of the digit totals
        uint32_t tv[kPer], sum = 0;
#pragma unroll
        for (int r = 0; r < kPer; ++r) { tv[r] = totals[d0 + r]; sum += tv[r]; }
        uint32_t run = block_exclusive(sum, wsum);
#pragma unroll
        for (int r = 0; r < kPer; ++r) {
            goff[d0 + r] = run + hist[(size_t)(d0 + r) * tiles + blockIdx.x];
            run += tv[r];
        }
    }
    __syncthreads();
    const size_t tbase = (size_t)blockIdx.x * kTile;
    const size_t wbase = tbase + (size_t)warp * 32 * kItems;
    K k[kItems];
    uint32_t v[kItems], rank[kItems];
    const uint32_t lt = (1u << lane) - 1u;
    // all loads first (independent, in flight together), then the ranking
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        const size_t idx = wbase + (size_t)i * 32 + lane;
        const bool ok = idx < n;
        k[i] = ok ? keys[idx] : (K)0;
        v[i] = ok ? vals[idx] : 0u;
    }
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        const size_t idx = wbase + (size_t)i * 32 + lane;
        const bool ok = idx < n;
        const uint32_t d = (uint32_t)(k[i] >> shift) & kMask;
        // lanes with the same digit: one ballot per digit bit (padding lanes
        // are left out by the first ballot and never use their own mask)
        uint32_t peers = __ballot_sync(0xFFFFFFFFu, ok);
#pragma unroll
        for (int b = 0; b < kBits; ++b) {
            const bool bit = (d >> b) & 1u;
            const uint32_t m = __ballot_sync(0xFFFFFFFFu, bit);
            peers &= bit ? m : ~m;
        }
        uint32_t prev = 0;
        if (ok) prev = wh[warp][d];
        __syncwarp();
        if (ok && (peers & lt) == 0) wh[warp][d] = prev + __popc(peers);
        __syncwarp();
        rank[i] = prev + __popc(peers & lt);
    }
    __syncthreads();
    // per digit: exclusive prefix across warps; tile-local digit starts:
    // exclusive scan of the digits' tile counts
    {
        uint32_t cnt[kPer], tot = 0;
#pragma unroll
        for (int r = 0; r < kPer; ++r) {
            uint32_t run = 0;
            for (int w = 0; w < kWarps; ++w) {
                const uint32_t c = wh[w][d0 + r];
                wh[w][d0 + r] = run;
                run += c;
            }
            cnt[r] = run;
            tot += run;
        }
        uint32_t start = block_exclusive(tot, wsum);
#pragma unroll
        for (int r = 0; r < kPer; ++r) {
            tstart[d0 + r] = start;
            start += cnt[r];
        }
    }
    __syncthreads();
    // tile-local sorted position of every key, then the keys go to shared
    // memory in that order (over the digit counts, which are read first)
    uint32_t pos[kItems];
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        const uint32_t d = (uint32_t)(k[i] >> shift) & kMask;
        pos[i] = tstart[d] + wh[warp][d] + rank[i];
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        const size_t idx = wbase + (size_t)i * 32 + lane;
        if (idx < n) {
            skeys[pos[i]] = k[i];
            svals[pos[i]] = v[i];
        }
    }
    __syncthreads();
    // consecutive threads write consecutive slots of each digit's run
    const uint32_t tn = (uint32_t)min((size_t)kTile, (size_t)n - tbase);
    for (uint32_t j = threadIdx.x; j < tn; j += kThreads) {
        const K key = skeys[j];
        const uint32_t d = (uint32_t)(key >> shift) & kMask;
        const uint32_t dst = goff[d] + (j - tstart[d]);
        okeys[dst] = key;
        ovals[dst] = svals[j];
    }
}
} // namespace

namespace {
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__global__ void __launch_bounds__(kScanThreads) k_block_reduce(const uint32_t* __restrict__ a, uint32_t n,
    uint32_t* __restrict__ bsum)
{
    __shared__ uint32_t ws[32];
    const size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
    uint32_t s = 0;
    for (int i = 0; i < kScanItems; ++i)
        if (base + i < n) s += a[base + i];
    for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xFFFFFFFFu, s, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = ws[threadIdx.x];
        for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xFFFFFFFFu, s, o);
        if (threadIdx.x == 0) bsum[blockIdx.x] = s;
    }
}

__global__ void __launch_bounds__(kScanThreads) k_block_scan(uint32_t* __restrict__ a, uint32_t n,
    const uint32_t* __restrict__ boff, uint32_t* __restrict__ total_out)
{
    __shared__ uint32_t ws[32];
    const size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
    uint32_t v[kScanItems], s = 0;
    for (int i = 0; i < kScanItems; ++i) {
        v[i] = base + i < n ? a[base + i] : 0u;
        s += v[i];
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t inc = s;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xFFFFFFFFu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) ws[w] = inc;
    __syncthreads();
    if (w == 0) {
        uint32_t x = ws[lane], y = x;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xFFFFFFFFu, y, o);
            if (lane >= o) y += t;
        }
        ws[lane] = y - x;
    }
    __syncthreads();
    uint32_t run = boff[blockIdx.x] + ws[w] + inc - s;
    for (int i = 0; i < kScanItems; ++i) {
        if (base + i < n) a[base + i] = run;
        run += v[i];
    }
    if (total_out && blockIdx.x == gridDim.x - 1 && threadIdx.x == kScanThreads - 1) *total_out = run;
}
} // namespace

size_t scan_temp_bytes(uint32_t n)
{
    const uint32_t nb = (n + kScanTile - 1) / kScanTile;
    return (size_t)(nb ? nb : 1) * sizeof(uint32_t);
}

void exclusive_scan(uint32_t* a, uint32_t n, uint32_t* total_out, uint32_t* temp, cudaStream_t s)
{
    if (n == 0) {
        if (total_out) cudaMemsetAsync(total_out, 0, sizeof(uint32_t), s);
        return;
    }
    const uint32_t nb = (n + kScanTile - 1) / kScanTile;
    g_launches += 3;
    k_block_reduce<<<nb, kScanThreads, 0, s>>>(a, n, temp);
    k_scan<<<1, 1024, 0, s>>>(temp, nb);
    k_block_scan<<<nb, kScanThreads, 0, s>>>(a, n, temp, total_out);
}

template <typename K>
int radix_sort_pairs(K* keys, uint32_t* vals, K* keys_alt, uint32_t* vals_alt, uint32_t n, int begin_bit, int end_bit,
    uint32_t* temp, cudaStream_t s)
{
    if (n == 0) return 0;
    static std::atomic<unsigned long long> attr { 0 };
    set_smem_once((const void*)k_downsweep<K>, (int)downsweep_smem<K>(), attr);
    const uint32_t tiles = (n + kTile - 1) / kTile;
    int cur = 0;
    K* kb[2] = { keys, keys_alt };
    uint32_t* vb[2] = { vals, vals_alt };
    for (int shift = begin_bit; shift < end_bit; shift += kBits) {
        uint32_t* totals = temp + (size_t)kDigits * tiles;
        g_launches += 3;
        k_upsweep<K><<<tiles, kThreads, 0, s>>>(kb[cur], n, shift, temp, tiles);
        k_digit_scan<<<kDigits, kThreads, 0, s>>>(temp, tiles, totals);
        k_downsweep<K><<<tiles, kThreads, downsweep_smem<K>(), s>>>(kb[cur], vb[cur], kb[cur ^ 1], vb[cur ^ 1], n,
            shift, temp, tiles, totals);
        cur ^= 1;
    }
    return cur;
}

template int radix_sort_pairs<uint32_t>(uint32_t*, uint32_t*, uint32_t*, uint32_t*, uint32_t, int, int, uint32_t*,
    cudaStream_t);
template int radix_sort_pairs<unsigned long long>(unsigned long long*, uint32_t*, unsigned long long*, uint32_t*,
    uint32_t, int, int, uint32_t*, cudaStream_t);

} // namespace mcgpu
