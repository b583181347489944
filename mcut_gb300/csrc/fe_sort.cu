// LSD radix sort of (key, uint32 value) pairs, 8-bit digits, stable.
//
// One pass = three launches:
//   upsweep  : per-tile digit histogram (shared-memory atomics)
//   scan     : exclusive scan of the digit-major [256 x tiles] table (one CTA)
//   downsweep: each warp ranks its keys with __match_any_sync in input order,
//              warps are combined per digit in shared memory, keys scatter to
//              their global rank.
// A tile is 256 threads x 16 keys. Keys and values stream through HBM once
// per launch; the histogram table stays in L2.
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
constexpr int kDigits = 256;

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
        if (idx < n) atomicAdd(&h[(uint32_t)(k[i] >> shift) & 0xFFu], 1u);
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

template <typename K>
__global__ void __launch_bounds__(kThreads) k_downsweep(const K* __restrict__ keys, const uint32_t* __restrict__ vals,
    K* __restrict__ okeys, uint32_t* __restrict__ ovals, uint32_t n, int shift, const uint32_t* __restrict__ hist,
    uint32_t tiles, const uint32_t* __restrict__ totals)
{
    __shared__ uint32_t wh[kWarps][kDigits];
    __shared__ uint32_t goff[kDigits];
    __shared__ uint32_t wsum[kWarps];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < kWarps * kDigits; i += kThreads) (&wh[0][0])[i] = 0;
    {
        // digit bases: exclusive scan of the 256 digit totals (kThreads == kDigits)
        const uint32_t v = totals[threadIdx.x];
        uint32_t inc = v;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, inc, o);
            if (lane >= o) inc += t;
        }
        if (lane == 31) wsum[warp] = inc;
        __syncthreads();
        uint32_t wpre = 0;
        for (int k = 0; k < warp; ++k) wpre += wsum[k];
        goff[threadIdx.x] = wpre + inc - v + hist[(size_t)threadIdx.x * tiles + blockIdx.x];
    }
    __syncthreads();

    const size_t wbase = (size_t)blockIdx.x * kTile + (size_t)warp * 32 * kItems;
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
        const uint32_t d = ok ? ((uint32_t)(k[i] >> shift) & 0xFFu) : 0x100u; // 0x100: padding, no digit
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
        uint32_t prev = 0;
        if (ok) prev = wh[warp][d];
        __syncwarp();
        if (ok && (peers & lt) == 0) wh[warp][d] = prev + __popc(peers);
        __syncwarp();
        rank[i] = prev + __popc(peers & lt);
    }
    __syncthreads();
    // per digit: exclusive prefix across warps, plus the tile's global offset
    for (int d = threadIdx.x; d < kDigits; d += kThreads) {
        uint32_t run = goff[d];
        for (int w = 0; w < kWarps; ++w) {
            const uint32_t c = wh[w][d];
            wh[w][d] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        const size_t idx = wbase + (size_t)i * 32 + lane;
        if (idx < n) {
            const uint32_t d = (uint32_t)(k[i] >> shift) & 0xFFu;
            const uint32_t dst = wh[warp][d] + rank[i];
            okeys[dst] = k[i];
            ovals[dst] = v[i];
        }
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

size_t radix_sort_temp_bytes(uint32_t n)
{
    const uint32_t tiles = (n + kTile - 1) / kTile;
    const size_t table = (size_t)kDigits * (tiles ? tiles : 1);
    return (table + kDigits + 64) * sizeof(uint32_t);
}

template <typename K>
int radix_sort_pairs(K* keys, uint32_t* vals, K* keys_alt, uint32_t* vals_alt, uint32_t n, int begin_bit, int end_bit,
    uint32_t* temp, cudaStream_t s)
{
    if (n == 0) return 0;
    const uint32_t tiles = (n + kTile - 1) / kTile;
    int cur = 0;
    K* kb[2] = { keys, keys_alt };
    uint32_t* vb[2] = { vals, vals_alt };
    for (int shift = begin_bit; shift < end_bit; shift += 8) {
        uint32_t* totals = temp + (size_t)kDigits * tiles;
        g_launches += 3;
        k_upsweep<K><<<tiles, kThreads, 0, s>>>(kb[cur], n, shift, temp, tiles);
        k_digit_scan<<<kDigits, kThreads, 0, s>>>(temp, tiles, totals);
        k_downsweep<K><<<tiles, kThreads, 0, s>>>(kb[cur], vb[cur], kb[cur ^ 1], vb[cur ^ 1], n, shift, temp, tiles,
            totals);
        cur ^= 1;
    }
    return cur;
}

// One-CTA LSD radix sort for small inputs (n <= kSmallSort): every pass runs
// in shared memory, so the whole sort is one launch instead of three per
// pass. Keys carry their input position in the low 14 bits (composite
// uint64, so end_bit + 14 <= 64); 16 warps, warp w ranks its contiguous chunk
// in rounds of 32 keys (stable), digit offsets come from a (digit, warp) scan.
constexpr int kSmallThreads = 512;
constexpr int kSmallWarps = kSmallThreads / 32;
constexpr int kSmallIdxBits = 14;

__global__ void __launch_bounds__(kSmallThreads) k_sort_small(const unsigned long long* __restrict__ keys_in,
    const uint32_t* __restrict__ vals_in, unsigned long long* __restrict__ keys_out, uint32_t* __restrict__ vals_out,
    uint32_t n, int end_bit)
{
    extern __shared__ __align__(16) unsigned char sm[];
    unsigned long long* kb[2] = { reinterpret_cast<unsigned long long*>(sm),
        reinterpret_cast<unsigned long long*>(sm) + kSmallSort };
    uint32_t (*wh)[kDigits] = reinterpret_cast<uint32_t (*)[kDigits]>(kb[1] + kSmallSort);
    uint32_t* dbase = reinterpret_cast<uint32_t*>(wh + kSmallWarps);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t lt = (1u << lane) - 1u;
    for (uint32_t i = threadIdx.x; i < n; i += kSmallThreads) kb[0][i] = (keys_in[i] << kSmallIdxBits) | i;
    const uint32_t chunk = ((n + kSmallWarps - 1) / kSmallWarps + 31) & ~31u;
    int cur = 0;
    for (int shift = kSmallIdxBits; shift < end_bit + kSmallIdxBits; shift += 8) {
        for (int i = threadIdx.x; i < kSmallWarps * kDigits; i += kSmallThreads) (&wh[0][0])[i] = 0;
        __syncthreads();
        uint32_t rank[kSmallSort / kSmallWarps / 32];
        const uint32_t lo = w * chunk;
        for (uint32_t r = 0; r * 32 < chunk; ++r) {
            const uint32_t idx = lo + r * 32 + lane;
            const bool ok = idx < n;
            const uint32_t d = ok ? (uint32_t)(kb[cur][idx] >> shift) & 0xFFu : 0x100u;
            const uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
            uint32_t prev = 0;
            if (ok) prev = wh[w][d];
            __syncwarp();
            if (ok && (peers & lt) == 0) wh[w][d] = prev + __popc(peers);
            __syncwarp();
            rank[r] = prev + __popc(peers & lt);
        }
        __syncthreads();
        if (threadIdx.x < kDigits) {
            const int d = threadIdx.x;
            uint32_t run = 0;
            for (int k = 0; k < kSmallWarps; ++k) {
                const uint32_t c = wh[k][d];
                wh[k][d] = run;
                run += c;
            }
            dbase[d] = run;
        }
        __syncthreads();
        if (threadIdx.x < 32) {
            // exclusive scan of the 256 digit totals by one warp (8 per lane)
            uint32_t v[8], sum = 0;
            for (int k = 0; k < 8; ++k) { v[k] = dbase[lane * 8 + k]; sum += v[k]; }
            uint32_t inc = sum;
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, inc, o);
                if (lane >= o) inc += t;
            }
            uint32_t run = inc - sum;
            for (int k = 0; k < 8; ++k) { dbase[lane * 8 + k] = run; run += v[k]; }
        }
        __syncthreads();
        for (uint32_t r = 0; r * 32 < chunk; ++r) {
            const uint32_t idx = lo + r * 32 + lane;
            if (idx < n) {
                const unsigned long long k = kb[cur][idx];
                const uint32_t d = (uint32_t)(k >> shift) & 0xFFu;
                kb[cur ^ 1][dbase[d] + wh[w][d] + rank[r]] = k;
            }
        }
        __syncthreads();
        cur ^= 1;
    }
    for (uint32_t i = threadIdx.x; i < n; i += kSmallThreads) {
        const unsigned long long c = kb[cur][i];
        keys_out[i] = c >> kSmallIdxBits;
        vals_out[i] = vals_in[c & ((1u << kSmallIdxBits) - 1u)];
    }
}

size_t sort_small_smem() { return (size_t)kSmallSort * 16 + (size_t)kSmallWarps * kDigits * 4 + kDigits * 4; }

void sort_small_pairs(const unsigned long long* keys_in, const uint32_t* vals_in, unsigned long long* keys_out,
    uint32_t* vals_out, uint32_t n, int end_bit, cudaStream_t s)
{
    static std::atomic<unsigned long long> attr { 0 };
    set_smem_once((const void*)k_sort_small, (int)sort_small_smem(), attr);
    g_launches++;
    k_sort_small<<<1, kSmallThreads, sort_small_smem(), s>>>(keys_in, vals_in, keys_out, vals_out, n, end_bit);
}

template int radix_sort_pairs<uint32_t>(uint32_t*, uint32_t*, uint32_t*, uint32_t*, uint32_t, int, int, uint32_t*,
    cudaStream_t);
template int radix_sort_pairs<unsigned long long>(unsigned long long*, uint32_t*, unsigned long long*, uint32_t*,
    uint32_t, int, int, uint32_t*, cudaStream_t);

} // namespace mcgpu
