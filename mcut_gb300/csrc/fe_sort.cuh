// Device radix sort and scan used by the front-end kernels.
#pragma once
#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>

namespace mcgpu {

// kernels launched by the calling thread (each API call reports its own difference)
extern thread_local unsigned long long g_launches;
// cudaFuncSetAttribute(MaxDynamicSharedMemorySize) once per device (`done`: bit per device)
void set_smem_once(const void* func, int bytes, std::atomic<unsigned long long>& done);

// Digit width of one radix pass and keys per tile.
#ifndef MCGPU_SORT_BITS
#define MCGPU_SORT_BITS 8
#endif
constexpr int kSortDigitBits = MCGPU_SORT_BITS;
constexpr uint32_t kSortDigits = 1u << kSortDigitBits;
constexpr uint32_t kSortTile = 4096;

// Scratch (bytes) the sort needs for n keys: the [digit x tile] count table
// and the digit totals.
constexpr size_t radix_sort_temp_bytes(uint32_t n)
{
    return ((size_t)kSortDigits * (n ? (n + kSortTile - 1) / kSortTile : 1) + kSortDigits + 64) * sizeof(uint32_t);
}

// Sorts (keys, vals) by bits [begin_bit, end_bit) of the key, stably.
// Ping-pongs between (keys, vals) and (keys_alt, vals_alt); returns 0 if the
// result is in (keys, vals), 1 if in the alternates.
template <typename K>
int radix_sort_pairs(K* keys, uint32_t* vals, K* keys_alt, uint32_t* vals_alt, uint32_t n, int begin_bit, int end_bit,
    uint32_t* temp, cudaStream_t s);

// In-place exclusive scan of n uint32 (n+1-th element receives the total if
// total_out != nullptr). temp: scan_temp_bytes(n).
size_t scan_temp_bytes(uint32_t n);
void exclusive_scan(uint32_t* a, uint32_t n, uint32_t* total_out, uint32_t* temp, cudaStream_t s);

} // namespace mcgpu
