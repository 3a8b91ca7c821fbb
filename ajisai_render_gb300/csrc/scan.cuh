// Device-wide inclusive / exclusive scan of uint32 (reduce-then-scan over
// tiles of 2048, recursing on the tile totals).  Used by the radix sort
// (digit offsets), the PLOC merge compaction and the BVH layout pass.
#pragma once
#include "common.cuh"

namespace ajg {
// (internal linkage: several translation units include this header)
namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

// Block-level inclusive scan of kScanTile elements held 8 per thread.
__device__ __forceinline__ void block_scan_tile(uint32_t v[kScanItems],
                                                uint32_t* s_warp,
                                                uint32_t* total) {
  uint32_t run = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    run += v[k];
    v[k] = run;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = run;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < (kScanThreads / 32) ? s_warp[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < (kScanThreads / 32)) s_warp[lane] = w;
  }
  __syncthreads();
  const uint32_t before = (x - run) + (warp ? s_warp[warp - 1] : 0);
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) v[k] += before;
  if (total && threadIdx.x == kScanThreads - 1) *total = v[kScanItems - 1];
}

__global__ void k_scan_tiles(const uint32_t* __restrict__ in,
                             uint32_t* __restrict__ out, uint64_t n,
                             uint32_t* __restrict__ tile_totals,
                             int exclusive) {
  __shared__ uint32_t s_warp[kScanThreads / 32];
  const uint64_t base = (uint64_t)blockIdx.x * kScanTile +
                        (uint64_t)threadIdx.x * kScanItems;
  uint32_t v[kScanItems], orig[kScanItems];
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    uint64_t i = base + k;
    v[k] = i < n ? in[i] : 0u;
    orig[k] = v[k];
  }
  block_scan_tile(v, s_warp, tile_totals ? &tile_totals[blockIdx.x] : nullptr);
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    uint64_t i = base + k;
    if (i < n) out[i] = exclusive ? v[k] - orig[k] : v[k];
  }
}

__global__ void k_scan_add(uint32_t* __restrict__ out, uint64_t n,
                           const uint32_t* __restrict__ tile_prefix) {
  const uint32_t add = blockIdx.x ? tile_prefix[blockIdx.x - 1] : 0u;
  if (!add) return;
  const uint64_t base = (uint64_t)blockIdx.x * kScanTile;
  for (int k = threadIdx.x; k < kScanTile; k += blockDim.x) {
    uint64_t i = base + k;
    if (i < n) out[i] += add;
  }
}

// Scratch words the scan of n elements needs (all recursion levels).
inline uint64_t scan_scratch_words(uint64_t n) {
  uint64_t words = 0;
  while (n > (uint64_t)kScanTile) {
    n = (n + kScanTile - 1) / kScanTile;
    words += n;
  }
  return words + 1;
}

// out may alias in.  scratch: scan_scratch_words(n) uint32.
inline void device_scan(const uint32_t* in, uint32_t* out, uint64_t n,
                        bool exclusive, uint32_t* scratch, cudaStream_t s) {
  if (n == 0) return;
  const uint64_t tiles = (n + kScanTile - 1) / kScanTile;
  if (tiles == 1) {
    k_scan_tiles<<<1, kScanThreads, 0, s>>>(in, out, n, nullptr, exclusive);
    return;
  }
  uint32_t* totals = scratch;
  // inclusive scan within tiles (exclusive fix-up below needs the inclusive
  // tile totals either way)
  k_scan_tiles<<<(unsigned)tiles, kScanThreads, 0, s>>>(in, out, n, totals,
                                                        exclusive);
  device_scan(totals, totals, tiles, false, scratch + tiles, s);
  k_scan_add<<<(unsigned)tiles, kScanThreads, 0, s>>>(out, n, totals);
}

}  // namespace
}  // namespace ajg
