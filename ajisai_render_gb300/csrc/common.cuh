// Shared device helpers: float3 arithmetic in the reference's operation
// order, the counter sampler, launch geometry and error plumbing.
//
// Every .cu file of the library is compiled with -fmad=false so that no
// multiply-add is contracted: results of the non-transcendental arithmetic
// (Morton codes, PLOC distances, Moller-Trumbore, film sums) are bit-equal to
// the reference compiled for baseline x86-64.  Where a fused multiply-add is
// wanted it is written explicitly with __fmaf_rn.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/ajisai_gpu.h"

namespace ajg {

constexpr int kSMs = 152;  // GB300: 2 dies x 76 SMs

// ---------------------------------------------------------------- float3 --
struct F3 {
  float x, y, z;
};
__host__ __device__ __forceinline__ F3 mk3(float x, float y, float z) {
  return F3{x, y, z};
}
__host__ __device__ __forceinline__ F3 operator+(F3 a, F3 b) {
  return mk3(a.x + b.x, a.y + b.y, a.z + b.z);
}
__host__ __device__ __forceinline__ F3 operator-(F3 a, F3 b) {
  return mk3(a.x - b.x, a.y - b.y, a.z - b.z);
}
__host__ __device__ __forceinline__ F3 operator*(F3 a, F3 b) {
  return mk3(a.x * b.x, a.y * b.y, a.z * b.z);
}
__host__ __device__ __forceinline__ F3 operator*(F3 a, float s) {
  return mk3(a.x * s, a.y * s, a.z * s);
}
__host__ __device__ __forceinline__ F3 operator*(float s, F3 a) {
  return mk3(a.x * s, a.y * s, a.z * s);
}
__host__ __device__ __forceinline__ F3 operator/(F3 a, F3 b) {
  return mk3(a.x / b.x, a.y / b.y, a.z / b.z);
}
__host__ __device__ __forceinline__ F3 operator/(F3 a, float s) {
  return mk3(a.x / s, a.y / s, a.z / s);
}
__host__ __device__ __forceinline__ F3 operator-(F3 a) {
  return mk3(-a.x, -a.y, -a.z);
}
// math/vector.h:63-69: accumulated from 0 in index order
__host__ __device__ __forceinline__ float dot3(F3 a, F3 b) {
  float o = 0.f;
  o += a.x * b.x;
  o += a.y * b.y;
  o += a.z * b.z;
  return o;
}
// the same without the leading 0 (sign of zero is irrelevant at call site)
__host__ __device__ __forceinline__ float dot3f(F3 a, F3 b) {
  return (a.x * b.x + a.y * b.y) + a.z * b.z;
}
// math/vector3.h:90-95
__host__ __device__ __forceinline__ F3 cross3(F3 a, F3 b) {
  return mk3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x,
             a.x * b.y - b.x * a.y);
}
__device__ __forceinline__ float len3(F3 v) { return sqrtf(dot3(v, v)); }
// math/vector.h:201-216: v * (1 / length)
__device__ __forceinline__ F3 normalize3(F3 v) { return v * (1.f / len3(v)); }
// math/vector.h:36-45
__host__ __device__ __forceinline__ float ref_min(float a, float b) {
  return b < a ? b : a;
}
__host__ __device__ __forceinline__ float ref_max(float a, float b) {
  return a < b ? b : a;
}
__host__ __device__ __forceinline__ F3 vmin3(F3 a, F3 b) {
  return mk3(ref_min(a.x, b.x), ref_min(a.y, b.y), ref_min(a.z, b.z));
}
__host__ __device__ __forceinline__ F3 vmax3(F3 a, F3 b) {
  return mk3(ref_max(a.x, b.x), ref_max(a.y, b.y), ref_max(a.z, b.z));
}
__host__ __device__ __forceinline__ float maxc3(F3 v) {
  return ref_max(ref_max(v.x, v.y), v.z);
}
__host__ __device__ __forceinline__ bool black3(F3 v) {
  return maxc3(v) <= 0.f;
}
__device__ __forceinline__ F3 ld3(const float* p) {
  return mk3(p[0], p[1], p[2]);
}
__device__ __forceinline__ F3 xyz(float4 v) { return mk3(v.x, v.y, v.z); }

// math/constants.h:35-37
constexpr float kPi = 3.141592654f;
constexpr float kPi2 = 1.570796327f;
constexpr float kPi4 = 0.785398163f;
constexpr float kInvPi = 1.f / kPi;
constexpr float kRayEps = 1e-4f;  // Ray::Eps (ray.h:43)

// ---------------------------------------------------------------- sampler --
// Counter sampler: one float per (seed, pixel, sample, dimension), the
// SplitMix64 finaliser (Steele, Lea, Flood 2014) keyed by the path and
// offset by the dimension, mapped to [0,1) as PCG32::NextFloat does
// (core/random.h:46-53).
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__host__ __device__ __forceinline__ uint64_t path_key(uint64_t seed,
                                                      uint32_t pixel,
                                                      uint32_t sample) {
  return mix64(seed * 0x9E3779B97F4A7C15ull +
               (((uint64_t)pixel << 32) | (uint64_t)sample));
}
__device__ __forceinline__ float key_float(uint64_t key, uint32_t dim) {
  uint32_t u = (uint32_t)(mix64(key + (uint64_t)(dim + 1) *
                                          0x9E3779B97F4A7C15ull) >> 32);
  return __uint_as_float((u >> 9) | 0x3f800000u) - 1.0f;
}

// ------------------------------------------------------------ error flag --
// Kernels never trap: a guard that trips records a code in this word and
// the ray or path in question stops; the host turns it into AJG_ERR_DEVICE.
enum DeviceError : uint32_t {
  kDevOk = 0,
  kDevStackOverflow = 1,
  kDevQueueOverflow = 2,
  kDevIterationBound = 3,
  kDevSortOutOfBounds = 4,
  kDevTableOutOfBounds = 5  // a multi-job wave's job, scene or chunk index
};
__device__ __forceinline__ void raise_device_error(uint32_t* flag,
                                                   uint32_t code) {
  atomicCAS(flag, 0u, code);
}

// Warp-aggregated append to a queue: one atomic per warp.
__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, bool pred) {
  const unsigned mask = __activemask();
  const unsigned ballot = __ballot_sync(mask, pred);
  if (!ballot) return 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(ballot) - 1;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(ballot));
  base = __shfl_sync(mask, base, leader);
  return pred ? base + __popc(ballot & ((1u << lane) - 1)) : 0xffffffffu;
}

// 0: queue appends a warp at a time (warp_append) in every kernel.
#ifndef AJG_BLOCK_APPEND
#define AJG_BLOCK_APPEND 1
#endif

// Stream compaction of a whole block into NC queues at once: each thread
// passes the queue of its item (-1: none) and gets the item's slot in it.
// One atomicAdd per queue and block replaces one per warp -- the queue
// counters are single addresses shared by the whole grid, and same-address
// atomics otherwise bound the short kernels that fill the queues.  Every
// thread of the block must call it (block-uniform control flow); NW is the
// number of warps of the block.
template <int NC, int NW>
__device__ __forceinline__ uint32_t block_append(uint32_t* counters,
                                                 int cls) {
  __shared__ uint32_t s_cnt[NC][NW];
  __shared__ uint32_t s_base[NC][NW];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  uint32_t rank = 0;
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    const unsigned b = __ballot_sync(0xffffffffu, cls == c);
    if (lane == 0) s_cnt[c][warp] = (uint32_t)__popc(b);
    if (cls == c) rank = (uint32_t)__popc(b & lt);
  }
  __syncthreads();
  if (threadIdx.x < NC) {
    const int c = threadIdx.x;
    uint32_t tot = 0;
#pragma unroll
    for (int v = 0; v < NW; ++v) {
      const uint32_t x = s_cnt[c][v];
      s_base[c][v] = tot;
      tot += x;
    }
    const uint32_t g = tot ? atomicAdd(&counters[c], tot) : 0u;
#pragma unroll
    for (int v = 0; v < NW; ++v) s_base[c][v] += g;
  }
  __syncthreads();
  return cls >= 0 ? s_base[cls][warp] + rank : 0xffffffffu;
}

// Maximum of v over the block (every thread must call it).
template <int NW>
__device__ __forceinline__ uint32_t block_max(uint32_t v) {
  __shared__ uint32_t s_m[NW];
  v = __reduce_max_sync(0xffffffffu, v);
  if ((threadIdx.x & 31) == 0) s_m[threadIdx.x >> 5] = v;
  __syncthreads();
  uint32_t m = 0;
#pragma unroll
  for (int w = 0; w < NW; ++w) m = m > s_m[w] ? m : s_m[w];
  __syncthreads();
  return m;
}

inline int grid_for(uint64_t n, int block, int max_blocks = kSMs * 32) {
  uint64_t g = (n + block - 1) / block;
  if (g < 1) g = 1;
  if (g > (uint64_t)max_blocks) g = max_blocks;
  return (int)g;
}

}  // namespace ajg
