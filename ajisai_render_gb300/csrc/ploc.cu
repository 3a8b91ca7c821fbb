// GPU PLOC build (Meister and Bittner, "Parallel Locally-Ordered
// Clustering for Bounding Volume Hierarchy Construction", TVCG 2018), in the
// exact form of the reference's PLOCAggregate::Build
// (core/aggregate/ploc_aggregate.cpp:252-327):
//   1. 30-bit Morton codes of the triangle-box centres in the scene box
//      (ploc_aggregate.cpp:37-82, 513-541);
//   2. a stable LSD radix sort over three 10-bit digits
//      (ploc_aggregate.cpp:84-132) -- optionally reproducing the reference's
//      stale digit-0 offset, so that the tree is the reference's own;
//   3. leaves in sorted order, then Cluster iterations until one node is left
//      (ploc_aggregate.cpp:400-511): nearest neighbour by joined-box area
//      within +-r (first minimum in index order), mutual pairs merge, an
//      inclusive scan places parents and children.
// The result is bit-identical to the reference's node array; it is then
// re-laid out for traversal (two child boxes per interior node, leaf slots
// holding the triangles in Morton order).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>

#include "scan.cuh"
#include "scene.cuh"

namespace ajg {
namespace {

constexpr int kBuckets = 1024;
constexpr int kRadixThreads = 256;
constexpr int kRadixWarps = kRadixThreads / 32;
constexpr int kKeysPerWarp = 512;
constexpr int kRadixTile = kRadixWarps * kKeysPerWarp;  // 4096
constexpr int kClusterThreads = 256;

struct PNode {  // reference Node: bound, primitive_count, first_child
  float4 a;     // lo.xyz, first (int bits)
  float4 b;     // hi.xyz, count (int bits)
};

__device__ __forceinline__ bool is_point(const F3& lo, const F3& hi) {
  return lo.x == hi.x && lo.y == hi.y && lo.z == hi.z;
}
// math/bounds.h:108-113
__device__ __forceinline__ void join(F3 alo, F3 ahi, F3 blo, F3 bhi, F3& lo,
                                     F3& hi) {
  if (is_point(alo, ahi)) {
    lo = blo;
    hi = bhi;
  } else if (is_point(blo, bhi)) {
    lo = alo;
    hi = ahi;
  } else {
    lo = vmin3(alo, blo);
    hi = vmax3(ahi, bhi);
  }
}
// math/bounds.h:98-101
__device__ __forceinline__ float area(F3 lo, F3 hi) {
  F3 d = hi - lo;
  return 2.f * (d.x * d.y + d.x * d.z + d.y * d.z);
}
// ploc_aggregate.cpp:168-182
__device__ __forceinline__ void tri_box(const float* t, F3& lo, F3& hi) {
  lo = mk3(FLT_MAX, FLT_MAX, FLT_MAX);
  hi = mk3(-FLT_MAX, -FLT_MAX, -FLT_MAX);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    F3 v = mk3(t[3 * k], t[3 * k + 1], t[3 * k + 2]);
    lo = vmin3(lo, v);
    hi = vmax3(hi, v);
  }
}

__device__ __forceinline__ uint32_t morton_split(uint32_t x) {
  x &= 0x3ffu;
  x = (x | (x << 16)) & 0x030000FFu;
  x = (x | (x << 8)) & 0x0300F00Fu;
  x = (x | (x << 4)) & 0x030C30C3u;
  x = (x | (x << 2)) & 0x09249249u;
  return x;
}
__device__ __forceinline__ uint32_t grid_coord(float f) {
  float g = ref_max(f, 0.f);
  if (g != g) return 0u;  // flat axis: NaN converts to 0
  uint32_t m = __float2uint_rz(g);
  return m < 1023u ? m : 1023u;
}

__global__ void k_morton(const float* __restrict__ tris, uint64_t n, F3 w2g,
                         F3 off, uint32_t* __restrict__ codes,
                         int32_t* __restrict__ vals) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    F3 lo, hi;
    tri_box(tris + 9 * i, lo, hi);
    F3 c = (hi + lo) / 2.f;
    F3 g = c * w2g + off;
    codes[i] = morton_split(grid_coord(g.x)) |
               (morton_split(grid_coord(g.y)) << 1) |
               (morton_split(grid_coord(g.z)) << 2);
    vals[i] = (int32_t)i;
  }
}

__global__ void k_radix_hist(const uint32_t* __restrict__ keys, uint64_t n,
                             int bit, uint32_t* __restrict__ hist,
                             uint32_t nb) {
  __shared__ uint32_t h[kBuckets];
  for (int d = threadIdx.x; d < kBuckets; d += blockDim.x) h[d] = 0;
  __syncthreads();
  const uint64_t t0 = (uint64_t)blockIdx.x * kRadixTile;
  for (int k = threadIdx.x; k < kRadixTile; k += blockDim.x) {
    uint64_t i = t0 + k;
    if (i < n) atomicAdd(&h[(keys[i] >> bit) & (kBuckets - 1)], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < kBuckets; d += blockDim.x)
    hist[(uint64_t)d * nb + blockIdx.x] = h[d];
}

// Stable scatter: warp w owns keys [t0 + w*512, t0 + (w+1)*512) and walks
// them in order, 32 at a time; lanes with equal digits rank by lane.
__global__ void __launch_bounds__(kRadixThreads)
    k_radix_scatter(const uint32_t* __restrict__ keys_in,
                    const int32_t* __restrict__ vals_in,
                    uint32_t* __restrict__ keys_out,
                    int32_t* __restrict__ vals_out, uint64_t n, int bit,
                    const uint32_t* __restrict__ offsets, uint32_t nb,
                    int compat, const uint32_t* __restrict__ compat_base,
                    int32_t* __restrict__ owner, uint32_t* __restrict__ pos_of,
                    uint32_t* __restrict__ err) {
  __shared__ uint32_t wh[kRadixWarps][kBuckets];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int k = threadIdx.x; k < kRadixWarps * kBuckets; k += blockDim.x)
    (&wh[0][0])[k] = 0;
  __syncthreads();
  const uint64_t wbase = (uint64_t)blockIdx.x * kRadixTile +
                         (uint64_t)w * kKeysPerWarp;
  for (int s = 0; s < kKeysPerWarp; s += 32) {
    uint64_t i = wbase + s + lane;
    if (i < n) atomicAdd(&wh[w][(keys_in[i] >> bit) & (kBuckets - 1)], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < kBuckets; d += blockDim.x) {
    uint32_t run = offsets[(uint64_t)d * nb + blockIdx.x];
#pragma unroll
    for (int q = 0; q < kRadixWarps; ++q) {
      uint32_t c = wh[q][d];
      wh[q][d] = run;
      run += c;
    }
  }
  __syncthreads();
  const uint32_t base0 = compat ? *compat_base : 0u;
  const unsigned lt = (1u << lane) - 1u;
  for (int s = 0; s < kKeysPerWarp; s += 32) {
    uint64_t i = wbase + s + lane;
    const bool valid = i < n;
    uint32_t key = valid ? keys_in[i] : 0u;
    uint32_t d = valid ? ((key >> bit) & (kBuckets - 1)) : 0xffffffffu;
    unsigned peers = __match_any_sync(0xffffffffu, d);
    uint32_t pos = 0;
    if (valid) pos = wh[w][d] + __popc(peers & lt);
    __syncwarp();
    if (valid && lane == __ffs(peers) - 1) wh[w][d] += __popc(peers);
    __syncwarp();
    if (!valid) continue;
    if (!compat) {
      keys_out[pos] = key;
      vals_out[pos] = vals_in[i];
    } else {
      uint64_t p = pos;
      if (d == 0) p += base0;
      if (p >= n) {
        raise_device_error(err, kDevSortOutOfBounds);
        pos_of[i] = 0xffffffffu;
      } else {
        atomicMax(&owner[p], (int32_t)i);
        pos_of[i] = (uint32_t)p;
      }
    }
  }
}

// Reference-compatible pass: the later key (in input order) wins a slot,
// unwritten slots keep the stale contents of the destination.
__global__ void k_radix_compat_write(const uint32_t* __restrict__ keys_in,
                                     const int32_t* __restrict__ vals_in,
                                     uint32_t* __restrict__ keys_out,
                                     int32_t* __restrict__ vals_out,
                                     uint64_t n,
                                     const int32_t* __restrict__ owner,
                                     const uint32_t* __restrict__ pos_of) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t p = pos_of[i];
    if (p != 0xffffffffu && owner[p] == (int32_t)i) {
      keys_out[p] = keys_in[i];
      vals_out[p] = vals_in[i];
    }
  }
}

// After pass p's offset scan: base = sum of digit-0 counts of passes < p.
__global__ void k_compat_base(const uint32_t* __restrict__ offsets,
                              uint32_t nb, uint32_t* acc) {
  const uint32_t count0 = offsets[(uint64_t)1 * nb + 0];
  acc[0] = acc[1];
  acc[1] += count0;
}

__global__ void k_leaf_init(const float* __restrict__ tris,
                            const int32_t* __restrict__ perm,
                            PNode* __restrict__ nodes, uint64_t begin,
                            uint64_t n) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    F3 lo, hi;
    tri_box(tris + 9 * (uint64_t)perm[i], lo, hi);
    nodes[begin + i].a = make_float4(lo.x, lo.y, lo.z, __int_as_float((int)i));
    nodes[begin + i].b = make_float4(hi.x, hi.y, hi.z, __int_as_float(1));
  }
}

// Nearest neighbour within [i-r, i+r] (ploc_aggregate.cpp:408-459): scan in
// ascending index order with a strict comparison.
__global__ void __launch_bounds__(kClusterThreads)
    k_neighbors(const PNode* __restrict__ in, uint32_t begin, uint32_t end,
                int r, uint32_t* __restrict__ nb) {
  extern __shared__ float sb[];
  const uint32_t i0 = begin + blockIdx.x * kClusterThreads;
  const uint32_t lo_idx = i0 > begin + (uint32_t)r ? i0 - r : begin;
  const uint64_t hi_lim = (uint64_t)i0 + kClusterThreads + r;
  const uint32_t hi_idx = hi_lim < end ? (uint32_t)hi_lim : end;
  const uint32_t cnt = hi_idx - lo_idx;
  for (uint32_t k = threadIdx.x; k < cnt; k += blockDim.x) {
    float4 a = in[lo_idx + k].a, b = in[lo_idx + k].b;
    sb[6 * k + 0] = a.x;
    sb[6 * k + 1] = a.y;
    sb[6 * k + 2] = a.z;
    sb[6 * k + 3] = b.x;
    sb[6 * k + 4] = b.y;
    sb[6 * k + 5] = b.z;
  }
  __syncthreads();
  const uint32_t i = i0 + threadIdx.x;
  if (i >= end) return;
  const uint32_t s0 = i > begin + (uint32_t)r ? i - r : begin;
  const uint64_t e_lim = (uint64_t)i + r + 1;
  const uint32_t s1 = e_lim < end ? (uint32_t)e_lim : end;
  const float* mi = sb + 6 * (i - lo_idx);
  const F3 ilo = mk3(mi[0], mi[1], mi[2]), ihi = mk3(mi[3], mi[4], mi[5]);
  float best = FLT_MAX;
  uint32_t bj = 0xffffffffu;
  for (uint32_t j = s0; j < s1; ++j) {
    if (j == i) continue;
    const float* mj = sb + 6 * (j - lo_idx);
    F3 lo, hi;
    join(ilo, ihi, mk3(mj[0], mj[1], mj[2]), mk3(mj[3], mj[4], mj[5]), lo, hi);
    float d = area(lo, hi);
    if (d < best) {
      best = d;
      bj = j;
    }
  }
  nb[i] = bj;
}

__global__ void k_merge_flags(const uint32_t* __restrict__ nb, uint32_t begin,
                              uint32_t end, uint32_t* __restrict__ flags) {
  for (uint32_t i = begin + blockIdx.x * blockDim.x + threadIdx.x; i < end;
       i += gridDim.x * blockDim.x) {
    uint32_t j = nb[i];
    flags[i - begin] = (j != 0xffffffffu && i < j && nb[j] == i) ? 1u : 0u;
  }
}

// ploc_aggregate.cpp:481-501
__global__ void k_cluster_scatter(const PNode* __restrict__ in,
                                  PNode* __restrict__ out,
                                  const uint32_t* __restrict__ nb,
                                  const uint32_t* __restrict__ mi,
                                  uint32_t begin, uint32_t end,
                                  uint32_t unmerged_begin,
                                  uint32_t children_begin) {
  for (uint32_t i = begin + blockIdx.x * blockDim.x + threadIdx.x; i < end;
       i += gridDim.x * blockDim.x) {
    const uint32_t j = nb[i];
    if (j != 0xffffffffu && nb[j] == i) {
      if (i < j) {
        const uint32_t fc = children_begin + (mi[i - begin] - 1) * 2;
        const PNode ni = in[i], nj = in[j];
        F3 lo, hi;
        join(xyz(nj.a), xyz(nj.b), xyz(ni.a), xyz(ni.b), lo, hi);
        PNode p;
        p.a = make_float4(lo.x, lo.y, lo.z, __int_as_float((int)fc));
        p.b = make_float4(hi.x, hi.y, hi.z, __int_as_float(0));
        out[unmerged_begin + j - begin - mi[j - begin]] = p;
        out[fc + 0] = ni;
        out[fc + 1] = nj;
      }
    } else {
      out[unmerged_begin + i - begin - mi[i - begin]] = in[i];
    }
  }
}

__global__ void k_inner_flags(const PNode* __restrict__ nodes, uint64_t m,
                              uint32_t* __restrict__ flags) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
       i += (uint64_t)gridDim.x * blockDim.x)
    flags[i] = __float_as_int(nodes[i].b.w) == 0 ? 1u : 0u;
}

__device__ __forceinline__ int child_ref(const PNode* nodes,
                                         const uint32_t* compact, uint32_t c) {
  const PNode x = nodes[c];
  if (__float_as_int(x.b.w) != 0) return ~__float_as_int(x.a.w);
  return (int)compact[c];
}

__global__ void k_bvh2(const PNode* __restrict__ nodes, uint64_t m,
                       const uint32_t* __restrict__ compact,
                       float4* __restrict__ bvh) {
  for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < m;
       k += (uint64_t)gridDim.x * blockDim.x) {
    const PNode x = nodes[k];
    if (__float_as_int(x.b.w) != 0) continue;
    const uint32_t c0 = (uint32_t)__float_as_int(x.a.w);
    const PNode a = nodes[c0], b = nodes[c0 + 1];
    float4* o = bvh + 4 * (uint64_t)compact[k];
    o[0] = make_float4(a.a.x, a.b.x, a.a.y, a.b.y);
    o[1] = make_float4(b.a.x, b.b.x, b.a.y, b.b.y);
    o[2] = make_float4(a.a.z, a.b.z, b.a.z, b.b.z);
    o[3] = make_float4(__int_as_float(child_ref(nodes, compact, c0)),
                       __int_as_float(child_ref(nodes, compact, c0 + 1)), 0.f,
                       0.f);
  }
}

// A single triangle: one node whose two children are the same leaf.
__global__ void k_bvh2_single(const PNode* __restrict__ nodes,
                              float4* __restrict__ bvh) {
  const PNode a = nodes[0];
  bvh[0] = make_float4(a.a.x, a.b.x, a.a.y, a.b.y);
  bvh[1] = bvh[0];
  bvh[2] = make_float4(a.a.z, a.b.z, a.a.z, a.b.z);
  bvh[3] = make_float4(__int_as_float(~0), __int_as_float(~0), 0.f, 0.f);
}

// Collapse of the binary tree into W-wide nodes, top down, one level of
// wide nodes per launch: a wide node takes its binary node and expands the
// interior child with the largest surface area until it has W children (or
// only leaves); its interior children become the wide nodes of the next
// level, allocated contiguously.  Node layout (2W float4, 32W bytes): the
// children's lo.x, hi.x, lo.y, hi.y, lo.z, hi.z in groups of four, then the
// references (>= 0 wide node, ~slot leaf, kEmptyRef unused), then padding.
constexpr int kWideEmpty = (int)0x80000000;

template <int W>
__global__ void k_collapse(const PNode* __restrict__ nodes,
                           const uint2* __restrict__ fin, uint32_t n_in,
                           uint2* __restrict__ fout,
                           uint32_t* __restrict__ counters,
                           float4* __restrict__ wide) {
  constexpr int G = W / 4;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_in;
       i += gridDim.x * blockDim.x) {
    const uint2 e = fin[i];  // (binary node, wide slot)
    uint32_t ch[W];
    int nc = 1;
    ch[0] = e.x;
    while (nc < W) {
      int best = -1;
      float ba = 0.f;
      for (int c = 0; c < nc; ++c) {
        const PNode x = nodes[ch[c]];
        if (__float_as_int(x.b.w) != 0) continue;  // leaf
        const float a = area(xyz(x.a), xyz(x.b));
        if (best < 0 || a > ba) {
          best = c;
          ba = a;
        }
      }
      if (best < 0) break;
      const uint32_t f = (uint32_t)__float_as_int(nodes[ch[best]].a.w);
      ch[best] = f;
      ch[nc++] = f + 1;
    }
    int ni = 0;
    for (int c = 0; c < nc; ++c)
      ni += __float_as_int(nodes[ch[c]].b.w) == 0 ? 1 : 0;
    uint32_t base = 0, fo = 0;
    if (ni) {
      base = atomicAdd(&counters[1], (uint32_t)ni);
      fo = atomicAdd(&counters[0], (uint32_t)ni);
    }
    float pl[6][W];
    int rf[W];
    int j = 0;
    for (int c = 0; c < W; ++c) {
      if (c < nc) {
        const PNode x = nodes[ch[c]];
        pl[0][c] = x.a.x;
        pl[1][c] = x.b.x;
        pl[2][c] = x.a.y;
        pl[3][c] = x.b.y;
        pl[4][c] = x.a.z;
        pl[5][c] = x.b.z;
        if (__float_as_int(x.b.w) != 0) {
          rf[c] = ~__float_as_int(x.a.w);
        } else {
          rf[c] = (int)(base + j);
          fout[fo + j] = make_uint2(ch[c], base + j);
          ++j;
        }
      } else {
        for (int k = 0; k < 6; ++k) pl[k][c] = 0.f;
        rf[c] = kWideEmpty;
      }
    }
    float4* o = wide + (uint64_t)e.y * (2 * W);
    for (int g = 0; g < G; ++g) {
      for (int k = 0; k < 6; ++k)
        o[k * G + g] = make_float4(pl[k][4 * g], pl[k][4 * g + 1],
                                   pl[k][4 * g + 2], pl[k][4 * g + 3]);
      o[6 * G + g] = make_float4(
          __int_as_float(rf[4 * g]), __int_as_float(rf[4 * g + 1]),
          __int_as_float(rf[4 * g + 2]), __int_as_float(rf[4 * g + 3]));
      o[7 * G + g] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
}

// SAH-optimal collapse into 4-wide nodes (the dynamic program of Ylitie,
// Karras, Laine, "Efficient incoherent ray traversal on GPUs through
// compressed wide BVHs", HPG 2017, with one triangle per leaf): cost[n].i
// (i = 1..4 slots) is the least sum of wide-node surface areas with which
// the subtree of binary node n fills at most i children of a wide node --
// one slot holding n itself (a leaf, or a wide node of its own: its area
// plus its children's best use of 4 slots), or its two children sharing
// the slots.  Leaves cost 0 in every slot count (a leaf's triangle test is
// the same whatever the tree).  choice[n] packs the decisions: byte 0 the
// left child's share of a wide node's 4 slots, byte i-1 (i = 2..4) for i
// slots 0 (n itself) or (left share << 4 | slots used).  One launch per
// block of nodes the PLOC loop finalised, in the order they were
// finalised: children always come before their parents.
#ifndef AJG_SAH_COLLAPSE
#define AJG_SAH_COLLAPSE 1
#endif
__global__ void k_sah_dp(const PNode* __restrict__ nodes, uint32_t lo,
                         uint32_t hi, float4* __restrict__ cost,
                         uint32_t* __restrict__ choice) {
  for (uint32_t n = lo + blockIdx.x * blockDim.x + threadIdx.x; n < hi;
       n += gridDim.x * blockDim.x) {
    const PNode x = nodes[n];
    if (__float_as_int(x.b.w) != 0) {  // leaf
      cost[n] = make_float4(0.f, 0.f, 0.f, 0.f);
      choice[n] = 0u;
      continue;
    }
    const uint32_t f = (uint32_t)__float_as_int(x.a.w);
    const float4 L = cost[f], R = cost[f + 1];
    const float l[5] = {0.f, L.x, L.y, L.z, L.w};
    const float r[5] = {0.f, R.x, R.y, R.z, R.w};
    float dist[5];
    uint32_t dk[5];
#pragma unroll
    for (int j = 2; j <= 4; ++j) {
      dist[j] = __int_as_float(0x7f800000);
      dk[j] = 1;
#pragma unroll
      for (int k = 1; k < j; ++k) {
        const float v = l[k] + r[j - k];
        if (v < dist[j]) {
          dist[j] = v;
          dk[j] = (uint32_t)k;
        }
      }
    }
    float c[5];
    uint32_t kind[5] = {0u, 0u, 0u, 0u, 0u};
    c[1] = area(xyz(x.a), xyz(x.b)) + dist[4];
#pragma unroll
    for (int i = 2; i <= 4; ++i) {
      if (dist[i] < c[i - 1]) {
        c[i] = dist[i];
        kind[i] = (dk[i] << 4) | (uint32_t)i;
      } else {
        c[i] = c[i - 1];
        kind[i] = kind[i - 1];
      }
    }
    cost[n] = make_float4(c[1], c[2], c[3], c[4]);
    choice[n] = dk[4] | (kind[2] << 8) | (kind[3] << 16) | (kind[4] << 24);
  }
}

// k_collapse with the children of each wide node taken from the dynamic
// program above instead of by expanding the largest-area child.
__global__ void k_collapse_sah(const PNode* __restrict__ nodes,
                               const uint32_t* __restrict__ choice,
                               const uint2* __restrict__ fin, uint32_t n_in,
                               uint2* __restrict__ fout,
                               uint32_t* __restrict__ counters,
                               float4* __restrict__ wide) {
  constexpr int W = 4;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_in;
       i += gridDim.x * blockDim.x) {
    const uint2 e = fin[i];  // (binary node, wide slot)
    uint32_t ch[W];
    int nc = 0;
    const PNode root = nodes[e.x];
    if (__float_as_int(root.b.w) != 0) {
      ch[nc++] = e.x;  // a one-triangle tree
    } else {
      // (node, slots) still to resolve; each entry holds >= 1 of the 4 slots
      uint32_t sn[W], sj[W];
      int sp = 0;
      const uint32_t f = (uint32_t)__float_as_int(root.a.w);
      const uint32_t k = choice[e.x] & 0xffu;
      sn[sp] = f + 1;
      sj[sp++] = W - k;
      sn[sp] = f;
      sj[sp++] = k;
      while (sp > 0) {
        --sp;
        const uint32_t c = sn[sp], j = sj[sp];
        const uint32_t kd = j < 2 ? 0u : (choice[c] >> (8 * (j - 1))) & 0xffu;
        if (kd == 0u || nc + sp + 2 > W) {  // (the second never holds)
          ch[nc++] = c;
        } else {
          const uint32_t fc = (uint32_t)__float_as_int(nodes[c].a.w);
          const uint32_t k2 = kd >> 4, used = kd & 15u;
          sn[sp] = fc + 1;
          sj[sp++] = used - k2;
          sn[sp] = fc;
          sj[sp++] = k2;
        }
      }
    }
    int ni = 0;
    for (int c = 0; c < nc; ++c)
      ni += __float_as_int(nodes[ch[c]].b.w) == 0 ? 1 : 0;
    uint32_t base = 0, fo = 0;
    if (ni) {
      base = atomicAdd(&counters[1], (uint32_t)ni);
      fo = atomicAdd(&counters[0], (uint32_t)ni);
    }
    float pl[6][W];
    int rf[W];
    int jn = 0;
    for (int c = 0; c < W; ++c) {
      if (c < nc) {
        const PNode x = nodes[ch[c]];
        pl[0][c] = x.a.x;
        pl[1][c] = x.b.x;
        pl[2][c] = x.a.y;
        pl[3][c] = x.b.y;
        pl[4][c] = x.a.z;
        pl[5][c] = x.b.z;
        if (__float_as_int(x.b.w) != 0) {
          rf[c] = ~__float_as_int(x.a.w);
        } else {
          rf[c] = (int)(base + jn);
          fout[fo + jn] = make_uint2(ch[c], base + jn);
          ++jn;
        }
      } else {
        for (int k = 0; k < 6; ++k) pl[k][c] = 0.f;
        rf[c] = kWideEmpty;
      }
    }
    float4* o = wide + (uint64_t)e.y * (2 * W);
    for (int k = 0; k < 6; ++k)
      o[k] = make_float4(pl[k][0], pl[k][1], pl[k][2], pl[k][3]);
    o[6] = make_float4(__int_as_float(rf[0]), __int_as_float(rf[1]),
                       __int_as_float(rf[2]), __int_as_float(rf[3]));
    o[7] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

// The same collapse into compressed nodes (layout in scene.cuh), moving the
// leaf triangles of every node next to each other in `tris_new`.
template <int W>
__global__ void k_collapse_c(const PNode* __restrict__ nodes,
                             const float4* __restrict__ tris_old,
                             const uint2* __restrict__ fin, uint32_t n_in,
                             uint2* __restrict__ fout,
                             uint32_t* __restrict__ counters,
                             float4* __restrict__ wide,
                             float4* __restrict__ tris_new) {
  constexpr int NF = CwLayout<W>::kFloat4;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_in;
       i += gridDim.x * blockDim.x) {
    const uint2 e = fin[i];
    uint32_t ch[W];
    int nc = 1;
    ch[0] = e.x;
    while (nc < W) {
      int best = -1;
      float ba = 0.f;
      for (int c = 0; c < nc; ++c) {
        const PNode x = nodes[ch[c]];
        if (__float_as_int(x.b.w) != 0) continue;
        const float a = area(xyz(x.a), xyz(x.b));
        if (best < 0 || a > ba) {
          best = c;
          ba = a;
        }
      }
      if (best < 0) break;
      const uint32_t f = (uint32_t)__float_as_int(nodes[ch[best]].a.w);
      ch[best] = f;
      ch[nc++] = f + 1;
    }
    // quantisation grid: origin = lo of the union, 255 steps of 2^e cover
    // the union's extent per axis
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
    float hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int c = 0; c < nc; ++c) {
      const PNode x = nodes[ch[c]];
      lo[0] = fminf(lo[0], x.a.x);
      lo[1] = fminf(lo[1], x.a.y);
      lo[2] = fminf(lo[2], x.a.z);
      hi[0] = fmaxf(hi[0], x.b.x);
      hi[1] = fmaxf(hi[1], x.b.y);
      hi[2] = fmaxf(hi[2], x.b.z);
    }
    uint32_t eb[3];
    float sc[3];
    double step[3];
    for (int a = 0; a < 3; ++a) {
      const double ext = (double)hi[a] - (double)lo[a];
      int ex = -126;
      if (ext > 0.0) {
        int k = 0;
        frexp(ext / 255.0, &k);  // ext / 255 < 2^k
        ex = k;
      }
      ex = ex < -126 ? -126 : (ex > 127 ? 127 : ex);
      eb[a] = (uint32_t)(ex + 127);
      sc[a] = cw_scale(eb[a]);
      step[a] = ldexp(1.0, ex);
    }
    uint32_t vmask = 0, imask = 0;
    uint8_t q[6][W];
    for (int c = 0; c < W; ++c) {
      if (c >= nc) {
        for (int k = 0; k < 6; ++k) q[k][c] = 0;
        continue;
      }
      const PNode x = nodes[ch[c]];
      vmask |= 1u << c;
      if (__float_as_int(x.b.w) == 0) imask |= 1u << c;
      const float cl[3] = {x.a.x, x.a.y, x.a.z};
      const float chh[3] = {x.b.x, x.b.y, x.b.z};
      for (int a = 0; a < 3; ++a) {
        double fl = floor(((double)cl[a] - (double)lo[a]) / step[a]);
        double fh = ceil(((double)chh[a] - (double)lo[a]) / step[a]);
        uint32_t ql = fl < 0.0 ? 0u : (fl > 255.0 ? 255u : (uint32_t)fl);
        uint32_t qh = fh < 0.0 ? 0u : (fh > 255.0 ? 255u : (uint32_t)fh);
        // the decoded planes must enclose the child's box
        while (ql > 0 &&
               cw_decode(lo[a], cw_qfloat(0x4B000000u | ql), sc[a]) > cl[a])
          --ql;
        while (qh < 255 &&
               cw_decode(lo[a], cw_qfloat(0x4B000000u | qh), sc[a]) < chh[a])
          ++qh;
        q[2 * a][c] = (uint8_t)ql;
        q[2 * a + 1][c] = (uint8_t)qh;
      }
    }
    const int ni = __popc(imask), nl = __popc(vmask & ~imask);
    uint32_t base = 0, fo = 0, tb = 0;
    if (ni) {
      base = atomicAdd(&counters[1], (uint32_t)ni);
      fo = atomicAdd(&counters[0], (uint32_t)ni);
    }
    if (nl) tb = atomicAdd(&counters[2], (uint32_t)nl);
    int ji = 0, jl = 0;
    for (int c = 0; c < nc; ++c) {
      const PNode x = nodes[ch[c]];
      if ((imask >> c) & 1u) {
        fout[fo + ji] = make_uint2(ch[c], base + ji);
        ++ji;
      } else {
        const uint32_t slot = (uint32_t)__float_as_int(x.a.w);
        for (int k = 0; k < 3; ++k)
          tris_new[3 * (uint64_t)(tb + jl) + k] = tris_old[3 * (uint64_t)slot + k];
        ++jl;
      }
    }
    float4* o = wide + (uint64_t)e.y * NF;
    o[0] = make_float4(lo[0], lo[1], lo[2],
                       __uint_as_float(eb[0] | (eb[1] << 8) | (eb[2] << 16) |
                                       (imask << 24)));
    o[1] = make_float4(__uint_as_float(base), __uint_as_float(tb),
                       __uint_as_float(vmask), 0.f);
    uint32_t words[4 * (NF - 2)];
    for (int k = 0; k < 4 * (NF - 2); ++k) words[k] = 0;
    for (int k = 0; k < 6; ++k)
      for (int c = 0; c < W; ++c) {
        const int byte = k * W + c;
        words[byte >> 2] |= (uint32_t)q[k][c] << (8 * (byte & 3));
      }
    for (int f = 0; f < NF - 2; ++f)
      o[2 + f] = make_float4(
          __uint_as_float(words[4 * f]), __uint_as_float(words[4 * f + 1]),
          __uint_as_float(words[4 * f + 2]), __uint_as_float(words[4 * f + 3]));
  }
}

__global__ void k_slot_tris(const float* __restrict__ tris,
                            const int32_t* __restrict__ perm, uint64_t n,
                            float4* __restrict__ out) {
  for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < n;
       s += (uint64_t)gridDim.x * blockDim.x) {
    const int32_t p = perm[s];
    const float* t = tris + 9 * (uint64_t)p;
    out[3 * s + 0] = make_float4(t[0], t[1], t[2], __int_as_float(p));
    out[3 * s + 1] = make_float4(t[3], t[4], t[5], 0.f);
    out[3 * s + 2] = make_float4(t[6], t[7], t[8], 0.f);
  }
}

// Geometric normal of each primitive as its PostIntersect leaves it:
// normalize(cross(b-a, c-a)) (Triangle::Intersect, quad.cpp, mesh.cpp) or
// from the tuple order (c, b, a) for cubes (cube.cpp:96-108).
__global__ void k_shade_data(const float* __restrict__ tris,
                             const int32_t* __restrict__ mat,
                             const int32_t* __restrict__ flags, uint64_t n,
                             float4* __restrict__ out) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const float* t = tris + 9 * i;
    F3 a = ld3(t), b = ld3(t + 3), c = ld3(t + 6);
    const int fl = flags[i];
    F3 ng = (fl & AJG_MESH_NG_REVERSED) ? normalize3(cross3(b - c, a - c))
                                        : normalize3(cross3(b - a, c - a));
    const uint32_t w = ((uint32_t)mat[i] & 0xffffffu) | ((uint32_t)fl << 24);
    out[i] = make_float4(ng.x, ng.y, ng.z, __uint_as_float(w));
  }
}

__global__ void k_lum(const float* __restrict__ mats, uint32_t m,
                      float4* __restrict__ out) {
  for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
    const float* r = mats + 16 * i;
    // spectrum.h:80-82, evaluated in double as the reference does
    float lum = (float)(0.2126 * (double)r[1] + 0.7152 * (double)r[2] +
                        0.0722 * (double)r[3]);
    out[i] = make_float4(lum, 0.f, 0.f, 0.f);
  }
}

struct Arena {
  std::vector<void*> ptrs;
  cudaError_t err = cudaSuccess;
  template <class T>
  T* get(uint64_t count) {
    void* p = nullptr;
    if (err != cudaSuccess) return nullptr;
    err = cudaMalloc(&p, count * sizeof(T) > 0 ? count * sizeof(T) : 16);
    if (err != cudaSuccess) return nullptr;
    ptrs.push_back(p);
    return static_cast<T*>(p);
  }
  ~Arena() {
    for (void* p : ptrs) cudaFree(p);
  }
};

int set_err(ajg_ctx* ctx, int code, const std::string& msg) {
  ctx->last_error = msg;
  return code;
}

// The scene's typical triangle size: the median longest edge over up to
// 4,096 evenly spaced triangles.
float median_edge(const float* t, uint64_t n) {
  const uint64_t k = std::min<uint64_t>(n, 4096);
  std::vector<float> e(k);
  for (uint64_t i = 0; i < k; ++i) {
    const float* p = t + 9 * (i * n / k);
    float m = 0.f;
    for (int a = 0; a < 3; ++a) {
      const float* u = p + 3 * a;
      const float* v = p + 3 * ((a + 1) % 3);
      const float dx = u[0] - v[0], dy = u[1] - v[1], dz = u[2] - v[2];
      m = std::max(m, dx * dx + dy * dy + dz * dz);
    }
    e[i] = std::sqrt(m);
  }
  std::nth_element(e.begin(), e.begin() + k / 2, e.end());
  return e[k / 2];
}

}  // namespace

int build_scene(ajg_ctx* ctx, ajg_scene* s, const float* h_tris,
                const float* h_corner, const int32_t* h_mat,
                const int32_t* h_flags, uint64_t n, const float* world,
                const ajg_scene_opts& opts) {
  cudaStream_t st = ctx->stream;
  if (n == 0 || n > (1ull << 30))
    return set_err(ctx, AJG_ERR_INVALID, "triangle count must be in [1, 2^30]");
  const int r = (int)opts.search_radius;
  if (r < 1 || r > 1024)
    return set_err(ctx, AJG_ERR_INVALID, "search_radius must be in [1, 1024]");
  const uint64_t m = 2 * n - 1;
  bool any_normals = false;
  for (uint64_t i = 0; i < n && h_corner; ++i)
    if (h_flags[i] & AJG_MESH_HAS_NORMALS) {
      any_normals = true;
      break;
    }

  // persistent scene buffers
  auto keep = [&](size_t bytes) -> void* {
    void* p = nullptr;
    if (cudaMalloc(&p, bytes > 0 ? bytes : 16) != cudaSuccess) return nullptr;
    s->allocations.push_back(p);
    s->info.device_bytes += bytes;
    return p;
  };
  const uint64_t inner = n > 1 ? n - 1 : 1;
  // default: the 4-wide tree (the fastest measured on GB300 for the
  // workloads here; 8-wide nodes cost occupancy)
  const int width = opts.bvh_width ? (int)opts.bvh_width : 4;
  const bool compressed = (width & kBvhCompressed) != 0;
  const int wn = width & 0xff;  // children per node
  if (!(width == 2 || wn == 4 || wn == 8) || (width & ~0x1ff))
    return set_err(ctx, AJG_ERR_INVALID,
                   "bvh_width must be 0, 2, 4 or 8 (4 and 8 optionally "
                   "| AJG_BVH_COMPRESSED)");
  // the binary layout: the tree itself (width 2), or beside a plain 4-wide
  // tree for the closest-hit traversal (closest_width)
  const bool hybrid = closest_width(width) != width;
  float4* bvh =
      width == 2 ? (float4*)keep(inner * 4 * sizeof(float4)) : nullptr;
  float4* bvh_bin = hybrid ? (float4*)keep(inner * 4 * sizeof(float4)) : nullptr;
  float4* slot_tris = (float4*)keep(n * 3 * sizeof(float4));
  float4* shade = (float4*)keep(n * sizeof(float4));
  float* corner = any_normals ? (float*)keep(n * 9 * sizeof(float)) : nullptr;
  float4* ploc_nodes = (float4*)keep(m * sizeof(PNode));
  int32_t* perm_keep = (int32_t*)keep(n * sizeof(int32_t));
  if ((width == 2 && !bvh) || (hybrid && !bvh_bin) || !slot_tris || !shade ||
      (any_normals && !corner) ||
      !ploc_nodes || !perm_keep)
    return set_err(ctx, AJG_ERR_OOM, "device allocation failed (scene)");

  Arena tmp;
  float* d_tris = tmp.get<float>(n * 9);
  int32_t* d_mat = tmp.get<int32_t>(n);
  int32_t* d_flags = tmp.get<int32_t>(n);
  uint32_t* ka = tmp.get<uint32_t>(n);
  uint32_t* kb = tmp.get<uint32_t>(n);
  int32_t* va = tmp.get<int32_t>(n);
  int32_t* vb = tmp.get<int32_t>(n);
  const uint32_t nbt = (uint32_t)((n + kRadixTile - 1) / kRadixTile);
  const uint64_t hist_n = (uint64_t)kBuckets * nbt;
  uint32_t* hist = tmp.get<uint32_t>(hist_n);
  uint32_t* scratch =
      tmp.get<uint32_t>(scan_scratch_words(hist_n > m ? hist_n : m));
  int32_t* owner = opts.radix_compat ? tmp.get<int32_t>(n) : nullptr;
  uint32_t* pos_of = opts.radix_compat ? tmp.get<uint32_t>(n) : nullptr;
  uint32_t* acc = tmp.get<uint32_t>(2);
  PNode* na = tmp.get<PNode>(m);
  PNode* nbuf = tmp.get<PNode>(m);
  uint32_t* nbr = tmp.get<uint32_t>(m);
  uint32_t* mi = tmp.get<uint32_t>(m);
  uint32_t* flags = tmp.get<uint32_t>(m);
  if (tmp.err != cudaSuccess)
    return set_err(ctx, AJG_ERR_OOM, "device allocation failed (PLOC build)");

  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaMemcpyAsync(d_tris, h_tris, n * 9 * sizeof(float),
                  cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(d_mat, h_mat, n * sizeof(int32_t), cudaMemcpyHostToDevice,
                  st);
  cudaMemcpyAsync(d_flags, h_flags, n * sizeof(int32_t),
                  cudaMemcpyHostToDevice, st);
  if (corner)
    cudaMemcpyAsync(corner, h_corner, n * 9 * sizeof(float),
                    cudaMemcpyHostToDevice, st);
  cudaMemsetAsync(ctx->d_error, 0, sizeof(uint32_t), st);
  cudaEventRecord(e0, st);

  // MortonEncoder (ploc_aggregate.cpp:61-66): grid = 1024 / size, offset =
  // -min * grid, all in float
  const F3 wlo = mk3(world[0], world[1], world[2]);
  const F3 whi = mk3(world[3], world[4], world[5]);
  const F3 size = whi - wlo;
  const F3 inv = mk3(1.f / size.x, 1.f / size.y, 1.f / size.z);
  const F3 w2g = inv * 1024.f;
  const F3 off = (-wlo) * w2g;
  const int gb = grid_for(n, 256);
  k_morton<<<gb, 256, 0, st>>>(d_tris, n, w2g, off, ka, va);

  // three 10-bit passes; compat passes scatter into buffers whose stale
  // contents match the reference's (zeroed copies, then originals, ...)
  if (opts.radix_compat) {
    cudaMemsetAsync(kb, 0, n * sizeof(uint32_t), st);
    cudaMemsetAsync(vb, 0, n * sizeof(int32_t), st);
    cudaMemsetAsync(acc, 0, 2 * sizeof(uint32_t), st);
  }
  uint32_t* kin = ka;
  uint32_t* kout = kb;
  int32_t* vin = va;
  int32_t* vout = vb;
  for (int bit = 0; bit < 30; bit += 10) {
    k_radix_hist<<<nbt, kRadixThreads, 0, st>>>(kin, n, bit, hist, nbt);
    device_scan(hist, hist, hist_n, true, scratch, st);
    if (opts.radix_compat) {
      k_compat_base<<<1, 1, 0, st>>>(hist, nbt, acc);
      cudaMemsetAsync(owner, 0xff, n * sizeof(int32_t), st);
    }
    k_radix_scatter<<<nbt, kRadixThreads, 0, st>>>(
        kin, vin, kout, vout, n, bit, hist, nbt, opts.radix_compat ? 1 : 0,
        acc, owner, pos_of, ctx->d_error);
    if (opts.radix_compat)
      k_radix_compat_write<<<gb, 256, 0, st>>>(kin, vin, kout, vout, n, owner,
                                               pos_of);
    std::swap(kin, kout);
    std::swap(vin, vout);
  }
  const int32_t* perm = vin;  // sorted values after three passes

  // leaves, then cluster until one node remains
  uint64_t begin = m - n, end = m, pre_end = m;
  k_leaf_init<<<gb, 256, 0, st>>>(d_tris, perm, na, begin, n);
  PNode* in = na;
  PNode* out = nbuf;
  uint32_t iters = 0;
  const size_t smem = (size_t)(kClusterThreads + 2 * r) * 6 * sizeof(float);
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(k_neighbors,
                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
  uint32_t merged_h = 0;
  // the blocks of nodes each iteration finalises, in order (children
  // before their parents), for the SAH collapse
  std::vector<std::pair<uint64_t, uint64_t>> fin_blocks;
  while (end - begin > 1) {
    if (++iters > 100000)
      return set_err(ctx, AJG_ERR_DEVICE, "PLOC did not converge");
    const uint32_t cnt = (uint32_t)(end - begin);
    const unsigned blocks = (cnt + kClusterThreads - 1) / kClusterThreads;
    k_neighbors<<<blocks, kClusterThreads, smem, st>>>(
        in, (uint32_t)begin, (uint32_t)end, r, nbr);
    k_merge_flags<<<grid_for(cnt, 256), 256, 0, st>>>(nbr, (uint32_t)begin,
                                                     (uint32_t)end, flags);
    device_scan(flags, mi, cnt, false, scratch, st);
    cudaMemcpyAsync(&merged_h, mi + cnt - 1, sizeof(uint32_t),
                    cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess)
      return set_err(ctx, AJG_ERR_CUDA,
                     std::string("PLOC build: ") +
                         cudaGetErrorString(cudaGetLastError()));
    if (merged_h == 0)
      return set_err(ctx, AJG_ERR_DEVICE, "PLOC iteration merged no pair");
    const uint64_t merged = merged_h;
    const uint64_t unmerged = cnt - merged;
    const uint64_t children = merged * 2;
    const uint64_t children_begin = end - children;
    const uint64_t unmerged_begin = end - (children + unmerged);
    fin_blocks.emplace_back(children_begin, end);
    k_cluster_scatter<<<grid_for(cnt, 256), 256, 0, st>>>(
        in, out, nbr, mi, (uint32_t)begin, (uint32_t)end,
        (uint32_t)unmerged_begin, (uint32_t)children_begin);
    if (pre_end > end)
      cudaMemcpyAsync(out + end, in + end, (pre_end - end) * sizeof(PNode),
                      cudaMemcpyDeviceToDevice, st);
    std::swap(in, out);
    pre_end = end;
    begin = unmerged_begin;
    end = children_begin;
  }
  const PNode* nodes = in;
  fin_blocks.emplace_back(begin, end);  // the root

  // traversal layout
  cudaMemcpyAsync(ploc_nodes, nodes, m * sizeof(PNode),
                  cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(perm_keep, perm, n * sizeof(int32_t),
                  cudaMemcpyDeviceToDevice, st);
  uint32_t num_nodes = (uint32_t)inner;
  if (width == 2) {
    if (n > 1) {
      k_inner_flags<<<grid_for(m, 256), 256, 0, st>>>(nodes, m, flags);
      device_scan(flags, mi, m, true, scratch, st);
      k_bvh2<<<grid_for(m, 256), 256, 0, st>>>(nodes, m, mi, bvh);
    } else {
      k_bvh2_single<<<1, 1, 0, st>>>(nodes, bvh);
    }
  } else {
    if (hybrid && n > 1) {
      k_inner_flags<<<grid_for(m, 256), 256, 0, st>>>(nodes, m, flags);
      device_scan(flags, mi, m, true, scratch, st);
      k_bvh2<<<grid_for(m, 256), 256, 0, st>>>(nodes, m, mi, bvh_bin);
    } else if (hybrid) {
      k_bvh2_single<<<1, 1, 0, st>>>(nodes, bvh_bin);
    }
    // wide layout: collapse level by level into a worst-case buffer, then
    // keep the nodes made
    const uint64_t node_f4 =
        compressed ? (wn == 8 ? CwLayout<8>::kFloat4 : CwLayout<4>::kFloat4)
                   : 2 * (uint64_t)wn;
    // the triangles move into node order for compressed nodes
    k_slot_tris<<<gb, 256, 0, st>>>(d_tris, perm, n, slot_tris);
    float4* wtmp = tmp.get<float4>(inner * node_f4);
    float4* tri_tmp = compressed ? tmp.get<float4>(3 * n) : nullptr;
    uint2* fa = tmp.get<uint2>(inner);
    uint2* fb = tmp.get<uint2>(inner);
    uint32_t* wc = tmp.get<uint32_t>(3);
    if (tmp.err != cudaSuccess)
      return set_err(ctx, AJG_ERR_OOM, "device allocation failed (wide BVH)");
    const bool sah = AJG_SAH_COLLAPSE && wn == 4 && !compressed;
    uint32_t* choice = nullptr;
    if (sah) {
      float4* cost = tmp.get<float4>(m);
      choice = tmp.get<uint32_t>(m);
      if (tmp.err != cudaSuccess)
        return set_err(ctx, AJG_ERR_OOM, "device allocation failed (SAH collapse)");
      for (const auto& b : fin_blocks) {
        const uint32_t cnt = (uint32_t)(b.second - b.first);
        k_sah_dp<<<grid_for(cnt, 256), 256, 0, st>>>(
            nodes, (uint32_t)b.first, (uint32_t)b.second, cost, choice);
      }
    }
    const uint32_t init[3] = {0u, 1u, 0u};
    cudaMemcpyAsync(wc, init, sizeof(init), cudaMemcpyHostToDevice, st);
    const uint2 root = make_uint2(0u, 0u);
    cudaMemcpyAsync(fa, &root, sizeof(root), cudaMemcpyHostToDevice, st);
    uint32_t n_in = 1, levels = 0;
    while (n_in) {
      cudaMemsetAsync(wc, 0, sizeof(uint32_t), st);
      const int g = grid_for(n_in, 128);
      if (compressed && wn == 4)
        k_collapse_c<4><<<g, 128, 0, st>>>(nodes, slot_tris, fa, n_in, fb, wc,
                                           wtmp, tri_tmp);
      else if (compressed)
        k_collapse_c<8><<<g, 128, 0, st>>>(nodes, slot_tris, fa, n_in, fb, wc,
                                           wtmp, tri_tmp);
      else if (sah)
        k_collapse_sah<<<g, 128, 0, st>>>(nodes, choice, fa, n_in, fb, wc,
                                          wtmp);
      else if (wn == 4)
        k_collapse<4><<<g, 128, 0, st>>>(nodes, fa, n_in, fb, wc, wtmp);
      else
        k_collapse<8><<<g, 128, 0, st>>>(nodes, fa, n_in, fb, wc, wtmp);
      uint32_t h[2] = {0, 0};
      if (cudaMemcpyAsync(h, wc, sizeof(h), cudaMemcpyDeviceToHost, st) !=
              cudaSuccess ||
          cudaStreamSynchronize(st) != cudaSuccess)
        return set_err(ctx, AJG_ERR_CUDA, "wide BVH collapse failed");
      n_in = h[0];
      num_nodes = h[1];
      std::swap(fa, fb);
      if (++levels > inner + 1)
        return set_err(ctx, AJG_ERR_DEVICE, "wide BVH collapse did not end");
    }
    bvh = (float4*)keep((uint64_t)num_nodes * node_f4 * sizeof(float4));
    if (!bvh)
      return set_err(ctx, AJG_ERR_OOM, "device allocation failed (wide BVH)");
    cudaMemcpyAsync(bvh, wtmp, (uint64_t)num_nodes * node_f4 * sizeof(float4),
                    cudaMemcpyDeviceToDevice, st);
    if (compressed)
      cudaMemcpyAsync(slot_tris, tri_tmp, 3 * n * sizeof(float4),
                      cudaMemcpyDeviceToDevice, st);
  }
  if (width == 2) k_slot_tris<<<gb, 256, 0, st>>>(d_tris, perm, n, slot_tris);
  k_shade_data<<<gb, 256, 0, st>>>(d_tris, d_mat, d_flags, n, shade);
  cudaEventRecord(e1, st);
  cudaError_t ce = cudaStreamSynchronize(st);
  uint32_t derr = 0;
  if (ce == cudaSuccess)
    ce = cudaMemcpy(&derr, ctx->d_error, sizeof(uint32_t),
                    cudaMemcpyDeviceToHost);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (ce != cudaSuccess)
    return set_err(ctx, AJG_ERR_CUDA,
                   std::string("PLOC build: ") + cudaGetErrorString(ce));
  if (derr == kDevSortOutOfBounds)
    return set_err(ctx, AJG_ERR_INVALID,
                   "radix_compat: the reference's sort would write out of "
                   "bounds on this input");
  if (derr)
    return set_err(ctx, AJG_ERR_DEVICE, "device guard tripped in PLOC build");

  s->d.bvh = bvh;
  s->d.bvh_closest = bvh_bin;
  s->d.num_inner_closest = hybrid ? (uint32_t)inner : 0u;
  s->info.closest_node_bytes = 0;  // set with bvh_node_bytes below
  s->d.tris = slot_tris;
  s->d.shade = shade;
  s->d.corner = corner;
  s->d.n = n;
  s->d.num_inner = num_nodes;
  s->d.width = width;
  s->d.tri_test = (int32_t)opts.tri_test;
  s->ploc_nodes = ploc_nodes;
  s->perm = perm_keep;
  s->info.num_triangles = n;
  s->info.num_nodes = m;
  s->info.ploc_iterations = iters;
  s->info.build_ms = ms;
  s->info.bvh_width = (uint32_t)width;
  s->info.bvh_node_bytes =
      width == 2 ? 64u
                 : (compressed ? 16u * (wn == 8 ? CwLayout<8>::kFloat4
                                                : CwLayout<4>::kFloat4)
                               : 32u * (uint32_t)wn);
  s->info.bvh_nodes = num_nodes;
  s->info.closest_node_bytes = hybrid ? 64u : s->info.bvh_node_bytes;
  for (int k = 0; k < 6; ++k) s->world[k] = world[k];
  // lights are fitted to the world bounds (default_scene.cpp:41-48)
  const F3 center = (whi + wlo) / 2.f;
  const F3 half = whi - center;
  float d = 0.f;
  d += half.x * half.x;
  d += half.y * half.y;
  d += half.z * half.z;
  s->d.radius = sqrtf(d);
  s->d.packet_spread = kPacketSpread * median_edge(h_tris, n);
  return AJG_OK;
}

}  // namespace ajg
