// Closest-hit and any-hit traversal over the PLOC tree: the binary tree as
// built, or (the default) the tree collapsed into 4-wide nodes, 8-wide, or
// 4/8-wide with quantised boxes.
//
// Results are defined independently of the tree shape and of the visiting
// order: the closest hit is the minimum t over every triangle the test
// accepts, ties in t going to the lowest primitive index, and the node test
// does not cull a box that can hold a nearer hit -- it is the reference's
// slab test, (bound - o) * inv_dir (ploc_aggregate.cpp:154-162), with the
// far distance widened by 1 + 2*gamma(3) (Pharr, Jakob, Humphreys, PBRT 3rd
// ed., 3.9.2) and inclusive comparisons against the current best t.  The
// one exception is an exact tie in t (a ray through an edge two triangles
// share) whose lower-index triangle's box is entered at a distance that
// rounds above that t: found second, that triangle's box is culled, so the
// visiting order picks the winner; a ray's order is fixed, so its result is
// reproducible.  Any hits do not depend on the order at all.  Lanes are
// persistent (trace_persistent): one node visit per iteration, a lane whose
// ray finished takes the next from a shared counter.  Closest-hit rays visit
// the nearest interior child and push the others farthest first; any-hit
// rays take the children in order; a wide node's passing leaf children are
// tested after its box tests, or -- any-hit rays over the plain wide tree --
// held until the warp's next leaf pass, in which every lane holding some
// tests one (the lanes that found leaves in a visit are a few of the 32, and
// the pass gathers their tests into fewer warp instructions).  Each lane's
// stack keeps its top 16 entries
// in a shared-memory ring and the rest in local memory, and is guarded:
// overflow sets the device error word and ends the ray.  Coherent rays -- a
// pixel's shadow rays toward a directional light, and on request its camera
// rays -- are traced as masked packets instead (trace_packet_any,
// trace_packet_closest): a warp walks the tree once for its 32 rays, each
// lane testing the boxes and triangles its own ray reaches.
#pragma once
#include <type_traits>

#include "scene.cuh"

namespace ajg {

constexpr float kSlabWiden = 1.0000003576278687f;  // 1 + 2*gamma(3)

struct Hit {
  float t, u, v;
  int prim;
};

struct RayQ {
  F3 o, d, inv;
  float tmin, tmax;
};

// Triangle::Intersect / Occlude's Moller-Trumbore test
// (ploc_aggregate.cpp:184-242), with the reference's absolute determinant
// cull and open (t_min, t_max) interval.
__device__ __forceinline__ bool mt_test(const RayQ& r, float4 A, float4 B,
                                        float4 Cv, float& t_out, float& u_out,
                                        float& v_out) {
  const F3 v0 = xyz(A), v1 = xyz(B), v2 = xyz(Cv);
  const F3 e0 = v1 - v0, e1 = v2 - v0;
  const F3 h = cross3(r.d, e1);
  const float a = dot3f(e0, h);
  if (a > -1e-6f && a < 1e-6f) return false;
  const float f = __frcp_rn(a);  // == 1.f / a, correctly rounded
  const F3 s = r.o - v0;
  const float u = f * dot3f(s, h);
  if (u < 0.f || u > 1.f) return false;
  const F3 q = cross3(s, e0);
  const float v = f * dot3f(r.d, q);
  if (v < 0.f || u + v > 1.f) return false;
  const float t = f * dot3f(e1, q);
  if (!(t > r.tmin && t < r.tmax)) return false;
  t_out = t;
  u_out = u;
  v_out = v;
  return true;
}

// Watertight test (Woop, Benthin, Wald, JCGT 2(1), 2013), no double
// fallback; barycentrics reported for b and c as Moller-Trumbore does.
struct WtSetup {
  int kx, ky, kz;
  float sx, sy, sz;
};
__device__ __forceinline__ WtSetup wt_setup(const RayQ& r) {
  WtSetup w;
  const float ax = fabsf(r.d.x), ay = fabsf(r.d.y), az = fabsf(r.d.z);
  int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
  int kx = kz + 1 == 3 ? 0 : kz + 1;
  int ky = kx + 1 == 3 ? 0 : kx + 1;
  const float d[3] = {r.d.x, r.d.y, r.d.z};
  if (d[kz] < 0.f) {
    int t = kx;
    kx = ky;
    ky = t;
  }
  w.kx = kx;
  w.ky = ky;
  w.kz = kz;
  w.sx = d[kx] / d[kz];
  w.sy = d[ky] / d[kz];
  w.sz = 1.f / d[kz];
  return w;
}
__device__ __forceinline__ float comp(F3 v, int k) {
  return k == 0 ? v.x : (k == 1 ? v.y : v.z);
}
__device__ __forceinline__ bool wt_test(const RayQ& r, const WtSetup& w,
                                        float4 A4, float4 B4, float4 C4,
                                        float& t_out, float& u_out,
                                        float& v_out) {
  const F3 A = xyz(A4) - r.o, B = xyz(B4) - r.o, C = xyz(C4) - r.o;
  const float Az0 = comp(A, w.kz), Bz0 = comp(B, w.kz), Cz0 = comp(C, w.kz);
  const float Ax = comp(A, w.kx) - w.sx * Az0, Ay = comp(A, w.ky) - w.sy * Az0;
  const float Bx = comp(B, w.kx) - w.sx * Bz0, By = comp(B, w.ky) - w.sy * Bz0;
  const float Cx = comp(C, w.kx) - w.sx * Cz0, Cy = comp(C, w.ky) - w.sy * Cz0;
  const float U = Cx * By - Cy * Bx;
  const float V = Ax * Cy - Ay * Cx;
  const float W = Bx * Ay - By * Ax;
  if ((U < 0.f || V < 0.f || W < 0.f) && (U > 0.f || V > 0.f || W > 0.f))
    return false;
  const float det = U + V + W;
  if (det == 0.f) return false;
  const float T = U * (w.sz * Az0) + V * (w.sz * Bz0) + W * (w.sz * Cz0);
  const float rcp = __frcp_rn(det);
  const float t = T * rcp;
  if (!(t > r.tmin && t < r.tmax)) return false;
  t_out = t;
  u_out = V * rcp;
  v_out = W * rcp;
  return true;
}

__device__ __forceinline__ bool slab2(float lox, float hix, float loy,
                                      float hiy, float loz, float hiz,
                                      const RayQ& r, float lim, float& tn) {
  const float tx0 = (lox - r.o.x) * r.inv.x, tx1 = (hix - r.o.x) * r.inv.x;
  const float ty0 = (loy - r.o.y) * r.inv.y, ty1 = (hiy - r.o.y) * r.inv.y;
  const float tz0 = (loz - r.o.z) * r.inv.z, tz1 = (hiz - r.o.z) * r.inv.z;
  tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fminf(tz0, tz1));
  float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fmaxf(tz0, tz1));
  tf = tf * kSlabWiden;
  return tn <= tf && tn <= lim && tf >= r.tmin;
}

// Two consecutive float4 of a node (32-byte aligned: node arrays come from
// cudaMalloc and their strides are multiples of 64 bytes).  With
// AJG_WIDE_LOADS one 256-bit load per lane (sm_100 and later): one sector
// and one load instruction instead of two.
#ifndef AJG_WIDE_LOADS
#define AJG_WIDE_LOADS 1
#endif
__device__ __forceinline__ void ldg_node(const float4* p, float4& a,
                                         float4& b) {
#if AJG_WIDE_LOADS
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y),
        "=f"(b.z), "=f"(b.w)
      : "l"(p));
#else
  a = __ldg(p);
  b = __ldg(p + 1);
#endif
}

__device__ __forceinline__ RayQ make_query(F3 o, F3 d, float tmin,
                                           float tmax) {
  RayQ r;
  r.o = o;
  r.d = d;
  r.inv = mk3(1.f / d.x, 1.f / d.y, 1.f / d.z);
  r.tmin = tmin;
  r.tmax = tmax;
  return r;
}

// The tree a ray is traced against.  FETCH(k, ts) may retarget `ts` per
// ray (waves that mix scenes); single-scene callers leave it untouched.
struct TraceScene {
  const float4* bvh;
  const float4* tris;
  uint32_t max_visits;  // a ray visits each node of the tree at most once
};
__device__ __forceinline__ TraceScene trace_scene(const DeviceScene& s) {
  TraceScene t;
  t.bvh = s.bvh;
  t.tris = s.tris;
  t.max_visits = s.num_inner + 1;
  return t;
}

// Stack depth per lane: a node visit pushes at most W-1 siblings.
template <int W>
struct StackDepth {
  static constexpr int value = W == 2 ? 96 : (W == 4 ? 128 : 192);
};

// Tests one triangle of a leaf slot against the ray and keeps the closest
// hit (ties in t to the lowest primitive index); any-hit queries stop at the
// first accepted triangle.
template <int TEST, bool ANY>
__device__ __forceinline__ bool leaf_test(const float4* __restrict__ tris,
                                          int slot, const RayQ& r,
                                          const WtSetup& w, Hit& hit) {
  const float4 A = __ldg(tris + 3 * slot + 0);
  const float4 B = __ldg(tris + 3 * slot + 1);
  const float4 C = __ldg(tris + 3 * slot + 2);
  float t, u, v;
  const bool ok = TEST == AJG_TRI_WATERTIGHT ? wt_test(r, w, A, B, C, t, u, v)
                                             : mt_test(r, A, B, C, t, u, v);
  if (!ok) return false;
  const int prim = __float_as_int(A.w);
  if (ANY || t < hit.t || (t == hit.t && prim < hit.prim)) {
    hit.t = t;
    hit.u = u;
    hit.v = v;
    hit.prim = prim;
  }
  return ANY;
}

// Persistent-lane traversal.  Each lane owns one ray at a time and runs one
// node visit per loop iteration; lanes whose ray finished take new rays from
// a shared counter (warp-aggregated, once at least AJG_REFILL (closest hit)
// or AJG_REFILL_ANY (any hit) lanes of the warp are idle), so lanes are not
// left idle at ray boundaries waiting for the warp's slowest ray.  FETCH(k, ts) returns the k-th ray; FINISH(k, hit,
// occluded) stores its result.
//
// L is the tree layout: 2 is the binary PLOC tree (64-byte nodes holding
// both children's boxes); 4 and 8 are the collapsed wide trees (32*W-byte
// nodes: the children's boxes as lo.x, hi.x, lo.y, hi.y, lo.z, hi.z groups
// of four, then the child references); 4 or 8 | kBvhCompressed the
// quantised wide nodes (scene.cuh).  In a wide node the leaf children whose
// box passes are gathered during the box tests and then tested in one loop
// (one call site, so the lanes with an i-th leaf test it together); for
// closest hits the nearest interior child is visited next and the others
// are pushed farthest first.
#ifndef AJG_REFILL
#define AJG_REFILL 24  // closest-hit queries
#endif
// Blocks of 128 threads per SM the traversal kernels over 2- and 4-wide
// trees are compiled for: 8 caps them at 64 registers, which they fit without
// spills.  The 8-wide ones would spill there and stay uncapped (1).
#ifndef AJG_TRACE_MIN_BLOCKS
#define AJG_TRACE_MIN_BLOCKS 8
#endif
#ifndef AJG_TRACE_MIN_BLOCKS_BIN
#define AJG_TRACE_MIN_BLOCKS_BIN AJG_TRACE_MIN_BLOCKS  // the binary layout
#endif
template <int L>
constexpr int trace_min_blocks() {
  return (L & ~kBvhCompressed) == 8 ? 1
         : L == 2                   ? AJG_TRACE_MIN_BLOCKS_BIN
                                    : AJG_TRACE_MIN_BLOCKS;
}
#ifndef AJG_SMEM_STACK
#define AJG_SMEM_STACK 16  // stack entries per lane in shared memory (a power
                           // of two; 0: the whole stack in local memory)
#endif
#ifndef AJG_ANY_RING
#define AJG_ANY_RING AJG_SMEM_STACK  // the same for any-hit queries
#endif
#ifndef AJG_CLOSEST_STACK_T
#define AJG_CLOSEST_STACK_T 1  // 0: closest-hit entries without the box's
                               // entry distance (popped boxes are re-tested)
#endif
#ifndef AJG_LEAF_BATCH
#define AJG_LEAF_BATCH 1  // 0: test each leaf child at its own call site
#endif
#ifndef AJG_REFILL_ANY
#define AJG_REFILL_ANY 12  // any-hit queries
#endif
#ifndef AJG_LEAF_DEFER
#define AJG_LEAF_DEFER 6  // any-hit queries over a plain wide tree: lanes
                          // keep a node's leaf children pending, and the warp
                          // tests pending leaves together once this many
                          // lanes hold some (0: each visit tests its leaves)
#endif
#ifndef AJG_LEAF_DEFER_CLOSEST
#define AJG_LEAF_DEFER_CLOSEST 0  // the same for closest-hit queries over
                                  // the binary layout
#endif
constexpr int kRefill = AJG_REFILL;
constexpr int kEmptyRef = (int)0x80000000;  // unused child of a wide node

template <int TEST, bool ANY, int L, class FETCH, class FINISH>
__device__ __forceinline__ void trace_persistent(
    TraceScene ts, uint32_t n, uint32_t* next, FETCH fetch, FINISH finish,
    uint32_t& n_rays, uint32_t& n_nodes, uint32_t& n_tris, uint32_t* err) {
  constexpr int W = L & 0xff;  // children per node
  constexpr bool CMP = (L & (int)kBvhCompressed) != 0;
  constexpr int kIdle = -1, kDone = 0x7fffffff;
  constexpr int kStack = StackDepth<W>::value;
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  int k = kIdle;
  RayQ r;
  WtSetup w;
  Hit hit;
  int node = 0, sp = 0;
  uint32_t visits = 0;
  // Deferred leaves: a node visit records its leaf children (mask `pend`,
  // slots pend_slot[child]) instead of testing them, and a lane holding
  // pending leaves visits no node (nor pops one) until the warp's next leaf
  // pass.  That pass comes once kLeafPass lanes (or all active ones) hold
  // some; each of them tests one, and a lane whose leaves are done pops its
  // next node against the hit they left.  Every node is visited with the
  // same hit as without deferral, so the visits and the result are the
  // same: only the grouping of the leaf tests into warp instructions moves.
  constexpr int kLeafPass = ANY ? ((!CMP && W >= 4) ? AJG_LEAF_DEFER : 0)
                                : (W == 2 ? AJG_LEAF_DEFER_CLOSEST : 0);
  constexpr bool kDefer = kLeafPass > 0;
  unsigned pend = 0;
  int pend_slot[W];
  int stack_node[kStack];
  float stack_t[kStack];
#if AJG_SMEM_STACK > 0
  // The top kShort entries of each lane's stack live in shared memory (a
  // ring: entry i in slot i % kShort, lane-interleaved); a push evicts the
  // entry kShort below the top to the local array, a pop refills its slot.
  // Any-hit entries hold the node alone: every pushed box passed against
  // the ray's fixed t_max, so the pop needs no distance.
  constexpr bool kNodeOnly = ANY || !AJG_CLOSEST_STACK_T;
  constexpr int kShort = ANY ? AJG_ANY_RING : AJG_SMEM_STACK;
  static_assert((kShort & (kShort - 1)) == 0, "a power of two");
  using Slot = std::conditional_t<kNodeOnly, int, int2>;
  __shared__ Slot s_ring[kShort * 128];
  Slot* const ring = s_ring + threadIdx.x;
  auto push = [&](int nd, float t) {
    const int slot = sp & (kShort - 1);
    if constexpr (kNodeOnly) {
      if (sp >= kShort) stack_node[sp - kShort] = ring[slot * 128];
      ring[slot * 128] = nd;
    } else {
      if (sp >= kShort) {
        const int2 old = ring[slot * 128];
        stack_node[sp - kShort] = old.x;
        stack_t[sp - kShort] = __int_as_float(old.y);
      }
      ring[slot * 128] = make_int2(nd, __float_as_int(t));
    }
    ++sp;
  };
  auto pop = [&](int& nd, float& t) {
    --sp;
    const int slot = sp & (kShort - 1);
    if constexpr (kNodeOnly) {
      nd = ring[slot * 128];
      t = -__int_as_float(0x7f800000);
      if (sp >= kShort) ring[slot * 128] = stack_node[sp - kShort];
    } else {
      const int2 v = ring[slot * 128];
      nd = v.x;
      t = __int_as_float(v.y);
      if (sp >= kShort)
        ring[slot * 128] = make_int2(stack_node[sp - kShort],
                                     __float_as_int(stack_t[sp - kShort]));
    }
  };
#else
  auto push = [&](int nd, float t) {
    stack_node[sp] = nd;
    stack_t[sp] = t;
    ++sp;
  };
  auto pop = [&](int& nd, float& t) {
    --sp;
    nd = stack_node[sp];
    t = stack_t[sp];
  };
#endif
  for (;;) {
    const unsigned idle = __ballot_sync(full, k == kIdle);
    const unsigned done = __ballot_sync(full, k == kDone);
    constexpr int kRefillQ = ANY ? AJG_REFILL_ANY : kRefill;
    if (idle && (__popc(idle) >= kRefillQ || (idle | done) == full)) {
      const int leader = __ffs(idle) - 1;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(next, (uint32_t)__popc(idle));
      base = __shfl_sync(full, base, leader);
      if (k == kIdle) {
        const uint32_t kk = base + __popc(idle & lt);
        if (kk < n) {
          k = (int)kk;
          r = fetch(kk, ts);
          if (TEST == AJG_TRI_WATERTIGHT) w = wt_setup(r);
          hit.t = __int_as_float(0x7f800000);
          hit.prim = -1;
          hit.u = hit.v = 0.f;
          node = 0;
          sp = 0;
          visits = 0;
        } else {
          k = kDone;
        }
      }
    }
    if (__all_sync(full, k == kDone)) break;
    if constexpr (kDefer) {
      const bool act = k >= 0 && k != kDone;
      const unsigned pm = __ballot_sync(full, act && pend != 0);
      const unsigned am = __ballot_sync(full, act);
      if (pm && (__popc(pm) >= kLeafPass || pm == am)) {
        // the leaf pass
        if (pend) {
          const int c = __ffs(pend) - 1;
          pend &= pend - 1;
          int slot = 0;
#pragma unroll
          for (int j = 0; j < W; ++j)
            if (j == c) slot = pend_slot[j];
          ++n_tris;
          bool fin = leaf_test<TEST, ANY>(ts.tris, slot, r, w, hit);
          if (!fin && !pend && node < 0) {
            // the visit's deferred pop
            fin = true;
            while (sp > 0) {
              int nd;
              float st;
              pop(nd, st);
              if (st <= (ANY ? r.tmax : fminf(hit.t, r.tmax))) {
                node = nd;
                fin = false;
                break;
              }
            }
          }
          if (fin) {
            pend = 0;
            ++n_rays;
            finish((uint32_t)k, hit, hit.prim >= 0);
            k = kIdle;
          }
        }
        continue;
      }
      if (pend) continue;  // waits for the leaf pass
    }
    if (k < 0 || k == kDone) continue;

    // one node visit
    bool finished = false;
    ++n_nodes;
    if (++visits > ts.max_visits) {
      raise_device_error(err, kDevIterationBound);
      finish((uint32_t)k, hit, hit.prim >= 0);
      k = kIdle;
      pend = 0;
      continue;
    }
    const float4* __restrict__ bvh = ts.bvh;
    const float4* __restrict__ tris = ts.tris;
    const float lim = ANY ? r.tmax : fminf(hit.t, r.tmax);
    bool descend = false;  // `node` holds the next node to visit
    if constexpr (W == 2) {
      float4 n0, n1, n2, n3;
      ldg_node(bvh + 4 * (uint64_t)node, n0, n1);
      ldg_node(bvh + 4 * (uint64_t)node + 2, n2, n3);
      float tn0, tn1;
      bool h0 = slab2(n0.x, n0.y, n0.z, n0.w, n2.x, n2.y, r, lim, tn0);
      bool h1 = slab2(n1.x, n1.y, n1.z, n1.w, n2.z, n2.w, r, lim, tn1);
      const int r0 = __float_as_int(n3.x), r1 = __float_as_int(n3.y);
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const bool hc = c == 0 ? h0 : h1;
        const int rc = c == 0 ? r0 : r1;
        if (kDefer && hc && rc < 0) {
          pend |= 1u << c;
          pend_slot[c] = ~rc;
        } else if (hc && rc < 0 && !finished) {
          ++n_tris;
          finished = leaf_test<TEST, ANY>(tris, ~rc, r, w, hit);
        }
        if (hc && rc < 0) {
          if (c == 0)
            h0 = false;
          else
            h1 = false;
        }
      }
      if (!finished) {
        if (h0 && h1) {
          const bool first0 = tn0 <= tn1;
          if (sp >= kStack) {
            raise_device_error(err, kDevStackOverflow);
            finished = true;
          } else {
            push(first0 ? r1 : r0, first0 ? tn1 : tn0);
            node = first0 ? r0 : r1;
            descend = true;
          }
        } else if (h0) {
          node = r0;
          descend = true;
        } else if (h1) {
          node = r1;
          descend = true;
        }
      }
    } else {
      float tn[W];
      int ref[W];
      unsigned inner = 0;  // interior children whose box passed
#if AJG_LEAF_BATCH
      // leaf children whose box passed (mask `leaves`, slot per child, both
      // indexed by the child so that they stay in registers), tested after
      // the box tests from one call site (all lanes with an i-th leaf test
      // it together)
      int leaf_slot[W];
      unsigned leaves = 0;
#endif
      if constexpr (!CMP) {
        constexpr int G = W / 4;  // float4 groups per plane
        const float4* nd = bvh + (uint64_t)node * (2 * W);
        float4 q[8 * G];  // the node's 2W float4, the last G padding
#pragma unroll
        for (int i = 0; i < 7 * G; i += 2) ldg_node(nd + i, q[i], q[i + 1]);
#pragma unroll
        for (int g = 0; g < G; ++g) {
          const float4 lx = q[0 * G + g], hx = q[1 * G + g];
          const float4 ly = q[2 * G + g], hy = q[3 * G + g];
          const float4 lz = q[4 * G + g], hz = q[5 * G + g];
          const float4 rf = q[6 * G + g];
          const float* plx = &lx.x;
          const float* phx = &hx.x;
          const float* ply = &ly.x;
          const float* phy = &hy.x;
          const float* plz = &lz.x;
          const float* phz = &hz.x;
          const float* prf = &rf.x;
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int c = 4 * g + j;
            ref[c] = __float_as_int(prf[j]);
            float t0;
            const bool h = ref[c] != kEmptyRef &&
                           slab2(plx[j], phx[j], ply[j], phy[j], plz[j],
                                 phz[j], r, lim, t0);
            tn[c] = t0;
#if AJG_LEAF_BATCH
            if (kDefer && h && ref[c] < 0) {
              pend |= 1u << c;
              pend_slot[c] = ~ref[c];
            } else if (h && ref[c] < 0) {
              leaf_slot[c] = ~ref[c];
              leaves |= 1u << c;
            }
#else
            if (h && ref[c] < 0 && !finished) {
              ++n_tris;
              finished = leaf_test<TEST, ANY>(tris, ~ref[c], r, w, hit);
            }
#endif
            if (h && ref[c] >= 0) inner |= 1u << c;
          }
        }
      } else {
        constexpr int NF = CwLayout<W>::kFloat4;
        const float4* nd = bvh + (uint64_t)node * NF;
        const float4 h0 = __ldg(nd), h1 = __ldg(nd + 1);
        uint32_t qw[4 * (NF - 2)];
#pragma unroll
        for (int f = 0; f < NF - 2; ++f) {
          const float4 v = __ldg(nd + 2 + f);
          qw[4 * f] = __float_as_uint(v.x);
          qw[4 * f + 1] = __float_as_uint(v.y);
          qw[4 * f + 2] = __float_as_uint(v.z);
          qw[4 * f + 3] = __float_as_uint(v.w);
        }
        const uint32_t hb = __float_as_uint(h0.w);
        const float sx = cw_scale(hb & 0xffu);
        const float sy = cw_scale((hb >> 8) & 0xffu);
        const float sz = cw_scale((hb >> 16) & 0xffu);
        const uint32_t imask = hb >> 24;
        const uint32_t cbase = __float_as_uint(h1.x);
        const uint32_t tbase = __float_as_uint(h1.y);
        const uint32_t vmask = __float_as_uint(h1.z);
        const uint32_t lmask = vmask & ~imask;
#pragma unroll
        for (int c = 0; c < W; ++c) {
          tn[c] = 0.f;
          ref[c] = 0;
          if (!((vmask >> c) & 1u)) continue;
          // plane k of child c: byte c of the plane's W bytes, decoded
          // exactly as the build checked it
          auto plane = [&](int k, float origin, float sc) {
            const uint32_t word = qw[k * (W / 4) + (c >> 2)];
            const uint32_t bits =
                __byte_perm(word, 0x4B000000u, (uint32_t)(c & 3) | 0x7540u);
            return cw_decode(origin, cw_qfloat(bits), sc);
          };
          float t0;
          if (!slab2(plane(0, h0.x, sx), plane(1, h0.x, sx),
                     plane(2, h0.y, sy), plane(3, h0.y, sy),
                     plane(4, h0.z, sz), plane(5, h0.z, sz), r, lim, t0))
            continue;
          tn[c] = t0;
          const uint32_t below = (1u << c) - 1u;
          if ((imask >> c) & 1u) {
            ref[c] = (int)(cbase + __popc(imask & below));
            inner |= 1u << c;
          } else {
#if AJG_LEAF_BATCH
            leaf_slot[c] = (int)(tbase + __popc(lmask & below));
            leaves |= 1u << c;
#else
            if (!finished) {
              ++n_tris;
              finished = leaf_test<TEST, ANY>(
                  tris, (int)(tbase + __popc(lmask & below)), r, w, hit);
            }
#endif
          }
        }
      }
#if AJG_LEAF_BATCH
      while (leaves && !finished) {
        const int c = __ffs(leaves) - 1;
        leaves &= leaves - 1;
        ++n_tris;
        int slot = 0;
#pragma unroll
        for (int j = 0; j < W; ++j)
          if (j == c) slot = leaf_slot[j];
        finished = leaf_test<TEST, ANY>(tris, slot, r, w, hit);
      }
#endif
      if (!finished && inner && ANY) {
        // occlusion: any order will do -- visit the first, push the rest
        const int c0 = __ffs(inner) - 1;
        inner &= inner - 1;
        while (inner && !finished) {
          const int c = __ffs(inner) - 1;
          inner &= inner - 1;
          if (sp >= kStack) {
            raise_device_error(err, kDevStackOverflow);
            finished = true;
            break;
          }
          int fr = 0;
          float ft = 0.f;
#pragma unroll
          for (int cc = 0; cc < W; ++cc)
            if (cc == c) {
              fr = ref[cc];
              ft = tn[cc];
            }
          push(fr, ft);
        }
        if (!finished) {
          int nr = 0;
#pragma unroll
          for (int cc = 0; cc < W; ++cc)
            if (cc == c0) nr = ref[cc];
          node = nr;
          descend = true;
        }
      } else if (!finished && inner) {
        // push all but the nearest, farthest first
        while (__popc(inner) > 1) {
          int far_c = -1;
          float far_t = -__int_as_float(0x7f800000);
#pragma unroll
          for (int c = 0; c < W; ++c)
            if (((inner >> c) & 1u) && (far_c < 0 || tn[c] > far_t)) {
              far_c = c;
              far_t = tn[c];
            }
          if (sp >= kStack) {
            raise_device_error(err, kDevStackOverflow);
            finished = true;
            break;
          }
          int fr = 0;
#pragma unroll
          for (int c = 0; c < W; ++c)
            if (c == far_c) fr = ref[c];
          push(fr, far_t);
          inner &= ~(1u << far_c);
        }
        if (!finished) {
          const int c = __ffs(inner) - 1;
          int nr = 0;
#pragma unroll
          for (int cc = 0; cc < W; ++cc)
            if (cc == c) nr = ref[cc];
          node = nr;
          descend = true;
        }
      }
    }
    if (kDefer && !finished && !descend && pend) {
      node = -1;  // pops after the leaf pass
    } else if (!finished && !descend) {
      // pop, skipping boxes a closer hit has since excluded
      finished = true;
      while (sp > 0) {
        int nd;
        float st;
        pop(nd, st);
        const float lim2 = ANY ? r.tmax : fminf(hit.t, r.tmax);
        if (st <= lim2) {
          node = nd;
          finished = false;
          break;
        }
      }
    }
    if (finished) {
      ++n_rays;
      finish((uint32_t)k, hit, hit.prim >= 0);
      k = kIdle;
      pend = 0;
    }
  }
}

// Any hits of coherent rays (a pixel's samples toward one light) as masked
// packets over the plain 4-wide tree.  A warp takes 32 consecutive rays and
// walks the tree once for all of them: one node fetch per visit, the same
// address in every lane (one broadcast transaction instead of up to 32
// gathers), each lane testing the node's child boxes against its own ray.
// A child is visited for the lanes whose ray passed its box, and a leaf's
// triangle is tested by exactly those lanes, so a lane tests the triangles
// it would test alone -- the leaves whose every ancestor box its ray passes
// -- and its occlusion is the same; lanes leave the packet once occluded.
// Control flow is uniform across the warp (node, lane masks and stack come
// from broadcast loads and ballots), and the stack of (node, lanes) pairs is
// the warp's, in shared memory.  The packet visits each node at most once
// (the tree's interior nodes + 1 bound its visits, as for one ray) and its
// stack holds at most 3 entries per level, as one ray's does.
// Rays of a multi-job wave carry their scene: FETCH(k, sid) returns the ray
// and its scene index, SCENE(sid, ts) points `ts` at that scene's tree, and
// the warp walks one packet per scene its 32 rays hold.
constexpr int kPacketThreads = 128;
template <int TEST, class FETCH, class FINISH, class SCENE>
__device__ __forceinline__ void trace_packet_any(
    TraceScene ts0, uint32_t n, uint32_t* next, FETCH fetch, FINISH finish,
    SCENE scene_of, uint32_t& n_rays, uint32_t& n_nodes, uint32_t& n_tris,
    uint32_t* err) {
  constexpr int W = 4;
  constexpr int kStack = StackDepth<W>::value;
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  __shared__ int2 s_pstack[kPacketThreads / 32][kStack];
  int2* const stk = s_pstack[threadIdx.x >> 5];
  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(next, 32u);
    base = __shfl_sync(full, base, 0);
    if (base >= n) break;
    const uint32_t kk = base + (uint32_t)lane;
    const bool act = kk < n;
    uint32_t sid = 0;
    const RayQ r = act ? fetch(kk, sid)
                       : make_query(mk3(0.f, 0.f, 0.f), mk3(0.f, 0.f, 1.f),
                                    0.f, 0.f);
    WtSetup w;
    if (TEST == AJG_TRI_WATERTIGHT) w = wt_setup(r);
    Hit hit;
    hit.t = __int_as_float(0x7f800000);
    hit.prim = -1;
    hit.u = hit.v = 0.f;
    unsigned todo = __ballot_sync(full, act);  // lanes of scenes not walked
    while (todo) {
      const uint32_t s0 = __shfl_sync(full, sid, __ffs(todo) - 1);
      // lanes not yet occluded: the packet of scene s0
      unsigned live = __ballot_sync(full, ((todo >> lane) & 1u) && sid == s0);
      todo &= ~live;
      TraceScene ts = ts0;
      scene_of(s0, ts);
      unsigned mask = live;  // lanes visiting `node`
      int node = 0, sp = 0;
      uint32_t visits = 0;
      while (mask) {
        if (++visits > ts.max_visits) {
          raise_device_error(err, kDevIterationBound);
          break;
        }
        const bool in = (mask >> lane) & 1u;
        if (in) ++n_nodes;
        const float4* nd = ts.bvh + (uint64_t)node * (2 * W);
        float4 q[8];
#pragma unroll
        for (int i = 0; i < 8; i += 2) ldg_node(nd + i, q[i], q[i + 1]);
        const float* plx = &q[0].x;
        const float* phx = &q[1].x;
        const float* ply = &q[2].x;
        const float* phy = &q[3].x;
        const float* plz = &q[4].x;
        const float* phz = &q[5].x;
        const float* prf = &q[6].x;
        int ref[W];
        unsigned hm[W];
#pragma unroll
        for (int j = 0; j < W; ++j) {
          ref[j] = __float_as_int(prf[j]);
          float t0;
          const bool h = in && ref[j] != kEmptyRef &&
                         slab2(plx[j], phx[j], ply[j], phy[j], plz[j],
                               phz[j], r, r.tmax, t0);
          hm[j] = __ballot_sync(full, h);
        }
        // leaf children first: the lanes whose ray passed the box test them
#pragma unroll
        for (int j = 0; j < W; ++j) {
          if (ref[j] < 0 && ref[j] != kEmptyRef) {
            const unsigned m = hm[j] & live;
            if (m) {
              bool occ = false;
              if ((m >> lane) & 1u) {
                ++n_tris;
                occ = leaf_test<TEST, true>(ts.tris, ~ref[j], r, w, hit);
              }
              live &= ~__ballot_sync(full, occ);
            }
          }
        }
        // interior children in child order: the first is visited next, the
        // others pushed (popped last first)
        int nxt = -1;
        unsigned nmask = 0;
#pragma unroll
        for (int j = 0; j < W; ++j) {
          if (ref[j] >= 0) {
            const unsigned m = hm[j] & live;
            if (m) {
              if (nxt < 0) {
                nxt = ref[j];
                nmask = m;
              } else if (sp < kStack) {
                stk[sp] = make_int2(ref[j], (int)m);  // every lane, same value
                ++sp;
              } else {
                raise_device_error(err, kDevStackOverflow);
                live = 0;
              }
            }
          }
        }
        if (!live) break;
        if (nxt >= 0) {
          node = nxt;
          mask = nmask;
          continue;
        }
        mask = 0;
        while (sp > 0) {
          --sp;
          const int2 e = stk[sp];
          const unsigned m = (unsigned)e.y & live;
          if (m) {
            node = e.x;
            mask = m;
            break;
          }
        }
      }
    }
    if (act) {
      ++n_rays;
      finish(kk, hit, hit.prim >= 0);
    }
  }
}

// Closest hits of coherent rays (a pixel's camera rays) as masked packets
// over the binary tree, the counterpart of trace_packet_any: each lane tests
// the node's two child boxes against its own ray and current hit, a child
// is visited for the lanes that passed it, and a leaf's triangle is tested
// by exactly those lanes -- a lane never skips a node it would visit alone.
// Of two children the packet takes first the one most of its lanes reach
// first; the other is pushed with the packet's nearest entry distance to
// it, and on the pop a lane whose hit is nearer than that distance (so
// nearer than its own) leaves the entry's lanes.  The packet visits in
// another order than a single ray, so an exact tie at a shared edge (see
// the top of this file) can resolve to the other triangle: the camera-ray
// packets that use it are off by default (AJG_PACKET_CAMERA).
//
// Rays of a multi-job wave carry their scene: FETCH(k, sid) returns the
// ray and its scene index, SCENE(sid, ts) points `ts` at that scene's tree,
// and the warp walks one packet per scene its 32 rays hold (one, in all but
// the warps that straddle two jobs' chunks).
template <int TEST, class FETCH, class FINISH, class SCENE>
__device__ __forceinline__ void trace_packet_closest(
    TraceScene ts0, uint32_t n, uint32_t* next, FETCH fetch, FINISH finish,
    SCENE scene_of, uint32_t& n_rays, uint32_t& n_nodes, uint32_t& n_tris,
    uint32_t* err) {
  constexpr int kStack = StackDepth<2>::value;
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  __shared__ int2 s_cstack[kPacketThreads / 32][kStack];
  __shared__ float s_ctstack[kPacketThreads / 32][kStack];
  int2* const stk = s_cstack[threadIdx.x >> 5];
  float* const stt = s_ctstack[threadIdx.x >> 5];
  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(next, 32u);
    base = __shfl_sync(full, base, 0);
    if (base >= n) break;
    const uint32_t kk = base + (uint32_t)lane;
    const bool act = kk < n;
    uint32_t sid = 0;
    const RayQ r = act ? fetch(kk, sid)
                       : make_query(mk3(0.f, 0.f, 0.f), mk3(0.f, 0.f, 1.f),
                                    0.f, 0.f);
    WtSetup w;
    if (TEST == AJG_TRI_WATERTIGHT) w = wt_setup(r);
    Hit hit;
    hit.t = __int_as_float(0x7f800000);
    hit.prim = -1;
    hit.u = hit.v = 0.f;
    unsigned todo = __ballot_sync(full, act);  // lanes of scenes not walked
    while (todo) {
      const uint32_t s0 = __shfl_sync(full, sid, __ffs(todo) - 1);
      // lanes visiting `node`: the packet of scene s0
      unsigned mask = __ballot_sync(full, ((todo >> lane) & 1u) && sid == s0);
      todo &= ~mask;
      TraceScene ts = ts0;
      scene_of(s0, ts);
      int node = 0, sp = 0;
      uint32_t visits = 0;
      while (mask) {
        if (++visits > ts.max_visits) {
          raise_device_error(err, kDevIterationBound);
          break;
        }
        const bool in = (mask >> lane) & 1u;
        if (in) ++n_nodes;
        float4 n0, n1, n2, n3;
        ldg_node(ts.bvh + 4 * (uint64_t)node, n0, n1);
        ldg_node(ts.bvh + 4 * (uint64_t)node + 2, n2, n3);
        const float lim = fminf(hit.t, r.tmax);
        float tn0 = 0.f, tn1 = 0.f;
        const bool h0 =
            in && slab2(n0.x, n0.y, n0.z, n0.w, n2.x, n2.y, r, lim, tn0);
        const bool h1 =
            in && slab2(n1.x, n1.y, n1.z, n1.w, n2.z, n2.w, r, lim, tn1);
        const int r0 = __float_as_int(n3.x), r1 = __float_as_int(n3.y);
        unsigned m0 = __ballot_sync(full, h0), m1 = __ballot_sync(full, h1);
        if (r0 < 0) {
          if (h0) {
            ++n_tris;
            leaf_test<TEST, false>(ts.tris, ~r0, r, w, hit);
          }
          m0 = 0;
        }
        if (r1 < 0) {
          if (h1) {
            ++n_tris;
            leaf_test<TEST, false>(ts.tris, ~r1, r, w, hit);
          }
          m1 = 0;
        }
        if (m0 && m1) {
          const unsigned both = m0 & m1;
          const unsigned pref0 =
              __ballot_sync(full, ((both >> lane) & 1u) && tn0 <= tn1);
          const bool go0 = 2 * __popc(pref0) >= __popc(both);
          const unsigned far_m = go0 ? m1 : m0;
          float ft = ((far_m >> lane) & 1u) ? (go0 ? tn1 : tn0)
                                            : __int_as_float(0x7f800000);
#pragma unroll
          for (int o = 16; o > 0; o >>= 1)
            ft = fminf(ft, __shfl_xor_sync(full, ft, o));
          if (sp >= kStack) {
            raise_device_error(err, kDevStackOverflow);
            break;
          }
          stk[sp] = make_int2(go0 ? r1 : r0, (int)far_m);  // every lane, same
          stt[sp] = ft;                                    // values
          ++sp;
          node = go0 ? r0 : r1;
          mask = go0 ? m0 : m1;
          continue;
        }
        if (m0 | m1) {
          node = m0 ? r0 : r1;
          mask = m0 | m1;
          continue;
        }
        mask = 0;
        while (sp > 0) {
          --sp;
          const int2 e = stk[sp];
          const float et = stt[sp];
          const unsigned m =
              (unsigned)e.y & __ballot_sync(full, et <= fminf(hit.t, r.tmax));
          if (m) {
            node = e.x;
            mask = m;
            break;
          }
        }
      }
    }
    if (act) {
      ++n_rays;
      finish(kk, hit, hit.prim >= 0);
    }
  }
}

// Calls f(TEST, L) with the triangle test and the tree layout as
// compile-time constants (std::integral_constant), for launching the
// matching kernel.
template <class F, class T>
inline void dispatch_layout(int layout, F&& f, T test) {
  using L2 = std::integral_constant<int, 2>;
  using L4 = std::integral_constant<int, 4>;
  using L8 = std::integral_constant<int, 8>;
  using C4 = std::integral_constant<int, 4 | (int)kBvhCompressed>;
  using C8 = std::integral_constant<int, 8 | (int)kBvhCompressed>;
  switch (layout) {
    case 4: f(test, L4{}); break;
    case 8: f(test, L8{}); break;
    case 4 | (int)kBvhCompressed: f(test, C4{}); break;
    case 8 | (int)kBvhCompressed: f(test, C8{}); break;
    default: f(test, L2{}); break;
  }
}
template <class F>
inline void dispatch_trace(int tri_test, int layout, F&& f) {
  if (tri_test == AJG_TRI_WATERTIGHT)
    dispatch_layout(layout, f,
                    std::integral_constant<int, AJG_TRI_WATERTIGHT>{});
  else
    dispatch_layout(layout, f,
                    std::integral_constant<int, AJG_TRI_MOLLER_TRUMBORE>{});
}

__device__ __forceinline__ void flush_counters(TraceCounters* c, uint32_t rays,
                                               uint32_t nodes, uint32_t tris) {
  if (!c) return;
  unsigned long long a = rays, b = nodes, t = tris;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
    t += __shfl_down_sync(0xffffffffu, t, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&c->rays, a);
    atomicAdd(&c->nodes, b);
    atomicAdd(&c->tris, t);
  }
}

}  // namespace ajg
