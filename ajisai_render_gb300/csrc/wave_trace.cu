// Traversal kernels of the path waves: closest hits of a path queue
// (k_extend), any hits of the shadow queue (k_shadow) and closest hits of
// the MIS BSDF rays of scenes with emitters (k_bsdf_trace), each in a
// single-job form and a multi-job form whose rays carry their scene index;
// and the packet traversals of bounce 0's directional-light shadow rays
// (k_shadow_packet) and, on request, camera rays (k_extend_packet).
// A translation unit of its own: the traversal's arithmetic (the slab and
// triangle tests) must not be contracted into multiply-adds, so that hits
// stay bit-exact, while the shading kernels may be built with contraction.
#include "trace.cuh"

namespace ajg {
namespace {

constexpr int kTraceThreads = 128;
#ifndef AJG_PACKET_MIN_BLOCKS
#define AJG_PACKET_MIN_BLOCKS 8  // blocks of 128 per SM the packet kernels
                                 // are compiled for (64 registers)
#endif

// The tree of the ray's scene; closest-hit kernels of the binary layout
// (W = 2) take the binary tree a 4-wide scene keeps beside its wide one.
template <int W>
__device__ __forceinline__ void retarget(TraceScene& ts, const MJTables& t,
                                         uint32_t sid) {
  const DeviceScene& sc = t.scenes[mj_scene(t, sid)];
  if (W == 2 && sc.bvh_closest) {
    ts.bvh = sc.bvh_closest;
    ts.max_visits = sc.num_inner_closest + 1;
  } else {
    ts.bvh = sc.bvh;
    ts.max_visits = sc.num_inner + 1;
  }
  ts.tris = sc.tris;
}

// Closest hits of the path queue.
template <int TEST, bool MJ, int W>
__global__ void __launch_bounds__(kTraceThreads, trace_min_blocks<W>())
    k_extend(DeviceScene s, MJTables t, const float4* __restrict__ ro,
             const float4* __restrict__ rd, const uint32_t* __restrict__ count,
             uint32_t* fetch_next, ajg_hit* __restrict__ hits,
             TraceCounters* ctr, uint32_t* err) {
  const uint32_t n = *count;
  uint32_t nn = 0, nt = 0, nr = 0;
  auto fetch = [&](uint32_t k, TraceScene& ts) {
    const float4 o = ro[k], d = rd[k];
    if constexpr (MJ) retarget<W>(ts, t, __float_as_uint(o.w));
    return make_query(xyz(o), xyz(d), kRayEps, __int_as_float(0x7f800000));
  };
  auto finish = [&](uint32_t k, const Hit& h, bool) {
    ajg_hit o2;
    o2.t = h.t;
    o2.u = h.u;
    o2.v = h.v;
    o2.prim = h.prim;
    hits[k] = o2;
  };
  trace_persistent<TEST, false, W>(trace_scene(s), n, fetch_next, fetch,
                                   finish, nr, nn, nt, err);
  flush_counters(ctr, nr, nn, nt);
}

template <int TEST, bool MJ, int W>
__global__ void __launch_bounds__(kTraceThreads, trace_min_blocks<W>())
    k_shadow(DeviceScene s, MJTables t, const float4* __restrict__ sq_o,
             const float4* __restrict__ sq_d,
             const uint16_t* __restrict__ sq_scene,
             const uint32_t* __restrict__ count, uint32_t* fetch_next,
             uint8_t* __restrict__ vis, TraceCounters* ctr, uint32_t* err) {
  const uint32_t n = *count;
  uint32_t nn = 0, nt = 0, nr = 0;
  // the queue entry of the lane's current ray (a lane traces one at a time)
  uint32_t cur = 0;
  auto fetch = [&](uint32_t k, TraceScene& ts) {
    cur = k;
    const float4 o = sq_o[cur], d = sq_d[cur];
    if constexpr (MJ) retarget<W>(ts, t, sq_scene[cur]);
    return make_query(xyz(o), xyz(d), kRayEps, o.w);
  };
  auto finish = [&](uint32_t, const Hit&, bool occ) {
    if (!occ) vis[__float_as_uint(sq_d[cur].w)] = 1;
  };
  trace_persistent<TEST, true, W>(trace_scene(s), n, fetch_next, fetch,
                                  finish, nr, nn, nt, err);
  flush_counters(ctr, nr, nn, nt);
}

// Closest hits of bounce 0's camera rays (a pixel's samples side by side in
// the path queue) as masked packets over the binary layout; in multi-job
// waves a packet per scene the warp's rays hold.
template <int TEST, bool MJ>
__global__ void __launch_bounds__(kPacketThreads, AJG_PACKET_MIN_BLOCKS)
    k_extend_packet(DeviceScene s, MJTables t, const float4* __restrict__ ro,
                    const float4* __restrict__ rd,
                    const uint32_t* __restrict__ count, uint32_t* fetch_next,
                    ajg_hit* __restrict__ hits, TraceCounters* ctr,
                    uint32_t* err) {
  const uint32_t n = *count;
  uint32_t nn = 0, nt = 0, nr = 0;
  auto fetch = [&](uint32_t k, uint32_t& sid) {
    const float4 o = ro[k], d = rd[k];
    if constexpr (MJ) sid = __float_as_uint(o.w);
    return make_query(xyz(o), xyz(d), kRayEps, __int_as_float(0x7f800000));
  };
  auto scene_of = [&](uint32_t sid, TraceScene& ts) {
    if constexpr (MJ) retarget<2>(ts, t, sid);
  };
  auto finish = [&](uint32_t k, const Hit& h, bool) {
    ajg_hit o2;
    o2.t = h.t;
    o2.u = h.u;
    o2.v = h.v;
    o2.prim = h.prim;
    hits[k] = o2;
  };
  trace_packet_closest<TEST>(trace_scene(s), n, fetch_next, fetch, finish,
                             scene_of, nr, nn, nt, err);
  flush_counters(ctr, nr, nn, nt);
}

// Any hits of bounce 0's coherent shadow rays (the queue at the top of the
// shadow queue's storage: entry k at cap - 1 - k) as masked packets over the
// plain 4-wide tree; in multi-job waves a packet per scene the warp's rays
// hold.
template <int TEST, bool MJ>
__global__ void __launch_bounds__(kPacketThreads, AJG_PACKET_MIN_BLOCKS)
    k_shadow_packet(DeviceScene s, MJTables t, const float4* __restrict__ sq_o,
                    const float4* __restrict__ sq_d,
                    const uint16_t* __restrict__ sq_scene,
                    const uint32_t* __restrict__ count, uint32_t* fetch_next,
                    uint32_t cap, uint8_t* __restrict__ vis,
                    TraceCounters* ctr, uint32_t* err) {
  const uint32_t n = min(*count, cap);
  uint32_t nn = 0, nt = 0, nr = 0;
  auto fetch = [&](uint32_t k, uint32_t& sid) {
    const uint32_t i = cap - 1 - k;
    const float4 o = sq_o[i], d = sq_d[i];
    if constexpr (MJ) sid = sq_scene[i];
    return make_query(xyz(o), xyz(d), kRayEps, o.w);
  };
  auto scene_of = [&](uint32_t sid, TraceScene& ts) {
    if constexpr (MJ) retarget<4>(ts, t, sid);
  };
  auto finish = [&](uint32_t k, const Hit&, bool occ) {
    if (!occ) vis[__float_as_uint(sq_d[cap - 1 - k].w)] = 1;
  };
  trace_packet_any<TEST>(trace_scene(s), n, fetch_next, fetch, finish,
                         scene_of, nr, nn, nt, err);
  flush_counters(ctr, nr, nn, nt);
}

// Closest hits of the MIS BSDF rays of scenes with emitters (the queue at
// the top of the shadow queue's storage, see emit_closest); t and the
// primitive go to two arrays the material lists' storage lends.
template <int TEST, bool MJ, int W>
__global__ void __launch_bounds__(kTraceThreads, trace_min_blocks<W>())
    k_bsdf_trace(DeviceScene s, MJTables t, const float4* __restrict__ sq_o,
                 const float4* __restrict__ sq_d,
                 const uint16_t* __restrict__ sq_scene,
                 const uint32_t* __restrict__ count, uint32_t* fetch_next,
                 uint32_t cap, uint32_t n_max, float* __restrict__ t_hit,
                 int32_t* __restrict__ prim_hit, TraceCounters* ctr,
                 uint32_t* err) {
  // at most one entry per path (n_max = paths of the arena)
  const uint32_t n = min(*count, n_max);
  uint32_t nn = 0, nt = 0, nr = 0;
  auto fetch = [&](uint32_t k, TraceScene& ts) {
    const uint32_t i = cap - 1 - k;
    const float4 o = sq_o[i], d = sq_d[i];
    if constexpr (MJ) retarget<W>(ts, t, sq_scene[i]);
    return make_query(xyz(o), xyz(d), kRayEps, __int_as_float(0x7f800000));
  };
  auto finish = [&](uint32_t k, const Hit& h, bool) {
    t_hit[k] = h.t;
    prim_hit[k] = h.prim;
  };
  trace_persistent<TEST, false, W>(trace_scene(s), n, fetch_next, fetch,
                                   finish, nr, nn, nt, err);
  flush_counters(ctr, nr, nn, nt);
}

}  // namespace

void launch_wave_extend(bool mj, int tri_test, int width, const DeviceScene& s,
                        const MJTables& t, const float4* ro, const float4* rd,
                        const uint32_t* count, uint32_t* fetch_next,
                        ajg_hit* hits, TraceCounters* ctr, uint32_t* err,
                        cudaStream_t st) {
  dispatch_trace(tri_test, width, [&](auto T, auto Wd) {
    constexpr int TT = decltype(T)::value, WW = decltype(Wd)::value;
    if (mj) {
      const int g = resident_grid((const void*)k_extend<TT, true, WW>, kTraceThreads);
      k_extend<TT, true, WW><<<g, kTraceThreads, 0, st>>>(
          s, t, ro, rd, count, fetch_next, hits, ctr, err);
    } else {
      const int g = resident_grid((const void*)k_extend<TT, false, WW>, kTraceThreads);
      k_extend<TT, false, WW><<<g, kTraceThreads, 0, st>>>(
          s, t, ro, rd, count, fetch_next, hits, ctr, err);
    }
  });
}

void launch_wave_shadow(bool mj, int tri_test, int width, const DeviceScene& s,
                        const MJTables& t, const float4* sq_o,
                        const float4* sq_d, const uint16_t* sq_scene,
                        const uint32_t* count, uint32_t* fetch_next,
                        uint8_t* vis, TraceCounters* ctr, uint32_t* err,
                        cudaStream_t st) {
  dispatch_trace(tri_test, width, [&](auto T, auto Wd) {
    constexpr int TT = decltype(T)::value, WW = decltype(Wd)::value;
    if (mj) {
      const int g = resident_grid((const void*)k_shadow<TT, true, WW>, kTraceThreads);
      k_shadow<TT, true, WW><<<g, kTraceThreads, 0, st>>>(
          s, t, sq_o, sq_d, sq_scene, count, fetch_next, vis, ctr, err);
    } else {
      const int g = resident_grid((const void*)k_shadow<TT, false, WW>, kTraceThreads);
      k_shadow<TT, false, WW><<<g, kTraceThreads, 0, st>>>(
          s, t, sq_o, sq_d, sq_scene, count, fetch_next, vis, ctr, err);
    }
  });
}

void launch_wave_extend_packet(bool mj, int tri_test, const DeviceScene& s,
                               const MJTables& t, const float4* ro,
                               const float4* rd, const uint32_t* count,
                               uint32_t* fetch_next, ajg_hit* hits,
                               TraceCounters* ctr, uint32_t* err,
                               cudaStream_t st) {
  auto go = [&](auto T, auto M) {
    constexpr int TT = decltype(T)::value;
    constexpr bool MM = decltype(M)::value;
    const int g = resident_grid((const void*)k_extend_packet<TT, MM>, kPacketThreads);
    k_extend_packet<TT, MM><<<g, kPacketThreads, 0, st>>>(
        s, t, ro, rd, count, fetch_next, hits, ctr, err);
  };
  using WT = std::integral_constant<int, AJG_TRI_WATERTIGHT>;
  using MT = std::integral_constant<int, AJG_TRI_MOLLER_TRUMBORE>;
  if (tri_test == AJG_TRI_WATERTIGHT) {
    if (mj)
      go(WT{}, std::true_type{});
    else
      go(WT{}, std::false_type{});
  } else {
    if (mj)
      go(MT{}, std::true_type{});
    else
      go(MT{}, std::false_type{});
  }
}

void launch_wave_shadow_packet(bool mj, int tri_test, const DeviceScene& s,
                               const MJTables& t, const float4* sq_o,
                               const float4* sq_d, const uint16_t* sq_scene,
                               const uint32_t* count, uint32_t* fetch_next,
                               uint32_t cap, uint8_t* vis, TraceCounters* ctr,
                               uint32_t* err, cudaStream_t st) {
  auto go = [&](auto T, auto M) {
    constexpr int TT = decltype(T)::value;
    constexpr bool MM = decltype(M)::value;
    const int g = resident_grid((const void*)k_shadow_packet<TT, MM>, kPacketThreads);
    k_shadow_packet<TT, MM><<<g, kPacketThreads, 0, st>>>(
        s, t, sq_o, sq_d, sq_scene, count, fetch_next, cap, vis, ctr, err);
  };
  using WT = std::integral_constant<int, AJG_TRI_WATERTIGHT>;
  using MT = std::integral_constant<int, AJG_TRI_MOLLER_TRUMBORE>;
  if (tri_test == AJG_TRI_WATERTIGHT) {
    if (mj)
      go(WT{}, std::true_type{});
    else
      go(WT{}, std::false_type{});
  } else {
    if (mj)
      go(MT{}, std::true_type{});
    else
      go(MT{}, std::false_type{});
  }
}

void launch_wave_bsdf_trace(bool mj, int tri_test, int width,
                            const DeviceScene& s, const MJTables& t,
                            const float4* sq_o, const float4* sq_d,
                            const uint16_t* sq_scene, const uint32_t* count,
                            uint32_t* fetch_next, uint32_t cap, uint32_t n_max,
                            float* t_hit, int32_t* prim_hit,
                            TraceCounters* ctr, uint32_t* err, cudaStream_t st) {
  dispatch_trace(tri_test, width, [&](auto T, auto Wd) {
    constexpr int TT = decltype(T)::value, WW = decltype(Wd)::value;
    if (mj) {
      const int g =
          resident_grid((const void*)k_bsdf_trace<TT, true, WW>, kTraceThreads);
      k_bsdf_trace<TT, true, WW><<<g, kTraceThreads, 0, st>>>(
          s, t, sq_o, sq_d, sq_scene, count, fetch_next, cap, n_max, t_hit,
          prim_hit, ctr, err);
    } else {
      const int g =
          resident_grid((const void*)k_bsdf_trace<TT, false, WW>, kTraceThreads);
      k_bsdf_trace<TT, false, WW><<<g, kTraceThreads, 0, st>>>(
          s, t, sq_o, sq_d, sq_scene, count, fetch_next, cap, n_max, t_hit,
          prim_hit, ctr, err);
    }
  });
}

void prepare_mj_kernels() {
  for (int tt = 0; tt < 2; ++tt)
    for (int wd : {2, 4, 8, 4 | (int)kBvhCompressed, 8 | (int)kBvhCompressed})
      dispatch_trace(tt, wd, [&](auto T, auto Wd) {
        constexpr int TT = decltype(T)::value, WW = decltype(Wd)::value;
        resident_grid((const void*)k_extend<TT, true, WW>, kTraceThreads);
        resident_grid((const void*)k_shadow<TT, true, WW>, kTraceThreads);
        resident_grid((const void*)k_bsdf_trace<TT, true, WW>, kTraceThreads);
      });
  resident_grid((const void*)k_extend_packet<AJG_TRI_MOLLER_TRUMBORE, true>,
                kPacketThreads);
  resident_grid((const void*)k_extend_packet<AJG_TRI_WATERTIGHT, true>,
                kPacketThreads);
  resident_grid((const void*)k_shadow_packet<AJG_TRI_MOLLER_TRUMBORE, true>,
                kPacketThreads);
  resident_grid((const void*)k_shadow_packet<AJG_TRI_WATERTIGHT, true>,
                kPacketThreads);
}

}  // namespace ajg
