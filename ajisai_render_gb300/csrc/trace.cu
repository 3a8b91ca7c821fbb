// Ray-query kernels behind ajg_trace_closest / ajg_trace_any: one thread
// per ray, grid-stride over the batch.
#include "trace.cuh"

namespace ajg {
namespace {

constexpr int kTraceThreads = 128;

template <int TEST, int W>
__global__ void __launch_bounds__(kTraceThreads, trace_min_blocks<W>())
    k_trace_closest(DeviceScene s, const ajg_ray* __restrict__ rays,
                    uint64_t n, uint32_t* next, ajg_hit* __restrict__ hits,
                    TraceCounters* ctr, uint32_t* err) {
  uint32_t nn = 0, nt = 0, nr = 0;
  auto fetch = [&](uint32_t i, TraceScene&) {
    const ajg_ray q = rays[i];
    return make_query(mk3(q.o[0], q.o[1], q.o[2]), mk3(q.d[0], q.d[1], q.d[2]),
                      q.t_min, q.t_max);
  };
  auto finish = [&](uint32_t i, const Hit& h, bool) {
    ajg_hit o;
    o.t = h.t;
    o.u = h.u;
    o.v = h.v;
    o.prim = h.prim;
    hits[i] = o;
  };
  trace_persistent<TEST, false, W>(trace_scene(s), (uint32_t)n, next, fetch,
                                   finish, nr, nn, nt, err);
  flush_counters(ctr, nr, nn, nt);
}

template <int TEST, int W>
__global__ void __launch_bounds__(kTraceThreads, trace_min_blocks<W>())
    k_trace_any(DeviceScene s, const ajg_ray* __restrict__ rays, uint64_t n,
                uint32_t* next, uint8_t* __restrict__ occ, TraceCounters* ctr,
                uint32_t* err) {
  uint32_t nn = 0, nt = 0, nr = 0;
  auto fetch = [&](uint32_t i, TraceScene&) {
    const ajg_ray q = rays[i];
    return make_query(mk3(q.o[0], q.o[1], q.o[2]), mk3(q.d[0], q.d[1], q.d[2]),
                      q.t_min, q.t_max);
  };
  auto finish = [&](uint32_t i, const Hit&, bool o) { occ[i] = o ? 1 : 0; };
  trace_persistent<TEST, true, W>(trace_scene(s), (uint32_t)n, next, fetch,
                                  finish, nr, nn, nt, err);
  flush_counters(ctr, nr, nn, nt);
}

}  // namespace

// `next` is a zeroed device word (the persistent lanes' ray counter).
void launch_trace_closest(const DeviceScene& s, const ajg_ray* rays,
                          uint64_t n, ajg_hit* hits, uint32_t* next,
                          TraceCounters* ctr, uint32_t* err, cudaStream_t st) {
  if (!n) return;
  const int g = grid_for(n, kTraceThreads, kSMs * 10);
  dispatch_trace(s.tri_test, s.width, [&](auto T, auto W) {
    k_trace_closest<decltype(T)::value, decltype(W)::value>
        <<<g, kTraceThreads, 0, st>>>(s, rays, n, next, hits, ctr, err);
  });
}

void launch_trace_any(const DeviceScene& s, const ajg_ray* rays, uint64_t n,
                      uint8_t* occluded, uint32_t* next, TraceCounters* ctr,
                      uint32_t* err, cudaStream_t st) {
  if (!n) return;
  const int g = grid_for(n, kTraceThreads, kSMs * 10);
  dispatch_trace(s.tri_test, s.width, [&](auto T, auto W) {
    k_trace_any<decltype(T)::value, decltype(W)::value>
        <<<g, kTraceThreads, 0, st>>>(s, rays, n, next, occluded, ctr, err);
  });
}

}  // namespace ajg
