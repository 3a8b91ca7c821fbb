// Device-resident scene and the host objects behind the C ABI handles.
#pragma once
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"

namespace ajg {

// HBM layout of a built scene (all arrays are device pointers):
//   bvh    [inner][4] float4  two child boxes per interior node:
//          (c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y), (c1 ... same),
//          (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z), (ref0, ref1, -, -) where a
//          ref >= 0 is an interior node and ~slot a leaf
//   tris   [slots][3] float4  vertices a, b, c of the triangle in each leaf
//          slot (Morton order); a.w carries the primitive index
//   shade  [n] float4         per primitive: geometric normal, w = material |
//          flags << 24
//   corner [n][9] float       per-corner shading normals (HAS_NORMALS only)
struct DeviceScene {
  const float4* bvh = nullptr;
  const float4* tris = nullptr;
  const float4* shade = nullptr;
  const float* corner = nullptr;
  const float* materials = nullptr;  // [m][16]
  const float* lights = nullptr;     // [l][12]; env records carry in [10]
                                     // "sampling has mass" and in [11]
                                     // "pdf is nonzero" (1x1 Distribution2D)
  float4* mat_lum = nullptr;         // [m]: luminance of base colour
  uint64_t n = 0;
  uint32_t num_inner = 0;
  uint32_t num_materials = 0;
  uint32_t num_lights = 0;
  int32_t env = -1;      // the scene's environment light (the last one)
  float radius = 0.f;    // (world.max - world.center).length()
  int32_t tri_test = 0;
};

// Counters the traversal kernels accumulate (algorithmic bytes for the
// roofline: nodes * 64 B + triangles * 48 B).
struct TraceCounters {
  unsigned long long rays;
  unsigned long long nodes;
  unsigned long long tris;
};

struct Buffer {
  void* ptr = nullptr;
  size_t bytes = 0;
};

// Event pairs recorded around launches while profiling is on; resolved into
// milliseconds when the stats are read.
enum KernelKind { kKindClosest = 0, kKindAny = 1, kKindShade = 2, kKinds = 3 };
struct PendingTiming {
  cudaEvent_t a, b;
  int kind;
};

}  // namespace ajg

struct ajg_ctx {
  int device = 0;
  uint32_t wave_paths = 1u << 22;
  uint64_t hbm_budget = 0;
  uint64_t resident_bytes = 0;
  cudaStream_t stream = nullptr;
  std::mutex mu;
  std::string last_error;
  uint32_t* d_error = nullptr;            // device error flag
  uint32_t* d_fetch = nullptr;            // ray counter of query launches
  ajg::TraceCounters* d_counters = nullptr;  // [2]: closest, any
  unsigned long long paths_total = 0;
  unsigned long long kernel_launches = 0;
  bool profiling = false;
  std::vector<ajg::PendingTiming> pending;
  double kind_ms[ajg::kKinds] = {0, 0, 0};
  unsigned long long kind_launches[ajg::kKinds] = {0, 0, 0};
  // wavefront arena (grown on demand, reused across renders)
  std::vector<ajg::Buffer> arena;
  uint64_t arena_paths = 0;
};

struct ajg_scene {
  ajg_ctx* ctx = nullptr;
  ajg::DeviceScene d;
  std::vector<void*> allocations;
  // the tree in the reference layout, kept for download
  float4* ploc_nodes = nullptr;  // [2n-1][2]
  int32_t* perm = nullptr;       // [n]
  ajg_scene_info info{};
  std::vector<float> host_lights;
  std::vector<float> host_materials;
};

namespace ajg {
// Brackets one launch of a given kind with events when profiling.
struct KernelTimer {
  ajg_ctx* ctx;
  cudaStream_t st;
  int kind;
  cudaEvent_t a = nullptr, b = nullptr;
  KernelTimer(ajg_ctx* c, cudaStream_t s, int k) : ctx(c), st(s), kind(k) {
    ++ctx->kernel_launches;
    if (kind >= 0) ++ctx->kind_launches[kind];
    if (ctx->profiling && kind >= 0) {
      cudaEventCreate(&a);
      cudaEventCreate(&b);
      cudaEventRecord(a, st);
    }
  }
  ~KernelTimer() {
    if (a) {
      cudaEventRecord(b, st);
      ctx->pending.push_back(PendingTiming{a, b, kind});
    }
  }
};
// ploc.cu
int build_scene(ajg_ctx* ctx, ajg_scene* s, const float* h_tris,
                const float* h_corner, const int32_t* h_mat,
                const int32_t* h_flags, uint64_t n, const float* world,
                const ajg_scene_opts& opts);
// integrator.cu
int render_impl(ajg_scene* sc, const ajg_camera& cam,
                const ajg_render_params& prm, float4* d_out,
                uint64_t li_begin, uint64_t li_end, float* d_li,
                cudaStream_t st);
// The same render over caller-provided scratch (film accumulators first,
// then one wave); allocates nothing.  Runs on `st`; no profiling events.
int render_in_scratch(ajg_scene* sc, const ajg_camera& cam,
                      const ajg_render_params& prm, float4* d_out,
                      cudaStream_t st, char* scratch, uint64_t bytes);
// trace.cu
void launch_trace_closest(const DeviceScene& s, const ajg_ray* rays,
                          uint64_t n, ajg_hit* hits, uint32_t* next,
                          TraceCounters* ctr, uint32_t* err, cudaStream_t st);
void launch_trace_any(const DeviceScene& s, const ajg_ray* rays, uint64_t n,
                      uint8_t* occluded, uint32_t* next, TraceCounters* ctr,
                      uint32_t* err, cudaStream_t st);
}  // namespace ajg
