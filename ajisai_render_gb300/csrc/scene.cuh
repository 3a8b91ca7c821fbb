// Device-resident scene and the host objects behind the C ABI handles.
#pragma once
#include <atomic>
#include <chrono>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"

namespace ajg {

// HBM layout of a built scene (all arrays are device pointers):
//   bvh    width 2: [inner][4] float4, two child boxes per interior node:
//          (c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y), (c1 ... same),
//          (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z), (ref0, ref1, -, -) where a
//          ref >= 0 is an interior node and ~slot a leaf;
//          width W = 4, 8: [nodes][2W] float4 of the collapsed tree (see
//          k_collapse in ploc.cu)
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
  int32_t width = 2;     // layout of `bvh`: 2 (binary PLOC tree), 4, 8, or
                         // 4 / 8 | kBvhCompressed
  // area lights (emissive primitives): the first num_area light records
  // (kLightArea), the corner points their samplers read, and per triangle
  // (indexed like `shade`) the light it emits as, or -1; all null / 0 in a
  // scene without emitters
  const int32_t* tri_emit = nullptr;
  const float* emit_pts = nullptr;  // [k][3]
  uint32_t num_area = 0;
  uint32_t mat_mask = 0;  // bit t: a material of type t is present
  // the binary layout of the same tree kept beside a plain 4-wide one for
  // the closest-hit traversal (null for other layouts and with
  // AJG_HYBRID_CLOSEST=0)
  const float4* bvh_closest = nullptr;
  uint32_t num_inner_closest = 0;
  // kPacketSpread times the scene's median triangle edge: a render traces
  // bounce 0's directional-light shadow rays as packets when a pixel's
  // footprint at the scene is within it
  float packet_spread = 0.f;
};
#ifndef AJG_PACKET_SPREAD
#define AJG_PACKET_SPREAD 4.0f
#endif
constexpr float kPacketSpread = AJG_PACKET_SPREAD;

// Closest-hit rays walk the binary layout of the tree, any-hit rays the
// 4-wide one, when the scene keeps both (the default for the 4-wide tree):
// measured on the single-job workload, closest-hit traversal is faster over
// the binary nodes (nearest child first, tighter culling by the current
// hit) and any-hit traversal over the wide ones.
#ifndef AJG_HYBRID_CLOSEST
#define AJG_HYBRID_CLOSEST 1
#endif
constexpr bool kHybridClosest = AJG_HYBRID_CLOSEST != 0;
// The layout closest-hit launches use for scenes of layout `width`.
inline int closest_width(int width) {
  return kHybridClosest && width == 4 ? 2 : width;
}

// The scene as the closest-hit launches see it: the binary layout where
// the build kept one beside the wide tree.
inline DeviceScene closest_view(const DeviceScene& s) {
  DeviceScene c = s;
  if (s.bvh_closest) {
    c.bvh = s.bvh_closest;
    c.num_inner = s.num_inner_closest;
    c.width = 2;
  }
  return c;
}

// Light record types ([12] floats, type in [0]): the two of the ABI, and the
// area light of an emissive primitive:
//   [1..3] radiance, [4] geometry (AJG_GEOM_*), [5] two-sided,
//   [6] triangles (uint bits), [7] 1 / area, [8] the quad's (a,b,c) share of
//   its area, [9] Geometry::Pdf (the same for every point of the surface),
//   [10] first corner in emit_pts (uint bits)
constexpr int kLightArea = 2;

// Per-job constants of the integrator, shared by the single-job and the
// multi-job waves.  The film of a job covers the window (x0, y0, win_w,
// win_h) of a film_w x film_h image; the sampler keys by the image pixel
// y * film_w + x, so a window renders exactly the samples the whole image
// would render there.
struct JobParams {
  uint64_t seed;
  int32_t min_b, max_b;
  float cont;
  int32_t use_mis;
  int32_t nd;   // sampler draws per bounce without the roulette draw
  int32_t nl;   // lights of the job's scene
  float4 env_rgb;  // scaler * texel of the scene's env light
  int32_t env_mass;  // the env light's Distribution2D::Pdf is nonzero
  int32_t drop_nonfinite;
  uint32_t film_w, film_h;
  uint32_t x0, y0, win_w, win_h;
  int32_t packets;  // bounce 0's directional-light shadow rays as packets
  int32_t pad;
};

// SPPM's visible point (TracerVP's result, sppm.cpp:77-92): the hit, its
// throughput and what EvalAll needs there; pos.w carries the material
// index bits, 0xffffffff for a pixel without one.
struct VisPointD {
  float4 pos, wr, thr, ng, ns;
};
constexpr uint32_t kNoVisPoint = 0xffffffffu;

// Device record of a job in a multi-job wave.
struct JobRec {
  JobParams j;
  ajg_camera cam;
  uint32_t scene;  // index into the wave's scene table
  uint32_t pad;
  float4* fsum;    // film (window-sized): float32 sum + Kahan compensation
  float4* fcomp;
  double* fsum64;  // or a float64 sum
};

// One job's share of a wave: window pixels [pix0, pix0 + n_pix), samples
// [s0, s0 + S) each; its paths are [path_off, path_off + n_pix * S) of the
// wave (pixel-major) and its pixels [pix_off, pix_off + n_pix) of the
// wave's film pass.
struct Chunk {
  uint32_t job, pix0, n_pix, S, s0, path_off, pix_off, pad;
};

// Header of the per-wave tables in device memory.
struct WaveHeader {
  uint32_t n_chunks, n_paths, n_pix, n_jobs;
  // bounds the multi-job kernels check every table index against: the
  // scene table's entries and the wave arena's paths
  uint32_t n_scenes, cap_paths, pad0, pad1;
};

constexpr int kMaxWaveChunks = 1024;

// Device state of one wave (carved from a wave arena).
struct WaveBufs {
  // by path
  float4* thr;
  float4* thr_shade;
  float4* rad;
  uint32_t* pjob;  // multi-job waves: the path's job
  uint64_t* pkey;  // multi-job waves: the path's sampler key
  // by queue slot (double buffered); ro.w carries the scene index in
  // multi-job waves
  uint32_t* qpath[2];
  float4* ro[2];
  float4* rd[2];
  ajg_hit* hits;
  ajg_hit* hits2;  // single-job waves: bounce parity 1's hits (overlap)
  // light terms: slot = path * NT + term (lights first, the MIS BSDF term
  // last at NT - 1)
  float4* term_f;
  uint8_t* term_vis;
  float4* sq_o;  // shadow queue: o.xyz, t_max
  float4* sq_d;  // d.xyz, slot bits
  uint16_t* sq_scene;  // multi-job waves: scene index per shadow ray
  uint32_t* lists;   // [4][P]: queue slots of misses, Lambertian, Disney
                     // and other hits
  uint32_t* counts;  // [0],[1] path queues, [2] shadow queue, [3] shadow
                     // fetch, [4..7] lists, [8] extend fetch, [9] closest
                     // MIS BSDF queue, [10] its fetch, [11] coherent shadow
                     // queue (single jobs without emitters), [12] its fetch
};

// Tables of a multi-job wave in device memory.
struct MJTables {
  const DeviceScene* scenes;
  const JobRec* jobs;
  const Chunk* chunks;
  const WaveHeader* hdr;
  uint32_t* err;  // the request loop's device error word
};

// Multi-job table guards: a job or scene index past its table records
// kDevTableOutOfBounds in the request loop's error word (the wave's jobs
// then fail with AJG_ERR_DEVICE) and is replaced by 0, so that no read
// leaves the tables the host uploaded for the wave.
__device__ __forceinline__ uint32_t mj_job(const MJTables& t, uint32_t jid) {
  if (jid < t.hdr->n_jobs) return jid;
  raise_device_error(t.err, kDevTableOutOfBounds);
  return 0;
}
__device__ __forceinline__ uint32_t mj_scene(const MJTables& t, uint32_t sid) {
  if (sid < t.hdr->n_scenes) return sid;
  raise_device_error(t.err, kDevTableOutOfBounds);
  return 0;
}
// A wave whose header is out of range (more chunks than the kernels'
// shared offset tables hold, or more paths than the arena) runs nothing.
__device__ __forceinline__ bool mj_wave_ok(const MJTables& t) {
  const WaveHeader& h = *t.hdr;
  if (h.n_chunks <= (uint32_t)kMaxWaveChunks && h.n_jobs <= (uint32_t)kMaxWaveChunks &&
      h.n_scenes <= (uint32_t)kMaxWaveChunks && h.n_paths <= h.cap_paths)
    return true;
  if (blockIdx.x == 0 && threadIdx.x == 0)
    raise_device_error(t.err, kDevTableOutOfBounds);
  return false;
}

// Compressed wide nodes (bvh_width W | kBvhCompressed, W = 4 or 8; 80 bytes
// for W = 8, 64 for W = 4):
//   float4 0: node origin (lo corner of the children's union), and
//             e_x | e_y << 8 | e_z << 16 | imask << 24 (e biased by 127)
//   float4 1: child_base, tri_base, vmask (uint bits)
//   then six planes (lo.x, hi.x, lo.y, hi.y, lo.z, hi.z) of W bytes each
// Child c is valid when vmask bit c is set; an interior child is the wide
// node child_base + (interior children before c), a leaf the triangle
// tri_base + (leaf children before c).  A plane decodes as
// origin + q * 2^e with exactly one rounding (cw_decode); the build picks q
// so that the decoded box contains the child's box, so the box test stays
// conservative and the hits are the same as over the binary tree.
constexpr uint32_t kBvhCompressed = 0x100;
template <int W>
struct CwLayout {
  static constexpr int kFloat4 = (32 + 6 * W + 15) / 16;
};
__device__ __forceinline__ float cw_scale(uint32_t eb) {
  return __uint_as_float(eb << 23);
}
__device__ __forceinline__ float cw_qfloat(uint32_t q_bits) {
  // q_bits = 0x4B000000 | q: the float 2^23 + q, minus 2^23 is exactly q
  return __uint_as_float(q_bits) - 8388608.f;
}
__device__ __forceinline__ float cw_decode(float origin, float fq,
                                           float scale) {
  return origin + fq * scale;
}

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
// Launch kinds of the profiling log; the packet traversals count their
// rays in the closest-hit (kKindClosestPacket) and any-hit (kKindAnyPacket)
// counters.
enum KernelKind {
  kKindClosest = 0,
  kKindAny = 1,
  kKindShade = 2,
  kKindAnyPacket = 3,
  kKindClosestPacket = 4,
  kKinds = 5
};
// The traversal counters (ajg_ctx::d_counters) a launch kind adds to.
inline int counter_slot(int kind) {
  return kind == kKindAnyPacket ? kKindAny
         : kind == kKindClosestPacket ? kKindClosest
                                      : kind;
}
struct PendingTiming {
  cudaEvent_t a, b;
  int kind;
  int64_t snap;  // the traversal counters' snapshot after it (-1: none)
};
constexpr int kLaunchLogCap = 65536;

}  // namespace ajg

namespace ajg {
struct Server;
}

struct ajg_ctx {
  int device = 0;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  ajg::Server* server = nullptr;  // the request loop, started on first use
  std::mutex server_mu;
  // paths in flight per single-job wave: big enough that the persistent
  // traversal launches are long against their drain (a render takes no
  // more than it needs, and at most 48 GB of wave state)
  uint32_t wave_paths = 1u << 28;
  uint64_t hbm_budget = 0;
  uint64_t resident_bytes = 0;
  cudaStream_t stream = nullptr;
  // single-job waves trace bounce b+1's closest hits on trace_stream while
  // bounce b's shadow rays run on the render's stream (ev_queue: the next
  // queue is written; ev_hits: its hits are); AJG_TRACE_OVERLAP=0 keeps one
  // stream
  cudaStream_t trace_stream = nullptr;
  cudaEvent_t ev_queue = nullptr, ev_hits = nullptr;
  bool overlap = true;
  // single jobs without emitters over the plain 4-wide tree: the light terms
  // of bounce 0 whose shadow rays are traced as masked packets
  // (AJG_PACKET_SHADOW: 0 none, 1 directional lights, 2 every term, 3
  // directional lights and the MIS BSDF ray)
  int packet_shadow = 1;
  int packet_bounces = 1;  // bounces 0 .. packet_bounces-1 (AJG_PACKET_BOUNCES)
  // bounce 0's camera rays traced as masked packets over the binary layout
  // (AJG_PACKET_CAMERA=1; off by default: an exact tie in t between two
  // triangles, a ray through their shared edge, can resolve to the other
  // primitive when the packet visits them in another order, so the hits
  // are not bit-identical with the per-lane traversal's)
  bool packet_camera = false;
  std::mutex mu;
  std::string last_error;
  uint32_t* d_error = nullptr;            // device error flag
  uint32_t* d_fetch = nullptr;            // ray counter of query launches
  ajg::TraceCounters* d_counters = nullptr;  // [2]: closest, any
  unsigned long long paths_total = 0;
  unsigned long long kernel_launches = 0;
  bool profiling = false;
  std::vector<ajg::PendingTiming> pending;
  // per-launch log while profiling: pinned snapshots of the launching
  // kind's cumulative traversal counters, taken in stream order after each
  // timed traversal launch, and the resolved records
  ajg::TraceCounters* h_snaps = nullptr;  // [kLaunchLogCap]
  int64_t n_snaps = 0;
  std::vector<ajg_launch_record> launch_log;
  ajg::TraceCounters last_snap[2] = {};
  double kind_ms[ajg::kKinds] = {};
  unsigned long long kind_launches[ajg::kKinds] = {};
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
  std::atomic<int> jobs{0};  // unfinished jobs of the request loop
  std::vector<float> host_lights;
  std::vector<float> host_materials;
  float world[6] = {0, 0, 0, 0, 0, 0};  // the primitives' joined bounds
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
      int64_t snap = -1;
      if (kind != kKindShade && ctx->h_snaps && ctx->n_snaps < kLaunchLogCap) {
        snap = ctx->n_snaps++;
        cudaMemcpyAsync(ctx->h_snaps + snap, ctx->d_counters + counter_slot(kind),
                        sizeof(TraceCounters), cudaMemcpyDeviceToHost, st);
      }
      ctx->pending.push_back(PendingTiming{a, b, kind, snap});
    }
  }
};
// ploc.cu
int build_scene(ajg_ctx* ctx, ajg_scene* s, const float* h_tris,
                const float* h_corner, const int32_t* h_mat,
                const int32_t* h_flags, uint64_t n, const float* world,
                const ajg_scene_opts& opts);
// integrator.cu
uint64_t wave_bytes(uint64_t P, int nt, bool mj);
WaveBufs carve_wave(char* base, uint64_t P, int nt, bool mj);
// Enqueues one multi-job wave on `st` (capturable: fixed arguments, queue
// lengths and table contents read on the device): raygen, `bounces` bounce
// iterations, film update.  NT = light terms per path of the arena; `emit`:
// a scene of the wave has emitters (the closest-hit MIS BSDF pass runs).
// With a trace stream and two events, bounce b+1's closest hits run there
// beside bounce b's shadow rays (null: one stream).
void enqueue_mj_wave(const MJTables& t, const WaveBufs& w, uint64_t P,
                     int NT, int bounces, int tri_test, int width, bool emit,
                     TraceCounters* ctr, uint32_t* err, cudaStream_t st,
                     cudaStream_t ts = nullptr, cudaEvent_t ev_queue = nullptr,
                     cudaEvent_t ev_hits = nullptr, bool cam_packets = false,
                     bool shadow_packets = false);
// Kernels of a multi-job wave launched per wave (for launch counts):
// `shadow_packets` adds bounce 0's packet traversal of its directional-light
// rays (waves without emitters over plain 4-wide trees).
inline int mj_wave_kernels(int bounces, bool emit, int width = 0,
                           bool shadow_packets = false) {
  return 2 + (emit ? 10 : 8) * bounces +
         (shadow_packets && !emit && width == 4 && bounces > 0 ? 1 : 0);
}
// Looks up the persistent grids of the multi-job kernels (call before a
// stream capture).
void prepare_mj_kernels();
// The traversal launches of the path waves (wave_trace.cu, a translation
// unit of its own so that its arithmetic is compiled without contraction
// whatever the shading kernels are compiled with): closest hits of a path
// queue, any hits of the shadow queue, closest hits of the MIS BSDF queue
// at the top of the shadow queue's storage.  `mj`: multi-job waves (the
// scene of each ray from the wave tables).  Grids are the kernels' resident
// blocks (persistent lanes).
void launch_wave_extend(bool mj, int tri_test, int width, const DeviceScene& s,
                        const MJTables& t, const float4* ro, const float4* rd,
                        const uint32_t* count, uint32_t* fetch_next,
                        ajg_hit* hits, TraceCounters* ctr, uint32_t* err,
                        cudaStream_t st);
void launch_wave_shadow(bool mj, int tri_test, int width, const DeviceScene& s,
                        const MJTables& t, const float4* sq_o,
                        const float4* sq_d, const uint16_t* sq_scene,
                        const uint32_t* count, uint32_t* fetch_next,
                        uint8_t* vis, TraceCounters* ctr, uint32_t* err,
                        cudaStream_t st);
// A single job's camera rays (the binary layout) and coherent shadow rays
// (entry k at cap - 1 - k of the shadow queue's storage; the plain 4-wide
// tree) as masked packets.
void launch_wave_extend_packet(bool mj, int tri_test, const DeviceScene& s,
                               const MJTables& t, const float4* ro,
                               const float4* rd, const uint32_t* count,
                               uint32_t* fetch_next, ajg_hit* hits,
                               TraceCounters* ctr, uint32_t* err,
                               cudaStream_t st);
void launch_wave_shadow_packet(bool mj, int tri_test, const DeviceScene& s,
                               const MJTables& t, const float4* sq_o,
                               const float4* sq_d, const uint16_t* sq_scene,
                               const uint32_t* count, uint32_t* fetch_next,
                               uint32_t cap, uint8_t* vis, TraceCounters* ctr,
                               uint32_t* err, cudaStream_t st);
void launch_wave_bsdf_trace(bool mj, int tri_test, int width,
                            const DeviceScene& s, const MJTables& t,
                            const float4* sq_o, const float4* sq_d,
                            const uint16_t* sq_scene, const uint32_t* count,
                            uint32_t* fetch_next, uint32_t cap, uint32_t n_max,
                            float* t_hit, int32_t* prim_hit,
                            TraceCounters* ctr, uint32_t* err, cudaStream_t st);
// Blocks of `fn` (launched with `threads` threads) resident on the device at
// once: the grid of a persistent kernel.
int resident_grid(const void* fn, int threads);
// SPPM's camera pass (TracerVP, sppm.cpp:35-101) through the path-tracing
// wave: one path per pixel (sample 0), no roulette, depth `fmd`; fills
// vp[npix] (kNoVisPoint where none) and the direct light direct[npix].
int sppm_camera_pass(ajg_scene* sc, const ajg_camera& cam, int fmd,
                     uint64_t seed, VisPointD* vp, float4* direct,
                     cudaStream_t st);
// SPPMRenderer::Render on `st`: the footprint film (d_out, [h][w] float4, or
// null) and ComputePixelRadiance per pixel (d_rad, [h][w][3], or null).
int sppm_render(ajg_scene* sc, const ajg_camera& cam,
                const ajg_sppm_params& p, float4* d_out, float* d_rad,
                cudaStream_t st);
// Resolves a window-sized film into (sum rgb, sum w) per target pixel.
void enqueue_resolve(const float4* fsum, const float4* fcomp,
                     const double* fsum64, uint32_t w, uint32_t h,
                     bool fold_x, bool fold_y, float4* out, cudaStream_t st);
int check_render(ajg_ctx* ctx, const DeviceScene& s, const ajg_camera& cam,
                 const ajg_render_params& prm);
JobParams make_job_params(const ajg_scene* sc, const ajg_camera& cam,
                          const ajg_render_params& prm);
int render_impl(ajg_scene* sc, const ajg_camera& cam,
                const ajg_render_params& prm, float4* d_out,
                uint64_t li_begin, uint64_t li_end, float* d_li,
                cudaStream_t st);
// The same render over caller-provided scratch (film accumulators first,
// then one wave); allocates nothing.  Runs on `st`; no profiling events.
int render_in_scratch(ajg_scene* sc, const ajg_camera& cam,
                      const ajg_render_params& prm, float4* d_out,
                      cudaStream_t st, char* scratch, uint64_t bytes);
// serve.cu
void server_shutdown(ajg_ctx* ctx);
void server_sync(ajg_ctx* ctx);
// trace.cu
void launch_trace_closest(const DeviceScene& s, const ajg_ray* rays,
                          uint64_t n, ajg_hit* hits, uint32_t* next,
                          TraceCounters* ctr, uint32_t* err, cudaStream_t st);
void launch_trace_any(const DeviceScene& s, const ajg_ray* rays, uint64_t n,
                      uint8_t* occluded, uint32_t* next, TraceCounters* ctr,
                      uint32_t* err, cudaStream_t st);
}  // namespace ajg
