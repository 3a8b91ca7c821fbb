// The C ABI of include/ajisai_gpu.h: contexts, scenes, ray and shading
// queries, renders.  Every entry point validates its arguments, runs on the
// context's stream under the context mutex, and turns CUDA or device-guard
// failures into a status code plus a message for ajg_last_error().
#include <cfloat>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "shade.cuh"
#include "trace.cuh"

using namespace ajg;

namespace {

thread_local std::string g_error;  // errors before a context exists

int fail(ajg_ctx* ctx, int code, const std::string& m) {
  if (ctx)
    ctx->last_error = m;
  else
    g_error = m;
  return code;
}

int cuda_fail(ajg_ctx* ctx, cudaError_t e, const char* what) {
  return fail(ctx, e == cudaErrorMemoryAllocation ? AJG_ERR_OOM : AJG_ERR_CUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}

// After a synchronised call: surface a device guard as AJG_ERR_DEVICE and
// clear the flag so the context stays usable.
int check_device(ajg_ctx* ctx) {
  uint32_t e = 0;
  cudaError_t ce =
      cudaMemcpy(&e, ctx->d_error, sizeof(uint32_t), cudaMemcpyDeviceToHost);
  if (ce != cudaSuccess) return cuda_fail(ctx, ce, "reading the error flag");
  if (!e) return AJG_OK;
  cudaMemset(ctx->d_error, 0, sizeof(uint32_t));
  const char* what = e == kDevStackOverflow      ? "traversal stack overflow"
                     : e == kDevQueueOverflow    ? "queue capacity exceeded"
                     : e == kDevIterationBound   ? "iteration bound reached"
                     : e == kDevSortOutOfBounds  ? "sort out of bounds"
                     : e == kDevTableOutOfBounds ? "wave table index out of bounds"
                                                 : "unknown device guard";
  return fail(ctx, AJG_ERR_DEVICE, std::string("device guard: ") + what);
}

// Run work on the context stream ordered after `user`, and make `user` wait
// for it: one arena per context, so work of a context never overlaps.  A
// NULL `user` is the legacy default stream (the context stream is
// non-blocking, so it has to be joined explicitly like any other).
struct StreamJoin {
  cudaStream_t ctx_s, user;
  StreamJoin(cudaStream_t c, cudaStream_t u)
      : ctx_s(c), user(u ? u : cudaStreamLegacy) {
    if (user != ctx_s) {
      cudaEvent_t e;
      cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
      cudaEventRecord(e, user);
      cudaStreamWaitEvent(ctx_s, e, 0);
      cudaEventDestroy(e);
    }
  }
  ~StreamJoin() {
    if (user != ctx_s) {
      cudaEvent_t e;
      cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
      cudaEventRecord(e, ctx_s);
      cudaStreamWaitEvent(user, e, 0);
      cudaEventDestroy(e);
    }
  }
};

// Fresnel::computeDiffuseFresnel(ior, 1000000) (bsdf/helper.h:36-73), the
// term PlasticBsdf divides its albedo by; a million steps, so cached per
// ior.  (The reference computes it once per process, for the first
// PlasticBsdf it constructs; here each material uses its own ior.)
float host_dielectric_reflectance(float eta, float cos_i) {
  if (cos_i < 0.0f) {
    eta = 1.0f / eta;
    cos_i = -cos_i;
  }
  const float sin_t2 = eta * eta * (1.0f - cos_i * cos_i);
  if (sin_t2 > 1.0f) return 1.0f;
  const float cos_t = std::sqrt(ref_max(1.0f - sin_t2, 0.0f));
  const float rs = (eta * cos_i - cos_t) / (eta * cos_i + cos_t);
  const float rp = (eta * cos_t - cos_i) / (eta * cos_t + cos_i);
  return (rs * rs + rp * rp) * 0.5f;
}
float diffuse_fresnel(float ior) {
  static std::mutex mu;
  static std::map<uint32_t, float> cache;
  uint32_t key;
  std::memcpy(&key, &ior, 4);
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
  }
  const int n = 1000000;
  double acc = 0.0;
  float fb = host_dielectric_reflectance(ior, 0.0f);
  for (int i = 1; i <= n; ++i) {
    const float cos2 = float(i) / n;
    const float fa =
        host_dielectric_reflectance(ior, std::min(std::sqrt(cos2), 1.0f));
    acc += double(fa + fb) * (0.5 / n);
    fb = fa;
  }
  const float v = float(acc);
  std::lock_guard<std::mutex> lk(mu);
  cache[key] = v;
  return v;
}

// The device record of a material: the ABI record with the type as a float
// and, for plastic, the constructor's terms (plastic_bsdf.cpp:32-45) in the
// two reserved floats.
void material_record(const ajg_material& in, float r[16]) {
  std::memcpy(r, &in, sizeof(ajg_material));
  r[0] = (float)in.type;
  r[14] = r[15] = 0.f;
  if (in.type == AJG_MAT_PLASTIC) {
    const float ior = in.params[0], sc = in.params[1] * in.params[2];
    const float avg = (sc + sc + sc) / 3.f;
    r[14] = std::exp(-2.0f * avg);
    r[15] = diffuse_fresnel(ior);
  }
}

float host_lum(const float* rgb) {  // spectrum.h:80-82 in double
  return (float)(0.2126 * (double)rgb[0] + 0.7152 * (double)rgb[1] +
                 0.0722 * (double)rgb[2]);
}

__global__ void k_bsdf_query(const ajg_material* __restrict__ mats,
                             const float* __restrict__ ng,
                             const float* __restrict__ ns,
                             const float* __restrict__ wo,
                             const float* __restrict__ wi,
                             const float* __restrict__ sam,
                             const int32_t* __restrict__ op, uint64_t n,
                             float* __restrict__ out) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    // the record in global memory; its first word is the uint32 type, which
    // the BSDF routines do not read
    const float* m = reinterpret_cast<const float*>(mats + i);
    const float lum = (float)(0.2126 * (double)m[1] + 0.7152 * (double)m[2] +
                              0.0722 * (double)m[3]);
    Bsdf f;
    f.type = (int)mats[i].type;
    f.ng = ld3(ng + 3 * i);
    f.ns = ld3(ns + 3 * i);
    f.m = m;
    f.lum = lum;
    float* o = out + 8 * i;
    if (op[i] == 0) {
      const F3 v = f.eval(ld3(wi + 3 * i), ld3(wo + 3 * i));
      o[0] = v.x;
      o[1] = v.y;
      o[2] = v.z;
      o[3] = f.pdf(ld3(wi + 3 * i), ld3(wo + 3 * i));
      o[4] = o[5] = o[6] = 0.f;
      o[7] = 1.f;
    } else {
      const BsdfSample s = f.sample(ld3(wo + 3 * i), ld3(sam + 3 * i));
      o[0] = s.f.x;
      o[1] = s.f.y;
      o[2] = s.f.z;
      o[3] = s.pdf;
      o[4] = s.dir.x;
      o[5] = s.dir.y;
      o[6] = s.dir.z;
      const bool invalid = black3(s.f) && s.pdf == 0.f && maxc3(s.dir) <= 0.f &&
                           ref_min(ref_min(s.dir.x, s.dir.y), s.dir.z) >= 0.f;
      o[7] = invalid ? 0.f : (s.delta ? 3.f : 1.f);  // valid + 2 * delta
    }
  }
}

__global__ void k_camera_rays(ajg_camera cam, const float* __restrict__ raster,
                              uint64_t n, float* __restrict__ rays) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const float* q = raster + 4 * i;
    F3 o, d;
    camera_ray(cam, q[0], q[1], q[2], q[3], o, d);
    float* r = rays + 6 * i;
    r[0] = o.x;
    r[1] = o.y;
    r[2] = o.z;
    r[3] = d.x;
    r[4] = d.y;
    r[5] = d.z;
  }
}

template <class T>
struct DevBuf {
  T* p = nullptr;
  cudaStream_t s = nullptr;
  cudaError_t alloc(uint64_t count, cudaStream_t st) {
    s = st;
    return cudaMallocAsync((void**)&p, count * sizeof(T) > 0 ? count * sizeof(T) : 16,
                           st);
  }
  ~DevBuf() {
    if (p) cudaFreeAsync(p, s);
  }
};

#define CK(expr, what)                            \
  do {                                            \
    cudaError_t e_ = (expr);                      \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, what); \
  } while (0)

}  // namespace

extern "C" {

int ajg_abi_version(void) { return AJG_ABI_VERSION; }

const char* ajg_last_error(ajg_ctx* ctx) {
  return ctx ? ctx->last_error.c_str() : g_error.c_str();
}

int ajg_create_context(const ajg_config* cfg, ajg_ctx** out) {
  if (!out) return fail(nullptr, AJG_ERR_INVALID, "out is NULL");
  *out = nullptr;
  int dev = cfg ? cfg->device : 0;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0)
    return fail(nullptr, AJG_ERR_CUDA, "no CUDA device available");
  if (dev < 0 || dev >= count)
    return fail(nullptr, AJG_ERR_INVALID, "device ordinal out of range");
  e = cudaSetDevice(dev);
  if (e != cudaSuccess) return fail(nullptr, AJG_ERR_CUDA, cudaGetErrorString(e));
  // each render also keeps paths x light terms below 2^31 (job_wave_paths)
  if (cfg && cfg->wave_paths > (1u << 28))
    return fail(nullptr, AJG_ERR_INVALID, "wave_paths above 2^28");
  auto* ctx = new ajg_ctx();
  ctx->device = dev;
  if (cfg && cfg->wave_paths) ctx->wave_paths = cfg->wave_paths;
  if (ctx->wave_paths < 1024) ctx->wave_paths = 1024;
  if (cfg) ctx->hbm_budget = cfg->hbm_budget_bytes;
  if (const char* ov = std::getenv("AJG_TRACE_OVERLAP"))
    ctx->overlap = std::strcmp(ov, "0") != 0;
  if (const char* pk = std::getenv("AJG_PACKET_SHADOW"))
    ctx->packet_shadow = std::atoi(pk);
  if (const char* pb = std::getenv("AJG_PACKET_BOUNCES"))
    ctx->packet_bounces = std::atoi(pb);
  if (const char* pc = std::getenv("AJG_PACKET_CAMERA"))
    ctx->packet_camera = std::strcmp(pc, "0") != 0;
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) !=
          cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->trace_stream, cudaStreamNonBlocking) !=
          cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->ev_queue, cudaEventDisableTiming) !=
          cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->ev_hits, cudaEventDisableTiming) !=
          cudaSuccess ||
      cudaMalloc(&ctx->d_error, sizeof(uint32_t)) != cudaSuccess ||
      cudaMalloc(&ctx->d_fetch, sizeof(uint32_t)) != cudaSuccess ||
      cudaMalloc(&ctx->d_counters, 2 * sizeof(TraceCounters)) != cudaSuccess) {
    delete ctx;
    return fail(nullptr, AJG_ERR_CUDA, "context allocation failed");
  }
  cudaMemset(ctx->d_error, 0, sizeof(uint32_t));
  cudaMemset(ctx->d_counters, 0, 2 * sizeof(TraceCounters));
  *out = ctx;
  return AJG_OK;
}

int ajg_destroy_context(ajg_ctx* ctx) {
  if (!ctx) return AJG_ERR_INVALID;
  cudaSetDevice(ctx->device);
  server_shutdown(ctx);
  cudaStreamSynchronize(ctx->stream);
  for (auto& p : ctx->pending) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  for (auto& b : ctx->arena) cudaFree(b.ptr);
  cudaFree(ctx->d_error);
  cudaFree(ctx->d_fetch);
  cudaFree(ctx->d_counters);
  if (ctx->h_snaps) cudaFreeHost(ctx->h_snaps);
  cudaStreamSynchronize(ctx->trace_stream);
  cudaEventDestroy(ctx->ev_queue);
  cudaEventDestroy(ctx->ev_hits);
  cudaStreamDestroy(ctx->trace_stream);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return AJG_OK;
}

// Turns the recorded event pairs into milliseconds per kind and launch
// records (after the context's stream is synchronised).
static void resolve_timings(ajg_ctx* ctx) {
  for (auto& p : ctx->pending) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p.a, p.b);
    ctx->kind_ms[p.kind] += ms;
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
    ajg_launch_record r{};
    r.kind = (uint32_t)p.kind;
    r.ms = ms;
    if (p.snap >= 0) {
      const TraceCounters c = ctx->h_snaps[p.snap];
      const int slot = counter_slot(p.kind);
      const TraceCounters& l = ctx->last_snap[slot];
      r.rays = c.rays - l.rays;
      r.nodes = c.nodes - l.nodes;
      r.tris = c.tris - l.tris;
      ctx->last_snap[slot] = c;
    }
    if (ctx->launch_log.size() < (size_t)kLaunchLogCap)
      ctx->launch_log.push_back(r);
  }
  ctx->pending.clear();
}

int ajg_get_launch_log(ajg_ctx* ctx, ajg_launch_record* out, uint32_t capacity,
                       uint32_t* count, int reset) {
  if (!ctx || !count) return fail(ctx, AJG_ERR_INVALID, "NULL argument");
  std::lock_guard<std::mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  CK(cudaStreamSynchronize(ctx->stream), "launch log");
  CK(cudaStreamSynchronize(ctx->trace_stream), "launch log");
  resolve_timings(ctx);
  *count = (uint32_t)ctx->launch_log.size();
  if (out)
    std::memcpy(out, ctx->launch_log.data(),
                sizeof(ajg_launch_record) *
                    std::min<size_t>(capacity, ctx->launch_log.size()));
  if (reset) {
    ctx->launch_log.clear();
    ctx->n_snaps = 0;
  }
  return AJG_OK;
}

int ajg_get_stats(ajg_ctx* ctx, ajg_stats* out, int reset) {
  if (!ctx || !out) return fail(ctx, AJG_ERR_INVALID, "NULL argument");
  std::lock_guard<std::mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  TraceCounters c[2];
  CK(cudaStreamSynchronize(ctx->stream), "stats");
  CK(cudaMemcpy(c, ctx->d_counters, sizeof(c), cudaMemcpyDeviceToHost),
     "stats");
  out->closest_rays = c[0].rays;
  out->any_rays = c[1].rays;
  out->closest_nodes = c[0].nodes;
  out->closest_tris = c[0].tris;
  out->any_nodes = c[1].nodes;
  out->any_tris = c[1].tris;
  out->nodes_visited = c[0].nodes + c[1].nodes;
  out->tris_tested = c[0].tris + c[1].tris;
  out->paths = ctx->paths_total;
  resolve_timings(ctx);
  out->kernel_launches = ctx->kernel_launches;
  out->closest_launches =
      ctx->kind_launches[kKindClosest] + ctx->kind_launches[kKindClosestPacket];
  out->any_launches =
      ctx->kind_launches[kKindAny] + ctx->kind_launches[kKindAnyPacket];
  out->shade_launches = ctx->kind_launches[kKindShade];
  out->closest_ms = ctx->kind_ms[kKindClosest] + ctx->kind_ms[kKindClosestPacket];
  out->any_ms = ctx->kind_ms[kKindAny] + ctx->kind_ms[kKindAnyPacket];
  out->shade_ms = ctx->kind_ms[kKindShade];
  if (reset) {
    CK(cudaMemset(ctx->d_counters, 0, sizeof(c)), "stats");
    for (auto& l : ctx->last_snap) l = TraceCounters{};
    ctx->paths_total = 0;
    ctx->kernel_launches = 0;
    for (int k = 0; k < kKinds; ++k) {
      ctx->kind_ms[k] = 0;
      ctx->kind_launches[k] = 0;
    }
  }
  return AJG_OK;
}

int ajg_set_profiling(ajg_ctx* ctx, int enable) {
  if (!ctx) return fail(nullptr, AJG_ERR_INVALID, "NULL context");
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (enable && !ctx->h_snaps) {
    cudaSetDevice(ctx->device);
    CK(cudaHostAlloc((void**)&ctx->h_snaps,
                     sizeof(TraceCounters) * kLaunchLogCap, cudaHostAllocDefault),
       "launch log");
  }
  if (enable && !ctx->profiling) {
    // counters the log's first deltas start from
    CK(cudaStreamSynchronize(ctx->stream), "profiling");
    CK(cudaMemcpy(ctx->last_snap, ctx->d_counters, sizeof(ctx->last_snap),
                  cudaMemcpyDeviceToHost),
       "profiling");
  }
  ctx->profiling = enable != 0;
  return AJG_OK;
}

namespace {

// An emitter's AreaLight as the device reads it: the light record and the
// corner points of its sampler (quad: a, b, c, d; mesh: its corners in
// index order; cube: each triangle's corners in the order the cube's index
// tuples declare them, the reverse of its MeshView's).  Areas and pdfs are
// computed in float as the geometries compute them (quad.cpp:52-60,
// mesh.cpp:62-68 with the sum in double, cube.cpp:145-191 from its first
// triangle, two_sided.cpp:104-112).
void area_light_record(const float* tris, const ajg_emitter& e,
                       uint32_t pts_first, float rec[12],
                       std::vector<float>& pts) {
  auto corner = [&](uint64_t t, int k) {
    const float* v = tris + 9 * ((uint64_t)e.first_triangle + t) + 3 * k;
    return mk3(v[0], v[1], v[2]);
  };
  auto push = [&](F3 v) { pts.insert(pts.end(), {v.x, v.y, v.z}); };
  auto len = [](F3 v) { return std::sqrt(dot3(v, v)); };
  float inv_area = 0.f, share = 0.f, pdf = 0.f;
  if (e.geometry == AJG_GEOM_QUAD) {
    const F3 a = corner(0, 0), b = corner(0, 1), c = corner(0, 2),
             d = corner(1, 2);
    for (F3 v : {a, b, c, d}) push(v);
    const float abc = len(cross3(b - a, c - a)) * 0.5f;
    const float acd = len(cross3(c - a, d - a)) * 0.5f;
    const float area = abc + acd;
    share = abc / area;
    inv_area = 1.f / area;
    pdf = 1.f / area;
  } else if (e.geometry == AJG_GEOM_MESH) {
    float area = 0.f;
    for (uint32_t t = 0; t < e.num_triangles; ++t) {
      const F3 i = corner(t, 0), j = corner(t, 1), k = corner(t, 2);
      push(i);
      push(j);
      push(k);
      area = (float)((double)area + 0.5 * (double)len(cross3(j - i, k - i)));
    }
    inv_area = 1.f / area;
    pdf = 1.f / area;
  } else {
    for (uint32_t t = 0; t < 12; ++t)
      for (int k = 2; k >= 0; --k) push(corner(t, k));
    const F3 pa = corner(0, 2), pb = corner(0, 1), pc = corner(0, 0);
    pdf = 1.f / (12.f * len(cross3(pb - pa, pc - pa)) * 0.5f);
  }
  if (e.two_sided) pdf = pdf * 0.5f;
  std::memset(rec, 0, 12 * sizeof(float));
  rec[0] = (float)kLightArea;
  rec[1] = e.radiance[0];
  rec[2] = e.radiance[1];
  rec[3] = e.radiance[2];
  rec[4] = (float)e.geometry;
  rec[5] = e.two_sided ? 1.f : 0.f;
  std::memcpy(&rec[6], &e.num_triangles, 4);
  rec[7] = inv_area;
  rec[8] = share;
  rec[9] = pdf;
  std::memcpy(&rec[10], &pts_first, 4);
}

bool black_emission(const ajg_emitter& e) {
  return e.radiance[0] == 0.f && e.radiance[1] == 0.f && e.radiance[2] == 0.f;
}

}  // namespace

int ajg_scene_create_flat(ajg_ctx* ctx, const float* tris,
                          const float* corner_normals,
                          const int32_t* tri_material,
                          const int32_t* tri_flags, uint64_t n,
                          const float* world, const ajg_material* materials,
                          uint32_t num_materials, const ajg_light* lights,
                          uint32_t num_lights, const ajg_scene_opts* opts,
                          ajg_scene** out) {
  return ajg_scene_create_flat_ex(ctx, tris, corner_normals, tri_material,
                                  tri_flags, n, world, materials, num_materials,
                                  lights, num_lights, nullptr, 0, opts, out);
}

int ajg_scene_create_flat_ex(ajg_ctx* ctx, const float* tris,
                             const float* corner_normals,
                             const int32_t* tri_material,
                             const int32_t* tri_flags, uint64_t n,
                             const float* world, const ajg_material* materials,
                             uint32_t num_materials, const ajg_light* lights,
                             uint32_t num_lights, const ajg_emitter* emitters,
                             uint32_t num_emitters, const ajg_scene_opts* opts,
                             ajg_scene** out) {
  if (!ctx || !out) return fail(ctx, AJG_ERR_INVALID, "NULL argument");
  *out = nullptr;
  if (!tris || !tri_material || !tri_flags || !world || n == 0)
    return fail(ctx, AJG_ERR_INVALID, "empty scene or NULL arrays");
  if (!materials || num_materials == 0)
    return fail(ctx, AJG_ERR_INVALID, "a scene needs at least one material");
  if ((num_lights && !lights) || (num_emitters && !emitters))
    return fail(ctx, AJG_ERR_INVALID, "NULL light or emitter array");
  // emitters: each a disjoint triangle range of the shape its sampler needs
  std::vector<int32_t> tri_emit;
  uint32_t num_area = 0;
  for (uint32_t i = 0; i < num_emitters; ++i) {
    const ajg_emitter& e = emitters[i];
    if (e.geometry > AJG_GEOM_MESH)
      return fail(ctx, AJG_ERR_INVALID, "unknown emitter geometry");
    const uint32_t need = e.geometry == AJG_GEOM_QUAD   ? 2u
                          : e.geometry == AJG_GEOM_CUBE ? 12u
                                                        : 0u;
    if ((need && e.num_triangles != need) || e.num_triangles == 0)
      return fail(ctx, AJG_ERR_INVALID,
                  "emitter triangle count does not fit its geometry (quad 2, "
                  "cube 12, mesh >= 1)");
    if ((uint64_t)e.first_triangle + e.num_triangles > n)
      return fail(ctx, AJG_ERR_INVALID, "emitter triangles out of range");
    if (e.two_sided > 1) return fail(ctx, AJG_ERR_INVALID, "two_sided is 0 or 1");
    if (black_emission(e)) continue;
    if (tri_emit.empty()) tri_emit.assign(n, -1);
    for (uint32_t t = 0; t < e.num_triangles; ++t) {
      const uint64_t g = (uint64_t)e.first_triangle + t;
      if (tri_emit[g] >= 0)
        return fail(ctx, AJG_ERR_INVALID, "emitters share a triangle");
      if (((tri_flags[g] & AJG_MESH_TWO_SIDED) != 0) != (e.two_sided != 0))
        return fail(ctx, AJG_ERR_INVALID,
                    "emitter two_sided differs from its triangles' flags");
      tri_emit[g] = (int32_t)num_area;
    }
    ++num_area;
  }
  if (num_lights + num_area > 15)
    return fail(ctx, AJG_ERR_UNSUPPORTED,
                "at most 15 lights (emitters included)");
  ajg_scene_opts o{14, AJG_TRI_MOLLER_TRUMBORE, 0, 0};
  if (opts) o = *opts;
  if (o.tri_test > AJG_TRI_WATERTIGHT)
    return fail(ctx, AJG_ERR_INVALID, "unknown triangle test");
  for (uint64_t i = 0; i < n; ++i) {
    if (tri_material[i] < 0 || (uint32_t)tri_material[i] >= num_materials)
      return fail(ctx, AJG_ERR_INVALID, "triangle material index out of range");
    if ((tri_flags[i] & AJG_MESH_HAS_NORMALS) && !corner_normals)
      return fail(ctx, AJG_ERR_INVALID, "HAS_NORMALS without normals");
    if (tri_flags[i] & ~7)
      return fail(ctx, AJG_ERR_INVALID, "unknown triangle flag");
  }
  for (uint32_t m = 0; m < num_materials; ++m)
    if (materials[m].type > AJG_MAT_NULL)
      return fail(ctx, AJG_ERR_UNSUPPORTED, "unknown material type");
  for (uint32_t l = 0; l < num_lights; ++l)
    if (lights[l].type > AJG_LIGHT_ENV)
      return fail(ctx, AJG_ERR_UNSUPPORTED, "unknown light type");
  // admission by the HBM budget: resident scene bytes per triangle
  const uint64_t est = n * (64 + 48 + 16 + 32 + 4 + 36) + (1u << 20);
  if (ctx->hbm_budget && ctx->resident_bytes + est > ctx->hbm_budget)
    return fail(ctx, AJG_ERR_OOM, "scene exceeds the HBM admission budget");

  std::lock_guard<std::mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  auto* s = new ajg_scene();
  s->ctx = ctx;
  // lights: the emitters' area lights first (default_scene.cpp:33-48), then
  // the records as given; env records get the two mass flags of the 1x1
  // Distribution2D (utility/distribution.h:40-60, 135-144)
  const uint32_t nl_all = num_area + num_lights;
  s->host_lights.resize(12 * (size_t)nl_all);
  std::vector<float> emit_pts;
  for (uint32_t i = 0, a = 0; i < num_emitters; ++i) {
    if (black_emission(emitters[i])) continue;
    area_light_record(tris, emitters[i], (uint32_t)(emit_pts.size() / 3),
                      &s->host_lights[12 * (size_t)a++], emit_pts);
  }
  int env = -1;
  for (uint32_t l = 0; l < num_lights; ++l) {
    float* r = &s->host_lights[12 * (size_t)(num_area + l)];
    std::memcpy(r, &lights[l], sizeof(ajg_light));
    r[0] = (float)lights[l].type;
    if (lights[l].type == AJG_LIGHT_ENV) {
      env = (int)(num_area + l);
      const float w = host_lum(lights[l].rgb) * std::sin(kPi * (0 + 0.5f) / 1.f);
      const float func_int = 0.f + w * (1.f / 1.f);
      r[10] = func_int > 0.f ? 1.f : 0.f;
      r[11] = func_int * func_int != 0.f ? 1.f : 0.f;
    } else {
      r[10] = r[11] = 0.f;
    }
  }
  s->host_materials.resize(16 * (size_t)num_materials);
  std::vector<float4> lum(num_materials);
  uint32_t mat_mask = 0;
  for (uint32_t m = 0; m < num_materials; ++m) {
    material_record(materials[m], &s->host_materials[16 * m]);
    lum[m] = make_float4(host_lum(materials[m].base_color), 0, 0, 0);
    mat_mask |= 1u << materials[m].type;
  }
  auto keep = [&](size_t bytes) -> void* {
    void* p = nullptr;
    if (cudaMalloc(&p, bytes > 0 ? bytes : 16) != cudaSuccess) return nullptr;
    s->allocations.push_back(p);
    s->info.device_bytes += bytes;
    return p;
  };
  float* d_mat = (float*)keep(s->host_materials.size() * sizeof(float));
  float* d_light = (float*)keep(std::max<size_t>(1, s->host_lights.size()) *
                                sizeof(float));
  float4* d_lum = (float4*)keep(num_materials * sizeof(float4));
  int32_t* d_tri_emit =
      num_area ? (int32_t*)keep(n * sizeof(int32_t)) : nullptr;
  float* d_pts = num_area ? (float*)keep(emit_pts.size() * sizeof(float)) : nullptr;
  if (!d_mat || !d_light || !d_lum || (num_area && (!d_tri_emit || !d_pts))) {
    ajg_scene_release(s);
    return fail(ctx, AJG_ERR_OOM, "device allocation failed (scene tables)");
  }
  cudaMemcpy(d_mat, s->host_materials.data(),
             s->host_materials.size() * sizeof(float), cudaMemcpyHostToDevice);
  if (nl_all)
    cudaMemcpy(d_light, s->host_lights.data(),
               s->host_lights.size() * sizeof(float), cudaMemcpyHostToDevice);
  if (num_area) {
    cudaMemcpy(d_tri_emit, tri_emit.data(), n * sizeof(int32_t),
               cudaMemcpyHostToDevice);
    cudaMemcpy(d_pts, emit_pts.data(), emit_pts.size() * sizeof(float),
               cudaMemcpyHostToDevice);
  }
  s->d.tri_emit = d_tri_emit;
  s->d.emit_pts = d_pts;
  s->d.num_area = num_area;
  cudaMemcpy(d_lum, lum.data(), num_materials * sizeof(float4),
             cudaMemcpyHostToDevice);
  s->d.materials = d_mat;
  s->d.lights = d_light;
  s->d.mat_lum = d_lum;
  s->d.num_materials = num_materials;
  s->d.mat_mask = mat_mask;
  s->d.num_lights = nl_all;
  s->d.env = env;
  int rc = build_scene(ctx, s, tris, corner_normals, tri_material, tri_flags,
                       n, world, o);
  if (rc != AJG_OK) {
    std::string m = ctx->last_error;
    ajg_scene_release(s);
    ctx->last_error = m;
    return rc;
  }
  ctx->resident_bytes += s->info.device_bytes;
  *out = s;
  return AJG_OK;
}

int ajg_scene_create(ajg_ctx* ctx, const ajg_mesh_desc* meshes,
                     uint32_t num_meshes, const ajg_material* materials,
                     uint32_t num_materials, const ajg_light* lights,
                     uint32_t num_lights, const ajg_scene_opts* opts,
                     ajg_scene** out) {
  return ajg_scene_create_ex(ctx, meshes, num_meshes, materials, num_materials,
                             lights, num_lights, nullptr, 0, opts, out);
}

int ajg_scene_create_ex(ajg_ctx* ctx, const ajg_mesh_desc* meshes,
                        uint32_t num_meshes, const ajg_material* materials,
                        uint32_t num_materials, const ajg_light* lights,
                        uint32_t num_lights, const ajg_emitter* emitters,
                        uint32_t num_emitters, const ajg_scene_opts* opts,
                        ajg_scene** out) {
  if (!ctx || !out || (!meshes && num_meshes))
    return fail(ctx, AJG_ERR_INVALID, "NULL argument");
  uint64_t n = 0;
  bool any_normals = false;
  for (uint32_t m = 0; m < num_meshes; ++m) {
    const ajg_mesh_desc& d = meshes[m];
    if (d.num_triangles && (!d.positions || !d.indices))
      return fail(ctx, AJG_ERR_INVALID, "mesh without positions or indices");
    if ((d.flags & AJG_MESH_HAS_NORMALS) && !d.normals)
      return fail(ctx, AJG_ERR_INVALID, "HAS_NORMALS without normals");
    n += d.num_triangles;
    any_normals |= (d.flags & AJG_MESH_HAS_NORMALS) != 0;
  }
  std::vector<float> tris(9 * n), cn(any_normals ? 9 * n : 0);
  std::vector<int32_t> mat(n), flags(n);
  // world = Join of the primitives' AABBs (default_scene.cpp:32-39), each
  // primitive's AABB spanning all of its vertices (mesh.cpp:71-74)
  float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  uint64_t t = 0;
  for (uint32_t m = 0; m < num_meshes; ++m) {
    const ajg_mesh_desc& d = meshes[m];
    float plo[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
    float phi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (uint32_t v = 0; v < d.num_vertices; ++v)
      for (int k = 0; k < 3; ++k) {
        plo[k] = ref_min(plo[k], d.positions[3 * v + k]);
        phi[k] = ref_max(phi[k], d.positions[3 * v + k]);
      }
    const bool lpoint = lo[0] == hi[0] && lo[1] == hi[1] && lo[2] == hi[2];
    const bool ppoint = plo[0] == phi[0] && plo[1] == phi[1] && plo[2] == phi[2];
    if (d.num_vertices) {
      if (lpoint) {
        std::memcpy(lo, plo, sizeof(lo));
        std::memcpy(hi, phi, sizeof(hi));
      } else if (!ppoint) {
        for (int k = 0; k < 3; ++k) {
          lo[k] = ref_min(lo[k], plo[k]);
          hi[k] = ref_max(hi[k], phi[k]);
        }
      }
    }
    for (uint32_t i = 0; i < d.num_triangles; ++i, ++t) {
      for (int c = 0; c < 3; ++c) {
        const uint32_t vi = d.indices[3 * i + c];
        if (vi >= d.num_vertices)
          return fail(ctx, AJG_ERR_INVALID, "vertex index out of range");
        std::memcpy(&tris[9 * t + 3 * c], d.positions + 3 * (uint64_t)vi,
                    3 * sizeof(float));
        if (d.flags & AJG_MESH_HAS_NORMALS)
          std::memcpy(&cn[9 * t + 3 * c], d.normals + 3 * (uint64_t)vi,
                      3 * sizeof(float));
      }
      mat[t] = (int32_t)d.material;
      flags[t] = (int32_t)d.flags;
    }
  }
  const float world[6] = {lo[0], lo[1], lo[2], hi[0], hi[1], hi[2]};
  return ajg_scene_create_flat_ex(
      ctx, tris.data(), any_normals ? cn.data() : nullptr, mat.data(),
      flags.data(), n, world, materials, num_materials, lights, num_lights,
      emitters, num_emitters, opts, out);
}

int ajg_scene_release(ajg_scene* s) {
  if (!s) return AJG_ERR_INVALID;
  ajg_ctx* ctx = s->ctx;
  if (s->jobs.load() > 0)
    return fail(ctx, AJG_ERR_INVALID, "scene has unfinished jobs");
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  server_sync(ctx);
  for (void* p : s->allocations) cudaFree(p);
  if (ctx->resident_bytes >= s->info.device_bytes)
    ctx->resident_bytes -= s->info.device_bytes;
  delete s;
  return AJG_OK;
}

int ajg_scene_get_info(ajg_scene* s, ajg_scene_info* out) {
  if (!s || !out) return AJG_ERR_INVALID;
  *out = s->info;
  return AJG_OK;
}

int ajg_scene_download_bvh(ajg_scene* s, float* node_bounds,
                           int64_t* node_count_first, int64_t* perm) {
  if (!s || !node_bounds || !node_count_first || !perm) return AJG_ERR_INVALID;
  ajg_ctx* ctx = s->ctx;
  std::lock_guard<std::mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  const uint64_t m = s->info.num_nodes, n = s->info.num_triangles;
  std::vector<float4> nodes(2 * m);
  std::vector<int32_t> p(n);
  CK(cudaMemcpy(nodes.data(), s->ploc_nodes, 2 * m * sizeof(float4),
                cudaMemcpyDeviceToHost),
     "download_bvh");
  CK(cudaMemcpy(p.data(), s->perm, n * sizeof(int32_t), cudaMemcpyDeviceToHost),
     "download_bvh");
  for (uint64_t i = 0; i < m; ++i) {
    const float4 a = nodes[2 * i], b = nodes[2 * i + 1];
    float* o = node_bounds + 6 * i;
    o[0] = a.x; o[1] = a.y; o[2] = a.z;
    o[3] = b.x; o[4] = b.y; o[5] = b.z;
    int32_t first, count;
    std::memcpy(&first, &a.w, 4);
    std::memcpy(&count, &b.w, 4);
    node_count_first[2 * i] = count;
    node_count_first[2 * i + 1] = first;
  }
  for (uint64_t i = 0; i < n; ++i) perm[i] = p[i];
  return AJG_OK;
}

static int trace_host(ajg_scene* s, const ajg_ray* rays, uint64_t n,
                      void* out, bool any) {
  if (!s || (n && (!rays || !out))) return AJG_ERR_INVALID;
  ajg_ctx* ctx = s->ctx;
  if (n > (1ull << 31))
    return fail(ctx, AJG_ERR_INVALID, "at most 2^31 rays per call");
  if (n == 0) return AJG_OK;
  std::lock_guard<std::mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  cudaStream_t st = ctx->stream;
  DevBuf<ajg_ray> dr;
  CK(dr.alloc(n, st), "trace: alloc");
  CK(cudaMemcpyAsync(dr.p, rays, n * sizeof(ajg_ray), cudaMemcpyHostToDevice, st),
     "trace: copy in");
  CK(cudaMemsetAsync(ctx->d_fetch, 0, sizeof(uint32_t), st), "trace");
  KernelTimer tm(ctx, st, any ? kKindAny : kKindClosest);
  if (any) {
    DevBuf<uint8_t> dh;
    CK(dh.alloc(n, st), "trace: alloc");
    launch_trace_any(s->d, dr.p, n, dh.p, ctx->d_fetch, &ctx->d_counters[1],
                     ctx->d_error, st);
    CK(cudaMemcpyAsync(out, dh.p, n, cudaMemcpyDeviceToHost, st), "trace: copy out");
  } else {
    DevBuf<ajg_hit> dh;
    CK(dh.alloc(n, st), "trace: alloc");
    launch_trace_closest(closest_view(s->d), dr.p, n, dh.p, ctx->d_fetch,
                         &ctx->d_counters[0],
                         ctx->d_error, st);
    CK(cudaMemcpyAsync(out, dh.p, n * sizeof(ajg_hit), cudaMemcpyDeviceToHost, st),
       "trace: copy out");
  }
  CK(cudaStreamSynchronize(st), "trace");
  return check_device(ctx);
}

int ajg_trace_closest(ajg_scene* s, const ajg_ray* rays, uint64_t n,
                      ajg_hit* hits) {
  return trace_host(s, rays, n, hits, false);
}

int ajg_trace_any(ajg_scene* s, const ajg_ray* rays, uint64_t n,
                  uint8_t* occluded) {
  return trace_host(s, rays, n, occluded, true);
}

int ajg_trace_closest_device(ajg_scene* s, const ajg_ray* d_rays, uint64_t n,
                             ajg_hit* d_hits, void* stream) {
  if (!s || (n && (!d_rays || !d_hits))) return AJG_ERR_INVALID;
  ajg_ctx* ctx = s->ctx;
  if (n > (1ull << 31))
    return fail(ctx, AJG_ERR_INVALID, "at most 2^31 rays per call");
  std::lock_guard<std::mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  StreamJoin j(ctx->stream, (cudaStream_t)stream);
  CK(cudaMemsetAsync(ctx->d_fetch, 0, sizeof(uint32_t), ctx->stream),
     "trace_closest_device");
  KernelTimer tm(ctx, ctx->stream, kKindClosest);
  launch_trace_closest(closest_view(s->d), d_rays, n, d_hits, ctx->d_fetch,
                       &ctx->d_counters[0], ctx->d_error, ctx->stream);
  CK(cudaGetLastError(), "trace_closest_device");
  return AJG_OK;
}

int ajg_trace_any_device(ajg_scene* s, const ajg_ray* d_rays, uint64_t n,
                         uint8_t* d_occluded, void* stream) {
  if (!s || (n && (!d_rays || !d_occluded))) return AJG_ERR_INVALID;
  ajg_ctx* ctx = s->ctx;
  if (n > (1ull << 31))
    return fail(ctx, AJG_ERR_INVALID, "at most 2^31 rays per call");
  std::lock_guard<std::mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  StreamJoin j(ctx->stream, (cudaStream_t)stream);
  CK(cudaMemsetAsync(ctx->d_fetch, 0, sizeof(uint32_t), ctx->stream),
     "trace_any_device");
  KernelTimer tm(ctx, ctx->stream, kKindAny);
  launch_trace_any(s->d, d_rays, n, d_occluded, ctx->d_fetch,
                   &ctx->d_counters[1], ctx->d_error, ctx->stream);
  CK(cudaGetLastError(), "trace_any_device");
  return AJG_OK;
}

int ajg_bsdf_query(ajg_ctx* ctx, const ajg_material* materials,
                   const float* ng, const float* ns, const float* wo,
                   const float* wi, const float* sam, const int32_t* op,
                   uint64_t n, float* out) {
  if (!ctx) return fail(nullptr, AJG_ERR_INVALID, "NULL context");
  if (n && (!materials || !ng || !ns || !wo || !wi || !sam || !op || !out))
    return fail(ctx, AJG_ERR_INVALID, "NULL array");
  if (!n) return AJG_OK;
  std::lock_guard<std::mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  cudaStream_t st = ctx->stream;
  DevBuf<ajg_material> dm;
  DevBuf<float> dv, dout;
  DevBuf<int32_t> dop;
  CK(dm.alloc(n, st), "bsdf_query");
  CK(dv.alloc(15 * n, st), "bsdf_query");
  CK(dout.alloc(8 * n, st), "bsdf_query");
  CK(dop.alloc(n, st), "bsdf_query");
  // the device records: plastic's precomputed terms in the reserved floats
  std::vector<ajg_material> recs(materials, materials + n);
  for (uint64_t i = 0; i < n; ++i) {
    if (recs[i].type > AJG_MAT_NULL)
      return fail(ctx, AJG_ERR_UNSUPPORTED, "unknown material type");
    float r[16];
    material_record(recs[i], r);
    recs[i].pad[0] = r[14];
    recs[i].pad[1] = r[15];
  }
  cudaMemcpyAsync(dm.p, recs.data(), n * sizeof(ajg_material), cudaMemcpyHostToDevice, st);
  const float* srcs[5] = {ng, ns, wo, wi, sam};
  for (int k = 0; k < 5; ++k)
    cudaMemcpyAsync(dv.p + 3 * n * k, srcs[k], 3 * n * sizeof(float),
                    cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(dop.p, op, n * sizeof(int32_t), cudaMemcpyHostToDevice, st);
  k_bsdf_query<<<grid_for(n, 128), 128, 0, st>>>(
      dm.p, dv.p, dv.p + 3 * n, dv.p + 6 * n, dv.p + 9 * n, dv.p + 12 * n,
      dop.p, n, dout.p);
  cudaMemcpyAsync(out, dout.p, 8 * n * sizeof(float), cudaMemcpyDeviceToHost, st);
  CK(cudaStreamSynchronize(st), "bsdf_query");
  return AJG_OK;
}

int ajg_camera_rays(ajg_ctx* ctx, const ajg_camera* cam, const float* raster,
                    uint64_t n, float* rays) {
  if (!ctx) return fail(nullptr, AJG_ERR_INVALID, "NULL context");
  if (!cam || (n && (!raster || !rays)))
    return fail(ctx, AJG_ERR_INVALID, "NULL argument");
  if (!n) return AJG_OK;
  std::lock_guard<std::mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  cudaStream_t st = ctx->stream;
  DevBuf<float> din, dout;
  CK(din.alloc(4 * n, st), "camera_rays");
  CK(dout.alloc(6 * n, st), "camera_rays");
  cudaMemcpyAsync(din.p, raster, 4 * n * sizeof(float), cudaMemcpyHostToDevice, st);
  k_camera_rays<<<grid_for(n, 128), 128, 0, st>>>(*cam, din.p, n, dout.p);
  cudaMemcpyAsync(rays, dout.p, 6 * n * sizeof(float), cudaMemcpyDeviceToHost, st);
  CK(cudaStreamSynchronize(st), "camera_rays");
  return AJG_OK;
}

int ajg_render(ajg_scene* s, const ajg_camera* cam,
               const ajg_render_params* params, float* out_rgbw) {
  if (!s || !cam || !params || !out_rgbw) return AJG_ERR_INVALID;
  ajg_ctx* ctx = s->ctx;
  std::lock_guard<std::mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  cudaStream_t st = ctx->stream;
  const uint64_t npix = (uint64_t)cam->width * cam->height;
  DevBuf<float4> d;
  CK(d.alloc(npix, st), "render: alloc");
  int rc = render_impl(s, *cam, *params, d.p, 0, 0, nullptr, st);
  if (rc) return rc;
  CK(cudaMemcpyAsync(out_rgbw, d.p, npix * sizeof(float4),
                     cudaMemcpyDeviceToHost, st),
     "render: copy out");
  CK(cudaStreamSynchronize(st), "render");
  return check_device(ctx);
}

int ajg_render_sppm(ajg_scene* s, const ajg_camera* cam,
                    const ajg_sppm_params* params, float* out_rgbw,
                    float* out_radiance) {
  if (!s || !cam || !params) return AJG_ERR_INVALID;
  ajg_ctx* ctx = s->ctx;
  std::lock_guard<std::mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  cudaStream_t st = ctx->stream;
  const uint64_t npix = (uint64_t)cam->width * cam->height;
  DevBuf<float4> d;
  DevBuf<float> r;
  if (out_rgbw) CK(d.alloc(npix, st), "render_sppm: alloc");
  if (out_radiance) CK(r.alloc(3 * npix, st), "render_sppm: alloc");
  int rc = sppm_render(s, *cam, *params, out_rgbw ? d.p : nullptr,
                       out_radiance ? r.p : nullptr, st);
  if (rc) {
    cudaStreamSynchronize(st);
    return rc;
  }
  if (out_rgbw)
    CK(cudaMemcpyAsync(out_rgbw, d.p, npix * sizeof(float4),
                       cudaMemcpyDeviceToHost, st),
       "render_sppm: copy out");
  if (out_radiance)
    CK(cudaMemcpyAsync(out_radiance, r.p, 3 * npix * sizeof(float),
                       cudaMemcpyDeviceToHost, st),
       "render_sppm: copy out");
  CK(cudaStreamSynchronize(st), "render_sppm");
  return check_device(ctx);
}

int ajg_render_device(ajg_scene* s, const ajg_camera* cam,
                      const ajg_render_params* params, float* d_out_rgbw,
                      void* stream) {
  if (!s || !cam || !params || !d_out_rgbw) return AJG_ERR_INVALID;
  ajg_ctx* ctx = s->ctx;
  std::lock_guard<std::mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  StreamJoin j(ctx->stream, (cudaStream_t)stream);
  int rc = render_impl(s, *cam, *params, reinterpret_cast<float4*>(d_out_rgbw),
                       0, 0, nullptr, ctx->stream);
  if (rc) return rc;
  CK(cudaGetLastError(), "render_device");
  return AJG_OK;
}

int ajg_render_samples(ajg_scene* s, const ajg_camera* cam,
                       const ajg_render_params* params, uint64_t pixel_begin,
                       uint64_t pixel_end, float* out_li) {
  if (!s || !cam || !params || !out_li) return AJG_ERR_INVALID;
  ajg_ctx* ctx = s->ctx;
  const uint64_t npix = (uint64_t)cam->width * cam->height;
  if (pixel_begin >= pixel_end || pixel_end > npix)
    return fail(ctx, AJG_ERR_INVALID, "pixel range out of the film");
  std::lock_guard<std::mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  cudaStream_t st = ctx->stream;
  const uint64_t count = (pixel_end - pixel_begin) * params->spp * 3;
  DevBuf<float> d;
  CK(d.alloc(count, st), "render_samples: alloc");
  int rc = render_impl(s, *cam, *params, nullptr, pixel_begin, pixel_end, d.p,
                       st);
  if (rc) return rc;
  CK(cudaMemcpyAsync(out_li, d.p, count * sizeof(float), cudaMemcpyDeviceToHost,
                     st),
     "render_samples: copy out");
  CK(cudaStreamSynchronize(st), "render_samples");
  return check_device(ctx);
}

}  // extern "C"
