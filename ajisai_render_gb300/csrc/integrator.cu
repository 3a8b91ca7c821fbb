// Wavefront PT-MIS integrator: PathTracing::TraceMIS / Trace
// (core/renderer/pt.cpp:98-311) split into per-bounce kernels over SoA
// queues, driven by TiledIntegrator::Render's sample loop (pt.cpp:40-73).
//
// A single-job wave holds S samples of a range of pixels (path p -> pixel
// pix0 + p / S, sample s0 + p % S).  A multi-job wave holds chunks of many
// jobs (each its own scene, camera, film and parameters; see Chunk); every
// kernel exists in both forms (template flag MJ), and the multi-job form
// reads the per-path job, scene and sampler key from the wave's tables.
// Per bounce:
//   trace_closest(queue) -> shade (NEE candidates, MIS-BSDF escape ray,
//   continuation, Russian roulette for the next bounce) -> trace_any(shadow
//   queue) -> accumulate (the direct-lighting sum in the reference's order)
// Queues are compacted with warp-ballot appends; every kernel is a
// grid-stride loop that reads its queue length from device memory, so a wave
// needs no host synchronisation and a multi-job wave is one captured graph.
// After the last bounce each pixel adds its S samples to a Kahan-compensated
// float32 film (or a float64 one), and a resolve pass applies the
// reference's 2x2 box footprint.
//
// Sampler dimensions per path (the reference's draw order, pt.cpp:58-61,
// 107-108, 203-216, helper.h, directional_light.cpp:46, env_light.cpp:71):
//   0,1 pixel jitter; 2,3 lens; then per bounce b:
//   [Russian roulette if b > min_bounces]
//   2 per light in scene order (directional: cone u, v; env: v then u --
//     g++ evaluates SampleContinuous's two Next1D() arguments right to left),
//   3 for the MIS BSDF sample, 3 for the continuation sample.
#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <string>

#include "shade.cuh"
#include "trace.cuh"

namespace ajg {
namespace {

#ifndef AJG_SHADE_THREADS
#define AJG_SHADE_THREADS 256
#endif
constexpr int kShadeThreads = AJG_SHADE_THREADS;
constexpr int kClassifyThreads = 256;
// Queue appends of the shading kernels: a block at a time (block_append,
// block-uniform loops), or with AJG_BLOCK_APPEND=0 a warp at a time.
__device__ __forceinline__ uint32_t shade_append(uint32_t* counter,
                                                 bool pred) {
  if constexpr (AJG_BLOCK_APPEND)
    return block_append<1, kShadeThreads / 32>(counter, pred ? 0 : -1);
  else
    return warp_append(counter, pred);
}
#ifndef AJG_SHADE_MIN_BLOCKS
// blocks per SM the shading kernels are compiled for: 512 threads, up to
// 128 registers, no spills (1024 threads: 64)
#define AJG_SHADE_MIN_BLOCKS (512 / AJG_SHADE_THREADS)
#endif
#ifndef AJG_SHADE_GRID
#define AJG_SHADE_GRID 256  // single-job shading grid: blocks per SM
#endif
#ifndef AJG_MJ_SHADE_GRID
#define AJG_MJ_SHADE_GRID 8  // multi-job shading grid: blocks per SM
#endif
#ifndef AJG_SHADE_MIN_BLOCKS_DIFFUSE
// the Lambertian kernels: 1024 threads, 64 registers, no spills
#define AJG_SHADE_MIN_BLOCKS_DIFFUSE (1024 / AJG_SHADE_THREADS)
#endif
template <int MAT>
constexpr int shade_min_blocks() {
  return MAT == AJG_MAT_DIFFUSE ? AJG_SHADE_MIN_BLOCKS_DIFFUSE
                                : AJG_SHADE_MIN_BLOCKS;
}
constexpr int kMaxLights = 15;
constexpr unsigned kFull = 0xffffffffu;

struct WaveArgs {
  DeviceScene s;
  ajg_camera cam;
  JobParams j;
  uint32_t pix0, S, s0, n_paths;
  VisPointD* vp;  // SPPM camera pass: the visible points (else null)
};

// Where a kernel finds the job and the scene of a path: the kernel
// arguments (single job) or the wave tables (multi-job).
template <bool MJ>
struct Src;
template <>
struct Src<false> {
  static __device__ __forceinline__ const JobParams& job(const WaveArgs& a,
                                                         const MJTables&,
                                                         uint32_t) {
    return a.j;
  }
  static __device__ __forceinline__ const DeviceScene& scene(
      const WaveArgs& a, const MJTables&, uint32_t) {
    return a.s;
  }
};
template <>
struct Src<true> {
  static __device__ __forceinline__ const JobParams& job(const WaveArgs&,
                                                         const MJTables& t,
                                                         uint32_t jid) {
    return t.jobs[jid].j;
  }
  static __device__ __forceinline__ const DeviceScene& scene(
      const WaveArgs&, const MJTables& t, uint32_t jid) {
    return t.scenes[mj_scene(t, t.jobs[jid].scene)];
  }
};

__device__ __forceinline__ int dim_base(const JobParams& J, int b) {
  const int rr = b - J.min_b - 1;
  return 4 + b * J.nd + (rr > 0 ? rr : 0);
}

__device__ __forceinline__ void path_id(const WaveArgs& a, uint32_t p,
                                        uint32_t& pixel, uint32_t& sample) {
  pixel = a.pix0 + p / a.S;
  sample = a.s0 + p % a.S;
}

// Last index c in [0, n) with off[c] <= v (off ascending, off[0] == 0).
__device__ __forceinline__ uint32_t find_le(const uint32_t* off, uint32_t n,
                                            uint32_t v) {
  uint32_t lo = 0, hi = n;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (off[mid] <= v)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// The camera sample of one path (pt.cpp:58-61) and the roulette before
// bounce 0.
__device__ __forceinline__ void raygen_path(const ajg_camera& cam,
                                            const JobParams& J, uint64_t key,
                                            int x, int y, F3& ro, F3& rd,
                                            F3& T, bool& alive) {
  const float u = x + key_float(key, 0);
  const float v = y + key_float(key, 1);
  const float l0 = key_float(key, 2), l1 = key_float(key, 3);
  camera_ray(cam, u, v, l0, l1, ro, rd);
  T = mk3(1.f, 1.f, 1.f);
  alive = J.max_b > 0;
  if (alive && 0 > J.min_b) {  // roulette before bounce 0
    if (key_float(key, dim_base(J, 0)) > J.cont) alive = false;
    T = T / J.cont;
  }
}

template <bool MJ>
__global__ void __launch_bounds__(kShadeThreads)
    k_raygen(WaveArgs a, MJTables t, WaveBufs w) {
  __shared__ uint32_t s_off[MJ ? kMaxWaveChunks : 1];
  uint32_t n_paths = a.n_paths, n_chunks = 0;
  const bool all_alive =
      AJG_BLOCK_APPEND && !MJ && a.j.max_b > 0 && !(0 > a.j.min_b);
  if (all_alive && blockIdx.x == 0 && threadIdx.x == 0)
    atomicAdd(&w.counts[0], n_paths);
  if constexpr (MJ) {
    if (!mj_wave_ok(t)) return;  // uniform: every thread reads one header
    n_paths = t.hdr->n_paths;
    n_chunks = t.hdr->n_chunks;
    for (uint32_t c = threadIdx.x; c < n_chunks; c += blockDim.x)
      s_off[c] = t.chunks[c].path_off;
    __syncthreads();
  }
  // block-uniform iterations (block_append synchronises the block)
  for (uint32_t pb = blockIdx.x * blockDim.x; pb < n_paths;
       pb += gridDim.x * blockDim.x) {
    const uint32_t p = pb + threadIdx.x;
    F3 ro = mk3(0, 0, 0), rd = mk3(0, 0, 1), T = mk3(1, 1, 1);
    bool alive = false;
    uint32_t sid = 0;
    if (p >= n_paths) {
      // past the wave: only the queue append below
    } else if constexpr (MJ) {
      const Chunk C = t.chunks[find_le(s_off, n_chunks, p)];
      const uint32_t q = p - C.path_off;
      const uint32_t i = C.pix0 + q / C.S;
      const uint32_t sample = C.s0 + q % C.S;
      const uint32_t jid = mj_job(t, C.job);
      const JobRec& R = t.jobs[jid];
      const int x = (int)(R.j.x0 + i % R.j.win_w);
      const int y = (int)(R.j.y0 + i / R.j.win_w);
      const uint64_t key =
          path_key(R.j.seed, (uint32_t)y * R.j.film_w + (uint32_t)x, sample);
      w.pjob[p] = jid;
      w.pkey[p] = key;
      sid = mj_scene(t, R.scene);
      raygen_path(R.cam, R.j, key, x, y, ro, rd, T, alive);
    } else {
      uint32_t pixel, sample;
      path_id(a, p, pixel, sample);
      const uint64_t key = path_key(a.j.seed, pixel, sample);
      const int x = (int)(pixel % a.cam.width), y = (int)(pixel / a.cam.width);
      raygen_path(a.cam, a.j, key, x, y, ro, rd, T, alive);
    }
    if (p < n_paths) {
      w.thr[p] = make_float4(T.x, T.y, T.z, 0.f);
      w.rad[p] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    // a single job whose paths all start (no roulette before bounce 0) is
    // queued in path order without atomics (the count is added once above)
    const uint32_t k = all_alive ? p : shade_append(&w.counts[0], alive);
    if (alive) {
      w.qpath[0][k] = p;
      w.ro[0][k] = make_float4(ro.x, ro.y, ro.z, __uint_as_float(sid));
      w.rd[0][k] = make_float4(rd.x, rd.y, rd.z, 0.f);
    }
  }
}

// Files every queue slot under its hit's shading class (a miss, Lambertian,
// Disney, or one of the other material types), so that shading runs in
// class-specialised kernels; warps stay converged, so each list append is
// one atomic per warp.
template <bool MJ>
__global__ void __launch_bounds__(kClassifyThreads)
    k_classify(DeviceScene s, MJTables t,
                           const float4* __restrict__ ro,
                           const uint32_t* __restrict__ count,
                           const ajg_hit* __restrict__ hits,
                           uint32_t* __restrict__ lists,
                           uint32_t* __restrict__ list_counts,
                           uint32_t list_cap) {
  const uint32_t n = *count;
  const uint32_t stride = gridDim.x * blockDim.x;
  // block-uniform iterations: block_append synchronises the block
  for (uint32_t bb = blockIdx.x * blockDim.x; bb < n; bb += stride) {
    const uint32_t k = bb + threadIdx.x;
    int cls = -1;
    if (k < n) {
      const int prim = hits[k].prim;
      cls = 0;
      if (prim >= 0) {
        const float4* shade = s.shade;
        const float* materials = s.materials;
        if constexpr (MJ) {
          const DeviceScene& sc = t.scenes[mj_scene(t, __float_as_uint(ro[k].w))];
          shade = sc.shade;
          materials = sc.materials;
        }
        const uint32_t mat =
            __float_as_uint(__ldg(&shade[prim].w)) & 0xffffffu;
        const int type = (int)__ldg(materials + 16 * mat);
        cls = type == AJG_MAT_DIFFUSE ? 1 : (type == AJG_MAT_DISNEY ? 2 : 3);
      }
    }
#if AJG_BLOCK_APPEND
    const uint32_t j = block_append<4, kClassifyThreads / 32>(list_counts, cls);
    if (cls >= 0) lists[(uint64_t)cls * list_cap + j] = k;
#else
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const uint32_t j = warp_append(&list_counts[c], cls == c);
      if (cls == c) lists[(uint64_t)c * list_cap + j] = k;
    }
#endif
  }
}

// The MIS BSDF term from its closest hit (helper.h:223-264): an escaped ray
// sees the environment, one that hits the lit side of an emitter its
// radiance, weighted against AreaLight::Pdf; anything else adds nothing.
template <bool MJ>
__global__ void __launch_bounds__(kShadeThreads)
    k_bsdf_emit(WaveArgs a, MJTables t, WaveBufs w, uint32_t NT, uint32_t cap,
                uint32_t n_max, const float* __restrict__ t_hit,
                const int32_t* __restrict__ prim_hit) {
  const uint32_t n = min(w.counts[9], n_max);
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += gridDim.x * blockDim.x) {
    const uint32_t i = cap - 1 - k;
    const float4 o4 = w.sq_o[i], d4 = w.sq_d[i];
    const uint32_t slot = __float_as_uint(d4.w);
    const uint32_t p = slot / NT;
    const uint32_t jid = MJ ? mj_job(t, w.pjob[p]) : 0u;
    const JobParams& J = Src<MJ>::job(a, t, jid);
    const DeviceScene& s = Src<MJ>::scene(a, t, jid);
    const F3 o = xyz(o4), d = xyz(d4);
    const bool delta = signbit(o4.w);  // see k_shade
    const float pdf = fabsf(o4.w);
    const float4 fs = w.term_f[slot];
    const F3 bf = xyz(fs);
    const float cosv = fs.w;
    const int prim = prim_hit[k];
    F3 fo = mk3(0.f, 0.f, 0.f);
    bool vis = false;
    if (prim < 0) {
      const F3 rad = mk3(J.env_rgb.x, J.env_rgb.y, J.env_rgb.z);
      if (s.env >= 0 && !black3(rad)) {
        const F3 fv = rad * bf * cosv;
        if (delta) {
          fo = mk3(0, 0, 0) + fv / pdf;
        } else {
          const float lp = env_pdf(J.env_mass != 0, d);
          fo = mk3(0, 0, 0) + fv / pdf * power_heuristic(pdf, lp);
        }
        vis = true;
      }
    } else {
      const int li = __ldg(s.tri_emit + prim);
      if (li >= 0) {
        F3 pos, ng;
        emitter_hit(s, o, d, t_hit[k], prim, pos, ng);
        const float* L = s.lights + 12 * li;
        const F3 le =
            dot3(ng, -d) > 0 ? mk3(L[1], L[2], L[3]) : mk3(0.f, 0.f, 0.f);
        if (!black3(le)) {
          const F3 fv = le * bf * cosv;
          if (delta) {
            fo = fv / pdf;
          } else {
            const float lp = area_pdf(L[9], o, pos, ng);
            fo = fv / pdf * power_heuristic(pdf, lp);
          }
          vis = true;
        }
      }
    }
    w.term_f[slot] = make_float4(fo.x, fo.y, fo.z, 0.f);
    w.term_vis[slot] = vis ? 1 : 0;
  }
}

// A shadow ray: to the shadow queue, or -- `top`, the coherent rays of bounce
// 0 in waves without emitters -- to the coherent queue, whose entry k sits
// at cap - 1 - k of the same storage (the two cannot meet: a path appends at
// most NT entries to them together).  Without `split`, `top` is uniform over
// the block (one append); with `split` (uniform) each lane picks its queue
// (an append to each).
template <bool MJ>
__device__ __forceinline__ void emit_shadow(const WaveBufs& w, F3 o, F3 d,
                                            float tmax, uint32_t slot,
                                            uint32_t sid, bool pred,
                                            uint32_t cap, uint32_t* err,
                                            bool top = false,
                                            bool split = false) {
  uint32_t k;
  if (split) {
    const uint32_t kb = shade_append(&w.counts[2], pred && !top);
    const uint32_t kt = shade_append(&w.counts[11], pred && top);
    k = top ? kt : kb;
  } else {
    k = shade_append(&w.counts[top ? 11 : 2], pred);
  }
  if (!pred) return;
  if (k >= cap) {
    raise_device_error(err, kDevQueueOverflow);
    return;
  }
  const uint32_t i = top ? cap - 1 - k : k;
  w.sq_o[i] = make_float4(o.x, o.y, o.z, tmax);
  w.sq_d[i] = make_float4(d.x, d.y, d.z, __uint_as_float(slot));
  if constexpr (MJ) w.sq_scene[i] = (uint16_t)sid;
}

// The closest-hit queue of MIS BSDF rays in scenes with emitters: entry k
// sits at cap - 1 - k of the shadow queue's storage.  A path appends at most
// NT entries to the two queues together (its lights' shadow rays and one
// BSDF ray) and cap = P * NT, so the queues cannot meet.
template <bool MJ>
__device__ __forceinline__ void emit_closest(const WaveBufs& w, F3 o, F3 d,
                                             float pdf, uint32_t slot,
                                             uint32_t sid, bool pred,
                                             uint32_t cap, uint32_t* err) {
  const uint32_t k = shade_append(&w.counts[9], pred);
  if (!pred) return;
  if (k >= cap) {
    raise_device_error(err, kDevQueueOverflow);
    return;
  }
  const uint32_t i = cap - 1 - k;
  w.sq_o[i] = make_float4(o.x, o.y, o.z, pdf);
  w.sq_d[i] = make_float4(d.x, d.y, d.z, __uint_as_float(slot));
  if constexpr (MJ) w.sq_scene[i] = (uint16_t)sid;
}

// Escaped paths: the environment counts only for camera rays
// (pt.cpp:114-121), or on every bounce without MIS (pt.cpp:245-249).  The
// single-job launch is skipped on the host when neither applies.
template <bool MJ>
__global__ void k_shade_miss(WaveArgs a, MJTables t, WaveBufs w, int b,
                             int cur, const uint32_t* __restrict__ list,
                             const uint32_t* __restrict__ count) {
  const uint32_t n = *count;
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n;
       j += gridDim.x * blockDim.x) {
    const uint32_t p = w.qpath[cur][list[j]];
    float4 env = a.j.env_rgb;
    if constexpr (MJ) {
      const uint32_t jid = mj_job(t, w.pjob[p]);
      const JobParams& J = t.jobs[jid].j;
      if (!(b == 0 || !J.use_mis) || Src<true>::scene(a, t, jid).env < 0)
        continue;
      env = J.env_rgb;
    }
    float4 L = w.rad[p];
    L.x += env.x;
    L.y += env.y;
    L.z += env.z;
    w.rad[p] = L;
  }
}

// Shading of the hits on one material type: NEE to every light
// (helper.h:100-133), the MIS BSDF sample (helper.h:209-265), the
// continuation sample (pt.cpp:215-223) and the next bounce's roulette.
template <int MAT, bool MJ>
__global__ void __launch_bounds__(kShadeThreads, shade_min_blocks<MAT>())
    k_shade(WaveArgs a, MJTables t, WaveBufs w, int b, int cur,
            const uint32_t* __restrict__ list,
            const uint32_t* __restrict__ list_count, uint32_t NT,
            uint32_t shadow_cap, uint32_t* err, uint32_t coh = 0) {
  // coh: bit l set -- light term l's shadow rays go to the coherent queue
  // (bit 31: the MIS BSDF term's); multi-job waves: nonzero -- every lane's
  // directional-light rays go there.  Waves without emitters only.
  const uint32_t n = *list_count;
  const int nxt = cur ^ 1;
  // warp-uniform loop (block-uniform for a single job): every lane of a
  // warp (thread of the block) runs the same iterations, so the queue
  // appends see all of them
  constexpr bool kBlockLoop = AJG_BLOCK_APPEND;
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t first = kBlockLoop ? 0u : threadIdx.x - lane;
  for (uint32_t wb = blockIdx.x * blockDim.x + first; wb < n; wb += stride) {
    const uint32_t j = wb + (kBlockLoop ? threadIdx.x : lane);
    const bool hit = j < n;
    uint32_t p = 0, k = 0, jid = 0;
    if (hit) {
      k = list[j];
      p = w.qpath[cur][k];
      if constexpr (MJ) jid = mj_job(t, w.pjob[p]);
    }
    const JobParams& J = Src<MJ>::job(a, t, jid);
    const DeviceScene& s = Src<MJ>::scene(a, t, jid);
    const uint32_t sid = MJ ? mj_scene(t, t.jobs[jid].scene) : 0u;
    HitInfo hi;
    BsdfT<MAT> f;
    F3 T = mk3(0, 0, 0);
    uint64_t key = 0;
    int emitter = -1;
    if (hit) {
      const ajg_hit h = w.hits[k];
      if (s.tri_emit) emitter = __ldg(s.tri_emit + h.prim);
      const F3 ro = xyz(w.ro[cur][k]), rd = xyz(w.rd[cur][k]);
      if constexpr (MJ) {
        key = w.pkey[p];
      } else {
        uint32_t pixel, sample;
        path_id(a, p, pixel, sample);
        key = path_key(a.j.seed, pixel, sample);
      }
      T = xyz(w.thr[p]);
      hi = complete_hit(s, ro, rd, h.t, h.u, h.v, h.prim);
      f.m = s.materials + 16 * hi.mat;
      f.ng = hi.ng;
      f.ns = hi.ns;
      f.lum = __ldg(&s.mat_lum[hi.mat].x);
      w.thr_shade[p] = make_float4(T.x, T.y, T.z, 0.f);
      // an emitter seen by a camera ray, or by any ray without MIS
      // (pt.cpp:185-190, 282-286; AreaLight::Radiance, area_light.cpp:30-34)
      if (emitter >= 0 && (b == 0 || !J.use_mis)) {
        const float* L = s.lights + 12 * emitter;
        const F3 le = dot3(hi.ng, hi.wr) > 0 ? mk3(L[1], L[2], L[3])
                                               : mk3(0.f, 0.f, 0.f);
        const F3 c = T * le;
        float4 R = w.rad[p];
        R.x += c.x;
        R.y += c.y;
        R.z += c.z;
        w.rad[p] = R;
      }
    }
    int dim = dim_base(J, b) + (b > J.min_b ? 1 : 0);
    // lanes of a multi-job block differ in lights and MIS: loop over the
    // block's maximum with the lanes past their own count idle
    const int nl = (int)s.num_lights;
    const bool mis = hit && J.use_mis;
    int nl_loop = nl;
    bool any_mis = J.use_mis != 0;
    if constexpr (MJ && kBlockLoop) {
      nl_loop = (int)block_max<kShadeThreads / 32>(mis ? (unsigned)nl : 0u);
      any_mis = __syncthreads_or(mis) != 0;
    } else if constexpr (MJ) {
      nl_loop = (int)__reduce_max_sync(kFull, mis ? (unsigned)nl : 0u);
      any_mis = __any_sync(kFull, mis);
    }

    if (any_mis) {
      for (int l = 0; l < nl_loop; ++l) {
        const bool on = MJ ? (mis && l < nl) : hit;
        const float* L = s.lights + 12 * (MJ ? (l < nl ? l : 0) : l);
        bool emit = false;
        F3 fo = mk3(0, 0, 0), so = mk3(0, 0, 0), sd = mk3(0, 0, 1);
        float tmax = 0.f;
        int draws = 2;
        if (on) {
          F3 lpos, lrad;
          float lpdf;
          const int type = (int)L[0];
          bool ok = true;
          if (type == kLightArea) {
            // AreaLight::Sample (area_light.cpp:36-57): three draws
            draws = 3;
            const AreaSample g =
                area_sample(L, s.emit_pts, key_float(key, dim),
                            key_float(key, dim + 1), key_float(key, dim + 2));
            lrad = mk3(L[1], L[2], L[3]);
            lpos = g.pos;
            lpdf = 0.f;
            if (dot3(g.ng, hi.pos - g.pos) <= 0) {
              ok = false;
            } else {
              const F3 i2r = hi.pos - g.pos;
              const float dist2 = dot3(i2r, i2r);
              lpdf = g.pdf * dist2 / fabsf(dot3(g.ng, i2r));
            }
          } else if (type == AJG_LIGHT_DIRECTIONAL) {
            const float u0 = key_float(key, dim), u1 = key_float(key, dim + 1);
            const F3 dir = normalize3(mk3(L[4], L[5], L[6]));
            const F3 r2l = Frame(dir).to_world(uniform_cone(u0, u1, L[7]));
            lpdf = uniform_cone_pdf(L[7]);
            lpos = hi.pos + 2.f * s.radius * r2l;
            lrad = mk3(L[1], L[2], L[3]);
          } else {
            // g++ evaluates SampleContinuous's two Next1D() arguments right
            // to left: the first draw is v (env_light.cpp:71-72)
            const float v = key_float(key, dim);
            float u = key_float(key, dim + 1);
            lrad = mk3(L[1], L[2], L[3]);
            lpdf = 0.f;
            lpos = hi.pos;
            if (L[10] == 0.f) {  // the 1x1 distribution has no mass
              ok = false;
            } else {
              constexpr float inv_2_pi = 1.f / (2.f * kPi);
              constexpr float two_pi = 2.f * kPi;
              u -= L[9] / 180 * kPi * inv_2_pi;
              if (u > 1.f) u -= 1.f;
              if (u < 0.f) u += 1.f;
              const float phi = u * two_pi;
              const float theta = v * kPi;
              const float st = sinf(theta);
              lpdf = st != 0.f ? 1.f / (2.f * kPi * kPi * st) : 0.f;
              const F3 dir = mk3(-st * cosf(phi), cosf(theta), -st * sinf(phi));
              lpos = hi.pos + 2.f * s.radius * dir;
            }
          }
          if (ok && !(black3(lrad) || lpdf <= 0.f)) {
            const float len = len3(lpos - hi.pos) - kRayEps;
            if (!(len < kRayEps)) {
              const F3 wl = normalize3(lpos - hi.pos);
              F3 bf;
              float bp;
              f.eval_pdf(wl, hi.wr, bf, bp);
              if (!black3(bf)) {
                // MISSampleAreaLight takes the shading normal as it is, the
                // others normalise it (helper.h:64, 91, 120)
                const F3 nn = type == kLightArea ? hi.ns : normalize3(hi.ns);
                F3 fv;
                if (type != AJG_LIGHT_ENV)
                  fv = mk3(1.f, 1.f, 1.f) * lrad * bf * fabsf(dot3(wl, nn));
                else
                  fv = lrad * bf * fabsf(dot3(wl, nn));
                fo = fv / lpdf * power_heuristic(lpdf, bp);
                make_ray(hi.pos, wl, so, sd);
                tmax = 0.99f * len;
                emit = true;
              }
            }
          }
          const uint32_t slot = p * NT + l;
          w.term_f[slot] = make_float4(fo.x, fo.y, fo.z, 0.f);
          w.term_vis[slot] = 0;
        }
        // to the packet queue: this term's rays (a single job), or a lane's
        // directional-light rays when its job's footprint allows packets
        // (multi-job lanes differ in their l-th light and their job)
        const bool top =
            MJ ? (coh != 0 && on && J.packets &&
                  (int)L[0] == AJG_LIGHT_DIRECTIONAL)
               : (l < 31 && ((coh >> l) & 1u));
        emit_shadow<MJ>(w, so, sd, tmax, p * NT + l, sid, emit, shadow_cap,
                        err, top, MJ && coh != 0);
        if (on) dim += draws;
      }
      {
        // MISSampleBsdf (helper.h:209-265).  Without emitters only the
        // environment can answer, and an any-hit escape test decides; with
        // emitters the closest hit decides, so the ray goes to the closest
        // queue with the BSDF value and |cos| parked in its term and the pdf
        // in the ray (k_bsdf_emit completes the term).
        const bool on = MJ ? mis : hit;
        bool emit = false, closest = false;
        F3 fo = mk3(0, 0, 0), so = mk3(0, 0, 0), sd = mk3(0, 0, 1);
        float w_o = __int_as_float(0x7f800000);
        float cosv = 0.f;
        if (on) {
          const F3 sam = mk3(key_float(key, dim), key_float(key, dim + 1),
                             key_float(key, dim + 2));
          BsdfSample bs = f.sample(hi.wr, sam);
          if (!(black3(bs.f) || bs.pdf == 0.f)) {
            if (s.tri_emit) {
              bs.dir = normalize3(bs.dir);
              make_ray(eps_offset(hi, bs.dir), bs.dir, so, sd);
              fo = bs.f;
              cosv = fabsf(dot3(hi.ns, sd));
              w_o = bs.delta ? -bs.pdf : bs.pdf;  // a delta sample: negated
              closest = true;
            } else if (s.env >= 0) {
              bs.dir = normalize3(bs.dir);
              make_ray(eps_offset(hi, bs.dir), bs.dir, so, sd);
              const F3 rad = mk3(J.env_rgb.x, J.env_rgb.y, J.env_rgb.z);
              if (!black3(rad)) {
                const F3 fv = rad * bs.f * fabsf(dot3(hi.ns, sd));
                // a delta sample is not weighted (helper.h:236-241)
                if (bs.delta) {
                  fo = mk3(0, 0, 0) + fv / bs.pdf;
                } else {
                  const float lp = env_pdf(J.env_mass != 0, sd);
                  fo = mk3(0, 0, 0) +
                       fv / bs.pdf * power_heuristic(bs.pdf, lp);
                }
                emit = true;
              }
            }
          }
          const uint32_t slot = p * NT + (NT - 1);
          w.term_f[slot] = make_float4(fo.x, fo.y, fo.z, cosv);
          w.term_vis[slot] = 0;
          dim += 3;
        }
        emit_shadow<MJ>(w, so, sd, __int_as_float(0x7f800000),
                        p * NT + (NT - 1), sid, emit, shadow_cap, err,
                        !MJ && ((coh >> 31) & 1u));
        // (a single job's scene without emitters never fills this queue:
        // skip its block-wide append; the condition is uniform)
        if (MJ || s.tri_emit)
          emit_closest<MJ>(w, so, sd, w_o, p * NT + (NT - 1), sid, closest,
                           shadow_cap, err);
      }
    }

    // SPPM's camera pass ends a path at its first diffuse surface or its
    // last bounce with a visible point (sppm.cpp:77-92)
    bool vp_here = false;
    if constexpr (!MJ) {
      if (a.vp && hit) {
        bool diffuse;
        if (MAT == AJG_MAT_DIFFUSE)
          diffuse = true;
        else if (MAT == AJG_MAT_DISNEY)
          diffuse = f.m[5] < 1.f;  // DisneyBSDF: metallic < 1
        else
          diffuse = (int)f.m[0] == AJG_MAT_PLASTIC;
        vp_here = diffuse || b == J.max_b - 1;
        if (vp_here && isfinite(T.x) && isfinite(T.y) && isfinite(T.z)) {
          VisPointD v;
          v.pos = make_float4(hi.pos.x, hi.pos.y, hi.pos.z,
                              __uint_as_float(hi.mat));
          v.wr = make_float4(hi.wr.x, hi.wr.y, hi.wr.z, 0.f);
          v.thr = make_float4(T.x, T.y, T.z, 0.f);
          v.ng = make_float4(hi.ng.x, hi.ng.y, hi.ng.z, 0.f);
          v.ns = make_float4(hi.ns.x, hi.ns.y, hi.ns.z, 0.f);
          a.vp[a.pix0 + p / a.S] = v;
        }
      }
    }
    bool alive = false;
    F3 nro = mk3(0, 0, 0), nrd = mk3(0, 0, 1);
    if (hit && !vp_here && b + 1 < J.max_b) {
      const F3 sam = mk3(key_float(key, dim), key_float(key, dim + 1),
                         key_float(key, dim + 2));
      const BsdfSample bs = f.sample(hi.wr, sam);
      if (!(black3(bs.f) || bs.pdf < 0.f)) {
        T = T * (bs.f * fabsf(dot3(hi.ng, bs.dir)) / bs.pdf);
        make_ray(eps_offset(hi, bs.dir), bs.dir, nro, nrd);
        alive = true;
        if (b + 1 > J.min_b) {
          if (key_float(key, dim_base(J, b + 1)) > J.cont)
            alive = false;
          else
            T = T / J.cont;
        }
      }
      w.thr[p] = make_float4(T.x, T.y, T.z, 0.f);
    }
    const uint32_t kn = shade_append(&w.counts[nxt], alive);
    if (alive) {
      w.qpath[nxt][kn] = p;
      w.ro[nxt][kn] = make_float4(nro.x, nro.y, nro.z, __uint_as_float(sid));
      w.rd[nxt][kn] = make_float4(nrd.x, nrd.y, nrd.z, 0.f);
    }
  }
}

// direct_illum += throughput * MISSampleLight(...) for each light, then
// += throughput * MISSampleBsdf(...); pixel.value += direct (pt.cpp:200-213)
template <bool MJ>
__global__ void __launch_bounds__(kShadeThreads)
    k_accumulate(WaveArgs a, MJTables t, WaveBufs w, int cur, uint32_t NT) {
  const uint32_t n = w.counts[cur];
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += gridDim.x * blockDim.x) {
    if (w.hits[k].prim < 0) continue;
    const uint32_t p = w.qpath[cur][k];
    int nl = (int)a.s.num_lights;
    if constexpr (MJ) {
      const JobParams& J = t.jobs[mj_job(t, w.pjob[p])].j;
      if (!J.use_mis) continue;
      nl = J.nl;
      if (nl + 1 > (int)NT) {  // the arena holds NT terms per path
        raise_device_error(t.err, kDevTableOutOfBounds);
        continue;
      }
    }
    const F3 T = xyz(w.thr_shade[p]);
    F3 direct = mk3(0.f, 0.f, 0.f);
    for (int j = 0; j <= nl; ++j) {
      const uint32_t slot = p * NT + (j < nl ? (uint32_t)j : NT - 1);
      const F3 fv = w.term_vis[slot] ? xyz(w.term_f[slot]) : mk3(0, 0, 0);
      direct = direct + T * fv;
    }
    float4 L = w.rad[p];
    const F3 d1 = 1.f / 1 * direct;
    L.x += d1.x;
    L.y += d1.y;
    L.z += d1.z;
    w.rad[p] = L;
  }
}

// Adds S consecutive samples to one film pixel in sample order
// (Kahan-compensated float32, or float64).
__device__ __forceinline__ void film_pixel(const float4* __restrict__ rad,
                                           uint64_t base, uint32_t S,
                                           uint64_t pixel, float4* sum,
                                           float4* comp, double* sum64,
                                           bool drop_nonfinite) {
  if (sum64) {
    double* o = sum64 + 4 * pixel;
    double x = o[0], y = o[1], z = o[2], wsum = o[3];
    for (uint32_t j = 0; j < S; ++j) {
      const float4 L = rad[base + j];
      if (drop_nonfinite &&
          !(isfinite(L.x) && isfinite(L.y) && isfinite(L.z)))
        continue;
      x += L.x;
      y += L.y;
      z += L.z;
      wsum += 1.0;
    }
    o[0] = x;
    o[1] = y;
    o[2] = z;
    o[3] = wsum;
    return;
  }
  float4 s4 = sum[pixel], c4 = comp[pixel];
  for (uint32_t j = 0; j < S; ++j) {
    const float4 L = rad[base + j];
    if (drop_nonfinite && !(isfinite(L.x) && isfinite(L.y) && isfinite(L.z)))
      continue;
    s4.w += 1.f;
    float y, t;
    y = L.x - c4.x; t = s4.x + y; c4.x = (t - s4.x) - y; s4.x = t;
    y = L.y - c4.y; t = s4.y + y; c4.y = (t - s4.y) - y; s4.y = t;
    y = L.z - c4.z; t = s4.z + y; c4.z = (t - s4.z) - y; s4.z = t;
  }
  sum[pixel] = s4;
  comp[pixel] = c4;
}

// Each pixel of the wave adds its S samples in sample order.
template <bool MJ>
__global__ void k_film_add(WaveArgs a, MJTables t,
                           const float4* __restrict__ rad,
                           float4* __restrict__ sum, float4* __restrict__ comp,
                           double* __restrict__ sum64, uint32_t n_pix) {
  __shared__ uint32_t s_off[MJ ? kMaxWaveChunks : 1];
  uint32_t n_chunks = 0;
  if constexpr (MJ) {
    if (!mj_wave_ok(t)) return;  // uniform: every thread reads one header
    n_pix = t.hdr->n_pix;
    n_chunks = t.hdr->n_chunks;
    for (uint32_t c = threadIdx.x; c < n_chunks; c += blockDim.x)
      s_off[c] = t.chunks[c].pix_off;
    __syncthreads();
  }
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_pix;
       i += gridDim.x * blockDim.x) {
    if constexpr (MJ) {
      const Chunk C = t.chunks[find_le(s_off, n_chunks, i)];
      const JobRec& R = t.jobs[mj_job(t, C.job)];
      const uint32_t li = i - C.pix_off;
      if (C.path_off + (uint64_t)(li + 1) * C.S > t.hdr->n_paths) {
        raise_device_error(t.err, kDevTableOutOfBounds);
        continue;
      }
      film_pixel(rad, C.path_off + (uint64_t)li * C.S, C.S, C.pix0 + li,
                 R.fsum, R.fcomp, R.fsum64, R.j.drop_nonfinite != 0);
    } else {
      film_pixel(rad, (uint64_t)i * a.S, a.S, a.pix0 + i, sum, comp, sum64,
                 a.j.drop_nonfinite != 0);
    }
  }
}

// The reference's film convention (film.cpp:27-63, film.h:119-129,
// image.h:38-42): a sample at (x, y) lands on (x-1..x, y-1..y) with weight
// 1, and row/column -1 folds into 0.  Target (tx, ty) thus sums sources
// tx (twice when tx == 0) and tx + 1, likewise in y.  For a window of the
// image the fold applies only where the window starts at row/column 0, and
// sources past the window are absent.  The four terms are summed in
// double: the compensated float32 film carries more than float precision.
__global__ void k_resolve(const float4* __restrict__ sum,
                          const float4* __restrict__ comp,
                          const double* __restrict__ sum64, uint32_t W,
                          uint32_t H, int fold_x, int fold_y,
                          float4* __restrict__ out) {
  const uint64_t npix = (uint64_t)W * H;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < npix;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t tx = (uint32_t)(i % W), ty = (uint32_t)(i / W);
    double r = 0, g = 0, bl = 0, wt = 0;
    for (int dy = 0; dy < 2; ++dy) {
      const uint32_t sy = ty + dy;
      if (sy >= H) continue;
      const int my = (dy == 0 && ty == 0 && fold_y) ? 2 : 1;
      for (int dx = 0; dx < 2; ++dx) {
        const uint32_t sx = tx + dx;
        if (sx >= W) continue;
        const int mx = (dx == 0 && tx == 0 && fold_x) ? 2 : 1;
        const uint64_t src = (uint64_t)sy * W + sx;
        double x, y, z, ww;
        if (sum64) {
          x = sum64[4 * src];
          y = sum64[4 * src + 1];
          z = sum64[4 * src + 2];
          ww = sum64[4 * src + 3];
        } else {
          const float4 s4 = sum[src], c4 = comp[src];
          x = (double)s4.x - (double)c4.x;
          y = (double)s4.y - (double)c4.y;
          z = (double)s4.z - (double)c4.z;
          ww = s4.w;
        }
        const int m = mx * my;
        r += m * x;
        g += m * y;
        bl += m * z;
        wt += m * ww;
      }
    }
    out[i] = make_float4((float)r, (float)g, (float)bl, (float)wt);
  }
}

__global__ void k_copy_li(WaveArgs a, const float4* __restrict__ rad,
                          uint64_t pixel_begin, uint32_t spp,
                          float* __restrict__ out) {
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n_paths;
       p += gridDim.x * blockDim.x) {
    uint32_t pixel, sample;
    path_id(a, p, pixel, sample);
    float* o = out + 3 * (((uint64_t)pixel - pixel_begin) * spp + sample);
    const float4 L = rad[p];
    o[0] = L.x;
    o[1] = L.y;
    o[2] = L.z;
  }
}

int fail(ajg_ctx* ctx, int code, const std::string& m) {
  ctx->last_error = m;
  return code;
}

// SPPM's camera pass: each pixel's direct light (one path per pixel).
__global__ void k_copy_direct(WaveArgs a, const float4* __restrict__ rad,
                              float4* __restrict__ direct) {
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n_paths;
       p += gridDim.x * blockDim.x)
    direct[a.pix0 + p] = rad[p];
}

template <class T>
T* carve(char*& cur, uint64_t count) {
  T* p = reinterpret_cast<T*>(cur);
  cur += ((count * sizeof(T) + 255) / 256) * 256;
  return p;
}

}  // namespace

int resident_grid(const void* fn, int threads) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, int> cache;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(mu);
  auto key = std::make_pair(fn, dev);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  int sms = kSMs, per_sm = 1;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, 0) !=
          cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  const int g = sms * per_sm;
  cache[key] = g;
  return g;
}

uint64_t wave_bytes(uint64_t P, int nt, bool mj) {
  const uint64_t slots = P * nt;
  uint64_t b = 0;
  auto add = [&](uint64_t bytes) { b += ((bytes + 255) / 256) * 256; };
  add(P * 16); add(P * 16); add(P * 16);  // thr, thr_shade, rad
  if (mj) {
    add(P * 4);  // pjob
    add(P * 8);  // pkey
  }
  add(P * 4); add(P * 4);      // qpath
  add(P * 16); add(P * 16);    // ro
  add(P * 16); add(P * 16);    // rd
  add(P * sizeof(ajg_hit));
  add(P * sizeof(ajg_hit));    // hits2
  add(slots * 16);             // term_f
  add(slots);                  // term_vis
  add(slots * 16); add(slots * 16);  // shadow queue
  if (mj) add(slots * 2);      // sq_scene
  add(P * 4 * 4);              // shading-class lists
  add(64);                     // counts
  return b;
}

WaveBufs carve_wave(char* base, uint64_t P, int nt, bool mj) {
  char* cur = base;
  WaveBufs w{};
  w.thr = carve<float4>(cur, P);
  w.thr_shade = carve<float4>(cur, P);
  w.rad = carve<float4>(cur, P);
  if (mj) {
    w.pjob = carve<uint32_t>(cur, P);
    w.pkey = carve<uint64_t>(cur, P);
  }
  w.qpath[0] = carve<uint32_t>(cur, P);
  w.qpath[1] = carve<uint32_t>(cur, P);
  w.ro[0] = carve<float4>(cur, P);
  w.ro[1] = carve<float4>(cur, P);
  w.rd[0] = carve<float4>(cur, P);
  w.rd[1] = carve<float4>(cur, P);
  w.hits = carve<ajg_hit>(cur, P);
  w.hits2 = carve<ajg_hit>(cur, P);
  w.term_f = carve<float4>(cur, P * nt);
  w.term_vis = carve<uint8_t>(cur, P * nt);
  w.sq_o = carve<float4>(cur, P * nt);
  w.sq_d = carve<float4>(cur, P * nt);
  if (mj) w.sq_scene = carve<uint16_t>(cur, P * nt);
  w.lists = carve<uint32_t>(cur, P * 4);
  w.counts = carve<uint32_t>(cur, 16);
  return w;
}

// The wave arena: one device allocation reused across renders of the
// context, grown when a render needs more paths or light terms.
static int ensure_arena(ajg_ctx* ctx, uint64_t P, int nt, char** base) {
  const uint64_t need = wave_bytes(P, nt, false);
  if (ctx->arena.empty() || ctx->arena[0].bytes < need) {
    for (auto& b : ctx->arena) cudaFree(b.ptr);
    ctx->arena.clear();
    Buffer b;
    if (cudaMalloc(&b.ptr, need) != cudaSuccess)
      return fail(ctx, AJG_ERR_OOM, "device allocation failed (wave arena)");
    b.bytes = need;
    ctx->arena.push_back(b);
  }
  *base = static_cast<char*>(ctx->arena[0].ptr);
  return AJG_OK;
}

// Paths per wave of a single-job render: the context's wave size, but no
// more than the render needs (its paths, in whole KiB) and no more than
// kArenaBytes of wave state for its light count.
constexpr uint64_t kArenaBytes = 96ull << 30;
static uint64_t job_wave_paths(const ajg_ctx* ctx, uint64_t needed, int nt) {
  const uint64_t per_path = (wave_bytes(1u << 20, nt, false) >> 20) + 1;
  uint64_t P = std::min<uint64_t>(ctx->wave_paths, (needed + 1023) / 1024 * 1024);
  P = std::min<uint64_t>(P, kArenaBytes / per_path);
  // the shadow queue (P x nt entries) is indexed by the traversal's 32-bit
  // signed ray numbers, with 2^31 - 1 reserved
  P = std::min<uint64_t>(P, ((1ull << 31) - 2) / (uint64_t)nt);
  return std::max<uint64_t>(1024, P / 1024 * 1024);
}

int check_render(ajg_ctx* ctx, const DeviceScene& s, const ajg_camera& cam,
                 const ajg_render_params& prm) {
  if (cam.width == 0 || cam.height == 0 || prm.spp == 0)
    return fail(ctx, AJG_ERR_INVALID, "empty film or zero spp");
  if (prm.max_bounces < 0 || prm.max_bounces > 1024)
    return fail(ctx, AJG_ERR_INVALID, "max_bounces must be in [0, 1024]");
  if (s.num_lights > kMaxLights)
    return fail(ctx, AJG_ERR_UNSUPPORTED, "at most 15 lights");
  if ((uint64_t)cam.width * cam.height > (1ull << 31))
    return fail(ctx, AJG_ERR_INVALID, "film too large");
  return AJG_OK;
}

// Whether a pixel's samples fall within a few triangles of each other, so
// that bounce 0's directional-light shadow rays pay as packets (a packet
// walks the union of its rays' traversals, which near their origins grows
// with the triangles they span): the pixel's footprint at the world box's
// centre -- the angle between the rays through the film centre and the
// pixel beside it, times the camera's distance to that centre -- against
// kPacketSpread median triangle edges.
static bool packets_pay(const ajg_scene* sc, const ajg_camera& cam) {
  auto apply = [](const float* m, const float v[4], float o[4]) {
    for (int r = 0; r < 4; ++r) {
      o[r] = 0.f;
      for (int c = 0; c < 4; ++c) o[r] += m[c * 4 + r] * v[c];
    }
  };
  const float cx = 0.5f * (float)cam.width, cy = 0.5f * (float)cam.height;
  const float p0[4] = {cx, cy, 1.f, 1.f}, p1[4] = {cx + 1.f, cy, 1.f, 1.f};
  float q0[4], q1[4];
  apply(cam.raster2camera, p0, q0);
  apply(cam.raster2camera, p1, q1);
  auto unit = [](const float q[4], double u[3]) {
    const double n = std::sqrt((double)q[0] * q[0] + (double)q[1] * q[1] +
                               (double)q[2] * q[2]);
    for (int k = 0; k < 3; ++k) u[k] = n > 0 ? q[k] / n : 0.0;
  };
  double u0[3], u1[3];
  unit(q0, u0);
  unit(q1, u1);
  const double angle = std::sqrt((u1[0] - u0[0]) * (u1[0] - u0[0]) +
                                 (u1[1] - u0[1]) * (u1[1] - u0[1]) +
                                 (u1[2] - u0[2]) * (u1[2] - u0[2]));
  const float* m = cam.camera2world;  // column-major: translation in 12..14
  double dist2 = 0.0;
  for (int k = 0; k < 3; ++k) {
    const double c = 0.5 * ((double)sc->world[k] + sc->world[k + 3]);
    const double e = (double)m[12 + k] / (m[15] != 0.f ? m[15] : 1.f) - c;
    dist2 += e * e;
  }
  return angle * std::sqrt(dist2) <= (double)sc->d.packet_spread;
}

JobParams make_job_params(const ajg_scene* sc, const ajg_camera& cam,
                          const ajg_render_params& prm) {
  const DeviceScene& s = sc->d;
  JobParams j{};
  j.seed = prm.seed;
  j.min_b = prm.min_bounces;
  j.max_b = prm.max_bounces;
  j.cont = prm.cont_prob;
  j.use_mis = prm.use_mis ? 1 : 0;
  j.nl = (int)s.num_lights;
  // draws per bounce: 2 per directional or env light, 3 per area light,
  // 3 for the MIS BSDF sample and 3 for the continuation
  j.nd = j.use_mis ? (2 * j.nl + (int)s.num_area + 6) : 3;
  j.env_rgb = make_float4(0, 0, 0, 0);
  j.env_mass = 0;
  if (s.env >= 0) {
    const float* L = sc->host_lights.data() + 12 * s.env;
    // EnvLight::Radiance = scaler * texel (env_light.cpp:65)
    j.env_rgb = make_float4(L[8] * L[1], L[8] * L[2], L[8] * L[3], 0.f);
    j.env_mass = L[11] != 0.f ? 1 : 0;
  }
  j.drop_nonfinite = (prm.flags & AJG_RENDER_DROP_NONFINITE) ? 1 : 0;
  j.film_w = cam.width;
  j.film_h = cam.height;
  j.x0 = j.y0 = 0;
  j.win_w = cam.width;
  j.win_h = cam.height;
  j.packets = packets_pay(sc, cam) ? 1 : 0;
  return j;
}

// The sample loop of one render over zeroed film accumulators: waves of S
// samples of a pixel range, the bounce loop per wave, the film update per
// wave and the footprint resolve at the end.  `timers` enables the
// profiling events of the traversal and shading launches.
static void run_waves(ajg_scene* sc, const ajg_camera& cam,
                      const ajg_render_params& prm, const WaveBufs& w,
                      uint64_t P, float4* fsum, float4* fcomp, double* fsum64,
                      float4* d_out, uint64_t li_begin, uint64_t li_end,
                      float* d_li, cudaStream_t st, bool timers,
                      VisPointD* vp = nullptr, float4* d_direct = nullptr) {
  ajg_ctx* ctx = sc->ctx;
  const DeviceScene& s = sc->d;
  const int nt = (int)s.num_lights + 1;
  const uint64_t npix_all = (uint64_t)cam.width * cam.height;
  const bool want_film = d_out != nullptr;
  const int kc = timers ? kKindClosest : -1;
  const int ka = timers ? kKindAny : -1;
  const int ks = timers ? kKindShade : -1;
  const int kcp = timers ? kKindClosestPacket : -1;
  const int kap = timers ? kKindAnyPacket : -1;
  const MJTables t{};

  WaveArgs a;
  a.s = s;
  a.cam = cam;
  a.j = make_job_params(sc, cam, prm);
  a.vp = vp;

  const uint64_t pb = d_li ? li_begin : 0;
  const uint64_t pe = d_li ? li_end : npix_all;
  const uint64_t npix = pe - pb;
  uint64_t S = std::min<uint64_t>(prm.spp, std::max<uint64_t>(1, P / npix));
  const uint64_t chunk = std::min<uint64_t>(npix, P / S);
  const uint32_t shadow_cap = (uint32_t)(P * nt);
  const int gs = kSMs * 8;
  // persistent traversal: resident blocks only
  const DeviceScene s_closest = closest_view(s);
  // bounce 0's camera rays (a pixel's samples side by side in the queue) as
  // masked packets over the binary layout (AJG_PACKET_CAMERA)
  const bool cam_packets = ctx->packet_camera && s_closest.width == 2;
  auto extend = [&](int q, ajg_hit* hits, cudaStream_t es, bool cam) {
    if (cam)
      launch_wave_extend_packet(false, s_closest.tri_test, s_closest, t,
                                w.ro[q], w.rd[q], &w.counts[q], &w.counts[8],
                                hits, &ctx->d_counters[0], ctx->d_error, es);
    else
      launch_wave_extend(false, s_closest.tri_test, s_closest.width, s_closest,
                         t, w.ro[q], w.rd[q], &w.counts[q], &w.counts[8], hits,
                         &ctx->d_counters[0], ctx->d_error, es);
  };
  // Bounce b+1's closest hits run on the trace stream beside bounce b's
  // shadow rays: the two persistent launches fill each other's drain.  The
  // hits alternate between two buffers by bounce parity (k_accumulate of
  // bounce b still reads its own); everything else bounce b+1 touches is
  // written after k_accumulate of bounce b on the render stream.
  const bool overlap = ctx->overlap && !ctx->profiling && w.hits2 != nullptr;
  cudaStream_t ts = ctx->trace_stream;
  auto extend_ahead = [&](int q, ajg_hit* hits, bool cam) {
    cudaEventRecord(ctx->ev_queue, st);
    cudaStreamWaitEvent(ts, ctx->ev_queue, 0);
    cudaMemsetAsync(&w.counts[8], 0, sizeof(uint32_t), ts);
    KernelTimer tm(ctx, ts, cam ? kcp : kc);
    extend(q, hits, ts, cam);
    cudaEventRecord(ctx->ev_hits, ts);
  };
  auto bsdf_closest = [&]() {
    launch_wave_bsdf_trace(false, s_closest.tri_test, s_closest.width, s_closest, t,
                           w.sq_o, w.sq_d,
                           nullptr, &w.counts[9], &w.counts[10], shadow_cap,
                           (uint32_t)P, reinterpret_cast<float*>(w.lists),
                           reinterpret_cast<int32_t*>(w.lists + P),
                           &ctx->d_counters[0], ctx->d_error, st);
  };
  auto shadow = [&]() {
    launch_wave_shadow(false, s.tri_test, s.width, s, t, w.sq_o, w.sq_d, nullptr,
                       &w.counts[2], &w.counts[3], w.term_vis,
                       &ctx->d_counters[1], ctx->d_error, st);
  };
  // Coherent shadow rays: at bounce 0 a shading block's rays of one light
  // term are a pixel's samples (one origin region; toward a directional
  // light, one direction), traced as masked packets from a queue of their
  // own.  Single jobs without emitters (the BSDF rays of scenes with
  // emitters use the top of the storage) over the plain 4-wide tree.
  uint32_t coh0 = 0;
  if (ctx->packet_shadow > 0 && !s.tri_emit && s.width == 4 && a.j.use_mis &&
      (a.j.packets || ctx->packet_shadow >= 2)) {
    for (int l = 0; l < (int)s.num_lights && l < 31; ++l)
      if (ctx->packet_shadow == 2 ||
          (int)sc->host_lights[12 * l] == AJG_LIGHT_DIRECTIONAL)
        coh0 |= 1u << l;
    if (ctx->packet_shadow >= 2) coh0 |= 1u << 31;  // 3: directional + BSDF
  }
  auto shadow_packets = [&]() {
    launch_wave_shadow_packet(false, s.tri_test, s, t, w.sq_o, w.sq_d, nullptr,
                              &w.counts[11], &w.counts[12], shadow_cap,
                              w.term_vis, &ctx->d_counters[1], ctx->d_error,
                              st);
  };
  for (uint64_t s0 = 0; s0 < prm.spp; s0 += S) {
    const uint64_t Sw = std::min<uint64_t>(S, prm.spp - s0);
    for (uint64_t p0 = pb; p0 < pe; p0 += chunk) {
      const uint64_t n_pix = std::min<uint64_t>(chunk, pe - p0);
      a.pix0 = (uint32_t)p0;
      a.S = (uint32_t)Sw;
      a.s0 = (uint32_t)s0;
      a.n_paths = (uint32_t)(n_pix * Sw);
      // shading grids: many short blocks (the block-wide loop waits on its
      // slowest warp each round; small blocks of work keep the SMs evenly
      // busy to the end), never more than the wave's paths need
      const int gsh = grid_for(a.n_paths, kShadeThreads, kSMs * AJG_SHADE_GRID);
      cudaMemsetAsync(w.counts, 0, 64, st);
      KernelTimer{ctx, st, -1};
      k_raygen<false><<<grid_for(a.n_paths, kShadeThreads, gs), kShadeThreads,
                        0, st>>>(a, t, w);
      int q = 0;
      if (overlap && a.j.max_b > 0) extend_ahead(0, w.hits, cam_packets);
      for (int b = 0; b < a.j.max_b; ++b) {
        WaveBufs wb = w;
        const uint32_t coh = b < ctx->packet_bounces ? coh0 : 0u;
        if (overlap) {
          wb.hits = (b & 1) ? w.hits2 : w.hits;
          cudaStreamWaitEvent(st, ctx->ev_hits, 0);
        }
        // next queue, shadow queues, fetch counters and material lists
        cudaMemsetAsync(&w.counts[q ^ 1], 0, sizeof(uint32_t), st);
        if (overlap) {
          cudaMemsetAsync(&w.counts[2], 0, 6 * sizeof(uint32_t), st);
          cudaMemsetAsync(&w.counts[9], 0, 4 * sizeof(uint32_t), st);
        } else {
          cudaMemsetAsync(&w.counts[2], 0, 11 * sizeof(uint32_t), st);
          const bool cam = b == 0 && cam_packets;
          KernelTimer tm(ctx, st, cam ? kcp : kc);
          extend(q, w.hits, st, cam);
        }
        {
          KernelTimer tm(ctx, st, -1);
          k_classify<false><<<gs, kClassifyThreads, 0, st>>>(s, t, w.ro[q], &w.counts[q],
                                                wb.hits, w.lists, &w.counts[4],
                                                (uint32_t)P);
        }
        if ((b == 0 || !a.j.use_mis) && s.env >= 0) {
          KernelTimer tm(ctx, st, ks);
          k_shade_miss<false><<<gs, kShadeThreads, 0, st>>>(
              a, t, wb, b, q, w.lists, &w.counts[4]);
        }
        // one shading launch per material class the scene has
        if (s.mat_mask & (1u << AJG_MAT_DIFFUSE)) {
          KernelTimer tm(ctx, st, ks);
          k_shade<AJG_MAT_DIFFUSE, false><<<gsh, kShadeThreads, 0, st>>>(
              a, t, wb, b, q, w.lists + P, &w.counts[5], (uint32_t)nt,
              shadow_cap, ctx->d_error, coh);
        }
        if (s.mat_mask & (1u << AJG_MAT_DISNEY)) {
          KernelTimer tm(ctx, st, ks);
          k_shade<AJG_MAT_DISNEY, false><<<gsh, kShadeThreads, 0, st>>>(
              a, t, wb, b, q, w.lists + 2 * P, &w.counts[6], (uint32_t)nt,
              shadow_cap, ctx->d_error, coh);
        }
        if (s.mat_mask >> AJG_MAT_MIRROR) {
          KernelTimer tm(ctx, st, ks);
          k_shade<kMatOther, false><<<gsh, kShadeThreads, 0, st>>>(
              a, t, wb, b, q, w.lists + 3 * P, &w.counts[7], (uint32_t)nt,
              shadow_cap, ctx->d_error, coh);
        }
        if (overlap && b + 1 < a.j.max_b)
          extend_ahead(q ^ 1, (b & 1) ? w.hits : w.hits2, false);
        if (a.j.use_mis) {
          {
            KernelTimer tm(ctx, st, ka);
            shadow();
          }
          if (coh) {
            KernelTimer tm(ctx, st, kap);
            shadow_packets();
          }
          if (s.tri_emit) {
            {
              KernelTimer tm(ctx, st, kc);
              bsdf_closest();
            }
            KernelTimer{ctx, st, -1};
            k_bsdf_emit<false><<<gs, kShadeThreads, 0, st>>>(
                a, t, w, (uint32_t)nt, shadow_cap, (uint32_t)P,
                reinterpret_cast<const float*>(w.lists),
                reinterpret_cast<const int32_t*>(w.lists + P));
          }
          KernelTimer{ctx, st, -1};
          k_accumulate<false><<<gs, kShadeThreads, 0, st>>>(a, t, wb, q,
                                                            (uint32_t)nt);
        }
        q ^= 1;
      }
      if (want_film) KernelTimer{ctx, st, -1};
      if (want_film)
        k_film_add<false><<<grid_for(n_pix, 256, gs), 256, 0, st>>>(
            a, t, w.rad, fsum, fcomp, fsum64, (uint32_t)n_pix);
      if (d_li) KernelTimer{ctx, st, -1};
      if (d_li)
        k_copy_li<<<grid_for(a.n_paths, 256, gs), 256, 0, st>>>(
            a, w.rad, li_begin, prm.spp, d_li);
      if (d_direct) {
        KernelTimer{ctx, st, -1};
        k_copy_direct<<<grid_for(a.n_paths, 256, gs), 256, 0, st>>>(
            a, w.rad, d_direct);
      }
    }
  }
  if (want_film) {
    KernelTimer{ctx, st, -1};
    k_resolve<<<grid_for(npix_all, 256, gs), 256, 0, st>>>(
        fsum, fcomp, fsum64, cam.width, cam.height, 1, 1, d_out);
  }
  ctx->paths_total += (unsigned long long)npix * prm.spp;
}

void enqueue_mj_wave(const MJTables& t, const WaveBufs& w, uint64_t P,
                     int NT, int bounces, int tri_test, int width, bool emit,
                     TraceCounters* ctr, uint32_t* err, cudaStream_t st,
                     cudaStream_t ts, cudaEvent_t ev_queue,
                     cudaEvent_t ev_hits, bool cam_packets,
                     bool shadow_packets) {
  const DeviceScene s{};
  WaveArgs a{};
  const uint32_t shadow_cap = (uint32_t)(P * NT);
  const int gs = kSMs * 8;
  const int gsh = grid_for(P, kShadeThreads, kSMs * AJG_MJ_SHADE_GRID);
  // bounce 0's camera rays (each chunk's paths a pixel's samples side by
  // side) as masked packets when the closest hits walk binary trees
  const bool cam_ok = cam_packets && closest_width(width) == 2;
  // and its directional-light shadow rays, in waves without emitters over
  // plain 4-wide trees
  const bool shadow_ok = shadow_packets && !emit && width == 4;
  auto extend = [&](int q, ajg_hit* hits, cudaStream_t es, bool cam) {
    if (cam)
      launch_wave_extend_packet(true, tri_test, s, t, w.ro[q], w.rd[q],
                                &w.counts[q], &w.counts[8], hits, ctr, err, es);
    else
      launch_wave_extend(true, tri_test, closest_width(width), s, t, w.ro[q],
                         w.rd[q], &w.counts[q], &w.counts[8], hits, ctr, err,
                         es);
  };
  // bounce b+1's closest hits on the trace stream beside bounce b's shadow
  // rays, as in the single-job waves (run_waves)
  const bool overlap = ts && ev_queue && ev_hits && w.hits2;
  auto extend_ahead = [&](int q, ajg_hit* hits, bool cam) {
    cudaEventRecord(ev_queue, st);
    cudaStreamWaitEvent(ts, ev_queue, 0);
    cudaMemsetAsync(&w.counts[8], 0, sizeof(uint32_t), ts);
    extend(q, hits, ts, cam);
    cudaEventRecord(ev_hits, ts);
  };
  cudaMemsetAsync(w.counts, 0, 64, st);
  k_raygen<true><<<gs, kShadeThreads, 0, st>>>(a, t, w);
  int q = 0;
  if (overlap && bounces > 0) extend_ahead(0, w.hits, cam_ok);
  for (int b = 0; b < bounces; ++b) {
    WaveBufs wb = w;
    if (overlap) {
      wb.hits = (b & 1) ? w.hits2 : w.hits;
      cudaStreamWaitEvent(st, ev_hits, 0);
    }
    const uint32_t coh = b == 0 && shadow_ok ? 1u : 0u;
    cudaMemsetAsync(&w.counts[q ^ 1], 0, sizeof(uint32_t), st);
    if (overlap) {
      cudaMemsetAsync(&w.counts[2], 0, 6 * sizeof(uint32_t), st);
      cudaMemsetAsync(&w.counts[9], 0, 4 * sizeof(uint32_t), st);
    } else {
      cudaMemsetAsync(&w.counts[2], 0, 11 * sizeof(uint32_t), st);
      extend(q, w.hits, st, b == 0 && cam_ok);
    }
    k_classify<true><<<gs, kClassifyThreads, 0, st>>>(s, t, w.ro[q], &w.counts[q], wb.hits,
                                         w.lists, &w.counts[4], (uint32_t)P);
    k_shade_miss<true><<<gs, kShadeThreads, 0, st>>>(a, t, wb, b, q, w.lists,
                                                     &w.counts[4]);
    k_shade<AJG_MAT_DIFFUSE, true><<<gsh, kShadeThreads, 0, st>>>(
        a, t, wb, b, q, w.lists + P, &w.counts[5], (uint32_t)NT, shadow_cap,
        err, coh);
    k_shade<AJG_MAT_DISNEY, true><<<gsh, kShadeThreads, 0, st>>>(
        a, t, wb, b, q, w.lists + 2 * P, &w.counts[6], (uint32_t)NT,
        shadow_cap, err, coh);
    k_shade<kMatOther, true><<<gsh, kShadeThreads, 0, st>>>(
        a, t, wb, b, q, w.lists + 3 * P, &w.counts[7], (uint32_t)NT,
        shadow_cap, err, coh);
    if (overlap && b + 1 < bounces)
      extend_ahead(q ^ 1, (b & 1) ? w.hits : w.hits2, false);
    launch_wave_shadow(true, tri_test, width, s, t, w.sq_o, w.sq_d, w.sq_scene,
                       &w.counts[2], &w.counts[3], w.term_vis, ctr + 1, err, st);
    if (coh)
      launch_wave_shadow_packet(true, tri_test, s, t, w.sq_o, w.sq_d,
                                w.sq_scene, &w.counts[11], &w.counts[12],
                                shadow_cap, w.term_vis, ctr + 1, err, st);
    if (emit) {
      launch_wave_bsdf_trace(true, tri_test, closest_width(width), s, t, w.sq_o, w.sq_d,
                             w.sq_scene, &w.counts[9], &w.counts[10], shadow_cap,
                             (uint32_t)P, reinterpret_cast<float*>(w.lists),
                             reinterpret_cast<int32_t*>(w.lists + P), ctr, err,
                             st);
      k_bsdf_emit<true><<<gs, kShadeThreads, 0, st>>>(
          a, t, w, (uint32_t)NT, shadow_cap, (uint32_t)P,
          reinterpret_cast<const float*>(w.lists),
          reinterpret_cast<const int32_t*>(w.lists + P));
    }
    k_accumulate<true><<<gs, kShadeThreads, 0, st>>>(a, t, wb, q,
                                                     (uint32_t)NT);
    q ^= 1;
  }
  k_film_add<true><<<gs, 256, 0, st>>>(a, t, w.rad, nullptr, nullptr, nullptr,
                                       0);
}

void enqueue_resolve(const float4* fsum, const float4* fcomp,
                     const double* fsum64, uint32_t w, uint32_t h,
                     bool fold_x, bool fold_y, float4* out, cudaStream_t st) {
  k_resolve<<<grid_for((uint64_t)w * h, 256, kSMs * 8), 256, 0, st>>>(
      fsum, fcomp, fsum64, w, h, fold_x ? 1 : 0, fold_y ? 1 : 0, out);
}

int render_impl(ajg_scene* sc, const ajg_camera& cam,
                const ajg_render_params& prm, float4* d_out,
                uint64_t li_begin, uint64_t li_end, float* d_li,
                cudaStream_t st) {
  ajg_ctx* ctx = sc->ctx;
  const DeviceScene& s = sc->d;
  int rc = check_render(ctx, s, cam, prm);
  if (rc) return rc;
  const int nt = (int)s.num_lights + 1;
  const uint64_t npix_all = (uint64_t)cam.width * cam.height;
  const uint64_t npix_job = d_li ? std::min(li_end, npix_all) - li_begin : npix_all;
  const uint64_t P = job_wave_paths(ctx, npix_job * prm.spp, nt);
  char* base = nullptr;
  rc = ensure_arena(ctx, P, nt, &base);
  if (rc) return rc;
  const WaveBufs w = carve_wave(base, P, nt, false);

  // film accumulators: per pixel a float32 sum and Kahan compensation, or a
  // float64 sum
  const bool fp64 = (prm.flags & AJG_RENDER_FP64_FILM) != 0;
  float4 *fsum = nullptr, *fcomp = nullptr;
  double* fsum64 = nullptr;
  if (d_out) {
    if (fp64) {
      if (cudaMallocAsync((void**)&fsum64, npix_all * 32, st) != cudaSuccess)
        return fail(ctx, AJG_ERR_OOM, "device allocation failed (film)");
      cudaMemsetAsync(fsum64, 0, npix_all * 32, st);
    } else {
      if (cudaMallocAsync((void**)&fsum, npix_all * 32, st) != cudaSuccess)
        return fail(ctx, AJG_ERR_OOM, "device allocation failed (film)");
      fcomp = fsum + npix_all;
      cudaMemsetAsync(fsum, 0, npix_all * 32, st);
    }
  }
  run_waves(sc, cam, prm, w, P, fsum, fcomp, fsum64, d_out, li_begin, li_end,
            d_li, st, true);
  if (fsum) cudaFreeAsync(fsum, st);
  if (fsum64) cudaFreeAsync(fsum64, st);
  return AJG_OK;
}

int render_in_scratch(ajg_scene* sc, const ajg_camera& cam,
                      const ajg_render_params& prm, float4* d_out,
                      cudaStream_t st, char* scratch, uint64_t bytes) {
  ajg_ctx* ctx = sc->ctx;
  const DeviceScene& s = sc->d;
  int rc = check_render(ctx, s, cam, prm);
  if (rc) return rc;
  const int nt = (int)s.num_lights + 1;
  const uint64_t npix = (uint64_t)cam.width * cam.height;
  const uint64_t film_bytes = ((npix * 32 + 255) / 256) * 256;
  const uint64_t min_wave = wave_bytes(1024, nt, false);
  if (film_bytes + min_wave > bytes)
    return fail(ctx, AJG_ERR_INVALID,
                "film of " + std::to_string(npix) + " pixels needs " +
                    std::to_string(film_bytes + min_wave) +
                    " bytes of scratch; the static scratch holds " +
                    std::to_string(bytes) + " (at most " +
                    std::to_string((bytes - min_wave) / 32) + " pixels)");
  uint64_t P = 1024;
  while (wave_bytes(P + 1024, nt, false) + film_bytes <= bytes) P += 1024;
  float4* fsum = nullptr;
  float4* fcomp = nullptr;
  double* fsum64 = nullptr;
  // the scratch keeps the previous call's contents: zero the film
  if (prm.flags & AJG_RENDER_FP64_FILM) {
    fsum64 = reinterpret_cast<double*>(scratch);
  } else {
    fsum = reinterpret_cast<float4*>(scratch);
    fcomp = fsum + npix;
  }
  cudaMemsetAsync(scratch, 0, npix * 32, st);
  const WaveBufs w = carve_wave(scratch + film_bytes, P, nt, false);
  run_waves(sc, cam, prm, w, P, fsum, fcomp, fsum64, d_out, 0, 0, nullptr, st,
            false);
  return AJG_OK;
}

int sppm_camera_pass(ajg_scene* sc, const ajg_camera& cam, int fmd,
                     uint64_t seed, VisPointD* vp, float4* direct,
                     cudaStream_t st) {
  ajg_ctx* ctx = sc->ctx;
  // TracerVP is TraceMIS without roulette that stops at a visible point:
  // min = max bounces = fmd, sample 0 of each pixel (SetSeed(x + y W))
  ajg_render_params prm{};
  prm.spp = 1;
  prm.min_bounces = fmd;
  prm.max_bounces = fmd;
  prm.cont_prob = 1.f;
  prm.use_mis = 1;
  prm.seed = seed;
  int rc = check_render(ctx, sc->d, cam, prm);
  if (rc) return rc;
  const int nt = (int)sc->d.num_lights + 1;
  const uint64_t npix = (uint64_t)cam.width * cam.height;
  const uint64_t P = job_wave_paths(ctx, npix, nt);
  char* base = nullptr;
  rc = ensure_arena(ctx, P, nt, &base);
  if (rc) return rc;
  const WaveBufs w = carve_wave(base, P, nt, false);
  cudaMemsetAsync(vp, 0xff, npix * sizeof(VisPointD), st);
  run_waves(sc, cam, prm, w, P, nullptr, nullptr, nullptr, nullptr, 0, 0,
            nullptr, st, false, vp, direct);
  return AJG_OK;
}

}  // namespace ajg
