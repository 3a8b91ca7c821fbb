// Wavefront PT-MIS integrator: PathTracing::TraceMIS / Trace
// (core/renderer/pt.cpp:98-311) split into per-bounce kernels over SoA
// queues, driven by TiledIntegrator::Render's sample loop (pt.cpp:40-73).
//
// A wave holds S samples of a range of pixels (path p -> pixel pix0 + p / S,
// sample s0 + p % S).  Per bounce:
//   trace_closest(queue) -> shade (NEE candidates, MIS-BSDF escape ray,
//   continuation, Russian roulette for the next bounce) -> trace_any(shadow
//   queue) -> accumulate (the direct-lighting sum in the reference's order)
// Queues are compacted with warp-ballot appends; every kernel is a
// grid-stride loop that reads its queue length from device memory, so a wave
// needs no host synchronisation.  After the last bounce each pixel adds its
// S samples to a Kahan-compensated float32 film (or a float64 one), and a
// resolve pass applies the reference's 2x2 box footprint.
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
#include <string>

#include "shade.cuh"
#include "trace.cuh"

namespace ajg {
namespace {

constexpr int kShadeThreads = 128;
#ifndef AJG_SHADE_MIN_BLOCKS
#define AJG_SHADE_MIN_BLOCKS 8
#endif
#ifndef AJG_TRACE_MIN_BLOCKS
#define AJG_TRACE_MIN_BLOCKS 1
#endif
#ifndef AJG_TRACE_BLOCKS_PER_SM
#define AJG_TRACE_BLOCKS_PER_SM 10
#endif
constexpr int kMaxLights = 15;

struct WaveArgs {
  DeviceScene s;
  ajg_camera cam;
  uint64_t seed;
  uint32_t pix0, S, s0, n_paths;
  int32_t min_b, max_b;
  float cont;
  int use_mis;
  int nd;  // draws per bounce without the roulette draw
  float4 env_rgb;  // scaler * texel of the scene's env light
  int env_mass;    // the env light's Distribution2D::Pdf is nonzero
};

struct WaveBufs {
  // by path
  float4* thr;
  float4* thr_shade;
  float4* rad;
  // by queue slot (double buffered)
  uint32_t* qpath[2];
  float4* ro[2];
  float4* rd[2];
  ajg_hit* hits;
  // shadow terms: slot = path * (lights + 1) + term
  float4* term_f;
  uint8_t* term_vis;
  float4* sq_o;  // o.xyz, t_max
  float4* sq_d;  // d.xyz, slot bits
  uint32_t* lists;   // [3][P]: queue slots of misses, Lambertian and
                     // Disney hits
  uint32_t* counts;  // [0],[1] path queues, [2] shadow queue, [3] shadow
                     // fetch, [4..6] lists, [7] extend fetch
};

__device__ __forceinline__ int dim_base(const WaveArgs& a, int b) {
  const int rr = b - a.min_b - 1;
  return 4 + b * a.nd + (rr > 0 ? rr : 0);
}

__device__ __forceinline__ void path_id(const WaveArgs& a, uint32_t p,
                                        uint32_t& pixel, uint32_t& sample) {
  pixel = a.pix0 + p / a.S;
  sample = a.s0 + p % a.S;
}

__global__ void k_set(uint32_t* c, uint32_t v) { *c = v; }

__global__ void __launch_bounds__(kShadeThreads)
    k_raygen(WaveArgs a, WaveBufs w) {
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n_paths;
       p += gridDim.x * blockDim.x) {
    uint32_t pixel, sample;
    path_id(a, p, pixel, sample);
    const uint64_t key = path_key(a.seed, pixel, sample);
    const int x = (int)(pixel % a.cam.width), y = (int)(pixel / a.cam.width);
    const float u = x + key_float(key, 0);
    const float v = y + key_float(key, 1);
    const float l0 = key_float(key, 2), l1 = key_float(key, 3);
    F3 ro, rd;
    camera_ray(a.cam, u, v, l0, l1, ro, rd);
    F3 T = mk3(1.f, 1.f, 1.f);
    bool alive = a.max_b > 0;
    if (alive && 0 > a.min_b) {  // roulette before bounce 0
      if (key_float(key, dim_base(a, 0)) > a.cont) alive = false;
      T = T / a.cont;
    }
    w.thr[p] = make_float4(T.x, T.y, T.z, 0.f);
    w.rad[p] = make_float4(0.f, 0.f, 0.f, 0.f);
    const uint32_t k = warp_append(&w.counts[0], alive);
    if (alive) {
      w.qpath[0][k] = p;
      w.ro[0][k] = make_float4(ro.x, ro.y, ro.z, 0.f);
      w.rd[0][k] = make_float4(rd.x, rd.y, rd.z, 0.f);
    }
  }
}

// Closest hits of the path queue.
template <int TEST>
__global__ void __launch_bounds__(128, AJG_TRACE_MIN_BLOCKS)
    k_extend(DeviceScene s, const float4* __restrict__ ro,
             const float4* __restrict__ rd, const uint32_t* __restrict__ count,
             uint32_t* fetch_next, ajg_hit* __restrict__ hits,
             TraceCounters* ctr, uint32_t* err) {
  const uint32_t n = *count;
  uint32_t nn = 0, nt = 0, nr = 0;
  auto fetch = [&](uint32_t k) {
    const float4 o = ro[k], d = rd[k];
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
  trace_persistent<TEST, false>(s, n, fetch_next, fetch, finish, nr, nn, nt,
                                err);
  flush_counters(ctr, nr, nn, nt);
}

// Files every queue slot under its hit's material type (or as a miss), so
// that shading runs in material-specialised kernels; warps stay converged,
// so each list append is one atomic per warp.
__global__ void k_classify(DeviceScene s, const uint32_t* __restrict__ count,
                           const ajg_hit* __restrict__ hits,
                           uint32_t* __restrict__ lists,
                           uint32_t* __restrict__ list_counts,
                           uint32_t list_cap) {
  const uint32_t n = *count;
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t lane = threadIdx.x & 31;
  for (uint32_t wb = blockIdx.x * blockDim.x + (threadIdx.x - lane); wb < n;
       wb += stride) {
    const uint32_t k = wb + lane;
    int cls = -1;
    if (k < n) {
      const int prim = hits[k].prim;
      cls = 0;
      if (prim >= 0) {
        const uint32_t mat =
            __float_as_uint(__ldg(&s.shade[prim].w)) & 0xffffffu;
        cls = 1 + ((int)__ldg(s.materials + 16 * mat) == AJG_MAT_DISNEY);
      }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const uint32_t j = warp_append(&list_counts[c], cls == c);
      if (cls == c) lists[(uint64_t)c * list_cap + j] = k;
    }
  }
}

template <int TEST>
__global__ void __launch_bounds__(128, AJG_TRACE_MIN_BLOCKS)
    k_shadow(DeviceScene s, const float4* __restrict__ sq_o,
             const float4* __restrict__ sq_d, const uint32_t* __restrict__ count,
             uint32_t* fetch_next, uint8_t* __restrict__ vis,
             TraceCounters* ctr, uint32_t* err) {
  const uint32_t n = *count;
  uint32_t nn = 0, nt = 0, nr = 0;
  auto fetch = [&](uint32_t k) {
    const float4 o = sq_o[k], d = sq_d[k];
    return make_query(xyz(o), xyz(d), kRayEps, o.w);
  };
  auto finish = [&](uint32_t k, const Hit&, bool occ) {
    if (!occ) vis[__float_as_uint(sq_d[k].w)] = 1;
  };
  trace_persistent<TEST, true>(s, n, fetch_next, fetch, finish, nr, nn, nt,
                               err);
  flush_counters(ctr, nr, nn, nt);
}

__device__ __forceinline__ void emit_shadow(const WaveBufs& w, F3 o, F3 d,
                                            float tmax, uint32_t slot,
                                            bool pred, uint32_t cap,
                                            uint32_t* err) {
  const uint32_t k = warp_append(&w.counts[2], pred);
  if (!pred) return;
  if (k >= cap) {
    raise_device_error(err, kDevQueueOverflow);
    return;
  }
  w.sq_o[k] = make_float4(o.x, o.y, o.z, tmax);
  w.sq_d[k] = make_float4(d.x, d.y, d.z, __uint_as_float(slot));
}

// Escaped paths: the environment counts only for camera rays
// (pt.cpp:114-121), or on every bounce without MIS (pt.cpp:245-249).
__global__ void k_shade_miss(WaveArgs a, WaveBufs w, int cur,
                             const uint32_t* __restrict__ list,
                             const uint32_t* __restrict__ count) {
  const uint32_t n = *count;
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n;
       j += gridDim.x * blockDim.x) {
    const uint32_t p = w.qpath[cur][list[j]];
    float4 L = w.rad[p];
    L.x += a.env_rgb.x;
    L.y += a.env_rgb.y;
    L.z += a.env_rgb.z;
    w.rad[p] = L;
  }
}

// Shading of the hits on one material type: NEE to every light
// (helper.h:100-133), the MIS BSDF sample (helper.h:209-265), the
// continuation sample (pt.cpp:215-223) and the next bounce's roulette.
template <int MAT>
__global__ void __launch_bounds__(kShadeThreads, AJG_SHADE_MIN_BLOCKS)
    k_shade(WaveArgs a, WaveBufs w, int b, int cur,
            const uint32_t* __restrict__ list,
            const uint32_t* __restrict__ list_count, uint32_t shadow_cap,
            uint32_t* err) {
  const DeviceScene& s = a.s;
  const uint32_t n = *list_count;
  const int nt = (int)s.num_lights + 1;
  const int nxt = cur ^ 1;
  // warp-uniform loop: every lane of a warp runs the same iterations, so the
  // warp-wide queue appends see all lanes
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t lane = threadIdx.x & 31;
  for (uint32_t wb = blockIdx.x * blockDim.x + (threadIdx.x - lane); wb < n;
       wb += stride) {
    const uint32_t j = wb + lane;
    const bool hit = j < n;
    uint32_t p = 0;
    HitInfo hi;
    BsdfT<MAT> f;
    F3 T = mk3(0, 0, 0);
    uint64_t key = 0;
    if (hit) {
      const uint32_t k = list[j];
      p = w.qpath[cur][k];
      const ajg_hit h = w.hits[k];
      const F3 ro = xyz(w.ro[cur][k]), rd = xyz(w.rd[cur][k]);
      uint32_t pixel, sample;
      path_id(a, p, pixel, sample);
      key = path_key(a.seed, pixel, sample);
      T = xyz(w.thr[p]);
      hi = complete_hit(s, ro, rd, h.t, h.u, h.v, h.prim);
      f.m = s.materials + 16 * hi.mat;
      f.ng = hi.ng;
      f.ns = hi.ns;
      f.lum = __ldg(&s.mat_lum[hi.mat].x);
      w.thr_shade[p] = make_float4(T.x, T.y, T.z, 0.f);
    }
    int dim = dim_base(a, b) + (b > a.min_b ? 1 : 0);

    if (a.use_mis) {
      for (int l = 0; l < (int)s.num_lights; ++l) {
        const float* L = s.lights + 12 * l;
        bool emit = false;
        F3 fo = mk3(0, 0, 0), so = mk3(0, 0, 0), sd = mk3(0, 0, 1);
        float tmax = 0.f;
        if (hit) {
          F3 lpos, lrad;
          float lpdf;
          const int type = (int)L[0];
          bool ok = true;
          if (type == AJG_LIGHT_DIRECTIONAL) {
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
                const F3 nn = normalize3(hi.ns);
                F3 fv;
                if (type == AJG_LIGHT_DIRECTIONAL)
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
          const uint32_t slot = p * nt + l;
          w.term_f[slot] = make_float4(fo.x, fo.y, fo.z, 0.f);
          w.term_vis[slot] = 0;
        }
        emit_shadow(w, so, sd, tmax, p * nt + l, emit, shadow_cap, err);
        dim += 2;
      }
      {
        bool emit = false;
        F3 fo = mk3(0, 0, 0), so = mk3(0, 0, 0), sd = mk3(0, 0, 1);
        if (hit) {
          const F3 sam = mk3(key_float(key, dim), key_float(key, dim + 1),
                             key_float(key, dim + 2));
          BsdfSample bs = f.sample(hi.wr, sam);
          if (!(black3(bs.f) || bs.pdf == 0.f) && s.env >= 0) {
            bs.dir = normalize3(bs.dir);
            make_ray(eps_offset(hi, bs.dir), bs.dir, so, sd);
            const F3 rad = mk3(a.env_rgb.x, a.env_rgb.y, a.env_rgb.z);
            if (!black3(rad)) {
              const F3 fv = rad * bs.f * fabsf(dot3(hi.ns, sd));
              const float lp = env_pdf(a.env_mass != 0, sd);
              fo = mk3(0, 0, 0) + fv / bs.pdf * power_heuristic(bs.pdf, lp);
              emit = true;
            }
          }
          const uint32_t slot = p * nt + (nt - 1);
          w.term_f[slot] = make_float4(fo.x, fo.y, fo.z, 0.f);
          w.term_vis[slot] = 0;
        }
        emit_shadow(w, so, sd, __int_as_float(0x7f800000), p * nt + (nt - 1),
                    emit, shadow_cap, err);
        dim += 3;
      }
    }

    bool alive = false;
    F3 nro = mk3(0, 0, 0), nrd = mk3(0, 0, 1);
    if (hit && b + 1 < a.max_b) {
      const F3 sam = mk3(key_float(key, dim), key_float(key, dim + 1),
                         key_float(key, dim + 2));
      const BsdfSample bs = f.sample(hi.wr, sam);
      if (!(black3(bs.f) || bs.pdf < 0.f)) {
        T = T * (bs.f * fabsf(dot3(hi.ng, bs.dir)) / bs.pdf);
        make_ray(eps_offset(hi, bs.dir), bs.dir, nro, nrd);
        alive = true;
        if (b + 1 > a.min_b) {
          if (key_float(key, dim_base(a, b + 1)) > a.cont)
            alive = false;
          else
            T = T / a.cont;
        }
      }
      w.thr[p] = make_float4(T.x, T.y, T.z, 0.f);
    }
    const uint32_t kn = warp_append(&w.counts[nxt], alive);
    if (alive) {
      w.qpath[nxt][kn] = p;
      w.ro[nxt][kn] = make_float4(nro.x, nro.y, nro.z, 0.f);
      w.rd[nxt][kn] = make_float4(nrd.x, nrd.y, nrd.z, 0.f);
    }
  }
}

// direct_illum += throughput * MISSampleLight(...) for each light, then
// += throughput * MISSampleBsdf(...); pixel.value += direct (pt.cpp:200-213)
__global__ void __launch_bounds__(kShadeThreads)
    k_accumulate(WaveArgs a, WaveBufs w, int cur) {
  const uint32_t n = w.counts[cur];
  const int nt = (int)a.s.num_lights + 1;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += gridDim.x * blockDim.x) {
    if (w.hits[k].prim < 0) continue;
    const uint32_t p = w.qpath[cur][k];
    const F3 T = xyz(w.thr_shade[p]);
    F3 direct = mk3(0.f, 0.f, 0.f);
    for (int j = 0; j < nt; ++j) {
      const uint32_t slot = p * nt + j;
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

// Each pixel adds its S samples in sample order (Kahan-compensated float32,
// or float64).
__global__ void k_film_add(WaveArgs a, const float4* __restrict__ rad,
                           float4* __restrict__ sum, float4* __restrict__ comp,
                           double* __restrict__ sum64, uint32_t n_pix,
                           int drop_nonfinite) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_pix;
       i += gridDim.x * blockDim.x) {
    const uint32_t pixel = a.pix0 + i;
    if (sum64) {
      double* o = sum64 + 4 * (uint64_t)pixel;
      double x = o[0], y = o[1], z = o[2], wsum = o[3];
      for (uint32_t j = 0; j < a.S; ++j) {
        const float4 L = rad[(uint64_t)i * a.S + j];
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
      continue;
    }
    float4 s4 = sum[pixel], c4 = comp[pixel];
    for (uint32_t j = 0; j < a.S; ++j) {
      const float4 L = rad[(uint64_t)i * a.S + j];
      if (drop_nonfinite &&
          !(isfinite(L.x) && isfinite(L.y) && isfinite(L.z)))
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
}

// The reference's film convention (film.cpp:27-63, film.h:119-129,
// image.h:38-42): a sample at (x, y) lands on (x-1..x, y-1..y) with weight
// 1, and row/column -1 folds into 0.  Target (tx, ty) thus sums sources
// tx (twice when tx == 0) and tx + 1, likewise in y.
__global__ void k_resolve(const float4* __restrict__ sum,
                          const float4* __restrict__ comp,
                          const double* __restrict__ sum64, uint32_t W,
                          uint32_t H, float4* __restrict__ out) {
  const uint64_t npix = (uint64_t)W * H;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < npix;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t tx = (uint32_t)(i % W), ty = (uint32_t)(i / W);
    double r = 0, g = 0, bl = 0, wt = 0;
    for (int dy = 0; dy < 2; ++dy) {
      const uint32_t sy = ty + dy;
      if (sy >= H) continue;
      const int my = (dy == 0 && ty == 0) ? 2 : 1;
      for (int dx = 0; dx < 2; ++dx) {
        const uint32_t sx = tx + dx;
        if (sx >= W) continue;
        const int mx = (dx == 0 && tx == 0) ? 2 : 1;
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

template <class T>
T* carve(char*& cur, uint64_t count) {
  T* p = reinterpret_cast<T*>(cur);
  cur += ((count * sizeof(T) + 255) / 256) * 256;
  return p;
}

uint64_t wave_bytes(uint64_t P, int nt) {
  const uint64_t slots = P * nt;
  uint64_t b = 0;
  auto add = [&](uint64_t bytes) { b += ((bytes + 255) / 256) * 256; };
  add(P * 16); add(P * 16); add(P * 16);  // thr, thr_shade, rad
  add(P * 4); add(P * 4);      // qpath
  add(P * 16); add(P * 16);    // ro
  add(P * 16); add(P * 16);    // rd
  add(P * sizeof(ajg_hit));
  add(slots * 16);             // term_f
  add(slots);                  // term_vis
  add(slots * 16); add(slots * 16);  // shadow queue
  add(P * 4 * 3);              // material lists
  add(32);                     // counts
  return b;
}

}  // namespace

// The wave arena: one device allocation reused across renders of the
// context, grown when a render needs more paths or light terms.
static int ensure_arena(ajg_ctx* ctx, uint64_t P, int nt, char** base) {
  const uint64_t need = wave_bytes(P, nt);
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

static int check_render(ajg_ctx* ctx, const DeviceScene& s,
                        const ajg_camera& cam, const ajg_render_params& prm) {
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

static WaveBufs carve_wave(char* base, uint64_t P, int nt) {
  char* cur = base;
  WaveBufs w;
  w.thr = carve<float4>(cur, P);
  w.thr_shade = carve<float4>(cur, P);
  w.rad = carve<float4>(cur, P);
  w.qpath[0] = carve<uint32_t>(cur, P);
  w.qpath[1] = carve<uint32_t>(cur, P);
  w.ro[0] = carve<float4>(cur, P);
  w.ro[1] = carve<float4>(cur, P);
  w.rd[0] = carve<float4>(cur, P);
  w.rd[1] = carve<float4>(cur, P);
  w.hits = carve<ajg_hit>(cur, P);
  w.term_f = carve<float4>(cur, P * nt);
  w.term_vis = carve<uint8_t>(cur, P * nt);
  w.sq_o = carve<float4>(cur, P * nt);
  w.sq_d = carve<float4>(cur, P * nt);
  w.lists = carve<uint32_t>(cur, P * 3);
  w.counts = carve<uint32_t>(cur, 8);
  return w;
}

// The sample loop of one render over zeroed film accumulators: waves of S
// samples of a pixel range, the bounce loop per wave, the film update per
// wave and the footprint resolve at the end.  `timers` enables the
// profiling events of the traversal and shading launches.
static void run_waves(ajg_scene* sc, const ajg_camera& cam,
                      const ajg_render_params& prm, const WaveBufs& w,
                      uint64_t P, float4* fsum, float4* fcomp, double* fsum64,
                      float4* d_out, uint64_t li_begin, uint64_t li_end,
                      float* d_li, cudaStream_t st, bool timers) {
  ajg_ctx* ctx = sc->ctx;
  const DeviceScene& s = sc->d;
  const int nt = (int)s.num_lights + 1;
  const uint64_t npix_all = (uint64_t)cam.width * cam.height;
  const bool want_film = d_out != nullptr;
  const int kc = timers ? kKindClosest : -1;
  const int ka = timers ? kKindAny : -1;
  const int ks = timers ? kKindShade : -1;

  WaveArgs a;
  a.s = s;
  a.cam = cam;
  a.seed = prm.seed;
  a.min_b = prm.min_bounces;
  a.max_b = prm.max_bounces;
  a.cont = prm.cont_prob;
  a.use_mis = prm.use_mis ? 1 : 0;
  a.nd = a.use_mis ? (2 * (int)s.num_lights + 6) : 3;
  a.env_rgb = make_float4(0, 0, 0, 0);
  a.env_mass = 0;
  if (s.env >= 0) {
    const float* L = sc->host_lights.data() + 12 * s.env;
    // EnvLight::Radiance = scaler * texel (env_light.cpp:65)
    a.env_rgb = make_float4(L[8] * L[1], L[8] * L[2], L[8] * L[3], 0.f);
    a.env_mass = L[11] != 0.f ? 1 : 0;
  }

  const uint64_t pb = d_li ? li_begin : 0;
  const uint64_t pe = d_li ? li_end : npix_all;
  const uint64_t npix = pe - pb;
  uint64_t S = std::min<uint64_t>(prm.spp, std::max<uint64_t>(1, P / npix));
  const uint64_t chunk = std::min<uint64_t>(npix, P / S);
  const uint32_t shadow_cap = (uint32_t)(P * nt);
  const int gs = kSMs * 8;
  // persistent traversal: resident blocks only (occupancy-limited)
  const int trace_grid = kSMs * AJG_TRACE_BLOCKS_PER_SM;
  for (uint64_t s0 = 0; s0 < prm.spp; s0 += S) {
    const uint64_t Sw = std::min<uint64_t>(S, prm.spp - s0);
    for (uint64_t p0 = pb; p0 < pe; p0 += chunk) {
      const uint64_t n_pix = std::min<uint64_t>(chunk, pe - p0);
      a.pix0 = (uint32_t)p0;
      a.S = (uint32_t)Sw;
      a.s0 = (uint32_t)s0;
      a.n_paths = (uint32_t)(n_pix * Sw);
      cudaMemsetAsync(w.counts, 0, 32, st);
      KernelTimer{ctx, st, -1};
      k_raygen<<<grid_for(a.n_paths, kShadeThreads, gs), kShadeThreads, 0,
                 st>>>(a, w);
      int q = 0;
      for (int b = 0; b < a.max_b; ++b) {
        // next queue, shadow queue, fetch counters and material lists
        cudaMemsetAsync(&w.counts[q ^ 1], 0, sizeof(uint32_t), st);
        cudaMemsetAsync(&w.counts[2], 0, 6 * sizeof(uint32_t), st);
        {
          KernelTimer tm(ctx, st, kc);
          if (s.tri_test == AJG_TRI_WATERTIGHT)
            k_extend<AJG_TRI_WATERTIGHT><<<trace_grid, 128, 0, st>>>(
                s, w.ro[q], w.rd[q], &w.counts[q], &w.counts[7], w.hits,
                &ctx->d_counters[0], ctx->d_error);
          else
            k_extend<AJG_TRI_MOLLER_TRUMBORE><<<trace_grid, 128, 0, st>>>(
                s, w.ro[q], w.rd[q], &w.counts[q], &w.counts[7], w.hits,
                &ctx->d_counters[0], ctx->d_error);
        }
        {
          KernelTimer tm(ctx, st, -1);
          k_classify<<<gs, 256, 0, st>>>(s, &w.counts[q], w.hits, w.lists,
                                         &w.counts[4], (uint32_t)P);
        }
        if ((b == 0 || !a.use_mis) && s.env >= 0) {
          KernelTimer tm(ctx, st, ks);
          k_shade_miss<<<gs, kShadeThreads, 0, st>>>(a, w, q, w.lists,
                                                     &w.counts[4]);
        }
        {
          KernelTimer tm(ctx, st, ks);
          k_shade<AJG_MAT_DIFFUSE><<<gs, kShadeThreads, 0, st>>>(
              a, w, b, q, w.lists + P, &w.counts[5], shadow_cap, ctx->d_error);
        }
        {
          KernelTimer tm(ctx, st, ks);
          k_shade<AJG_MAT_DISNEY><<<gs, kShadeThreads, 0, st>>>(
              a, w, b, q, w.lists + 2 * P, &w.counts[6], shadow_cap,
              ctx->d_error);
        }
        if (a.use_mis) {
          {
            KernelTimer tm(ctx, st, ka);
            if (s.tri_test == AJG_TRI_WATERTIGHT)
              k_shadow<AJG_TRI_WATERTIGHT><<<trace_grid, 128, 0, st>>>(
                  s, w.sq_o, w.sq_d, &w.counts[2], &w.counts[3], w.term_vis,
                  &ctx->d_counters[1], ctx->d_error);
            else
              k_shadow<AJG_TRI_MOLLER_TRUMBORE><<<trace_grid, 128, 0, st>>>(
                  s, w.sq_o, w.sq_d, &w.counts[2], &w.counts[3], w.term_vis,
                  &ctx->d_counters[1], ctx->d_error);
          }
          KernelTimer{ctx, st, -1};
          k_accumulate<<<gs, kShadeThreads, 0, st>>>(a, w, q);
        }
        q ^= 1;
      }
      if (want_film) KernelTimer{ctx, st, -1};
      if (want_film)
        k_film_add<<<grid_for(n_pix, 256, gs), 256, 0, st>>>(
            a, w.rad, fsum, fcomp, fsum64, (uint32_t)n_pix,
            (prm.flags & AJG_RENDER_DROP_NONFINITE) ? 1 : 0);
      if (d_li) KernelTimer{ctx, st, -1};
      if (d_li)
        k_copy_li<<<grid_for(a.n_paths, 256, gs), 256, 0, st>>>(
            a, w.rad, li_begin, prm.spp, d_li);
    }
  }
  if (want_film) {
    KernelTimer{ctx, st, -1};
    k_resolve<<<grid_for(npix_all, 256, gs), 256, 0, st>>>(
        fsum, fcomp, fsum64, cam.width, cam.height, d_out);
  }
  ctx->paths_total += (unsigned long long)npix * prm.spp;
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
  const uint64_t P = ctx->wave_paths;
  const uint64_t npix_all = (uint64_t)cam.width * cam.height;
  char* base = nullptr;
  rc = ensure_arena(ctx, P, nt, &base);
  if (rc) return rc;
  const WaveBufs w = carve_wave(base, P, nt);

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
  const uint64_t min_wave = wave_bytes(1024, nt);
  if (film_bytes + min_wave > bytes)
    return fail(ctx, AJG_ERR_INVALID,
                "film of " + std::to_string(npix) + " pixels needs " +
                    std::to_string(film_bytes + min_wave) +
                    " bytes of scratch; the static scratch holds " +
                    std::to_string(bytes) + " (at most " +
                    std::to_string((bytes - min_wave) / 32) + " pixels)");
  uint64_t P = 1024;
  while (wave_bytes(P + 1024, nt) + film_bytes <= bytes) P += 1024;
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
  const WaveBufs w = carve_wave(scratch + film_bytes, P, nt);
  run_waves(sc, cam, prm, w, P, fsum, fcomp, fsum64, d_out, 0, 0, nullptr, st,
            false);
  return AJG_OK;
}

}  // namespace ajg
