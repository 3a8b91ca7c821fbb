// Stochastic progressive photon mapping: SPPMRenderer::Render
// (core/renderer/sppm.cpp:180-296) on the GPU.
//
// The camera pass (TracerVP) runs once through the path-tracing wave
// (sppm_camera_pass): the reference reseeds every pixel each iteration, so
// every iteration finds the same visible points and the same direct light.
// Per iteration:
//   the visible-point grid -- the reference's VisiblePointSearcher
//     (photon_mapping.h:69-148): 40960 hash entries, each visible point
//     filed under the cells [lo, hi) of its radius box -- built as count,
//     scan and fill over the entries instead of linked lists;
//   the photon pass (TracerPhoton, sppm.cpp:103-143) as a wavefront: emit
//     from a light chosen by the scene's uniform selector, then per depth a
//     closest-hit traversal and a shading kernel that deposits into the
//     grid (AddPhoton: EvalAll at the visible point, atomically summed) and
//     samples the BSDF; roulette draws as the reference draws them;
//   the radius reduction and UpdatePixel (sppm.cpp:145-169).
// Photon i of iteration k draws from path_key(photon_seed(seed), i, k).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "shade.cuh"
#include "trace.cuh"

namespace ajg {
namespace {

constexpr uint32_t kEntries = 40960;   // VisiblePointSearcher(..., 40960)
constexpr int kMaxCellsPerAxis = 4;    // a radius box spans <= 3 cells
constexpr int kThreads = 128;
constexpr unsigned kFull = 0xffffffffu;

int fail(ajg_ctx* ctx, int code, const std::string& m) {
  ctx->last_error = m;
  return code;
}

// photon streams (the oracle's ajg_photon_seed)
__host__ __device__ __forceinline__ uint64_t photon_seed(uint64_t seed) {
  return mix64(seed ^ 0x50484F544F4E5321ull);
}

// Per-render constants.
struct SppmArgs {
  DeviceScene s;
  F3 lo;              // world bounds grown by the initial radius
  F3 center;          // world centre (the lights' emission disks)
  float init_radius;
  uint64_t pseed;     // photon stream seed
  uint32_t npix;
  uint32_t it;        // iteration
  int pmin, pmax;
  float cont;
  // DefaultScene's light selector (default_scene.cpp:48-53, 77-86)
  float cdf[16];
  float lpdf;
  uint32_t nl;
};

// Per-pixel state (sppm::Pixel, photon_mapping.h:54-67).
struct SppmPixels {
  const VisPointD* vp;
  const float4* direct;
  float* radius;
  float* N;
  uint32_t* M;
  float4* phi;
  float4* tau;
};

struct Grid {
  uint32_t* counts;   // [kEntries]
  uint32_t* offsets;  // [kEntries + 1]
  uint32_t* cursor;   // [kEntries]
  uint32_t* items;    // pixel indices, entry by entry
  float4* spheres;    // per item: the visible point and radius^2, so the
                      // distance test of a deposit reads one 16-byte record
  uint32_t cap;
  const float* maxr;  // this iteration's max radius (the cell side / 1.05)
};

// VisiblePointSearcher::ToGrid and ToEntry (photon_mapping.h:123-139).
__device__ __forceinline__ void to_grid(F3 pos, F3 lo, float side, int c[3]) {
  const F3 hd = pos - lo;
  c[0] = (int)((hd.x < 0.f ? 0.f : hd.x) / side);
  c[1] = (int)((hd.y < 0.f ? 0.f : hd.y) / side);
  c[2] = (int)((hd.z < 0.f ? 0.f : hd.z) / side);
}
__device__ __forceinline__ uint64_t hash_combine(uint64_t a, uint64_t b) {
  return a ^ (b + 0x9e3779b97f4a7c15ull + (a << 6) + (a >> 2));
}
__device__ __forceinline__ uint32_t to_entry(int x, int y, int z) {
  const uint64_t low3 = (uint64_t)(((x & 1) << 0) | ((y & 1) << 1) | (z & 2));
  uint64_t h = (uint64_t)(int64_t)x;  // std::hash<int>
  h = hash_combine(h, (uint64_t)(int64_t)y);
  h = hash_combine(h, (uint64_t)(int64_t)z);
  return (uint32_t)(((h << 3) % kEntries) | low3);
}

__device__ __forceinline__ bool has_vp(const VisPointD& v) {
  return __float_as_uint(v.pos.w) != kNoVisPoint;
}

// AddVp's cell range of pixel i (photon_mapping.h:80-96); false when the
// box spans more cells than a radius below the cell side allows.
__device__ __forceinline__ bool vp_cells(const SppmArgs& a,
                                         const SppmPixels& px, const Grid& g,
                                         uint32_t i, int lo[3], int hi[3]) {
  const float side = 1.05f * *g.maxr;
  const F3 pos = xyz(px.vp[i].pos);
  const float r = px.radius[i];
  to_grid(pos - mk3(r, r, r), a.lo, side, lo);
  to_grid(pos + mk3(r, r, r), a.lo, side, hi);
  for (int k = 0; k < 3; ++k)
    if (hi[k] - lo[k] > kMaxCellsPerAxis) return false;
  return true;
}

__global__ void k_grid_count(SppmArgs a, SppmPixels px, Grid g,
                             uint32_t* err) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.npix;
       i += gridDim.x * blockDim.x) {
    if (!has_vp(px.vp[i])) continue;
    int lo[3], hi[3];
    if (!vp_cells(a, px, g, i, lo, hi)) {
      raise_device_error(err, kDevIterationBound);
      continue;
    }
    for (int z = lo[2]; z < hi[2]; ++z)
      for (int y = lo[1]; y < hi[1]; ++y)
        for (int x = lo[0]; x < hi[0]; ++x)
          atomicAdd(&g.counts[to_entry(x, y, z)], 1u);
  }
}

// Exclusive scan of the entry counts (one block).
__global__ void __launch_bounds__(1024) k_grid_scan(Grid g) {
  constexpr uint32_t kPer = (kEntries + 1023) / 1024;
  __shared__ uint32_t part[1024];
  const uint32_t t = threadIdx.x;
  const uint32_t b0 = t * kPer;
  uint32_t local = 0;
  for (uint32_t k = 0; k < kPer; ++k)
    if (b0 + k < kEntries) local += g.counts[b0 + k];
  part[t] = local;
  __syncthreads();
  for (uint32_t off = 1; off < 1024; off <<= 1) {
    const uint32_t v = t >= off ? part[t - off] : 0u;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  uint32_t run = part[t] - local;
  for (uint32_t k = 0; k < kPer; ++k)
    if (b0 + k < kEntries) {
      g.offsets[b0 + k] = run;
      g.cursor[b0 + k] = 0;
      run += g.counts[b0 + k];
    }
  if (t == 1023) g.offsets[kEntries] = part[1023];
}

__global__ void k_grid_fill(SppmArgs a, SppmPixels px, Grid g,
                            uint32_t* err) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.npix;
       i += gridDim.x * blockDim.x) {
    if (!has_vp(px.vp[i])) continue;
    int lo[3], hi[3];
    if (!vp_cells(a, px, g, i, lo, hi)) continue;
    for (int z = lo[2]; z < hi[2]; ++z)
      for (int y = lo[1]; y < hi[1]; ++y)
        for (int x = lo[0]; x < hi[0]; ++x) {
          const uint32_t e = to_entry(x, y, z);
          const uint32_t slot = g.offsets[e] + atomicAdd(&g.cursor[e], 1u);
          if (slot >= g.cap) {
            raise_device_error(err, kDevQueueOverflow);
            continue;
          }
          const float4 p4 = px.vp[i].pos;
          const float r = px.radius[i];
          g.items[slot] = i;
          g.spheres[slot] = make_float4(p4.x, p4.y, p4.z, r * r);
        }
  }
}

// The photon queue (double buffered): ro.w = photon index bits, rd.w = the
// photon's next sampler dimension, coef = its power.
struct PhotonQ {
  float4* ro[2];
  float4* rd[2];
  float4* coef[2];
  ajg_hit* hits;
  uint32_t* counts;  // [0],[1] queues, [2] extend fetch
  uint32_t cap;
};

__device__ __forceinline__ void push_photon(const PhotonQ& q, int qi, F3 o,
                                            F3 d, F3 c, uint32_t pid,
                                            uint32_t dim, bool pred,
                                            uint32_t* err) {
  const uint32_t k = warp_append(&q.counts[qi], pred);
  if (!pred) return;
  if (k >= q.cap) {
    raise_device_error(err, kDevQueueOverflow);
    return;
  }
  q.ro[qi][k] = make_float4(o.x, o.y, o.z, __uint_as_float(pid));
  q.rd[qi][k] = make_float4(d.x, d.y, d.z, __uint_as_float(dim));
  q.coef[qi][k] = make_float4(c.x, c.y, c.z, 0.f);
}

struct Emission {
  F3 pos, dir, normal, radiance;
  float pdf_pos = 0.f, pdf_dir = 0.f;
};

// Light::SampleEmit: directional_light.cpp:60-79, env_light.cpp:105-150,
// area_light.cpp:59-70.
__device__ Emission sample_emit(const SppmArgs& a, const float* L,
                                uint64_t key, uint32_t& dim) {
  Emission e;
  const int type = (int)L[0];
  if (type == kLightArea) {
    const float x = key_float(key, dim), y = key_float(key, dim + 1),
                z = key_float(key, dim + 2);
    dim += 3;
    const AreaSample g = area_sample(L, a.s.emit_pts, x, y, z);
    float pdf_dir;
    const F3 lwi =
        cosine_hemisphere(key_float(key, dim), key_float(key, dim + 1), &pdf_dir);
    dim += 2;
    e.pos = g.pos;
    e.dir = Frame(g.ng).to_world(lwi);
    e.normal = g.ng;
    e.radiance = mk3(L[1], L[2], L[3]);
    e.pdf_pos = g.pdf;
    e.pdf_dir = pdf_dir;
  } else if (type == AJG_LIGHT_DIRECTIONAL) {
    const float u0 = key_float(key, dim), u1 = key_float(key, dim + 1);
    dim += 2;
    const F3 r2l =
        Frame(normalize3(mk3(L[4], L[5], L[6]))).to_world(uniform_cone(u0, u1, L[7]));
    const float pdf_dir = uniform_cone_pdf(L[7]);
    const float radius = a.s.radius;
    float dx, dy;
    concentric(key_float(key, dim), key_float(key, dim + 1), dx, dy);
    dim += 2;
    const Frame dc(r2l);
    e.pos = a.center + (dx * dc.dx + dy * dc.dy + r2l) * radius;
    e.dir = -r2l;
    e.normal = normalize3(-r2l);
    e.radiance = mk3(L[1], L[2], L[3]);
    e.pdf_pos = 1.f / (kPi * radius * radius);
    e.pdf_dir = pdf_dir;
  } else {
    // g++ evaluates SampleContinuous's two Next1D() arguments right to
    // left: the first draw is v
    const float v = key_float(key, dim);
    float u = key_float(key, dim + 1);
    dim += 2;
    if (L[10] == 0.f) return Emission{};  // the 1x1 distribution has no mass
    float pdf = 1.f;
    constexpr float inv_2_pi = 1.f / (2.f * kPi);
    constexpr float two_pi = 2.f * kPi;
    u -= L[9] / 180 * kPi * inv_2_pi;
    if (u > 1.f) u -= 1.f;
    if (u < 0.f) u += 1.f;
    const float phi = u * two_pi;
    const float theta = v * kPi;
    const float st = sinf(theta);
    pdf = st != 0.f ? pdf / (2.f * kPi * kPi * st) : 0.f;
    F3 dir = mk3(-sinf(theta) * cosf(phi), cosf(theta), -sinf(theta) * sinf(phi));
    dir = -dir;
    const float radius = a.s.radius;
    float dx, dy;
    concentric(key_float(key, dim), key_float(key, dim + 1), dx, dy);
    dim += 2;
    const Frame dc(-dir);
    e.pos = a.center + (dx * dc.dx + dy * dc.dy - dir) * radius;
    e.dir = dir;
    e.normal = normalize3(dir);
    e.radiance = mk3(L[1], L[2], L[3]);  // the texel, without the scaler
    e.pdf_pos = 1.f / (kPi * radius * radius);
    e.pdf_dir = pdf;
  }
  return e;
}

// TracerPhoton's start (sppm.cpp:105-121) and depth 1's roulette.
__global__ void __launch_bounds__(kThreads)
    k_photon_emit(SppmArgs a, PhotonQ q, uint32_t i0, uint32_t n,
                  uint32_t* err) {
  const uint32_t lane = threadIdx.x & 31;
  for (uint32_t wb = blockIdx.x * blockDim.x + (threadIdx.x - lane); wb < n;
       wb += gridDim.x * blockDim.x) {
    const uint32_t t = wb + lane;
    bool live = false;
    F3 o = mk3(0, 0, 0), d = mk3(0, 0, 1), coef = mk3(0, 0, 0);
    uint32_t pid = i0 + t, dim = 0;
    if (t < n && a.nl > 0) {
      const uint64_t key = path_key(a.pseed, pid, a.it);
      const float u = key_float(key, dim++);
      // upper_bound with <=: the first j with u <= cdf[j]
      uint32_t j = 0;
      while (j <= a.nl && !(u <= a.cdf[j])) ++j;
      const int idx = min(max((int)j - 1, 0), (int)a.nl - 1);
      const Emission e = sample_emit(a, a.s.lights + 12 * idx, key, dim);
      if (!(black3(e.radiance) || e.pdf_dir == 0.f || e.pdf_pos == 0.f)) {
        coef = e.radiance * fabsf(dot3(e.normal, e.dir)) /
               (a.lpdf * e.pdf_pos * e.pdf_dir);
        make_ray(e.pos, e.dir, o, d);
        live = 1 <= a.pmax;
        if (live && 1 > a.pmin) {
          if (key_float(key, dim++) > a.cont)
            live = false;
          else
            coef = coef / a.cont;
        }
      }
    }
    push_photon(q, 0, o, d, coef, pid, dim, live, err);
  }
}

template <int TEST, int W>
__global__ void __launch_bounds__(128, trace_min_blocks<W>())
    k_photon_extend(DeviceScene s, const float4* __restrict__ ro,
                    const float4* __restrict__ rd,
                    const uint32_t* __restrict__ count, uint32_t* fetch_next,
                    ajg_hit* __restrict__ hits, TraceCounters* ctr,
                    uint32_t* err) {
  const uint32_t n = *count;
  uint32_t nn = 0, nt = 0, nr = 0;
  auto fetch = [&](uint32_t k, TraceScene&) {
    return make_query(xyz(ro[k]), xyz(rd[k]), kRayEps,
                      __int_as_float(0x7f800000));
  };
  auto finish = [&](uint32_t k, const Hit& h, bool) {
    ajg_hit o;
    o.t = h.t;
    o.u = h.u;
    o.v = h.v;
    o.prim = h.prim;
    hits[k] = o;
  };
  trace_persistent<TEST, false, W>(trace_scene(s), n, fetch_next, fetch,
                                   finish, nr, nn, nt, err);
  flush_counters(ctr, nr, nn, nt);
}

// A BSDF from a material record and its two normals.
__device__ __forceinline__ Bsdf bsdf_at(const DeviceScene& s, uint32_t mat,
                                        F3 ng, F3 ns) {
  Bsdf f;
  f.m = s.materials + 16 * mat;
  f.type = (int)f.m[0];
  f.ng = ng;
  f.ns = ns;
  f.lum = __ldg(&s.mat_lum[mat].x);
  return f;
}

// VisiblePointSearcher::AddPhoton (photon_mapping.h:101-120).
__device__ void add_photon(const SppmArgs& a, const SppmPixels& px,
                           const Grid& g, F3 pos, F3 phi, F3 wr) {
  const float side = 1.05f * *g.maxr;
  int c[3];
  to_grid(pos, a.lo, side, c);
  const uint32_t e = to_entry(c[0], c[1], c[2]);
  const uint32_t end = min(g.offsets[e + 1], g.cap);
  for (uint32_t j = g.offsets[e]; j < end; ++j) {
    const float4 sp = __ldg(&g.spheres[j]);
    const F3 d = xyz(sp) - pos;
    if (dot3(d, d) > sp.w) continue;
    const uint32_t i = g.items[j];
    const VisPointD v = px.vp[i];
    const Bsdf f = bsdf_at(a.s, __float_as_uint(v.pos.w), xyz(v.ng), xyz(v.ns));
    const F3 dp = phi * f.eval(wr, xyz(v.wr));
    if (!(isfinite(dp.x) && isfinite(dp.y) && isfinite(dp.z))) continue;
    atomicAdd(&px.phi[i].x, dp.x);
    atomicAdd(&px.phi[i].y, dp.y);
    atomicAdd(&px.phi[i].z, dp.z);
    atomicAdd(&px.M[i], 1u);
  }
}

// One depth of TracerPhoton (sppm.cpp:122-142) over the queue: deposit
// (from depth 2 on), sample the BSDF, and the next depth's roulette.
__global__ void __launch_bounds__(kThreads)
    k_photon_shade(SppmArgs a, SppmPixels px, Grid g, PhotonQ q, int cur,
                   int depth, uint32_t* err) {
  const uint32_t n = min(q.counts[cur], q.cap);
  const int nxt = cur ^ 1;
  const uint32_t lane = threadIdx.x & 31;
  for (uint32_t wb = blockIdx.x * blockDim.x + (threadIdx.x - lane); wb < n;
       wb += gridDim.x * blockDim.x) {
    const uint32_t k = wb + lane;
    bool live = false;
    F3 no = mk3(0, 0, 0), nd = mk3(0, 0, 1), coef = mk3(0, 0, 0);
    uint32_t pid = 0, dim = 0;
    if (k < n) {
      const ajg_hit h = q.hits[k];
      const float4 o4 = q.ro[cur][k], d4 = q.rd[cur][k];
      pid = __float_as_uint(o4.w);
      dim = __float_as_uint(d4.w);
      coef = xyz(q.coef[cur][k]);
      if (h.prim >= 0) {
        const uint64_t key = path_key(a.pseed, pid, a.it);
        const HitInfo hi =
            complete_hit(a.s, xyz(o4), xyz(d4), h.t, h.u, h.v, h.prim);
        if (depth > 1) add_photon(a, px, g, hi.pos, coef, hi.wr);
        const Bsdf f = bsdf_at(a.s, hi.mat, hi.ng, hi.ns);
        const F3 sam = mk3(key_float(key, dim), key_float(key, dim + 1),
                           key_float(key, dim + 2));
        dim += 3;
        const BsdfSample bs = f.sample(hi.wr, sam);
        if (!(black3(bs.f) || bs.pdf < 0.f)) {
          coef = coef * (bs.f / bs.pdf * fabsf(dot3(hi.ng, bs.dir)));
          make_ray(eps_offset(hi, bs.dir), bs.dir, no, nd);
          live = depth + 1 <= a.pmax;
          if (live && depth + 1 > a.pmin) {
            if (key_float(key, dim++) > a.cont)
              live = false;
            else
              coef = coef / a.cont;
          }
        }
      }
    }
    push_photon(q, nxt, no, nd, coef, pid, dim, live, err);
  }
}

// The largest radius of a pixel with a visible point (before the update).
__global__ void k_max_radius(SppmArgs a, SppmPixels px, uint32_t* bits) {
  uint32_t m = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.npix;
       i += gridDim.x * blockDim.x)
    if (has_vp(px.vp[i])) m = max(m, __float_as_uint(px.radius[i]));
  m = __reduce_max_sync(kFull, m);
  if ((threadIdx.x & 31) == 0 && m) atomicMax(bits, m);
}

// UpdatePixel (sppm.cpp:145-169) and the next iteration's cell size.
__global__ void k_update(SppmArgs a, SppmPixels px, float alpha,
                         const uint32_t* bits, float* maxr) {
  const uint32_t i0 = blockIdx.x * blockDim.x + threadIdx.x;
  if (i0 == 0) {
    const float m = __uint_as_float(*bits);
    *maxr = m == 0.f ? a.init_radius : m;
  }
  for (uint32_t i = i0; i < a.npix; i += gridDim.x * blockDim.x) {
    if (!has_vp(px.vp[i])) continue;
    const uint32_t M = px.M[i];
    if (M > 0) {
      const float N = px.N[i], r = px.radius[i];
      const float new_N = N + alpha * (float)M;
      const float new_R = r * sqrtf(new_N / (N + (float)M));
      const float4 p4 = px.phi[i];
      const F3 phi = mk3(p4.x, p4.y, p4.z);
      const F3 thr = xyz(px.vp[i].thr);
      const F3 tau = (xyz(px.tau[i]) + thr * phi) * (new_R * new_R) / (r * r);
      px.tau[i] = make_float4(tau.x, tau.y, tau.z, 0.f);
      px.N[i] = new_N;
      px.radius[i] = new_R;
      px.M[i] = 0;
      px.phi[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
}

// ComputePixelRadiance (sppm.cpp:171-180): the direct light summed over the
// iterations as the reference's per-pixel accumulator sums it, divided by
// their count, plus the photon estimate; written as one film sample.
__global__ void k_final(SppmArgs a, SppmPixels px, uint32_t iters,
                        uint64_t photon_n, float4* fsum, float4* fcomp,
                        float* rad) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.npix;
       i += gridDim.x * blockDim.x) {
    const F3 d1 = xyz(px.direct[i]);
    F3 acc = mk3(0.f, 0.f, 0.f);
    for (uint32_t k = 0; k < iters; ++k) acc = acc + d1;
    const F3 direct = acc / (float)iters;
    const float r = px.radius[i];
    const float dem = (float)photon_n * kPi * r * r;
    const F3 L = direct + xyz(px.tau[i]) / dem;
    fsum[i] = make_float4(L.x, L.y, L.z, 1.f);
    fcomp[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (rad) {
      rad[3 * (uint64_t)i] = L.x;
      rad[3 * (uint64_t)i + 1] = L.y;
      rad[3 * (uint64_t)i + 2] = L.z;
    }
  }
}

__global__ void k_fill_f(float* p, uint64_t n, float v) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    p[i] = v;
}

template <class T>
struct Dev {
  T* p = nullptr;
  cudaStream_t s = nullptr;
  cudaError_t alloc(uint64_t count, cudaStream_t st) {
    s = st;
    return cudaMallocAsync((void**)&p, std::max<uint64_t>(16, count * sizeof(T)),
                           st);
  }
  ~Dev() {
    if (p) cudaFreeAsync(p, s);
  }
};

}  // namespace

int sppm_render(ajg_scene* sc, const ajg_camera& cam, const ajg_sppm_params& p,
                float4* d_out, float* d_rad, cudaStream_t st) {
  ajg_ctx* ctx = sc->ctx;
  const DeviceScene& s = sc->d;
  const uint64_t npix = (uint64_t)cam.width * cam.height;
  if (npix == 0 || npix > (1ull << 30))
    return fail(ctx, AJG_ERR_INVALID, "empty or too large film");
  if (p.iterations == 0) return fail(ctx, AJG_ERR_INVALID, "no iterations");
  if (p.forward_max_depth < 1 || p.forward_max_depth > 1024 ||
      p.photon_max_depth < 0 || p.photon_max_depth > 1024)
    return fail(ctx, AJG_ERR_INVALID, "depths must be in [1, 1024]");
  if (!(p.init_radius != 0.f) || !std::isfinite(p.init_radius))
    return fail(ctx, AJG_ERR_INVALID, "init_radius must be nonzero and finite");

  // the world grown by the initial radius (sppm.cpp:184-194)
  const F3 wlo = mk3(sc->world[0], sc->world[1], sc->world[2]);
  const F3 whi = mk3(sc->world[3], sc->world[4], sc->world[5]);
  float init_radius = p.init_radius;
  if (init_radius < 0) {
    const F3 d = whi - wlo;
    float q = 0.f;
    q += d.x * d.x;
    q += d.y * d.y;
    q += d.z * d.z;
    init_radius = std::sqrt(q) / 1000.f;
  }
  SppmArgs a{};
  a.s = s;
  a.lo = wlo - mk3(init_radius, init_radius, init_radius);
  a.center = (whi + wlo) / 2.f;
  a.init_radius = init_radius;
  a.pseed = photon_seed(p.seed);
  a.npix = (uint32_t)npix;
  a.pmin = p.photon_min_depth;
  a.pmax = p.photon_max_depth;
  a.cont = p.photon_cont_prob;
  // DefaultScene's selector over its lights: pdf 1/n each, the cdf as
  // Distribution::SetFunction builds it (distribution.h:37-56)
  a.nl = s.num_lights;
  if (a.nl) {
    std::vector<float> table(a.nl, 1.f);
    float sum = 0.f;
    for (float t : table) sum += t;
    const float ratio = 1.f / sum;
    for (float& t : table) t *= ratio;
    const float inv = 1.f / float(a.nl);
    a.cdf[0] = 0.f;
    for (uint32_t i = 1; i <= a.nl; ++i) a.cdf[i] = a.cdf[i - 1] + table[i - 1] * inv;
    const float fi = a.cdf[a.nl];
    for (uint32_t i = 0; i <= a.nl; ++i)
      a.cdf[i] = fi > 0.f ? a.cdf[i] / fi : float(i) / float(a.nl);
    a.lpdf = table[0];
  }

  Dev<VisPointD> vp;
  Dev<float4> direct, phi, tau, film;
  Dev<float> radius, N, maxr;
  Dev<uint32_t> M, counts, offsets, cursor, items, bits;
  Dev<float4> spheres;
  const uint32_t cap = (uint32_t)std::min<uint64_t>(8 * npix, 0xffffffffull);
  cudaError_t e = cudaSuccess;
  auto A = [&](cudaError_t r) {
    if (e == cudaSuccess) e = r;
  };
  A(vp.alloc(npix, st));
  A(direct.alloc(npix, st));
  A(phi.alloc(npix, st));
  A(tau.alloc(npix, st));
  A(film.alloc(2 * npix, st));
  A(radius.alloc(npix, st));
  A(N.alloc(npix, st));
  A(maxr.alloc(1, st));
  A(M.alloc(npix, st));
  A(counts.alloc(kEntries, st));
  A(offsets.alloc(kEntries + 1, st));
  A(cursor.alloc(kEntries, st));
  A(items.alloc(cap, st));
  A(spheres.alloc(cap, st));
  A(bits.alloc(1, st));
  // the photon queue, in chunks of at most the context's wave size
  const uint64_t chunk = std::max<uint64_t>(
      1, std::min<uint64_t>(p.photons_per_iteration, ctx->wave_paths));
  Dev<float4> qro, qrd, qcoef;
  Dev<ajg_hit> qhits;
  Dev<uint32_t> qcounts;
  A(qro.alloc(2 * chunk, st));
  A(qrd.alloc(2 * chunk, st));
  A(qcoef.alloc(2 * chunk, st));
  A(qhits.alloc(chunk, st));
  A(qcounts.alloc(4, st));
  if (e != cudaSuccess)
    return fail(ctx, AJG_ERR_OOM, "device allocation failed (SPPM buffers)");

  int rc = sppm_camera_pass(sc, cam, p.forward_max_depth, p.seed, vp.p,
                            direct.p, st);
  if (rc) return rc;

  const int gs = kSMs * 8;
  cudaMemsetAsync(phi.p, 0, npix * sizeof(float4), st);
  cudaMemsetAsync(tau.p, 0, npix * sizeof(float4), st);
  cudaMemsetAsync(N.p, 0, npix * sizeof(float), st);
  cudaMemsetAsync(M.p, 0, npix * sizeof(uint32_t), st);
  k_fill_f<<<grid_for(npix, 256, gs), 256, 0, st>>>(radius.p, npix, init_radius);
  k_fill_f<<<1, 32, 0, st>>>(maxr.p, 1, init_radius);
  const SppmPixels px{vp.p, direct.p, radius.p, N.p, M.p, phi.p, tau.p};
  const Grid g{counts.p, offsets.p, cursor.p, items.p, spheres.p, cap, maxr.p};
  PhotonQ q{};
  q.ro[0] = qro.p;
  q.ro[1] = qro.p + chunk;
  q.rd[0] = qrd.p;
  q.rd[1] = qrd.p + chunk;
  q.coef[0] = qcoef.p;
  q.coef[1] = qcoef.p + chunk;
  q.hits = qhits.p;
  q.counts = qcounts.p;
  q.cap = (uint32_t)chunk;
  for (uint32_t it = 0; it < p.iterations; ++it) {
    a.it = it;
    cudaMemsetAsync(counts.p, 0, kEntries * sizeof(uint32_t), st);
    k_grid_count<<<grid_for(npix, 256, gs), 256, 0, st>>>(a, px, g, ctx->d_error);
    k_grid_scan<<<1, 1024, 0, st>>>(g);
    k_grid_fill<<<grid_for(npix, 256, gs), 256, 0, st>>>(a, px, g, ctx->d_error);
    for (uint64_t i0 = 0; i0 < p.photons_per_iteration; i0 += chunk) {
      const uint32_t n =
          (uint32_t)std::min<uint64_t>(chunk, p.photons_per_iteration - i0);
      cudaMemsetAsync(q.counts, 0, 4 * sizeof(uint32_t), st);
      k_photon_emit<<<grid_for(n, kThreads, gs), kThreads, 0, st>>>(
          a, q, (uint32_t)i0, n, ctx->d_error);
      int cur = 0;
      for (int depth = 1; depth <= p.photon_max_depth; ++depth) {
        cudaMemsetAsync(&q.counts[cur ^ 1], 0, sizeof(uint32_t), st);
        cudaMemsetAsync(&q.counts[2], 0, sizeof(uint32_t), st);
        // photon rays keep the wide tree: over the binary layout the
        // photon pass measured 8% slower (long rays from the lights)
        dispatch_trace(s.tri_test, s.width, [&](auto T, auto Wd) {
          constexpr int TT = decltype(T)::value, WW = decltype(Wd)::value;
          const int gr = resident_grid((const void*)k_photon_extend<TT, WW>, 128);
          k_photon_extend<TT, WW><<<gr, 128, 0, st>>>(
              s, q.ro[cur], q.rd[cur], &q.counts[cur], &q.counts[2], q.hits,
              &ctx->d_counters[0], ctx->d_error);
        });
        k_photon_shade<<<gs, kThreads, 0, st>>>(a, px, g, q, cur, depth,
                                                ctx->d_error);
        cur ^= 1;
      }
      ctx->paths_total += n;
    }
    cudaMemsetAsync(bits.p, 0, sizeof(uint32_t), st);
    k_max_radius<<<grid_for(npix, 256, gs), 256, 0, st>>>(a, px, bits.p);
    k_update<<<grid_for(npix, 256, gs), 256, 0, st>>>(a, px, p.update_alpha,
                                                      bits.p, maxr.p);
  }
  const uint64_t photon_n =
      (uint64_t)p.iterations * (uint64_t)p.photons_per_iteration;
  k_final<<<grid_for(npix, 256, gs), 256, 0, st>>>(
      a, px, p.iterations, photon_n, film.p, film.p + npix, d_rad);
  if (d_out)
    enqueue_resolve(film.p, film.p + npix, nullptr, cam.width, cam.height,
                    true, true, d_out, st);
  const cudaError_t le = cudaGetLastError();
  if (le != cudaSuccess) return fail(ctx, AJG_ERR_CUDA, cudaGetErrorString(le));
  return AJG_OK;
}

}  // namespace ajg
