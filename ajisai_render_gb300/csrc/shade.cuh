// Device shading for the PT-MIS path: hit completion (PostIntersect rules),
// the Lambertian AggregateBSDF and the Disney BSDF, directional and constant
// environment lights, and the thin-lens camera.  Each function keeps the
// reference's evaluation order (cited per function); transcendental
// functions are CUDA's own (sinf, cosf, acosf, atan2f, tanf), so shading is
// within a few ulp of the reference rather than bit-equal.
#pragma once
#include <cfloat>

#include "common.cuh"
#include "scene.cuh"

namespace ajg {

// libstdc++'s std::lerp for floats (C++20 <cmath>)
__device__ __forceinline__ float std_lerp(float a, float b, float t) {
  if ((a <= 0 && b >= 0) || (a >= 0 && b <= 0)) return t * b + (1 - t) * a;
  if (t == 1) return b;
  const float x = a + t * (b - a);
  return (t > 1) == (b > a) ? (b < x ? x : b) : (b > x ? x : b);
}
// core/material/disney.cpp:48-52
__device__ __forceinline__ float dlerp(float a, float b, float t) {
  return a * (1 - t) + b * t;
}
__device__ __forceinline__ F3 dlerp(F3 a, F3 b, float t) {
  return a * (1 - t) + b * t;
}
__device__ __forceinline__ float clampf(float v, float lo, float hi) {
  return v < lo ? lo : (hi < v ? hi : v);
}

// CoordinateSystem (core/coordinate_system.h:37-52)
struct Frame {
  F3 dx, dy, dz;
  __device__ __forceinline__ explicit Frame(F3 n) : dz(n) {
    const float sign = copysignf(1.f, n.z);
    const float a = -1.f / (sign + n.z);
    const float b = n.x * n.y * a;
    dx = mk3(1.f + sign * n.x * n.x * a, sign * b, -sign * n.x);
    dy = mk3(b, sign + n.y * n.y * a, -n.y);
  }
  __device__ __forceinline__ F3 to_local(F3 v) const {
    return mk3(dot3(v, dx), dot3(v, dy), dot3(v, dz));
  }
  __device__ __forceinline__ F3 to_world(F3 v) const {
    return dx * v.x + dy * v.y + dz * v.z;
  }
};

// core/warp.h:29-72
__device__ __forceinline__ void concentric(float sx, float sy, float& px,
                                           float& py) {
  const float ox = 2.f * sx - 1.f, oy = 2.f * sy - 1.f;
  float r, phi;
  if (ox == 0 && oy == 0) {
    px = 0.f;
    py = 0.f;
    return;
  } else if (fabsf(ox) > fabsf(oy)) {
    r = ox;
    phi = kPi4 * (oy / ox);
  } else {
    r = oy;
    phi = kPi2 - kPi4 * (ox / oy);
  }
  px = r * cosf(phi);
  py = r * sinf(phi);
}
__device__ __forceinline__ F3 cosine_hemisphere(float sx, float sy,
                                                float* pdf) {
  float px, py;
  concentric(sx, sy, px, py);
  float r = 0.f;
  r += px * px;
  r += py * py;
  float z = sqrtf(ref_max(0.0f, 1 - r));
  if (z == 0) z = 1e-10f;
  if (pdf) *pdf = z * kInvPi;
  return mk3(px, py, z);
}
// core/warp.h:74-80, 100-104
__device__ __forceinline__ F3 uniform_cone(float u0, float u1, float cmax) {
  const float ct = (1.f - u0) + u0 * cmax;
  const float st = sqrtf(ref_max(0.f, 1.f - ct * ct));
  const float phi = u1 * 2 * kPi;
  return mk3(cosf(phi) * st, sinf(phi) * st, ct);
}
__device__ __forceinline__ float uniform_cone_pdf(float cmax) {
  if (cmax == 1.0f) return 1.0f;
  return 1.0f / (2.0f * kPi * (1.0f - cmax));
}
// core/bsdf/bsdf.h:42-46
__device__ __forceinline__ float correct_shading_normal(F3 ng, F3 ns, F3 wi) {
  const float denom = fabsf(dot3(ng, wi));
  return denom == 0 ? 1.f : fabsf(dot3(ns, wi) / denom);
}

struct BsdfSample {
  F3 dir, f;
  float pdf;
  bool delta = false;  // BSDFSampleResult::is_delta
};
__device__ __forceinline__ BsdfSample invalid_sample() {
  BsdfSample s;
  s.dir = mk3(0, 0, 0);
  s.f = mk3(0, 0, 0);
  s.pdf = 0.f;
  s.delta = false;
  return s;
}

struct MatParams {
  int type;
  F3 base;
  float subsurface, metallic, specular, specular_tint, roughness, sheen,
      sheen_tint, clearcoat, clearcoat_gloss, lum;
};
__device__ __forceinline__ MatParams load_material(const float* m,
                                                   float lum) {
  MatParams p;
  p.type = (int)m[0];
  p.base = mk3(m[1], m[2], m[3]);
  p.subsurface = m[4];
  p.metallic = m[5];
  p.specular = m[6];
  p.specular_tint = m[7];
  p.roughness = m[8];
  p.sheen = m[10];
  p.sheen_tint = m[11];
  p.clearcoat = m[12];
  p.clearcoat_gloss = m[13];
  p.lum = lum;
  return p;
}

// ----------------------------------------------------------- Lambertian --
// Diffuse::Shade -> AggregateBSDF{DiffuseComponent, weight 1}
// (core/material/diffuse.cpp:35-48, core/bsdf/aggregate_bsdf.cpp:43-131,
// core/bsdf/diffuse_component.cpp:28-64, core/bsdf/bsdf.cpp:30-63)
struct Lambert {
  F3 ng, ns, albedo, coef;
  __device__ __forceinline__ Lambert(F3 ng_, F3 ns_, F3 alb)
      : ng(ng_), ns(ns_), albedo(alb), coef(alb / kPi) {}
  __device__ __forceinline__ bool fringes(F3 w) const {
    return (dot3(ng, w) > 0) != (dot3(ns, w) > 0);
  }
  __device__ __forceinline__ BsdfSample sample(F3 wo, F3 sam) const {
    if (fringes(wo)) {
      if (dot3(ng, wo) <= 0.f) return invalid_sample();
      float pdf;
      const F3 lwi = cosine_hemisphere(sam.x, sam.y, &pdf);
      if (pdf < FLT_EPSILON) return invalid_sample();
      const F3 wi = normalize3(Frame(ng).to_world(lwi));
      const float factor = correct_shading_normal(ng, ns, wi);
      BsdfSample s;
      s.dir = wi;
      s.f = albedo / kPi * factor;
      s.pdf = pdf;
      return s;
    }
    const Frame sf(ns);
    const F3 lwo = normalize3(sf.to_local(wo));
    if (lwo.z <= 0.f) return invalid_sample();
    float pdf;
    F3 lwi = cosine_hemisphere(sam.y, sam.z, &pdf);
    // pdf < 1e-3 compares in double in the reference
    // (diffuse_component.cpp:39); for a float pdf that is pdf < 1e-3f
    // exactly, as no float lies in [1e-3, 1e-3f)
    if (pdf < 1e-3f) return invalid_sample();
    lwi = normalize3(lwi);
    pdf *= 1.f;
    const F3 wi = sf.to_world(lwi);
    const float factor = correct_shading_normal(ng, ns, wi);
    BsdfSample s;
    s.dir = wi;
    s.f = coef * factor;
    s.pdf = pdf;
    return s;
  }
  __device__ F3 eval(F3 wi, F3 wo) const {
    if (fringes(wo)) {
      if ((dot3(ng, wi) <= 0.f) || (dot3(ng, wo) <= 0.f)) return mk3(0, 0, 0);
      return albedo / kPi;
    }
    const Frame sf(ns);
    const F3 lwi = normalize3(sf.to_local(wi));
    const F3 lwo = normalize3(sf.to_local(wo));
    if (lwi.z <= 0.f || lwo.z <= 0.f) return mk3(0, 0, 0);
    return mk3(0, 0, 0) + coef;
  }
  __device__ float pdf(F3 wi, F3 wo) const {
    if (fringes(wo)) {
      if ((dot3(ng, wi) > 0.f) != (dot3(ng, wo) > 0.f)) return 0.f;
      const F3 local = normalize3(Frame(ng).to_local(wi));
      return local.z * kInvPi;
    }
    const Frame sf(ns);
    const F3 lwi = normalize3(sf.to_local(wi));
    const F3 lwo = normalize3(sf.to_local(wo));
    if (lwi.z <= 0.f || lwo.z <= 0.f) return 0.f;
    float wsum = 0.f, p = 0.f;
    wsum += 1.f;
    p += 1.f * (lwi.z * kInvPi);
    return wsum > 0 ? p / wsum : 0;
  }
};

// ----------------------------------------------------- float-float helpers --
// The reference evaluates the VNDF slope fit in double (disney.cpp:400-407).
// GB300 issues FP64 at a small fraction of the FP32 rate, so the fit is
// evaluated in float-float arithmetic (unevaluated sums hi + lo; Dekker's
// and Knuth's error-free transformations, FMA-based products): about 48
// significant bits, against the fit's denominator cancelling to ~2e-5 near
// u2 = 1, so the result rounds to the same float as the double evaluation
// except when that lands within ~2^-32 relative of a rounding boundary.
struct FF {
  float hi, lo;
};
__host__ __device__ __forceinline__ float fma_rn(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return fmaf(a, b, c);
#endif
}
__host__ __device__ __forceinline__ FF ff_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return FF{s, (a - (s - bb)) + (b - bb)};
}
__host__ __device__ __forceinline__ FF ff_fast_two_sum(float a, float b) {
  const float s = a + b;
  return FF{s, b - (s - a)};
}
__host__ __device__ __forceinline__ FF ff_add(FF x, FF y) {
  FF s = ff_two_sum(x.hi, y.hi);
  const FF t = ff_two_sum(x.lo, y.lo);
  s.lo += t.hi;
  s = ff_fast_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return ff_fast_two_sum(s.hi, s.lo);
}
__host__ __device__ __forceinline__ FF ff_mul(FF x, FF y) {
  const float p = x.hi * y.hi;
  float e = fma_rn(x.hi, y.hi, -p);
  e = fma_rn(x.hi, y.lo, e);
  e = fma_rn(x.lo, y.hi, e);
  return ff_fast_two_sum(p, e);
}
__host__ __device__ __forceinline__ FF ff_div(FF x, FF y) {
  const float q1 = x.hi / y.hi;
  const FF r = ff_add(x, ff_mul(FF{-q1, 0.f}, y));
  const float q2 = r.hi / y.hi;
  const FF q = ff_fast_two_sum(q1, q2);
  const FF r2 = ff_add(x, ff_mul(FF{-q.hi, -q.lo}, y));
  return ff_add(q, FF{r2.hi / y.hi, 0.f});
}
#define AJG_FF_CONST(c) FF{(float)(c), (float)((c) - (double)(float)(c))}
// rounds hi + lo to the nearest float (hi is already the nearest float to
// the unevaluated sum after the final renormalisation)
__host__ __device__ __forceinline__ float ff_round(FF x) { return x.hi + x.lo; }

// z(u2) of the VNDF slope fit (disney.cpp:400-407)
__host__ __device__ __forceinline__ float vndf_fit_z(float u2f) {
  const FF u = FF{u2f, 0.f};
  FF num = ff_add(ff_mul(u, AJG_FF_CONST(-0.365728915865723)),
                  AJG_FF_CONST(0.790235037209296));
  num = ff_add(ff_mul(u, num), AJG_FF_CONST(-0.424965825137544));
  num = ff_add(ff_mul(u, num), AJG_FF_CONST(0.000152998850436920));
  FF den = ff_add(ff_mul(u, AJG_FF_CONST(0.169507819808272)),
                  AJG_FF_CONST(-0.397203533833404));
  den = ff_add(ff_mul(u, den), AJG_FF_CONST(-0.232500544458471));
  den = ff_add(ff_mul(u, den), FF{1.f, 0.f});
  den = ff_add(ff_mul(u, den), AJG_FF_CONST(-0.539825872510702));
  return ff_round(ff_div(num, den));
}

// --------------------------------------------------------------- Disney --
// DisneyBSDF (core/material/disney.cpp:58-473)
struct DisneyB {
  const MatParams& m;
  Frame sf;
  __device__ __forceinline__ DisneyB(const MatParams& mat, F3 ns)
      : m(mat), sf(ns) {}

  __device__ static float tan_theta(F3 v) {
    const float temp = 1 - v.z * v.z;
    if (temp <= 0.0f) return 0.0f;
    return sqrtf(temp) / v.z;
  }
  __device__ static float tan2(F3 v) {
    const float tmp = 1.f - v.z * v.z;
    if (tmp <= 0.f) return 0.f;
    return tmp / (v.z * v.z);
  }
  __device__ static F3 reflect(F3 vi, F3 n) {
    return vi + (2 * dot3(-vi, n) * n);
  }
  __device__ static float ggx_d(F3 wh, float alpha) {
    if (wh.z <= 0.f) return 0.f;
    const float t2 = tan2(wh);
    const float c2 = wh.z * wh.z;
    const float root = alpha / (c2 * (alpha * alpha + t2));
    return kInvPi * (root * root);
  }
  __device__ static float smith_g(F3 v, F3 wh, float alpha) {
    const float tt = fabsf(tan_theta(v));
    if (tt == 0.0f) return 1.0f;
    if (dot3(v, wh) * v.z <= 0) return 0.0f;
    const float root = alpha * tt;
    return 2.0f / (1.0f + sqrtf(1.0f + root * root));
  }
  __device__ static float ggx_g(F3 wi, F3 wo, F3 wh, float alpha) {
    return smith_g(wo, wh, alpha) * smith_g(wi, wh, alpha);
  }
  __device__ static float pdf_vn(F3 wi, F3 h, float alpha) {
    const float D = ggx_d(h, alpha);
    return smith_g(wi, h, alpha) * fabsf(dot3(wi, h)) * D /
           (fabsf(wi.z) + 1e-4f);
  }
  __device__ static void vn_unit(float thetaI, float u1, float u2, float& sx,
                                 float& sy) {
    if (thetaI < 1e-4f) {
      const float R = sqrtf(ref_max(u1 / ((1 - u1) + 1e-6f), 0.0f));
      const float SinPhi = sinf(2 * kPi * u2);
      const float CosPhi = cosf(2 * kPi * u2);
      sx = R * CosPhi;
      sy = R * SinPhi;
      return;
    }
    const float TanThetaI = tanf(thetaI);
    const float a = 1 / TanThetaI;
    const float G1 = 2.0f / (1.0f + sqrtf(ref_max(1.0f + 1.0f / (a * a), 0.0f)));
    float A = 2.0f * u1 / G1 - 1.0f;
    if (fabsf(A) == 1) A -= (A >= 0.0f ? 1.0f : -1.0f) * 1e-4f;
    const float Temp = 1.0f / (A * A - 1.0f);
    const float B = TanThetaI;
    const float D =
        sqrtf(ref_max(B * B * Temp * Temp - (A * A - B * B) * Temp, 0.0f));
    const float x1 = B * Temp - D;
    const float x2 = B * Temp + D;
    sx = (A < 0.0f || x2 > 1.0f / TanThetaI) ? x1 : x2;
    float S;
    if (u2 > 0.5f) {
      S = 1.0f;
      u2 = 2.0f * (u2 - 0.5f);
    } else {
      S = -1.0f;
      u2 = 2.0f * (0.5f - u2);
    }
    // the published rational fit of the slope distribution, which the
    // reference evaluates in double (disney.cpp:400-407): float-float here
    const float z = vndf_fit_z(u2);
    sy = S * z * sqrtf(1.0f + sx * sx);
  }
  __device__ static __forceinline__ F3 sample_vn(F3 wi_in, float u1, float u2,
                                                float Alpha) {
    const F3 wi = normalize3(mk3(Alpha * wi_in.x, Alpha * wi_in.y, wi_in.z));
    float Theta = 0, Phi = 0;
    if (wi.z < 0.99999f) {
      Theta = acosf(wi.z);
      Phi = atan2f(wi.y, wi.x);
    }
    const float SinPhi = sinf(Phi), CosPhi = cosf(Phi);
    float sx, sy;
    vn_unit(Theta, u1, u2, sx, sy);
    float rx = CosPhi * sx - SinPhi * sy;
    float ry = SinPhi * sx + CosPhi * sy;
    rx *= Alpha;
    ry *= Alpha;
    const float Norm = 1.f / sqrtf(rx * rx + ry * ry + 1.0f);
    return mk3(-rx * Norm, -ry * Norm, Norm);
  }
  __device__ float fresnel_conductor(float cosi, float eta, float k) const {
    const float tmp = (eta * eta + k * k) * cosi * cosi;
    const float Rparl2 =
        (tmp - (2.f * eta * cosi) + 1) / (tmp + (2.f * eta * cosi) + 1);
    const float tmp_f = eta * eta + k * k;
    const float Rperp2 = (tmp_f - (2.f * eta * cosi) + cosi * cosi) /
                         (tmp_f + (2.f * eta * cosi) + cosi * cosi);
    return 0.5f * (Rparl2 + Rperp2);
  }
  __device__ float fresnel_schlick(float cosD, float R0) const {
    const float omc = 1.f - cosD;
    const float omc2 = omc * omc;
    const float fr = R0 + (1.f - R0) * omc2 * omc2 * omc;
    const float fc = fresnel_conductor(cosD, 0.4f, 1.6f);
    return std_lerp(fr, fc, m.metallic);
  }
  __device__ static float fresnel_coat(float cosD) {
    const float omc = 1.0f - cosD;
    const float omc2 = omc * omc;
    return 0.04f + (1.0f - 0.04f) * omc2 * omc2 * omc;
  }
  __device__ float diffuse_term(F3 wi, F3 wo, float idh, float rough) const {
    if (m.metallic == 1.f) return 0.f;
    const float l = 1.f - fabsf(wi.z), l2 = l * l;
    const float v = 1.f - fabsf(wo.z), v2 = v * v;
    const float FD90 = 0.5f + 2.f * idh * rough;
    return kInvPi * (1.f + (FD90 - 1.f) * l2 * l2 * l) *
           (1.f + (FD90 - 1.f) * v2 * v2 * v);
  }
  __device__ float specular_term(F3 wi, F3 wo, F3 wh, float odh,
                                 float rough) const {
    if (wi.z * wo.z <= 0.f) return 0.f;
    const float D = ggx_d(wh, rough * rough);
    if (D == 0.f) return 0.f;
    const float nr = std_lerp(0.f, 0.08f, m.specular);
    const float F = fresnel_schlick(odh, nr);
    const float rg = (0.5f + 0.5f * rough);
    const float G = ggx_g(wi, wo, wh, rg * rg);
    return F * D * G / (4.f * fabsf(wi.z) * fabsf(wo.z));
  }
  __device__ float subsurface_term(F3 wi, F3 wo, float idh,
                                   float rough) const {
    if (m.subsurface == 0.0f) return 0.0f;
    const float l = 1.0f - fabsf(wi.z), l2 = l * l;
    const float v = 1.0f - fabsf(wo.z), v2 = v * v;
    const float F = idh * idh * rough;
    const float S = (1.0f + (F - 1.0f) * l2 * l2 * l) *
                    (1.0f + (F - 1.0f) * v2 * v2 * v);
    return kInvPi * 1.25f *
           (S * (1.0f / (fabsf(wo.z) + fabsf(wi.z)) - 0.5f) + 0.5f);
  }
  __device__ float clearcoat_term(F3 wi, F3 wo, F3 wh, float idh,
                                  float gloss) const {
    if (m.clearcoat == 0.0f) return 0.0f;
    const float rough = dlerp(0.005f, 0.1f, gloss);
    const float D = ggx_d(wh, rough);
    if (D == 0.0f) return 0.0f;
    const float F = fresnel_coat(idh);
    const float G = ggx_g(wo, wi, wh, 0.25f);
    return m.clearcoat * D * F * G / (4.0f * fabsf(wi.z) * fabsf(wo.z));
  }
  __device__ __forceinline__ F3 eval(F3 wi, F3 wo) const {
    const F3 lwi = normalize3(sf.to_local(wi));
    const F3 lwo = normalize3(sf.to_local(wo));
    if (fabsf(lwi.z) < FLT_EPSILON || fabsf(lwo.z) < FLT_EPSILON)
      return mk3(0, 0, 0);
    const float rough = clampf(m.roughness, 0.02f, 1.f);
    const F3 untinted = mk3(m.lum, m.lum, m.lum);
    F3 spec_alb = dlerp(dlerp(m.base, untinted, 1.0f - m.specular_tint),
                        m.base, m.metallic);
    const F3 sheen_alb = dlerp(untinted, m.base, m.sheen_tint);
    const F3 wh = normalize3(lwo + lwi);
    const float odh = dot3(lwo, wh);
    const float idh = dot3(lwi, wh);
    const float omo = 1.f - odh;
    spec_alb = dlerp(spec_alb, untinted, omo * omo * omo);
    const float F = fresnel_schlick(odh, 0.0f);
    const F3 sheen_term = F * m.sheen * sheen_alb;
    const float dl = dlerp(diffuse_term(lwi, lwo, idh, rough),
                           subsurface_term(lwi, lwo, idh, rough), m.subsurface);
    const F3 t1 = (1.0f - m.metallic) * (m.base * dl + sheen_term);
    const F3 t2 = spec_alb * specular_term(lwi, lwo, wh, odh, rough);
    const float cc = clearcoat_term(lwi, lwo, wh, idh, m.clearcoat_gloss);
    return t1 + t2 + mk3(cc, cc, cc);
  }
  __device__ __forceinline__ float pdf(F3 wi, F3 wo) const {
    const F3 lwi = normalize3(sf.to_local(wi));
    const F3 lwo = normalize3(sf.to_local(wo));
    const F3 wh = normalize3(lwo + lwi);
    if (maxc3(wh) <= 0.f) return 0.f;
    const float rough = clampf(m.roughness, 0.02f, 1.f);
    const float mpdf = pdf_vn(lwo, wh, rough * rough);
    float p = 0.f;
    const float dwhdwi = 1.f / (4.f * fabsf(dot3(lwi, wh)));
    const float spec_pdf = mpdf * dwhdwi;
    const float nr = std_lerp(0.f, 0.08f, m.specular);
    const float odh = dot3(lwo, wh);
    const float ps = fresnel_schlick(odh, nr);
    p += spec_pdf * ps;
    p += fabsf(lwi.z) * kInvPi * (1.f - ps);
    if (m.clearcoat > 0.f) {
      // the clearcoat lobe reads the world-space wo (disney.cpp:208-220)
      const float cw = m.clearcoat / (m.clearcoat + m.lum);
      const float fc = fresnel_coat(fabsf(wo.z));
      const float pc = (fc * cw) / (fc * cw + (1 - fc) * (1 - cw));
      const float cr = std_lerp(0.005f, 0.10f, m.clearcoat_gloss);
      const float chp = pdf_vn(wo, wh, cr);
      const float cp = chp * dwhdwi;
      p *= 1.0f - pc;
      p += cp * pc;
    }
    return p;
  }
  // eval() and pdf() of the same (wi, wo) with their common
  // subexpressions computed once (the same operations, so bit-identical).
  // pdf is left at 0 when f is black unless pdf_if_black.
  __device__ __forceinline__ void eval_pdf(F3 wi, F3 wo, F3& f, float& pdf,
                                           bool pdf_if_black) const {
    const F3 lwi = normalize3(sf.to_local(wi));
    const F3 lwo = normalize3(sf.to_local(wo));
    const float rough = clampf(m.roughness, 0.02f, 1.f);
    const F3 wh = normalize3(lwo + lwi);
    f = mk3(0, 0, 0);
    if (!(fabsf(lwi.z) < FLT_EPSILON || fabsf(lwo.z) < FLT_EPSILON)) {
      const F3 untinted = mk3(m.lum, m.lum, m.lum);
      F3 spec_alb = dlerp(dlerp(m.base, untinted, 1.0f - m.specular_tint),
                          m.base, m.metallic);
      const F3 sheen_alb = dlerp(untinted, m.base, m.sheen_tint);
      const float odh = dot3(lwo, wh);
      const float idh = dot3(lwi, wh);
      const float omo = 1.f - odh;
      spec_alb = dlerp(spec_alb, untinted, omo * omo * omo);
      const float F = fresnel_schlick(odh, 0.0f);
      const F3 sheen_term = F * m.sheen * sheen_alb;
      const float dl =
          dlerp(diffuse_term(lwi, lwo, idh, rough),
                subsurface_term(lwi, lwo, idh, rough), m.subsurface);
      const F3 t1 = (1.0f - m.metallic) * (m.base * dl + sheen_term);
      const F3 t2 = spec_alb * specular_term(lwi, lwo, wh, odh, rough);
      const float cc = clearcoat_term(lwi, lwo, wh, idh, m.clearcoat_gloss);
      f = t1 + t2 + mk3(cc, cc, cc);
    }
    pdf = 0.f;
    if (!pdf_if_black && black3(f)) return;
    if (maxc3(wh) <= 0.f) return;
    const float mpdf = pdf_vn(lwo, wh, rough * rough);
    float p = 0.f;
    const float dwhdwi = 1.f / (4.f * fabsf(dot3(lwi, wh)));
    const float spec_pdf = mpdf * dwhdwi;
    const float nr = std_lerp(0.f, 0.08f, m.specular);
    const float odh = dot3(lwo, wh);
    const float ps = fresnel_schlick(odh, nr);
    p += spec_pdf * ps;
    p += fabsf(lwi.z) * kInvPi * (1.f - ps);
    if (m.clearcoat > 0.f) {
      const float cw = m.clearcoat / (m.clearcoat + m.lum);
      const float fc = fresnel_coat(fabsf(wo.z));
      const float pc = (fc * cw) / (fc * cw + (1 - fc) * (1 - cw));
      const float cr = std_lerp(0.005f, 0.10f, m.clearcoat_gloss);
      const float chp = pdf_vn(wo, wh, cr);
      const float cp = chp * dwhdwi;
      p *= 1.0f - pc;
      p += cp * pc;
    }
    pdf = p;
  }
  __device__ __forceinline__ BsdfSample sample(F3 wo, F3 sam) const {
    const F3 lwo = normalize3(sf.to_local(wo));
    F3 lwi, lwh;
    bool coat = false;
    float r0 = sam.x, r1 = sam.y;
    const float r2 = sam.z;
    if (m.clearcoat > 0.f) {
      const float cw = m.clearcoat / (m.clearcoat + m.lum);
      const float fc = fresnel_coat(fabsf(lwo.z));
      const float pc = (fc * cw) / (fc * cw + (1.f - fc) * (1.f - cw));
      if (sam.y < pc) {
        coat = true;
        r1 /= pc;
        const float cr = std_lerp(0.005f, 0.1f, m.clearcoat_gloss);
        lwh = sample_vn(lwo, r0, r1, cr);
        lwi = reflect(-lwo, lwh);
      } else {
        r1 = (sam.y - pc) / (1.f - pc);
      }
    }
    if (!coat) {
      const float rough = clampf(m.roughness, 0.02f, 1.0f);
      lwh = sample_vn(lwo, r0, r1, rough * rough);
      const float nr = std_lerp(0.0f, 0.08f, m.specular);
      const float odh = dot3(lwo, lwh);
      const float ps = fresnel_schlick(odh, nr);
      if (r2 <= ps) {
        lwi = reflect(-lwo, lwh);
      } else {
        lwi = cosine_hemisphere(r0, r1, nullptr);
        if (lwo.z < 0.0f) lwi.z *= -1.0f;
      }
    }
    if (lwi.z <= 0.0f) return invalid_sample();
    BsdfSample s;
    s.dir = sf.to_world(lwi);
    eval_pdf(s.dir, wo, s.f, s.pdf, true);
    return s;
  }
};

// One out-of-line copy of each BSDF routine: the path kernel calls them from
// ten sites per hit, and inlining them all overflows the instruction cache.
static __device__ __noinline__ F3 disney_eval(const float* __restrict__ m, float lum,
                                       F3 ns, F3 wi, F3 wo) {
  const MatParams p = load_material(m, lum);
  return DisneyB(p, ns).eval(wi, wo);
}
static __device__ __noinline__ float disney_pdf(const float* __restrict__ m,
                                         float lum, F3 ns, F3 wi, F3 wo) {
  const MatParams p = load_material(m, lum);
  return DisneyB(p, ns).pdf(wi, wo);
}
static __device__ __noinline__ BsdfSample disney_sample(const float* __restrict__ m,
                                                 float lum, F3 ns, F3 wo,
                                                 F3 sam) {
  const MatParams p = load_material(m, lum);
  return DisneyB(p, ns).sample(wo, sam);
}
static __device__ __noinline__ void disney_eval_pdf(const float* __restrict__ m,
                                                    float lum, F3 ns, F3 wi,
                                                    F3 wo, F3& f, float& pdf,
                                                    bool pdf_if_black) {
  const MatParams p = load_material(m, lum);
  DisneyB(p, ns).eval_pdf(wi, wo, f, pdf, pdf_if_black);
}
static __device__ __noinline__ BsdfSample lambert_sample(F3 ng, F3 ns, F3 alb,
                                                  F3 wo, F3 sam) {
  return Lambert(ng, ns, alb).sample(wo, sam);
}
static __device__ __noinline__ F3 lambert_eval(F3 ng, F3 ns, F3 alb, F3 wi, F3 wo) {
  return Lambert(ng, ns, alb).eval(wi, wo);
}
static __device__ __noinline__ float lambert_pdf(F3 ng, F3 ns, F3 alb, F3 wi, F3 wo) {
  return Lambert(ng, ns, alb).pdf(wi, wo);
}

// ------------------------------------- mirror, glass, metal, plastic, null --
// Material records ([16] floats after the type): base colour in [1..3], the
// type's parameters in [4..13] (glass: refraction colour, ior; metal: k,
// eta, u/v roughness; plastic: ior, thickness, sigma_a), and for plastic
// the constructor's terms the host computes once (plastic_bsdf.cpp:32-45):
// [14] the average transmittance exp(-2 thickness sigma_a), [15] the
// diffuse Fresnel integral.
constexpr int kMatOther = 7;  // shading class of the types >= AJG_MAT_MIRROR

// Fresnel::dielectricReflectance (bsdf/helper.h:35-56)
__device__ __forceinline__ float dielectric_reflectance(float eta,
                                                        float cos_i) {
  if (cos_i < 0.0f) {
    eta = 1.0f / eta;
    cos_i = -cos_i;
  }
  const float sin_t2 = eta * eta * (1.0f - cos_i * cos_i);
  if (sin_t2 > 1.0f) return 1.0f;
  const float cos_t = sqrtf(ref_max(1.0f - sin_t2, 0.0f));
  const float rs = (eta * cos_i - cos_t) / (eta * cos_i + cos_t);
  const float rp = (eta * cos_t - cos_i) / (eta * cos_t + cos_i);
  return (rs * rs + rp * rp) * 0.5f;
}

// DielectricFresnel::Eval (material/fresnel.h:95-118), one channel
__device__ __forceinline__ float dielectric_fresnel(float eta_in,
                                                    float eta_out,
                                                    float cos_i) {
  if (cos_i < 0) {
    const float t = eta_in;
    eta_in = eta_out;
    eta_out = t;
    cos_i = -cos_i;
  }
  const float sin_i = sqrtf(ref_max(0.f, 1 - cos_i * cos_i));
  const float sin_t = eta_out / eta_in * sin_i;
  if (sin_t >= 1.f) return 1.f;
  const float cos_t = sqrtf(ref_max(0.f, 1 - sin_t * sin_t));
  const float para = ((eta_in * cos_i) - (eta_out * cos_t)) /
                     ((eta_in * cos_i) + (eta_out * cos_t));
  const float perp = ((eta_out * cos_i) - (eta_in * cos_t)) /
                     ((eta_out * cos_i) + (eta_in * cos_t));
  return 0.5f * (para * para + perp * perp);
}

// ConductorFresnel::Eval (material/fresnel.h:40-58) with eta_out = 1, one
// channel: e2 = eta^2, k2 = k^2
__device__ __forceinline__ float conductor_fresnel1(float e2, float k2,
                                                    float cos_i) {
  const float cos2 = cos_i * cos_i;
  const float sin2 = ref_max(0.f, 1 - cos2);
  const float t0 = e2 - k2 - sin2;
  const float a2b2 = sqrtf(t0 * t0 + 4.f * e2 * k2);
  const float t1 = a2b2 + cos2;
  const float a = sqrtf(0.5f * (a2b2 + t0));
  const float t2 = 2.f * cos_i * a;
  const float rs = (t1 - t2) / (t1 + t2);
  const float t3 = cos2 * a2b2 + sin2 * sin2;
  const float t4 = t2 * sin2;
  const float rp = rs * (t3 - t4) / (t3 + t4);
  return 0.5f * (rp + rs);
}

// The base BSDF's black-fringe fallbacks (bsdf.cpp:30-63) for a BSDF of
// albedo `alb` (Metal's AggregateBSDF: 1; PlasticBsdf: its albedo).
struct Fringe {
  F3 ng, ns, alb;
  __device__ __forceinline__ bool causes(F3 w) const {
    return (dot3(ng, w) > 0) != (dot3(ns, w) > 0);
  }
  __device__ __forceinline__ BsdfSample sample(F3 wo, F3 sam) const {
    if (dot3(ng, wo) <= 0.f) return invalid_sample();
    float pdf;
    const F3 lwi = cosine_hemisphere(sam.x, sam.y, &pdf);
    if (pdf < FLT_EPSILON) return invalid_sample();
    const F3 wi = normalize3(Frame(ng).to_world(lwi));
    const float factor = correct_shading_normal(ng, ns, wi);
    BsdfSample s;
    s.dir = wi;
    s.f = alb / kPi * factor;
    s.pdf = pdf;
    return s;
  }
  __device__ __forceinline__ F3 eval(F3 wi, F3 wo) const {
    if ((dot3(ng, wi) <= 0.f) || (dot3(ng, wo) <= 0.f)) return mk3(0, 0, 0);
    return alb / kPi;
  }
  __device__ __forceinline__ float pdf(F3 wi, F3 wo) const {
    if ((dot3(ng, wi) > 0.f) != (dot3(ng, wo) > 0.f)) return 0.f;
    const F3 local = normalize3(Frame(ng).to_local(wi));
    return local.z * kInvPi;
  }
};

// MirrorBSDF (mirror.cpp:32-66): delta reflection about the shading normal.
__device__ __forceinline__ BsdfSample mirror_sample(const float* m, F3 ng,
                                                    F3 ns, F3 wo) {
  const Frame sf(ns);
  const F3 lwo = normalize3(sf.to_local(wo));
  if (lwo.z <= 0.f) return invalid_sample();
  const F3 lwi = mk3(-lwo.x, -lwo.y, lwo.z);
  const F3 wi = sf.to_world(lwi);
  const float factor = correct_shading_normal(ng, ns, wi);
  BsdfSample s;
  s.dir = wi;
  s.f = mk3(m[1], m[2], m[3]) * factor / fabsf(lwi.z);
  s.pdf = 1.f;
  s.delta = true;
  return s;
}

// GlassBSDF (glass.cpp:31-116) with Glass::Shade's colours (glass.cpp:
// 128-150: the refraction colour's square root): reflect with probability
// Fr, else refract; both delta.
__device__ __forceinline__ BsdfSample glass_sample(const float* m, F3 ng,
                                                   F3 ns, F3 wo, F3 sam) {
  const Frame sf(ns);
  const float ior = m[7];
  const F3 lwo = normalize3(sf.to_local(wo));
  const F3 normal = lwo.z > 0 ? mk3(0.f, 0.f, 1.f) : mk3(0.f, 0.f, -1.f);
  const float fr = dielectric_fresnel(ior, 1.f, lwo.z);
  BsdfSample s;
  s.delta = true;
  if (sam.x < fr) {
    const F3 lwi = mk3(-lwo.x, -lwo.y, lwo.z);
    const F3 wi = sf.to_world(lwi);
    const F3 f = mk3(m[1], m[2], m[3]) * mk3(fr, fr, fr) / fabsf(lwi.z);
    s.dir = wi;
    s.f = f * correct_shading_normal(ng, ns, wi);
    s.pdf = fr;
    return s;
  }
  const float eta_i = lwo.z > 0 ? 1.f : ior;
  const float eta_t = lwo.z > 0 ? ior : 1.f;
  const float eta = eta_i / eta_t;
  const float cos_i = fabsf(lwo.z);
  const float sin2_i = ref_max(0.f, 1.f - cos_i * cos_i);
  const float sin2_t = eta * eta * sin2_i;
  if (sin2_t > 1.f) return invalid_sample();
  const float cos_t = sqrtf(1 - sin2_t);
  const F3 lwi = normalize3((eta * cos_i - cos_t) * normal - eta * lwo);
  const F3 dir = sf.to_world(lwi);
  const F3 refr = mk3(sqrtf(m[4]), sqrtf(m[5]), sqrtf(m[6]));
  const F3 f = eta * eta * refr * (1.f - fr) / fabsf(lwi.z);
  s.dir = dir;
  s.f = f * correct_shading_normal(ng, ns, dir);
  s.pdf = 1.f - fr;
  return s;
}

// TrowbridgeReitzDistribution and EvalPdf of the GGX reflection component
// (microfacet_reflection_component.cpp:26-135)
__device__ __forceinline__ float sqrf(float x) { return x * x; }
__device__ __forceinline__ float ggx_phi(F3 w) {
  if (w.x <= 0.f && w.y <= 0.f) return 0.f;
  const float r = atan2f(w.y, w.x);
  return r < 0.f ? (r + 2 * kPi) : r;
}
__device__ __forceinline__ float ggx_tan_theta(F3 w) {
  const float t = 1 - w.z * w.z;
  if (t <= 0) return 0;
  return sqrtf(t) / w.z;
}
__device__ __forceinline__ float ggx_g(float cos_phi, float sin_phi, float ax,
                                       float ay, float tan_theta) {
  const float t = sqrf(ax * cos_phi) + sqrf(ay * sin_phi);
  const float sq = 1 + t * sqrf(tan_theta);
  const float lambda = -0.5f + 0.5f * sqrtf(sq);
  return 1 / (1 + lambda);
}
// f (coloured conductor Fresnel) when `f` is given, and the pdf
__device__ __forceinline__ void ggx_eval_pdf(const float* m, F3 lwi, F3 lwo,
                                             F3* f, float* pdf) {
  if (lwi.z <= 0 || lwo.z <= 0) {
    if (f) *f = mk3(0, 0, 0);
    if (pdf) *pdf = 0.f;
    return;
  }
  const float ax = m[10], ay = m[11];
  const float cos_i = lwi.z, cos_o = lwo.z;
  const F3 lwh = normalize3(lwi + lwo);
  const float cos_d = dot3(lwi, lwh);
  const float phi_h = ggx_phi(lwh);
  const float sin_phi_h = sinf(phi_h), cos_phi_h = cosf(phi_h);
  const float cos_h = lwh.z;
  const float sin_h = sqrtf(ref_max(0.f, 1 - cos_h * cos_h));
  const float A = sqrf(cos_phi_h / ax) + sqrf(sin_phi_h / ay);
  const float RD = sqrf(sin_h) * A + sqrf(cos_h);
  const float D = 1.f / (kPi * ax * ay * sqrf(RD));
  const float phi_o = ggx_phi(lwo);
  const float Go = ggx_g(cosf(phi_o), sinf(phi_o), ax, ay, ggx_tan_theta(lwo));
  if (f) {
    const float phi_i = ggx_phi(lwi);
    const float Gi =
        ggx_g(cosf(phi_i), sinf(phi_i), ax, ay, ggx_tan_theta(lwi));
    const float G = Gi * Go;
    F3 F = mk3(0.f, 0.f, 0.f);
    if (cos_d > 0.f)
      F = mk3(conductor_fresnel1((m[7] / 1.f) * (m[7] / 1.f),
                                 (m[4] / 1.f) * (m[4] / 1.f), cos_d),
              conductor_fresnel1((m[8] / 1.f) * (m[8] / 1.f),
                                 (m[5] / 1.f) * (m[5] / 1.f), cos_d),
              conductor_fresnel1((m[9] / 1.f) * (m[9] / 1.f),
                                 (m[6] / 1.f) * (m[6] / 1.f), cos_d));
    F = mk3(m[1], m[2], m[3]) * F;
    *f = F * D * G / fabsf(4 * cos_i * cos_o);
  }
  if (pdf) *pdf = Go * D / (4 * lwo.z);
}

// Metal::Shade (metal.cpp:42-66): an AggregateBSDF of albedo 1 with one
// GGX reflection component of weight 1 (aggregate_bsdf.cpp:43-131,
// microfacet_reflection_component.cpp:137-183).
__device__ __forceinline__ BsdfSample metal_sample(const float* m, F3 ng,
                                                   F3 ns, F3 wo, F3 sam) {
  const Fringe fr{ng, ns, mk3(1.f, 1.f, 1.f)};
  if (fr.causes(wo)) return fr.sample(wo, sam);
  const Frame sf(ns);
  const F3 lwo = normalize3(sf.to_local(wo));
  if (lwo.z <= 0.f) return invalid_sample();
  const float ax = m[10], ay = m[11];
  // TrowbridgeReitzDistribution::SampleWh
  const F3 vh = normalize3(mk3(ax * lwo.x, ay * lwo.y, lwo.z));
  const float lensq = vh.x * vh.x + vh.y * vh.y;
  const F3 t1 = lensq > FLT_EPSILON ? mk3(-vh.y, vh.x, 0) / sqrtf(lensq)
                                    : mk3(1, 0, 0);
  const F3 t2 = cross3(vh, t1);
  const float r = sqrtf(sam.y);
  const float phi = 2 * kPi * sam.z;
  const float t_1 = r * cosf(phi);
  const float t_2s = r * sinf(phi);
  const float sv = 0.5f * (1 + vh.z);
  const float t_2 = (1 - sv) * sqrtf(1 - t_1 * t_1) + sv * t_2s;
  const F3 nh = t_1 * t1 + t_2 * t2 +
                sqrtf(ref_max(0.f, 1.f - t_1 * t_1 - t_2 * t_2)) * vh;
  const F3 ne = normalize3(mk3(ax * nh.x, ay * nh.y, ref_max(0.f, nh.z)));
  const F3 lwh = normalize3(ne);
  if (lwh.z <= 0) return invalid_sample();
  F3 lwi = normalize3(2 * dot3(lwo, lwh) * lwh - lwo);
  if (lwi.z <= 0) return invalid_sample();
  F3 f;
  float pdf;
  ggx_eval_pdf(m, lwi, lwo, &f, &pdf);
  if (pdf == 0) return invalid_sample();
  lwi = normalize3(lwi);
  pdf *= 1.f;
  const F3 wi = sf.to_world(lwi);
  BsdfSample s;
  s.dir = wi;
  s.f = f * correct_shading_normal(ng, ns, wi);
  s.pdf = pdf;
  return s;
}
__device__ __forceinline__ void metal_eval_pdf(const float* m, F3 ng, F3 ns,
                                               F3 wi, F3 wo, F3& f,
                                               float& pdf) {
  const Fringe fr{ng, ns, mk3(1.f, 1.f, 1.f)};
  if (fr.causes(wo)) {
    f = fr.eval(wi, wo);
    pdf = fr.pdf(wi, wo);
    return;
  }
  const Frame sf(ns);
  const F3 lwi = normalize3(sf.to_local(wi));
  const F3 lwo = normalize3(sf.to_local(wo));
  if (lwi.z <= 0.f || lwo.z <= 0.f) {
    f = mk3(0, 0, 0);
    pdf = 0.f;
    return;
  }
  F3 g;
  float p;
  ggx_eval_pdf(m, lwi, lwo, &g, &p);
  f = mk3(0, 0, 0) + g;
  float wsum = 0.f, acc = 0.f;
  wsum += 1.f;
  acc += 1.f * p;
  pdf = wsum > 0 ? acc / wsum : 0;
}

// checkReflectionConstraint (bsdf/helper.h:26-31)
__device__ __forceinline__ bool reflection_constraint(F3 wi, F3 wo) {
  return fabsf(wi.z * wo.z - wi.x * wo.x - wi.y * wo.y - 1.0f) < 1e-3f;
}

// PlasticBsdf (plastic_bsdf.cpp:47-185): a delta coat reflection with
// probability Fi / (Fi + T (1 - Fi)), else the cosine-sampled substrate; no
// shading-normal correction, and Eval does not reject wi below the surface.
struct PlasticB {
  F3 ng, ns, albedo, scaled;
  float ior, avg_t, dfres;
  __device__ __forceinline__ PlasticB(const float* m, F3 ng_, F3 ns_)
      : ng(ng_), ns(ns_), albedo(mk3(m[1], m[2], m[3])), ior(m[4]),
        avg_t(m[14]), dfres(m[15]) {
    const float sc = m[5] * m[6];
    scaled = mk3(sc, sc, sc);
  }
  // Sample's substrate f (k = (1 - Fi)(1 - Fo) eta^2), and Eval's, which
  // also carries lwi.z / pi inside the scalar
  __device__ __forceinline__ F3 substrate_albedo() const {
    return albedo / (mk3(1.0f, 1.0f, 1.0f) - albedo * dfres);
  }
  __device__ __forceinline__ F3 absorb(F3 lwi, F3 lwo) const {
    const F3 e = scaled * (-1.0f / lwi.z - 1.0f / lwo.z);
    return mk3(expf(e.x), expf(e.y), expf(e.z));
  }
  __device__ __forceinline__ float spec_prob(float Fi) const {
    const float substrate_weight = avg_t * (1.0f - Fi);
    const float specular_weight = Fi;
    return specular_weight / (specular_weight + substrate_weight);
  }
  __device__ BsdfSample sample(F3 wo, F3 sam) const {
    const Fringe fr{ng, ns, albedo};
    if (fr.causes(wo)) return fr.sample(wo, sam);
    const Frame sf(ns);
    const F3 lwo = normalize3(sf.to_local(wo));
    if (lwo.z <= 0.f) return invalid_sample();
    const float eta = 1.f / ior;
    const float Fi = dielectric_reflectance(eta, lwo.z);
    const float sp = spec_prob(Fi);
    BsdfSample s;
    F3 lwi;
    if (sam.x < sp) {
      lwi = mk3(-lwo.x, -lwo.y, lwo.z);
      s.pdf = sp;
      const float v = Fi / sp;
      s.f = mk3(v, v, v);
      s.delta = true;
    } else {
      float pdf;
      lwi = cosine_hemisphere(sam.y, sam.z, &pdf);
      const float Fo = dielectric_reflectance(eta, lwi.z);
      F3 f = ((1.0f - Fi) * (1.0f - Fo) * eta * eta) * substrate_albedo();
      if (maxc3(scaled) > 0.0f) f = f * absorb(lwi, lwo);
      pdf *= (1.0f - sp);
      s.f = f / (1.0f - sp);
      s.pdf = pdf;
      s.delta = false;
    }
    s.dir = normalize3(sf.to_world(lwi));
    return s;
  }
  __device__ void eval_pdf(F3 wi, F3 wo, F3& f, float& pdf) const {
    const Fringe fr{ng, ns, albedo};
    if (fr.causes(wo)) {
      f = fr.eval(wi, wo);
      pdf = fr.pdf(wi, wo);
      return;
    }
    const Frame sf(ns);
    const F3 lwi = normalize3(sf.to_local(wi));
    const F3 lwo = normalize3(sf.to_local(wo));
    const float eta = 1.0f / ior;
    const float Fi = dielectric_reflectance(eta, lwo.z);
    const float Fo = dielectric_reflectance(eta, lwi.z);
    const bool coat = reflection_constraint(lwo, lwi);
    if (coat) {
      f = mk3(Fi, Fi, Fi);
    } else {
      f = ((1.0f - Fi) * (1.0f - Fo) * eta * eta * lwi.z * (1.f / kPi)) *
          substrate_albedo();
      if (maxc3(scaled) > 0.0f) f = f * absorb(lwi, lwo);
    }
    if (lwi.z <= 0.0f || lwo.z <= 0.0f) {
      pdf = 0.f;
      return;
    }
    const float sp = spec_prob(dielectric_reflectance(1.0f / ior, lwo.z));
    pdf = coat ? sp : lwi.z * kInvPi * (1.0f - sp);
  }
};

// The types >= AJG_MAT_MIRROR (type passed separately: the record's first
// word is a float in the scene tables and a uint32 in ajg_bsdf_query's).
static __device__ __noinline__ BsdfSample other_sample(int type,
                                                       const float* m, F3 ng,
                                                       F3 ns, F3 wo, F3 sam) {
  switch (type) {
    case AJG_MAT_MIRROR: return mirror_sample(m, ng, ns, wo);
    case AJG_MAT_GLASS: return glass_sample(m, ng, ns, wo, sam);
    case AJG_MAT_METAL: return metal_sample(m, ng, ns, wo, sam);
    case AJG_MAT_PLASTIC: return PlasticB(m, ng, ns).sample(wo, sam);
    default: {  // NullBsdf (null.cpp:31-52): straight through
      BsdfSample s;
      s.dir = -wo;
      s.f = mk3(1.f, 1.f, 1.f);
      s.pdf = 1.f;
      s.delta = true;
      return s;
    }
  }
}
static __device__ __noinline__ void other_eval_pdf(int type, const float* m,
                                                   F3 ng, F3 ns, F3 wi, F3 wo,
                                                   F3& f, float& pdf) {
  if (type == AJG_MAT_METAL) {
    metal_eval_pdf(m, ng, ns, wi, wo, f, pdf);
  } else if (type == AJG_MAT_PLASTIC) {
    PlasticB(m, ng, ns).eval_pdf(wi, wo, f, pdf);
  } else {  // mirror, glass, null: Eval 0, Pdf 0
    f = mk3(0, 0, 0);
    pdf = 0.f;
  }
}

// The BSDF at a hit: material record (in global memory) and the two normals.
struct Bsdf {
  int type;
  F3 ng, ns;
  const float* m;  // [16] record
  float lum;
  __device__ __forceinline__ F3 albedo() const {
    return mk3(m[1], m[2], m[3]);
  }
  __device__ __forceinline__ BsdfSample sample(F3 wo, F3 s) const {
    if (type == AJG_MAT_DIFFUSE) return lambert_sample(ng, ns, albedo(), wo, s);
    if (type == AJG_MAT_DISNEY) return disney_sample(m, lum, ns, wo, s);
    return other_sample(type, m, ng, ns, wo, s);
  }
  __device__ __forceinline__ F3 eval(F3 wi, F3 wo) const {
    if (type == AJG_MAT_DIFFUSE) return lambert_eval(ng, ns, albedo(), wi, wo);
    if (type == AJG_MAT_DISNEY) return disney_eval(m, lum, ns, wi, wo);
    F3 f;
    float p;
    other_eval_pdf(type, m, ng, ns, wi, wo, f, p);
    return f;
  }
  __device__ __forceinline__ float pdf(F3 wi, F3 wo) const {
    if (type == AJG_MAT_DIFFUSE) return lambert_pdf(ng, ns, albedo(), wi, wo);
    if (type == AJG_MAT_DISNEY) return disney_pdf(m, lum, ns, wi, wo);
    F3 f;
    float p;
    other_eval_pdf(type, m, ng, ns, wi, wo, f, p);
    return p;
  }
};

// The same with the material type fixed at compile time (the specialised
// shading kernels): NEE needs f and, when f is not black, the pdf.
template <int MAT>
struct BsdfT {
  F3 ng, ns;
  const float* m;
  float lum;
  __device__ __forceinline__ F3 albedo() const {
    return mk3(m[1], m[2], m[3]);
  }
  __device__ __forceinline__ BsdfSample sample(F3 wo, F3 s) const {
    if (MAT == AJG_MAT_DIFFUSE) return Lambert(ng, ns, albedo()).sample(wo, s);
    if (MAT == kMatOther) return other_sample((int)m[0], m, ng, ns, wo, s);
    return disney_sample(m, lum, ns, wo, s);
  }
  __device__ __forceinline__ void eval_pdf(F3 wi, F3 wo, F3& f,
                                           float& pdf) const {
    if (MAT == AJG_MAT_DIFFUSE) {
      const Lambert l(ng, ns, albedo());
      f = l.eval(wi, wo);
      pdf = black3(f) ? 0.f : l.pdf(wi, wo);
      return;
    }
    if (MAT == kMatOther) {
      other_eval_pdf((int)m[0], m, ng, ns, wi, wo, f, pdf);
      return;
    }
    disney_eval_pdf(m, lum, ns, wi, wo, f, pdf, false);
  }
};

// ------------------------------------------------------------ hit record --
struct HitInfo {
  F3 pos, ng, ns, wr;
  uint32_t mat;
};

// Triangle::Intersect's normal and the primitive's PostIntersect
// (core/geometry/quad.cpp:73-90, cube.cpp:96-108, mesh.cpp:183-204,
// two_sided.cpp:44-53): pos = o + t d, wr = -d.
__device__ __forceinline__ HitInfo complete_hit(const DeviceScene& s, F3 o,
                                                F3 d, float t, float u,
                                                float v, int prim) {
  HitInfo h;
  const float4 sh = __ldg(s.shade + prim);
  const uint32_t w = __float_as_uint(sh.w);
  const uint32_t fl = w >> 24;
  h.pos = o + t * d;
  h.ng = mk3(sh.x, sh.y, sh.z);
  if (fl & AJG_MESH_HAS_NORMALS) {
    const float* cn = s.corner + 9 * (uint64_t)prim;
    h.ns = (1 - u - v) * ld3(cn) + u * ld3(cn + 3) + v * ld3(cn + 6);
  } else {
    h.ns = h.ng;
  }
  h.wr = -d;
  if (fl & AJG_MESH_TWO_SIDED) {
    if (dot3(h.ng, h.wr) < 0) {
      h.ng = h.ng * -1.f;
      h.ns = h.ns * -1.f;
    }
  }
  h.mat = w & 0xffffffu;
  return h;
}

// intersection.h:42-47
__device__ __forceinline__ F3 eps_offset(const HitInfo& h, F3 dir) {
  if (dot3(dir, h.ng) > 0.f) return h.pos + h.ng * kRayEps;
  return h.pos - h.ng * kRayEps;
}
// renderer/helper.h:38-42
__device__ __forceinline__ float power_heuristic(float a, float b) {
  a *= a;
  b *= b;
  return a / (a + b);
}

// The Ray constructor (ray.h:33-39).
__device__ __forceinline__ void make_ray(F3 o, F3 d, F3& ro, F3& rd) {
  const F3 dn = normalize3(d);
  ro = o + dn * kRayEps;
  rd = normalize3(d);
}

// EnvLight::Pdf for a 1x1 texture (env_light.cpp:152-170): the 2D
// distribution's density is 1 when the texel has luminance.
__device__ __forceinline__ float env_pdf(bool env_has_mass, F3 ref2light) {
  const F3 d = normalize3(ref2light);
  const float theta = acosf(clampf(d.y, -1.f, 1.f));
  const float st = sinf(theta);
  const float p2 = env_has_mass ? 1.f : 0.f;
  return p2 / (2.f * kPi * kPi * st);
}

// ------------------------------------------------------------ area lights --
struct AreaSample {
  F3 pos, ng;
  float pdf;  // per unit area
};

// Geometry::Sample(ref, pdf, sam) of an emitter's surface from its light
// record `L` (kLightArea layout) and corner points `pts`:
//   TwoSided: sam.x < 0.5 picks the back face, x rescaled to [0,1), pdf
//     halved, the normal flipped there (two_sided.cpp:86-103);
//   the triangle point: (u, v) reflected when u + v > 1, p = (1-u-v) a +
//     u b + v c, n = normalize(cross(b - a, c - a));
//   quad: (a,b,c) when sam.z is below its area share, else (a,c,d); pdf
//     1 / area (quad.cpp:128-150);
//   mesh: idx = min(int(sam.z * triangles), triangles - 1) and the corners
//     idx, idx+1, idx+2 of the index buffer -- without the factor 3, so the
//     windows that straddle two triangles (and repeat a vertex: a NaN
//     normal) are sampled as the reference samples them; pdf 1 / area
//     (mesh.cpp:251-275);
//   cube: triangle min(int(sam.z * 12), 11), pdf 1 / (12 * its area)
//     (cube.cpp:145-170).
__device__ __forceinline__ AreaSample area_sample(const float* L,
                                                  const float* pts, float x,
                                                  float y, float z) {
  const int kind = (int)L[4];
  const bool two = L[5] != 0.f;
  const uint32_t ntri = __float_as_uint(L[6]);
  const float* P = pts + 3 * (uint64_t)__float_as_uint(L[10]);
  F3 sam = mk3(x, y, z);
  bool back = false;
  if (two) {
    back = sam.x < 0.5f;
    if (back)
      sam.x = 2 * x;
    else
      sam.x = 2 * (x - 0.5f);
  }
  F3 sn = sam;
  if (sn.x + sn.y > 1.f) {
    sn.x = 1.f - sn.x;
    sn.y = 1.f - sn.y;
  }
  F3 a, b, c;
  AreaSample g;
  if (kind == AJG_GEOM_QUAD) {
    a = ld3(P);
    if (sam.z < L[8]) {
      b = ld3(P + 3);
      c = ld3(P + 6);
    } else {
      b = ld3(P + 6);
      c = ld3(P + 9);
    }
    g.pdf = L[7];
  } else if (kind == AJG_GEOM_MESH) {
    const int idx = min((int)(sam.z * (float)ntri), (int)ntri - 1);
    a = ld3(P + 3 * idx);
    b = ld3(P + 3 * idx + 3);
    c = ld3(P + 3 * idx + 6);
    g.pdf = L[7];
  } else {
    const int idx = min((int)(sam.z * (float)12), 11);
    a = ld3(P + 9 * idx);
    b = ld3(P + 9 * idx + 3);
    c = ld3(P + 9 * idx + 6);
    g.pdf = 1.f / (12.f * len3(cross3(b - a, c - a)) * 0.5f);
  }
  g.pos = (1 - sn.x - sn.y) * a + sn.x * b + sn.y * c;
  g.ng = normalize3(cross3(b - a, c - a));
  if (two) {
    g.pdf = g.pdf * 0.5f;
    if (back) g.ng = g.ng * -1.f;
  }
  return g;
}

// AreaLight::Pdf (area_light.cpp:68-79); `pdf_area` = Geometry::Pdf.
__device__ __forceinline__ float area_pdf(float pdf_area, F3 ref, F3 pos,
                                          F3 normal) {
  if (dot3(ref - pos, normal) <= 0.f) return 0.f;
  const F3 l2r = ref - pos;
  const float dist2 = dot3(l2r, l2r);
  const float abscos = fabsf(dot3(l2r, normal));
  return pdf_area * (dist2 / abscos);
}

// The part of PostIntersect an emitter hit needs: the position and the
// geometric normal, flipped toward the ray on two-sided primitives.
__device__ __forceinline__ void emitter_hit(const DeviceScene& s, F3 o, F3 d,
                                            float t, int prim, F3& pos,
                                            F3& ng) {
  const float4 sh = __ldg(s.shade + prim);
  pos = o + t * d;
  ng = mk3(sh.x, sh.y, sh.z);
  if (((__float_as_uint(sh.w) >> 24) & AJG_MESH_TWO_SIDED) &&
      dot3(ng, -d) < 0)
    ng = ng * -1.f;
}

// ----------------------------------------------------------------- camera --
__device__ __forceinline__ void mat_vec(const float* M, const float v[4],
                                        float out[4]) {
#pragma unroll
  for (int row = 0; row < 4; ++row) {
    float o = 0.f;
#pragma unroll
    for (int pos = 0; pos < 4; ++pos) o += M[pos * 4 + row] * v[pos];
    out[row] = o;
  }
}
// ThinLensCamera::GenerateRay (thin_lens.cpp:62-83), then the Ray ctor.
__device__ __forceinline__ void camera_ray(const ajg_camera& cam, float rx,
                                           float ry, float lx, float ly,
                                           F3& ro, F3& rd) {
  float p[4] = {rx, ry, 1.f, 1.f}, q[4];
  mat_vec(cam.raster2camera, p, q);
  const F3 cc = mk3(q[0], q[1], q[2]) / q[3];
  F3 o = mk3(0.f, 0.f, 0.f);
  F3 d = normalize3(cc);
  if (cam.lens_radius > 0 && cam.focal_distance > 0) {
    float px, py;
    concentric(lx, ly, px, py);
    const float lxp = px * cam.lens_radius, lyp = py * cam.lens_radius;
    const float ft = cam.focal_distance / d.z;
    const F3 focus = o + ft * d;
    o = mk3(lxp, lyp, 0.f);
    d = normalize3(focus - o);
  }
  float po[4] = {o.x, o.y, o.z, 1.f}, wo[4];
  mat_vec(cam.camera2world, po, wo);
  const F3 wpo = mk3(wo[0], wo[1], wo[2]) / wo[3];
  float pd[4] = {d.x, d.y, d.z, 0.f}, wd[4];
  mat_vec(cam.camera2world, pd, wd);
  make_ray(wpo, mk3(wd[0], wd[1], wd[2]), ro, rd);
}

}  // namespace ajg
