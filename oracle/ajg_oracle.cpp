/*
 * Oracle for the PT-MIS / PLOC path (TEST INFRASTRUCTURE ONLY, see
 * ajg_oracle.h).  A CPU restatement of the reference's algorithm, written to
 * reproduce its float arithmetic operation by operation: every expression
 * keeps the reference's evaluation order, and the file is compiled with
 * -ffp-contract=off so no multiply-add is fused.  References are to files of
 * siyuanpan/ajisai_render (paths relative to its root).
 */
#include "ajg_oracle.h"
#include "counter_rng.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

namespace {

/* ---------------------------------------------------------------- math --- */
/* ajisai/math/vector.h:63-69 (dot), vector3.h:90-95 (cross),
 * vector.h:201-216 (length, normalized = v * (1 / length)). */
struct V3 {
  float x, y, z;
};
inline V3 mk(float x, float y, float z) { return V3{x, y, z}; }
inline V3 operator+(V3 a, V3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator*(V3 a, V3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
inline V3 operator/(V3 a, V3 b) { return mk(a.x / b.x, a.y / b.y, a.z / b.z); }
inline V3 operator*(V3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
inline V3 operator*(float s, V3 a) { return a * s; }
inline V3 operator/(V3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
inline V3 operator-(V3 a) { return mk(-a.x, -a.y, -a.z); }
inline float dot(V3 a, V3 b) {
  float o = 0.f;
  o += a.x * b.x;
  o += a.y * b.y;
  o += a.z * b.z;
  return o;
}
inline V3 cross(V3 a, V3 b) {
  return mk(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x,
            a.x * b.y - b.x * a.y);
}
inline float length(V3 v) { return std::sqrt(dot(v, v)); }
inline V3 normalized(V3 v) { return v * (1.f / length(v)); }
/* vector.h:36-45: Min(a,b) = b < a ? b : a, Max(a,b) = a < b ? b : a */
inline float fmin_ref(float a, float b) { return b < a ? b : a; }
inline float fmax_ref(float a, float b) { return a < b ? b : a; }
inline V3 vmin(V3 a, V3 b) {
  return mk(fmin_ref(a.x, b.x), fmin_ref(a.y, b.y), fmin_ref(a.z, b.z));
}
inline V3 vmax(V3 a, V3 b) {
  return mk(fmax_ref(a.x, b.x), fmax_ref(a.y, b.y), fmax_ref(a.z, b.z));
}
inline float maxc(V3 v) { return fmax_ref(fmax_ref(v.x, v.y), v.z); }
inline float minc(V3 v) { return fmin_ref(fmin_ref(v.x, v.y), v.z); }
inline bool is_black(V3 v) { return maxc(v) <= 0.f; } /* spectrum.h:70 */
inline V3 ld3(const float* p) { return mk(p[0], p[1], p[2]); }

/* ajisai/math/constants.h:35-37 */
constexpr float kPi = 3.141592654f;
constexpr float kPi2 = 1.570796327f;
constexpr float kPi4 = 0.785398163f;
constexpr float kInvPi = 1.f / kPi;
constexpr float kEps = 1e-4f; /* Ray::Eps, ray.h:43 */

/* spectrum.h:80-82: evaluated in double, rounded to float */
inline float luminance(V3 c) {
  return (float)(0.2126 * c.x + 0.7152 * c.y + 0.0722 * c.z);
}

/* libstdc++'s std::lerp (C++20 <cmath>) for float operands */
inline float std_lerp(float a, float b, float t) {
  if ((a <= 0 && b >= 0) || (a >= 0 && b <= 0)) return t * b + (1 - t) * a;
  if (t == 1) return b;
  const float x = a + t * (b - a);
  return (t > 1) == (b > a) ? (b < x ? x : b) : (b > x ? x : b);
}
/* disney.cpp:48-52: the file-local Lerp, min * (1 - val) + max * val */
inline float dlerp(float a, float b, float t) { return a * (1 - t) + b * t; }
inline V3 dlerp(V3 a, V3 b, float t) { return a * (1 - t) + b * t; }
inline float clampf(float v, float lo, float hi) {
  return v < lo ? lo : (hi < v ? hi : v);
}

/* ------------------------------------------------------------- bounds --- */
struct Box {
  V3 lo, hi;
};
/* ajisai/math/bounds.h:108-113: a point box is absorbed */
inline bool is_point(const Box& b) {
  return b.lo.x == b.hi.x && b.lo.y == b.hi.y && b.lo.z == b.hi.z;
}
inline Box join(const Box& a, const Box& b) {
  if (is_point(a)) return b;
  if (is_point(b)) return a;
  return Box{vmin(a.lo, b.lo), vmax(a.hi, b.hi)};
}
/* bounds.h:98-101 */
inline float area(const Box& b) {
  V3 d = b.hi - b.lo;
  return 2.f * (d.x * d.y + d.x * d.z + d.y * d.z);
}
inline Box tri_box(const float* t) { /* ploc_aggregate.cpp:168-182 */
  Box b{mk(FLT_MAX, FLT_MAX, FLT_MAX), mk(-FLT_MAX, -FLT_MAX, -FLT_MAX)};
  for (int k = 0; k < 3; ++k) {
    V3 v = ld3(t + 3 * k);
    b.lo = vmin(b.lo, v);
    b.hi = vmax(b.hi, v);
  }
  return b;
}

/* ------------------------------------------------------------- morton --- */
/* ploc_aggregate.cpp:37-82: 10 bits per axis, 30-bit code in uint32 */
inline uint32_t morton_split(uint32_t x) {
  x &= 0x3ffu;
  x = (x | (x << 16)) & 0x030000FFu;
  x = (x | (x << 8)) & 0x0300F00Fu;
  x = (x | (x << 4)) & 0x030C30C3u;
  x = (x | (x << 2)) & 0x09249249u;
  return x;
}
struct MortonEnc {
  V3 w2g, off;
  explicit MortonEnc(const Box& bb) {
    V3 size = bb.hi - bb.lo;
    V3 inv = mk(1.f / size.x, 1.f / size.y, 1.f / size.z);
    w2g = inv * 1024.f;
    off = (-bb.lo) * w2g;
  }
  uint32_t enc(V3 p) const {
    V3 g = p * w2g + off;
    /* A flat axis makes size 0 and the grid coordinate NaN; the reference's
     * float-to-integer conversion yields 0 there on x86-64 and aarch64. */
    auto q = [](float f) -> uint32_t {
      float g = fmax_ref(f, 0.f);
      if (g != g) return 0u;
      uint32_t m = g >= 4294967296.f ? 0xffffffffu : (uint32_t)g;
      return std::min<uint32_t>(1023u, m);
    };
    return morton_split(q(g.x)) | (morton_split(q(g.y)) << 1) |
           (morton_split(q(g.z)) << 2);
  }
};
inline V3 box_center(const Box& b) { return (b.hi + b.lo) / 2.f; }

/* --------------------------------------------------------------- PLOC --- */
struct Node {
  Box b;
  int64_t count, first;
};

/* RadixSort<10> over 3 passes (ploc_aggregate.cpp:84-132): a stable LSD
 * counting sort, i.e. the stable order by 30-bit key. */
std::vector<int64_t> morton_order(const std::vector<uint32_t>& codes) {
  int64_t n = (int64_t)codes.size();
  std::vector<int64_t> idx(n), tmp(n);
  std::vector<uint32_t> k(codes), kt(n);
  for (int64_t i = 0; i < n; ++i) idx[i] = i;
  for (int bit = 0; bit < 30; bit += 10) {
    std::vector<int64_t> cnt(1025, 0);
    for (int64_t i = 0; i < n; ++i) cnt[((k[i] >> bit) & 1023u) + 1]++;
    for (int d = 0; d < 1024; ++d) cnt[d + 1] += cnt[d];
    for (int64_t i = 0; i < n; ++i) {
      int64_t j = cnt[(k[i] >> bit) & 1023u]++;
      kt[j] = k[i];
      tmp[j] = idx[i];
    }
    k.swap(kt);
    idx.swap(tmp);
  }
  return idx;
}

/* RadixSort<10>::Sort exactly as the reference runs it
 * (ploc_aggregate.cpp:89-131): buckets_accum[0] is zeroed once before the
 * pass loop, so from the second pass on the digit-0 keys are scattered from
 * the previous passes' digit-0 total instead of from 0.  Later writes win,
 * unwritten slots keep the stale contents of the destination buffer (the
 * zero-initialised copies, then the original arrays, then pass-1 output).
 * Returns false when a write would leave the array (undefined behaviour in
 * the reference). */
bool morton_order_compat(const std::vector<uint32_t>& codes,
                         std::vector<int64_t>& out) {
  int64_t n = (int64_t)codes.size();
  std::vector<uint32_t> ka(codes), kb(n, 0u);
  std::vector<int64_t> va(n), vb(n, 0);
  for (int64_t i = 0; i < n; ++i) va[i] = i;
  std::vector<uint32_t>* keys = &ka;
  std::vector<uint32_t>* kcopy = &kb;
  std::vector<int64_t>* vals = &va;
  std::vector<int64_t>* vcopy = &vb;
  std::vector<int64_t> accum(1024, 0);
  for (int bit = 0; bit < 30; bit += 10) {
    std::vector<int64_t> cnt(1024, 0);
    for (int64_t i = 0; i < n; ++i) cnt[((*keys)[i] >> bit) & 1023u]++;
    int64_t sum = cnt[0];
    for (int d = 1; d < 1024; ++d) {
      accum[d] = sum;
      sum += cnt[d];
    }
    for (int64_t i = 0; i < n; ++i) {
      int64_t j = accum[((*keys)[i] >> bit) & 1023u]++;
      if (j < 0 || j >= n) return false;
      (*kcopy)[j] = (*keys)[i];
      (*vcopy)[j] = (*vals)[i];
    }
    std::swap(kcopy, keys);
    std::swap(vcopy, vals);
  }
  out = *vals;
  return true;
}

/* PLOCAggregate::Cluster (ploc_aggregate.cpp:400-511).  Nearest neighbour by
 * area of the joined box within +-r, first minimum in ascending index order;
 * mutual pairs merge; the parent takes the right partner's slot. */
void ploc_cluster(const std::vector<Node>& in, std::vector<Node>& out,
                  std::vector<int64_t>& nb, std::vector<int64_t>& mi,
                  int64_t begin, int64_t end, int64_t pre_end, int64_t r,
                  int64_t* nbeg, int64_t* nend) {
  for (int64_t i = begin; i < end; ++i) {
    int64_t sb = i > begin + r ? i - r : begin;
    int64_t se = std::min(i + r + 1, end);
    float best = std::numeric_limits<float>::max();
    int64_t bj = -1;
    for (int64_t j = sb; j < se; ++j) {
      if (j == i) continue;
      float d = area(join(in[i].b, in[j].b));
      if (d < best) {
        best = d;
        bj = j;
      }
    }
    nb[i] = bj;
  }
  int64_t acc = 0;
  for (int64_t i = begin; i < end; ++i) {
    int64_t j = nb[i];
    acc += (i < j && nb[j] == i) ? 1 : 0;
    mi[i] = acc;
  }
  int64_t merged = mi[end - 1];
  int64_t unmerged = end - begin - merged;
  int64_t children = merged * 2;
  int64_t children_begin = end - children;
  int64_t unmerged_begin = end - (children + unmerged);
  for (int64_t i = begin; i < end; ++i) {
    int64_t j = nb[i];
    if (nb[j] == i) {
      if (i < j) {
        Node& p = out[unmerged_begin + j - begin - mi[j]];
        int64_t fc = children_begin + (mi[i] - 1) * 2;
        p.b = join(in[j].b, in[i].b);
        p.count = 0;
        p.first = fc;
        out[fc + 0] = in[i];
        out[fc + 1] = in[j];
      }
    } else {
      out[unmerged_begin + i - begin - mi[i]] = in[i];
    }
  }
  for (int64_t i = end; i < pre_end; ++i) out[i] = in[i];
  *nbeg = unmerged_begin;
  *nend = children_begin;
}

Box world_box(const float* w) { return Box{ld3(w), ld3(w + 3)}; }

bool ploc_build(const float* tris, int64_t n, const float* world, int64_t r,
                bool radix_compat, std::vector<Node>& nodes,
                std::vector<int64_t>& perm) {
  Box bb = world_box(world);
  MortonEnc enc(bb);
  std::vector<uint32_t> codes(n);
  for (int64_t i = 0; i < n; ++i)
    codes[i] = enc.enc(box_center(tri_box(tris + 9 * i)));
  if (radix_compat) {
    if (!morton_order_compat(codes, perm)) return false;
  } else {
    perm = morton_order(codes);
  }
  int64_t nn = 2 * n - 1;
  std::vector<Node> a(nn), b(nn);
  std::vector<int64_t> nb(nn), mi(nn);
  int64_t begin = nn - n, end = nn, pre_end = end;
  for (int64_t i = 0; i < n; ++i) {
    Node& x = a[begin + i];
    x.b = tri_box(tris + 9 * perm[i]);
    x.count = 1;
    x.first = i;
  }
  while (end - begin > 1) {
    int64_t nbg, nen;
    ploc_cluster(a, b, nb, mi, begin, end, pre_end, r, &nbg, &nen);
    a.swap(b);
    pre_end = end;
    begin = nbg;
    end = nen;
  }
  nodes.swap(a);
  return true;
}

/* ---------------------------------------------------------- ray tests --- */
struct Ray {
  V3 o, d;
  float tmin, tmax;
};
/* Ray ctor (ray.h:33-39): origin pushed by Eps along the normalised
 * direction, direction normalised. */
inline Ray make_ray(V3 o, V3 d, float tmin = kEps,
                    float tmax = std::numeric_limits<float>::infinity()) {
  V3 dn = normalized(d);
  Ray r;
  r.o = o + dn * kEps;
  r.d = normalized(d);
  r.tmin = tmin;
  r.tmax = tmax;
  return r;
}

/* Triangle::Intersect / Occlude test (ploc_aggregate.cpp:184-242):
 * Moller-Trumbore with the absolute determinant cull |a| < 1e-6. */
inline bool mt_test(const Ray& r, const float* tri, float* t_out, float* u_out,
                    float* v_out) {
  V3 v0 = ld3(tri), v1 = ld3(tri + 3), v2 = ld3(tri + 6);
  V3 e0 = v1 - v0, e1 = v2 - v0;
  V3 h = cross(r.d, e1);
  float a = dot(e0, h);
  if (a > -1e-6f && a < 1e-6f) return false;
  float f = 1.f / a;
  V3 s = r.o - v0;
  float u = f * dot(s, h);
  if (u < 0.f || u > 1.f) return false;
  V3 q = cross(s, e0);
  float v = f * dot(r.d, q);
  if (v < 0.f || u + v > 1.f) return false;
  float t = f * dot(e1, q);
  if (!(t > r.tmin && t < r.tmax)) return false;
  *t_out = t;
  *u_out = u;
  *v_out = v;
  return true;
}

/* Watertight test of Woop, Benthin and Wald, "Watertight Ray/Triangle
 * Intersection", JCGT 2(1), 2013, without the double-precision fallback.
 * Barycentrics are reported in the Moller-Trumbore convention (u for b,
 * v for c). */
struct WtRay {
  int kx, ky, kz;
  float sx, sy, sz;
};
inline WtRay wt_setup(const Ray& r) {
  WtRay w;
  float ax = std::fabs(r.d.x), ay = std::fabs(r.d.y), az = std::fabs(r.d.z);
  int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
  int kx = kz + 1 == 3 ? 0 : kz + 1;
  int ky = kx + 1 == 3 ? 0 : kx + 1;
  const float d[3] = {r.d.x, r.d.y, r.d.z};
  if (d[kz] < 0.f) std::swap(kx, ky);
  w.kx = kx;
  w.ky = ky;
  w.kz = kz;
  w.sx = d[kx] / d[kz];
  w.sy = d[ky] / d[kz];
  w.sz = 1.f / d[kz];
  return w;
}
inline bool wt_test(const Ray& r, const WtRay& w, const float* tri,
                    float* t_out, float* u_out, float* v_out) {
  const float o[3] = {r.o.x, r.o.y, r.o.z};
  float A[3], B[3], C[3];
  for (int k = 0; k < 3; ++k) {
    A[k] = tri[k] - o[k];
    B[k] = tri[3 + k] - o[k];
    C[k] = tri[6 + k] - o[k];
  }
  const float Ax = A[w.kx] - w.sx * A[w.kz], Ay = A[w.ky] - w.sy * A[w.kz];
  const float Bx = B[w.kx] - w.sx * B[w.kz], By = B[w.ky] - w.sy * B[w.kz];
  const float Cx = C[w.kx] - w.sx * C[w.kz], Cy = C[w.ky] - w.sy * C[w.kz];
  const float U = Cx * By - Cy * Bx;
  const float V = Ax * Cy - Ay * Cx;
  const float W = Bx * Ay - By * Ax;
  if ((U < 0.f || V < 0.f || W < 0.f) && (U > 0.f || V > 0.f || W > 0.f))
    return false;
  const float det = U + V + W;
  if (det == 0.f) return false;
  const float Az = w.sz * A[w.kz], Bz = w.sz * B[w.kz], Cz = w.sz * C[w.kz];
  const float T = U * Az + V * Bz + W * Cz;
  const float rcp = 1.f / det;
  const float t = T * rcp;
  if (!(t > r.tmin && t < r.tmax)) return false;
  *t_out = t;
  *u_out = V * rcp;
  *v_out = W * rcp;
  return true;
}

/* Conservative slab test shared with the GPU traversal: the reference's
 * (bound - o) * inv_dir form (ploc_aggregate.cpp:154-162) with the far
 * distance widened by 1 + 2*gamma(3) (Pharr, Jakob, Humphreys, PBRT 3rd ed.,
 * 3.9.2), and an inclusive comparison against the current best t so that an
 * equal-t hit on a lower primitive index is never culled. */
constexpr float kSlabWiden = 1.0000003576278687f; /* 1 + 2 * 3u/(1-3u) */
/* fminf / fmaxf semantics (a NaN operand yields the other one), inline; the
 * sign of a zero result may differ, which no comparison below can see */
inline float nmin(float a, float b) { return (b < a || a != a) ? b : a; }
inline float nmax(float a, float b) { return (a < b || a != a) ? b : a; }
inline bool slab(const Box& b, const Ray& r, V3 inv, float tlimit) {
  float tx0 = (b.lo.x - r.o.x) * inv.x, tx1 = (b.hi.x - r.o.x) * inv.x;
  float ty0 = (b.lo.y - r.o.y) * inv.y, ty1 = (b.hi.y - r.o.y) * inv.y;
  float tz0 = (b.lo.z - r.o.z) * inv.z, tz1 = (b.hi.z - r.o.z) * inv.z;
  float tn = nmax(nmax(nmin(tx0, tx1), nmin(ty0, ty1)), nmin(tz0, tz1));
  float tf = nmin(nmin(nmax(tx0, tx1), nmax(ty0, ty1)), nmax(tz0, tz1));
  tf = tf * kSlabWiden;
  return tn <= tf && tn <= tlimit && tf >= r.tmin;
}

struct Hit {
  float t, u, v;
  int32_t prim;
};

/* Traversal stack: 256 entries inline, growing on the heap only for
 * pathologically deep trees. */
struct SmallStack {
  int64_t inl[256];
  std::vector<int64_t> heap;
  int n = 0;
  void push(int64_t v) {
    if (n < 256)
      inl[n] = v;
    else
      heap.push_back(v);
    ++n;
  }
  int64_t pop() {
    --n;
    if (n < 256) return inl[n];
    int64_t v = heap.back();
    heap.pop_back();
    return v;
  }
  bool empty() const { return n == 0; }
};

struct Accel {
  const float* tris;
  int64_t n;
  const Node* nodes; /* reference layout */
  const int64_t* perm;
};

inline bool tri_test(int mode, const Ray& r, const WtRay& w, const float* tri,
                     float* t, float* u, float* v) {
  return mode == ORC_TEST_WATERTIGHT ? wt_test(r, w, tri, t, u, v)
                                     : mt_test(r, tri, t, u, v);
}

/* IntersectP (ploc_aggregate.cpp:152-160): the near corner chosen per axis
 * by the direction's sign, Vector::max()/min() folding Max(a, b) = a < b ?
 * b : a and Min(a, b) = b < a ? b : a (math/vector.h:36-45, 380-400), no
 * widening. */
inline float ref_max(float a, float b) { return a < b ? b : a; }
inline float ref_min(float a, float b) { return b < a ? b : a; }
inline bool ref_slab(const Box& b, const Ray& r, V3 inv) {
  const bool nx = inv.x < 0.f, ny = inv.y < 0.f, nz = inv.z < 0.f;
  const float n0 = ((nx ? b.hi.x : b.lo.x) - r.o.x) * inv.x;
  const float n1 = ((ny ? b.hi.y : b.lo.y) - r.o.y) * inv.y;
  const float n2 = ((nz ? b.hi.z : b.lo.z) - r.o.z) * inv.z;
  const float f0 = ((nx ? b.lo.x : b.hi.x) - r.o.x) * inv.x;
  const float f1 = ((ny ? b.lo.y : b.hi.y) - r.o.y) * inv.y;
  const float f2 = ((nz ? b.lo.z : b.hi.z) - r.o.z) * inv.z;
  const float tn = ref_max(ref_max(n0, n1), n2);
  const float tf = ref_min(ref_min(f0, f1), f2);
  if (tn > tf) return false;
  return tn < r.tmax && tf > r.tmin;
}

/* PLOCAggregate::Intersect / IntersectAux (ploc_aggregate.cpp:329-391):
 * depth first, left child before right, each node's slab test against the
 * current t_max, which a hit shrinks to its t (Triangle::Intersect,
 * :184-216, accepts t in (t_min, t_max)). */
Hit trace_closest_ref(const Accel& acc, Ray r) {
  Hit h{std::numeric_limits<float>::infinity(), 0.f, 0.f, -1};
  V3 inv = mk(1.f / r.d.x, 1.f / r.d.y, 1.f / r.d.z);
  SmallStack st;
  st.push(0);
  while (!st.empty()) {
    const Node& nd = acc.nodes[st.pop()];
    if (!ref_slab(nd.b, r, inv)) continue;
    if (nd.count) {
      const int32_t prim = (int32_t)acc.perm[nd.first];
      float t, u, v;
      if (mt_test(r, acc.tris + 9 * (int64_t)prim, &t, &u, &v) && t < h.t) {
        h = Hit{t, u, v, prim};
        r.tmax = t;
      }
    } else {
      st.push(nd.first + 1);
      st.push(nd.first);
    }
  }
  return h;
}

/* PLOCAggregate::Occlude / OccludeAux (ploc_aggregate.cpp:337-365). */
bool trace_any_ref(const Accel& acc, const Ray& r) {
  V3 inv = mk(1.f / r.d.x, 1.f / r.d.y, 1.f / r.d.z);
  SmallStack st;
  st.push(0);
  float t, u, v;
  while (!st.empty()) {
    const Node& nd = acc.nodes[st.pop()];
    if (!ref_slab(nd.b, r, inv)) continue;
    if (nd.count) {
      if (mt_test(r, acc.tris + 9 * acc.perm[nd.first], &t, &u, &v)) return true;
    } else {
      st.push(nd.first + 1);
      st.push(nd.first);
    }
  }
  return false;
}

Hit trace_closest(const Accel& acc, const Ray& r, int mode, bool use_bvh) {
  if (mode == ORC_TEST_REF_ORDER && use_bvh) return trace_closest_ref(acc, r);
  Hit h{std::numeric_limits<float>::infinity(), 0.f, 0.f, -1};
  WtRay w = wt_setup(r);
  auto consider = [&](int32_t prim) {
    float t, u, v;
    if (!tri_test(mode, r, w, acc.tris + 9 * (int64_t)prim, &t, &u, &v))
      return;
    if (t < h.t || (t == h.t && prim < h.prim)) h = Hit{t, u, v, prim};
  };
  if (!use_bvh) {
    for (int64_t i = 0; i < acc.n; ++i) consider((int32_t)i);
    return h;
  }
  V3 inv = mk(1.f / r.d.x, 1.f / r.d.y, 1.f / r.d.z);
  SmallStack st;
  st.push(0);
  while (!st.empty()) {
    int64_t k = st.pop();
    const Node& nd = acc.nodes[k];
    float lim = nmin(h.t, r.tmax);
    if (!slab(nd.b, r, inv, lim)) continue;
    if (nd.count) {
      consider((int32_t)acc.perm[nd.first]);
    } else {
      st.push(nd.first + 1);
      st.push(nd.first);
    }
  }
  return h;
}

bool trace_any(const Accel& acc, const Ray& r, int mode, bool use_bvh) {
  if (mode == ORC_TEST_REF_ORDER && use_bvh) return trace_any_ref(acc, r);
  WtRay w = wt_setup(r);
  float t, u, v;
  if (!use_bvh) {
    for (int64_t i = 0; i < acc.n; ++i)
      if (tri_test(mode, r, w, acc.tris + 9 * i, &t, &u, &v)) return true;
    return false;
  }
  V3 inv = mk(1.f / r.d.x, 1.f / r.d.y, 1.f / r.d.z);
  SmallStack st;
  st.push(0);
  while (!st.empty()) {
    int64_t k = st.pop();
    const Node& nd = acc.nodes[k];
    if (!slab(nd.b, r, inv, r.tmax)) continue;
    if (nd.count) {
      if (tri_test(mode, r, w, acc.tris + 9 * acc.perm[nd.first], &t, &u, &v))
        return true;
    } else {
      st.push(nd.first + 1);
      st.push(nd.first);
    }
  }
  return false;
}

template <class F>
void parallel_rows(int64_t n, int threads, F&& f, int64_t chunk = 64) {
  if (threads <= 1 || n < 2) {
    for (int64_t i = 0; i < n; ++i) f(i);
    return;
  }
  std::atomic<int64_t> next{0};
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t)
    pool.emplace_back([&]() {
      for (;;) {
        int64_t b = next.fetch_add(chunk);
        if (b >= n) break;
        int64_t e = std::min(n, b + chunk);
        for (int64_t i = b; i < e; ++i) f(i);
      }
    });
  for (auto& th : pool) th.join();
}

/* ------------------------------------------------------------- frames --- */
/* CoordinateSystem (coordinate_system.h:37-52, Duff et al. 2017) */
struct Frame {
  V3 dx, dy, dz;
  explicit Frame(V3 n) : dz(n) {
    float sign = std::copysign(1.f, n.z);
    const float a = -1.f / (sign + n.z);
    const float b = n.x * n.y * a;
    dx = mk(1.f + sign * n.x * n.x * a, sign * b, -sign * n.x);
    dy = mk(b, sign + n.y * n.y * a, -n.y);
  }
  V3 to_local(V3 v) const { return mk(dot(v, dx), dot(v, dy), dot(v, dz)); }
  V3 to_world(V3 v) const { return dx * v.x + dy * v.y + dz * v.z; }
};

/* warp.h:29-72 */
inline void concentric(float sx, float sy, float* px, float* py) {
  float ox = 2.f * sx - 1.f, oy = 2.f * sy - 1.f;
  float r, phi;
  if (ox == 0 && oy == 0) {
    *px = 0.f;
    *py = 0.f;
    return;
  } else if (std::fabs(ox) > std::fabs(oy)) {
    r = ox;
    phi = kPi4 * (oy / ox);
  } else {
    r = oy;
    phi = kPi2 - kPi4 * (ox / oy);
  }
  *px = r * std::cos(phi);
  *py = r * std::sin(phi);
}
inline V3 cosine_hemisphere(float sx, float sy, float* pdf) {
  float px, py;
  concentric(sx, sy, &px, &py);
  float r = 0.f;
  r += px * px;
  r += py * py;
  float z = std::sqrt(fmax_ref(0.0f, 1 - r));
  if (z == 0) z = 1e-10f;
  if (pdf) *pdf = z * kInvPi;
  return mk(px, py, z);
}
/* warp.h:74-80, 100-104 */
inline V3 uniform_cone(float u0, float u1, float cos_max) {
  float ct = (1.f - u0) + u0 * cos_max;
  float st = std::sqrt(fmax_ref(0.f, 1.f - ct * ct));
  float phi = u1 * 2 * kPi;
  return mk(std::cos(phi) * st, std::sin(phi) * st, ct);
}
inline float uniform_cone_pdf(float cos_max) {
  if (cos_max == 1.0f) return 1.0f;
  return 1.0f / (2.0f * kPi * (1.0f - cos_max));
}
/* bsdf.h:42-46 */
inline float correct_shading_normal(V3 ng, V3 ns, V3 wi) {
  const float denom = std::fabs(dot(ng, wi));
  return denom == 0 ? 1.f : std::fabs(dot(ns, wi) / denom);
}

/* ------------------------------------------------------------ Fresnel --- */
/* Fresnel::dielectricReflectance (bsdf/helper.h:35-56) */
inline float dielectric_reflectance(float eta, float cos_i) {
  if (cos_i < 0.0f) {
    eta = 1.0f / eta;
    cos_i = -cos_i;
  }
  const float sin_t2 = eta * eta * (1.0f - cos_i * cos_i);
  if (sin_t2 > 1.0f) return 1.0f;
  const float cos_t = std::sqrt(fmax_ref(1.0f - sin_t2, 0.0f));
  const float rs = (eta * cos_i - cos_t) / (eta * cos_i + cos_t);
  const float rp = (eta * cos_t - cos_i) / (eta * cos_t + cos_i);
  return (rs * rs + rp * rp) * 0.5f;
}

/* DielectricFresnel::Eval (material/fresnel.h:95-118), one channel */
inline float dielectric_fresnel(float eta_in, float eta_out, float cos_i) {
  if (cos_i < 0) {
    std::swap(eta_in, eta_out);
    cos_i = -cos_i;
  }
  const float sin_i = std::sqrt(fmax_ref(0.f, 1 - cos_i * cos_i));
  const float sin_t = eta_out / eta_in * sin_i;
  if (sin_t >= 1.f) return 1.f;
  const float cos_t = std::sqrt(fmax_ref(0.f, 1 - sin_t * sin_t));
  const float para = ((eta_in * cos_i) - (eta_out * cos_t)) /
                     ((eta_in * cos_i) + (eta_out * cos_t));
  const float perp = ((eta_out * cos_i) - (eta_in * cos_t)) /
                     ((eta_out * cos_i) + (eta_in * cos_t));
  return 0.5f * (para * para + perp * perp);
}

/* ConductorFresnel::Eval (material/fresnel.h:40-58), eta_out = 1:
 * eta2 = eta * eta, etak2 = k * k */
inline V3 conductor_fresnel(V3 eta2, V3 etak2, float cos_i) {
  if (cos_i <= 0.f) return mk(0, 0, 0);
  const float cos2 = cos_i * cos_i;
  const float sin2 = fmax_ref(0.f, 1 - cos2);
  V3 out;
  float* o = &out.x;
  const float* e2 = &eta2.x;
  const float* k2 = &etak2.x;
  for (int c = 0; c < 3; ++c) {
    const float t0 = e2[c] - k2[c] - sin2;
    const float a2b2 = std::sqrt(t0 * t0 + 4.f * e2[c] * k2[c]);
    const float t1 = a2b2 + cos2;
    const float a = std::sqrt(0.5f * (a2b2 + t0));
    const float t2 = 2.f * cos_i * a;
    const float rs = (t1 - t2) / (t1 + t2);
    const float t3 = cos2 * a2b2 + sin2 * sin2;
    const float t4 = t2 * sin2;
    const float rp = rs * (t3 - t4) / (t3 + t4);
    o[c] = 0.5f * (rp + rs);
  }
  return out;
}

}  // namespace

/* Fresnel::computeDiffuseFresnel (bsdf/helper.h:58-73) */
float orc_diffuse_fresnel(float ior, int n) {
  double acc = 0.0;
  float fb = dielectric_reflectance(ior, 0.0f);
  for (int i = 1; i <= n; ++i) {
    const float cos2 = float(i) / n;
    const float fa = dielectric_reflectance(ior, std::min(std::sqrt(cos2), 1.0f));
    acc += double(fa + fb) * (0.5 / n);
    fb = fa;
  }
  return float(acc);
}

namespace {

/* --------------------------------------------------------------- BSDF --- */
struct Sample {
  V3 dir, f;
  float pdf;
  bool valid;
  bool delta = false; /* BSDFSampleResult::is_delta */
};
inline Sample invalid_sample() {
  return Sample{mk(0, 0, 0), mk(0, 0, 0), 0.f, false, false};
}

struct Mat {
  int type;
  V3 base;
  float subsurface, metallic, specular, specular_tint, roughness, anisotropic,
      sheen, sheen_tint, clearcoat, clearcoat_gloss;
  float p[10]; /* the same ten floats, read by the other material types */
  float lum;   /* base.Luminance() */
  /* plastic: PlasticBsdf's constructor terms (plastic_bsdf.cpp:32-45) */
  float plastic_avg_t = 0.f, plastic_diffuse_fresnel = 0.f;
};
Mat load_mat(const float* m) {
  Mat x;
  x.type = (int)m[0];
  x.base = mk(m[1], m[2], m[3]);
  x.subsurface = m[4];
  x.metallic = m[5];
  x.specular = m[6];
  x.specular_tint = m[7];
  x.roughness = m[8];
  x.anisotropic = m[9];
  x.sheen = m[10];
  x.sheen_tint = m[11];
  x.clearcoat = m[12];
  x.clearcoat_gloss = m[13];
  for (int i = 0; i < 10; ++i) x.p[i] = m[4 + i];
  x.lum = luminance(x.base);
  if (x.type == ORC_MAT_PLASTIC) {
    const float ior = x.p[0], thickness = x.p[1], sigma_a = x.p[2];
    const float sc = thickness * sigma_a;
    const float avg = (sc + sc + sc) / 3.f;
    x.plastic_avg_t = std::exp(-2.0f * avg);
    /* a process-wide std::call_once in the reference: the first PlasticBsdf
     * constructed fixes it for every plastic; here each material's own */
    x.plastic_diffuse_fresnel = orc_diffuse_fresnel(ior, 1000000);
  }
  return x;
}

/* Lambertian: Diffuse::Shade builds an AggregateBSDF with one
 * DiffuseComponent of weight 1 (diffuse.cpp:35-48,
 * aggregate_bsdf.cpp:43-131, diffuse_component.cpp:28-64, bsdf.cpp:30-63). */
struct Lambert {
  V3 ng, ns, albedo, coef;
  Frame gf, sf;
  Lambert(V3 ng_, V3 ns_, V3 alb)
      : ng(ng_), ns(ns_), albedo(alb), coef(alb / kPi), gf(ng_), sf(ns_) {}
  bool fringes(V3 w) const { return (dot(ng, w) > 0) != (dot(ns, w) > 0); }
  Sample sample(V3 wo, V3 sam) const {
    if (fringes(wo)) {
      if (dot(ng, wo) <= 0.f) return invalid_sample();
      float pdf;
      V3 lwi = cosine_hemisphere(sam.x, sam.y, &pdf);
      if (pdf < FLT_EPSILON) return invalid_sample();
      V3 wi = normalized(gf.to_world(lwi));
      float factor = correct_shading_normal(ng, ns, wi);
      return Sample{wi, albedo / kPi * factor, pdf, true};
    }
    V3 lwo = normalized(sf.to_local(wo));
    if (lwo.z <= 0.f) return invalid_sample();
    /* component selection over one weight always picks index 0 */
    if (lwo.z < 0) return invalid_sample();
    float pdf;
    V3 lwi = cosine_hemisphere(sam.y, sam.z, &pdf);
    if ((double)pdf < 1e-3) return invalid_sample();
    if (pdf == 0) return invalid_sample();
    lwi = normalized(lwi);
    pdf *= 1.f;
    V3 wi = sf.to_world(lwi);
    float factor = correct_shading_normal(ng, ns, wi);
    return Sample{wi, coef * factor, pdf, true};
  }
  V3 eval(V3 wi, V3 wo) const {
    if (fringes(wo)) {
      if ((dot(ng, wi) <= 0.f) || (dot(ng, wo) <= 0.f)) return mk(0, 0, 0);
      return albedo / kPi;
    }
    V3 lwi = normalized(sf.to_local(wi));
    V3 lwo = normalized(sf.to_local(wo));
    if (lwi.z <= 0.f || lwo.z <= 0.f) return mk(0, 0, 0);
    return mk(0, 0, 0) + coef;
  }
  float pdf(V3 wi, V3 wo) const {
    if (fringes(wo)) {
      if ((dot(ng, wi) > 0.f) != (dot(ng, wo) > 0.f)) return 0.f;
      V3 local = normalized(gf.to_local(wi));
      return local.z * kInvPi;
    }
    V3 lwi = normalized(sf.to_local(wi));
    V3 lwo = normalized(sf.to_local(wo));
    if (lwi.z <= 0.f || lwo.z <= 0.f) return 0.f;
    float wsum = 0.f, p = 0.f;
    wsum += 1.f;
    p += 1.f * (lwi.z * kInvPi);
    return wsum > 0 ? p / wsum : 0;
  }
};

/* DisneyBSDF (disney.cpp:58-473), including the clearcoat pdf that reads the
 * world-space wo (disney.cpp:208-220). */
struct Disney {
  const Mat& m;
  Frame sf;
  Disney(const Mat& mat, V3 ns) : m(mat), sf(ns) {}

  static float cos2(V3 v) { return v.z * v.z; }
  static float tan_theta(V3 v) {
    float temp = 1 - v.z * v.z;
    if (temp <= 0.0f) return 0.0f;
    return std::sqrt(temp) / v.z;
  }
  static float tan2(V3 v) {
    float tmp = 1.f - v.z * v.z;
    if (tmp <= 0.f) return 0.f;
    return tmp / (v.z * v.z);
  }
  static V3 reflect(V3 vi, V3 n) { return vi + (2 * dot(-vi, n) * n); }
  static float ggx_d(V3 wh, float alpha) {
    if (wh.z <= 0.f) return 0.f;
    const float t2 = tan2(wh);
    const float c2 = cos2(wh);
    const float root = alpha / (c2 * (alpha * alpha + t2));
    return kInvPi * (root * root);
  }
  static float smith_g(V3 v, V3 wh, float alpha) {
    const float tt = std::fabs(tan_theta(v));
    if (tt == 0.0f) return 1.0f;
    if (dot(v, wh) * v.z <= 0) return 0.0f;
    const float root = alpha * tt;
    return 2.0f / (1.0f + std::sqrt(1.0f + root * root));
  }
  static float ggx_g(V3 wi, V3 wo, V3 wh, float alpha) {
    return smith_g(wo, wh, alpha) * smith_g(wi, wh, alpha);
  }
  static float pdf_vn(V3 wi, V3 h, float alpha) {
    float D = ggx_d(h, alpha);
    return smith_g(wi, h, alpha) * std::fabs(dot(wi, h)) * D /
           (std::fabs(wi.z) + 1e-4f);
  }
  static void vn_unit(float thetaI, float u1, float u2, float* sx, float* sy) {
    if (thetaI < 1e-4f) {
      float R = std::sqrt(fmax_ref(u1 / ((1 - u1) + 1e-6f), 0.0f));
      float SinPhi = std::sin(2 * kPi * u2);
      float CosPhi = std::cos(2 * kPi * u2);
      *sx = R * CosPhi;
      *sy = R * SinPhi;
      return;
    }
    float TanThetaI = std::tan(thetaI);
    float a = 1 / TanThetaI;
    float G1 =
        2.0f / (1.0f + std::sqrt(fmax_ref(1.0f + 1.0f / (a * a), 0.0f)));
    float A = 2.0f * u1 / G1 - 1.0f;
    if (std::fabs(A) == 1) A -= (A >= 0.0f ? 1.0f : -1.0f) * 1e-4f;
    float Temp = 1.0f / (A * A - 1.0f);
    float B = TanThetaI;
    float D = std::sqrt(
        fmax_ref(B * B * Temp * Temp - (A * A - B * B) * Temp, 0.0f));
    float x1 = B * Temp - D;
    float x2 = B * Temp + D;
    *sx = (A < 0.0f || x2 > 1.0f / TanThetaI) ? x1 : x2;
    float S;
    if (u2 > 0.5f) {
      S = 1.0f;
      u2 = 2.0f * (u2 - 0.5f);
    } else {
      S = -1.0f;
      u2 = 2.0f * (0.5f - u2);
    }
    /* the published rational fit, evaluated in double as in the source */
    float z = (float)((u2 * (u2 * (u2 * (-0.365728915865723) +
                                   0.790235037209296) -
                             0.424965825137544) +
                       0.000152998850436920) /
                      (u2 * (u2 * (u2 * (u2 * 0.169507819808272 -
                                         0.397203533833404) -
                                   0.232500544458471) +
                             1) -
                       0.539825872510702));
    *sy = S * z * std::sqrt(1.0f + (*sx) * (*sx));
  }
  static V3 sample_vn(V3 wi_in, float u1, float u2, float* pdf, float Alpha) {
    V3 wi = normalized(mk(Alpha * wi_in.x, Alpha * wi_in.y, wi_in.z));
    float Theta = 0, Phi = 0;
    if (wi.z < float(0.99999f)) {
      Theta = std::acos(wi.z);
      Phi = std::atan2(wi.y, wi.x);
    }
    float SinPhi = std::sin(Phi), CosPhi = std::cos(Phi);
    float sx, sy;
    vn_unit(Theta, u1, u2, &sx, &sy);
    float rx = CosPhi * sx - SinPhi * sy;
    float ry = SinPhi * sx + CosPhi * sy;
    rx *= Alpha;
    ry *= Alpha;
    float Norm = (float)1.f / std::sqrt(rx * rx + ry * ry + (float)1.0);
    V3 H = mk(-rx * Norm, -ry * Norm, Norm);
    *pdf = pdf_vn(wi_in, H, Alpha);
    return H;
  }
  float fresnel_conductor(float cosi, const float& eta, const float k) const {
    float tmp = (eta * eta + k * k) * cosi * cosi;
    float Rparl2 =
        (tmp - (2.f * eta * cosi) + 1) / (tmp + (2.f * eta * cosi) + 1);
    float tmp_f = eta * eta + k * k;
    float Rperp2 = (tmp_f - (2.f * eta * cosi) + cosi * cosi) /
                   (tmp_f + (2.f * eta * cosi) + cosi * cosi);
    return 0.5f * (Rparl2 + Rperp2);
  }
  float fresnel_schlick(float cosD, float R0) const {
    float omc = 1.f - cosD;
    float omc2 = omc * omc;
    float fr = R0 + (1.f - R0) * omc2 * omc2 * omc;
    float fc = fresnel_conductor(cosD, 0.4f, 1.6f);
    return std_lerp(fr, fc, m.metallic);
  }
  static float fresnel_coat(float cosD) {
    float omc = 1.0f - cosD;
    float omc2 = omc * omc;
    return 0.04f + (1.0f - 0.04f) * omc2 * omc2 * omc;
  }
  float diffuse_term(V3 wi, V3 wo, float idh, float rough) const {
    if (m.metallic == 1.f) return 0.f;
    float l = 1.f - std::fabs(wi.z), l2 = l * l;
    float v = 1.f - std::fabs(wo.z), v2 = v * v;
    float FD90 = 0.5f + 2.f * idh * rough;
    return kInvPi * (1.f + (FD90 - 1.f) * l2 * l2 * l) *
           (1.f + (FD90 - 1.f) * v2 * v2 * v);
  }
  float specular_term(V3 wi, V3 wo, V3 wh, float odh, float rough) const {
    if (wi.z * wo.z <= 0.f) return 0.f;
    float D = ggx_d(wh, rough * rough);
    if (D == 0.f) return 0.f;
    float nr = std_lerp(0.f, 0.08f, m.specular);
    float F = fresnel_schlick(odh, nr);
    float rg = (0.5f + 0.5f * rough);
    float G = ggx_g(wi, wo, wh, rg * rg);
    return F * D * G / (4.f * std::fabs(wi.z) * std::fabs(wo.z));
  }
  float subsurface_term(V3 wi, V3 wo, float idh, float rough) const {
    if (m.subsurface == 0.0f) return 0.0f;
    float l = 1.0f - std::fabs(wi.z), l2 = l * l;
    float v = 1.0f - std::fabs(wo.z), v2 = v * v;
    float F = idh * idh * rough;
    float S = (1.0f + (F - 1.0f) * l2 * l2 * l) *
              (1.0f + (F - 1.0f) * v2 * v2 * v);
    return kInvPi * 1.25f *
           (S * (1.0f / (std::fabs(wo.z) + std::fabs(wi.z)) - 0.5f) + 0.5f);
  }
  float clearcoat_term(V3 wi, V3 wo, V3 wh, float idh, float gloss) const {
    if (m.clearcoat == 0.0f) return 0.0f;
    float rough = dlerp(0.005f, 0.1f, gloss);
    float D = ggx_d(wh, rough);
    if (D == 0.0f) return 0.0f;
    float F = fresnel_coat(idh);
    float G = ggx_g(wo, wi, wh, 0.25f);
    return m.clearcoat * D * F * G /
           (4.0f * std::fabs(wi.z) * std::fabs(wo.z));
  }
  V3 eval(V3 wi, V3 wo) const {
    const V3 lwi = normalized(sf.to_local(wi));
    const V3 lwo = normalized(sf.to_local(wo));
    if (std::fabs(lwi.z) < FLT_EPSILON || std::fabs(lwo.z) < FLT_EPSILON)
      return mk(0, 0, 0);
    float rough = clampf(m.roughness, 0.02f, 1.f);
    V3 untinted = mk(m.lum, m.lum, m.lum);
    V3 spec_alb =
        dlerp(dlerp(m.base, untinted, 1.0f - m.specular_tint), m.base,
              m.metallic);
    V3 sheen_alb = dlerp(untinted, m.base, m.sheen_tint);
    V3 wh = normalized(lwo + lwi);
    float odh = dot(lwo, wh);
    float idh = dot(lwi, wh);
    float omo = 1.f - odh;
    spec_alb = dlerp(spec_alb, untinted, omo * omo * omo);
    float F = fresnel_schlick(odh, 0.0f);
    V3 sheen_term = F * m.sheen * sheen_alb;
    float dl = dlerp(diffuse_term(lwi, lwo, idh, rough),
                     subsurface_term(lwi, lwo, idh, rough), m.subsurface);
    V3 t1 = (1.0f - m.metallic) * (m.base * dl + sheen_term);
    V3 t2 = spec_alb * specular_term(lwi, lwo, wh, odh, rough);
    float cc = clearcoat_term(lwi, lwo, wh, idh, m.clearcoat_gloss);
    return t1 + t2 + mk(cc, cc, cc);
  }
  float pdf(V3 wi, V3 wo) const {
    const V3 lwi = normalized(sf.to_local(wi));
    const V3 lwo = normalized(sf.to_local(wo));
    V3 wh = normalized(lwo + lwi);
    if (maxc(wh) <= 0.f) return 0.f;
    float rough = clampf(m.roughness, 0.02f, 1.f);
    float mpdf = pdf_vn(lwo, wh, rough * rough);
    float p = 0.f;
    float dwhdwi = 1.f / (4.f * std::fabs(dot(lwi, wh)));
    float spec_pdf = mpdf * dwhdwi;
    float nr = std_lerp(0.f, 0.08f, m.specular);
    float odh = dot(lwo, wh);
    float ps = fresnel_schlick(odh, nr);
    p += spec_pdf * ps;
    p += std::fabs(lwi.z) * kInvPi * (1.f - ps);
    if (m.clearcoat > 0.f) {
      float cw = m.clearcoat / (m.clearcoat + m.lum);
      float fc = fresnel_coat(std::fabs(wo.z));
      float pc = (fc * cw) / (fc * cw + (1 - fc) * (1 - cw));
      float cr = std_lerp(0.005f, 0.10f, m.clearcoat_gloss);
      float chp = pdf_vn(wo, wh, cr);
      float cp = chp * dwhdwi;
      p *= 1.0f - pc;
      p += cp * pc;
    }
    return p;
  }
  Sample sample(V3 wo, V3 sam) const {
    const V3 lwo = normalized(sf.to_local(wo));
    V3 lwi, lwh;
    bool coat = false;
    float r0 = sam.x, r1 = sam.y, r2 = sam.z;
    if (m.clearcoat > 0.f) {
      float cw = m.clearcoat / (m.clearcoat + m.lum);
      float fc = fresnel_coat(std::fabs(lwo.z));
      float pc = (fc * cw) / (fc * cw + (1.f - fc) * (1.f - cw));
      if (sam.y < pc) {
        coat = true;
        r1 /= pc;
        float cr = std_lerp(0.005f, 0.1f, m.clearcoat_gloss);
        float cpdf;
        lwh = sample_vn(lwo, r0, r1, &cpdf, cr);
        lwi = reflect(-lwo, lwh);
      } else {
        coat = false;
        r1 = (sam.y - pc) / (1.f - pc);
      }
    }
    if (!coat) {
      float mpdf;
      float rough = clampf(m.roughness, 0.02f, 1.0f);
      lwh = sample_vn(lwo, r0, r1, &mpdf, rough * rough);
      float nr = std_lerp(0.0f, 0.08f, m.specular);
      float odh = dot(lwo, lwh);
      float ps = fresnel_schlick(odh, nr);
      if (r2 <= ps) {
        lwi = reflect(-lwo, lwh);
      } else {
        lwi = cosine_hemisphere(r0, r1, nullptr);
        if (lwo.z < 0.0f) lwi.z *= -1.0f;
      }
    }
    if (lwi.z <= 0.0f) return invalid_sample();
    const V3 wi = sf.to_world(lwi);
    return Sample{wi, eval(wi, wo), pdf(wi, wo), true};
  }
};

/* The base BSDF's black-fringe fallbacks (bsdf.cpp:30-63) for a BSDF of
 * albedo `alb` (Metal's AggregateBSDF: 1; PlasticBsdf: its albedo). */
struct Fringe {
  V3 ng, ns, alb;
  Frame gf;
  Fringe(V3 ng_, V3 ns_, V3 a) : ng(ng_), ns(ns_), alb(a), gf(ng_) {}
  bool causes(V3 w) const { return (dot(ng, w) > 0) != (dot(ns, w) > 0); }
  Sample sample(V3 wo, V3 sam) const {
    if (dot(ng, wo) <= 0.f) return invalid_sample();
    float pdf;
    V3 lwi = cosine_hemisphere(sam.x, sam.y, &pdf);
    if (pdf < FLT_EPSILON) return invalid_sample();
    V3 wi = normalized(gf.to_world(lwi));
    float factor = correct_shading_normal(ng, ns, wi);
    return Sample{wi, alb / kPi * factor, pdf, true, false};
  }
  V3 eval(V3 wi, V3 wo) const {
    if ((dot(ng, wi) <= 0.f) || (dot(ng, wo) <= 0.f)) return mk(0, 0, 0);
    return alb / kPi;
  }
  float pdf(V3 wi, V3 wo) const {
    if ((dot(ng, wi) > 0.f) != (dot(ng, wo) > 0.f)) return 0.f;
    V3 local = normalized(gf.to_local(wi));
    return local.z * kInvPi;
  }
};

/* MirrorBSDF (mirror.cpp:32-66): a delta reflection about the shading
 * normal, kr / |cos|, pdf 1; eval and pdf are 0. */
struct MirrorB {
  V3 ng, ns, kr;
  Frame sf;
  MirrorB(V3 ng_, V3 ns_, V3 kr_) : ng(ng_), ns(ns_), kr(kr_), sf(ns_) {}
  Sample sample(V3 wo) const {
    const V3 lwo = normalized(sf.to_local(wo));
    if (lwo.z <= 0.f) return invalid_sample();
    const V3 lwi = mk(-lwo.x, -lwo.y, lwo.z);
    const V3 wi = sf.to_world(lwi);
    const float factor = correct_shading_normal(ng, ns, wi);
    return Sample{wi, kr * factor / std::fabs(lwi.z), 1.f, true, true};
  }
};

/* GlassBSDF (glass.cpp:31-116) with Glass::Shade's colours (glass.cpp:
 * 128-150): reflection with probability Fr, else refraction, both delta. */
struct GlassB {
  V3 ng, ns, refl, refr;
  float ior;
  Frame sf;
  GlassB(V3 ng_, V3 ns_, const Mat& m)
      : ng(ng_), ns(ns_), refl(m.base), ior(m.p[3]), sf(ns_) {
    refr = mk(std::sqrt(m.p[0]), std::sqrt(m.p[1]), std::sqrt(m.p[2]));
  }
  Sample sample(V3 wo, V3 sam) const {
    const V3 lwo = normalized(sf.to_local(wo));
    const V3 normal = lwo.z > 0 ? mk(0.f, 0.f, 1.f) : mk(0.f, 0.f, -1.f);
    /* DielectricFresnel(eta_in = ior, eta_out = 1) */
    const float fr = dielectric_fresnel(ior, 1.f, lwo.z);
    if (sam.x < fr) {
      const V3 lwi = mk(-lwo.x, -lwo.y, lwo.z);
      const V3 wi = sf.to_world(lwi);
      const V3 f = refl * mk(fr, fr, fr) / std::fabs(lwi.z);
      const float factor = correct_shading_normal(ng, ns, wi);
      return Sample{wi, f * factor, fr, true, true};
    }
    const float eta_i = lwo.z > 0 ? 1.f : ior;
    const float eta_t = lwo.z > 0 ? ior : 1.f;
    const float eta = eta_i / eta_t;
    const float cos_i = std::fabs(lwo.z);
    const float sin2_i = fmax_ref(0.f, 1.f - cos_i * cos_i);
    const float sin2_t = eta * eta * sin2_i;
    if (sin2_t > 1.f) return invalid_sample();
    const float cos_t = std::sqrt(1 - sin2_t);
    const V3 w = (eta * cos_i - cos_t) * normal - eta * lwo;
    const V3 lwi = normalized(w);
    const V3 dir = sf.to_world(lwi);
    const V3 f = eta * eta * refr * (1.f - fr) / std::fabs(lwi.z);
    const float pdf = 1.f - fr;
    const float factor = correct_shading_normal(ng, ns, dir);
    return Sample{dir, f * factor, pdf, true, true};
  }
};

/* TrowbridgeReitzDistribution and EvalPdf of the GGX reflection component
 * (microfacet_reflection_component.cpp:26-135) */
inline float sqr(float x) { return x * x; }
inline float ggx_phi(V3 w) {
  if (w.x <= 0.f && w.y <= 0.f) return 0.f;
  const float r = std::atan2(w.y, w.x);
  return r < 0.f ? (r + 2 * kPi) : r;
}
inline float ggx_tan_theta(V3 w) {
  const float t = 1 - w.z * w.z;
  if (t <= 0) return 0;
  return std::sqrt(t) / w.z;
}
inline float ggx_d(float sin_phi_h, float cos_phi_h, float sin_theta_h,
                   float cos_theta_h, float ax, float ay) {
  const float A = sqr(cos_phi_h / ax) + sqr(sin_phi_h / ay);
  const float RD = sqr(sin_theta_h) * A + sqr(cos_theta_h);
  return 1.f / (kPi * ax * ay * sqr(RD));
}
inline float ggx_g(float cos_phi, float sin_phi, float ax, float ay,
                   float tan_theta) {
  const float t = sqr(ax * cos_phi) + sqr(ay * sin_phi);
  const float sq = 1 + t * sqr(tan_theta);
  const float lambda = -0.5f + 0.5f * std::sqrt(sq);
  return 1 / (1 + lambda);
}
inline V3 ggx_sample_wh(V3 ve, float ax, float ay, float sx, float sy) {
  const V3 vh = normalized(mk(ax * ve.x, ay * ve.y, ve.z));
  const float lensq = vh.x * vh.x + vh.y * vh.y;
  const V3 t1 = lensq > FLT_EPSILON ? mk(-vh.y, vh.x, 0) / std::sqrt(lensq)
                                    : mk(1, 0, 0);
  const V3 t2 = cross(vh, t1);
  const float r = std::sqrt(sx);
  const float phi = 2 * kPi * sy;
  const float t_1 = r * std::cos(phi);
  const float t_2s = r * std::sin(phi);
  const float s = 0.5f * (1 + vh.z);
  const float t_2 = (1 - s) * std::sqrt(1 - t_1 * t_1) + s * t_2s;
  const V3 nh = t_1 * t1 + t_2 * t2 +
                std::sqrt(fmax_ref(0.f, 1.f - t_1 * t_1 - t_2 * t_2)) * vh;
  return normalized(mk(ax * nh.x, ay * nh.y, fmax_ref(0.f, nh.z)));
}
/* EvalPdf<eval, pdf>: f (colored conductor Fresnel) and pdf */
inline void ggx_eval_pdf(V3 lwi, V3 lwo, V3 color, V3 eta2, V3 etak2,
                         float ax, float ay, V3* f, float* pdf) {
  if (lwi.z <= 0 || lwo.z <= 0) {
    if (f) *f = mk(0, 0, 0);
    if (pdf) *pdf = 0.f;
    return;
  }
  const float cos_i = lwi.z, cos_o = lwo.z;
  const V3 lwh = normalized(lwi + lwo);
  const float cos_d = dot(lwi, lwh);
  const float phi_h = ggx_phi(lwh);
  const float sin_phi_h = std::sin(phi_h), cos_phi_h = std::cos(phi_h);
  const float cos_h = lwh.z;
  const float sin_h = std::sqrt(fmax_ref(0.f, 1 - cos_h * cos_h));
  const float D = ggx_d(sin_phi_h, cos_phi_h, sin_h, cos_h, ax, ay);
  const float phi_i = ggx_phi(lwi), phi_o = ggx_phi(lwo);
  const float sin_phi_i = std::sin(phi_i), cos_phi_i = std::cos(phi_i);
  const float sin_phi_o = std::sin(phi_o), cos_phi_o = std::cos(phi_o);
  const float tan_i = ggx_tan_theta(lwi), tan_o = ggx_tan_theta(lwo);
  const float Go = ggx_g(cos_phi_o, sin_phi_o, ax, ay, tan_o);
  if (f) {
    const float Gi = ggx_g(cos_phi_i, sin_phi_i, ax, ay, tan_i);
    const float G = Gi * Go;
    const V3 F = color * conductor_fresnel(eta2, etak2, cos_d);
    *f = F * D * G / std::fabs(4 * cos_i * cos_o);
  }
  if (pdf) *pdf = Go * D / (4 * lwo.z);
}

/* Metal::Shade (metal.cpp:42-66): an AggregateBSDF of albedo 1 holding one
 * GGX reflection component of weight 1 with a ColoredConductorFresnel
 * (aggregate_bsdf.cpp:43-131). */
struct MetalB {
  V3 ng, ns, color, eta2, etak2;
  float ax, ay;
  Frame sf;
  Fringe fr;
  MetalB(V3 ng_, V3 ns_, const Mat& m)
      : ng(ng_), ns(ns_), color(m.base), ax(m.p[6]), ay(m.p[7]), sf(ns_),
        fr(ng_, ns_, mk(1.f, 1.f, 1.f)) {
    const V3 k = mk(m.p[0], m.p[1], m.p[2]);
    const V3 eta = mk(m.p[3], m.p[4], m.p[5]);
    eta2 = (eta / mk(1.f, 1.f, 1.f)) * (eta / mk(1.f, 1.f, 1.f));
    etak2 = (k / mk(1.f, 1.f, 1.f)) * (k / mk(1.f, 1.f, 1.f));
  }
  Sample sample(V3 wo, V3 sam) const {
    if (fr.causes(wo)) return fr.sample(wo, sam);
    const V3 lwo = normalized(sf.to_local(wo));
    if (lwo.z <= 0.f) return invalid_sample();
    /* GGXMicrofacetReflectionComponent::Sample (:137-154) */
    if (lwo.z <= 0) return invalid_sample();
    const V3 lwh = normalized(ggx_sample_wh(lwo, ax, ay, sam.y, sam.z));
    if (lwh.z <= 0) return invalid_sample();
    V3 lwi = normalized(2 * dot(lwo, lwh) * lwh - lwo);
    if (lwi.z <= 0) return invalid_sample();
    V3 f;
    float pdf;
    ggx_eval_pdf(lwi, lwo, color, eta2, etak2, ax, ay, &f, &pdf);
    if (pdf == 0) return invalid_sample();
    lwi = normalized(lwi);
    pdf *= 1.f;
    const V3 wi = sf.to_world(lwi);
    const float factor = correct_shading_normal(ng, ns, wi);
    return Sample{wi, f * factor, pdf, true, false};
  }
  V3 eval(V3 wi, V3 wo) const {
    if (fr.causes(wo)) return fr.eval(wi, wo);
    const V3 lwi = normalized(sf.to_local(wi));
    const V3 lwo = normalized(sf.to_local(wo));
    if (lwi.z <= 0.f || lwo.z <= 0.f) return mk(0, 0, 0);
    V3 f;
    ggx_eval_pdf(lwi, lwo, color, eta2, etak2, ax, ay, &f, nullptr);
    return mk(0, 0, 0) + f;
  }
  float pdf(V3 wi, V3 wo) const {
    if (fr.causes(wo)) return fr.pdf(wi, wo);
    const V3 lwi = normalized(sf.to_local(wi));
    const V3 lwo = normalized(sf.to_local(wo));
    if (lwi.z <= 0.f || lwo.z <= 0.f) return 0.f;
    float p;
    ggx_eval_pdf(lwi, lwo, color, eta2, etak2, ax, ay, nullptr, &p);
    float wsum = 0.f, acc = 0.f;
    wsum += 1.f;
    acc += 1.f * p;
    return wsum > 0 ? acc / wsum : 0;
  }
};

/* checkReflectionConstraint (bsdf/helper.h:26-31) */
inline bool reflection_constraint(V3 wi, V3 wo) {
  return std::fabs(wi.z * wo.z - wi.x * wo.x - wi.y * wo.y - 1.0f) < 1e-3f;
}

/* PlasticBsdf (plastic_bsdf.cpp:29-185): a delta coat reflection with
 * probability Fi / (Fi + T (1 - Fi)), else the cosine-sampled substrate.
 * No shading-normal correction; Eval does not reject wi below the
 * surface. */
struct PlasticB {
  V3 ng, ns, albedo;
  float ior, avg_t, dfres;
  V3 scaled;
  Frame sf;
  Fringe fr;
  PlasticB(V3 ng_, V3 ns_, const Mat& m)
      : ng(ng_), ns(ns_), albedo(m.base), ior(m.p[0]), avg_t(m.plastic_avg_t),
        dfres(m.plastic_diffuse_fresnel), sf(ns_), fr(ng_, ns_, m.base) {
    const float sc = m.p[1] * m.p[2];
    scaled = mk(sc, sc, sc);
  }
  V3 substrate(float Fi, float Fo, float eta) const {
    return ((1.0f - Fi) * (1.0f - Fo) * eta * eta) *
           (albedo / (mk(1.0f, 1.0f, 1.0f) - albedo * dfres));
  }
  V3 absorb(V3 lwi, V3 lwo) const {
    const V3 e = scaled * (-1.0f / lwi.z - 1.0f / lwo.z);
    return mk(std::exp(e.x), std::exp(e.y), std::exp(e.z));
  }
  Sample sample(V3 wo, V3 sam) const {
    if (fr.causes(wo)) return fr.sample(wo, sam);
    const V3 lwo = normalized(sf.to_local(wo));
    if (lwo.z <= 0.f) return invalid_sample();
    const float eta = 1.f / ior;
    const float Fi = dielectric_reflectance(eta, lwo.z);
    const float substrate_weight = avg_t * (1.0f - Fi);
    const float specular_weight = Fi;
    const float sp = specular_weight / (specular_weight + substrate_weight);
    V3 lwi, f;
    float pdf;
    bool delta;
    if (sam.x < sp) {
      lwi = mk(-lwo.x, -lwo.y, lwo.z);
      pdf = sp;
      const float v = Fi / sp;
      f = mk(v, v, v);
      delta = true;
    } else {
      lwi = cosine_hemisphere(sam.y, sam.z, &pdf);
      const float Fo = dielectric_reflectance(eta, lwi.z);
      f = substrate(Fi, Fo, eta);
      if (maxc(scaled) > 0.0f) f = f * absorb(lwi, lwo);
      pdf *= (1.0f - sp);
      f = f / (1.0f - sp);
      delta = false;
    }
    const V3 wi = sf.to_world(lwi);
    return Sample{normalized(wi), f, pdf, true, delta};
  }
  V3 eval(V3 wi, V3 wo) const {
    if (fr.causes(wo)) return fr.eval(wi, wo);
    const V3 lwi = normalized(sf.to_local(wi));
    const V3 lwo = normalized(sf.to_local(wo));
    const float eta = 1.0f / ior;
    const float Fi = dielectric_reflectance(eta, lwo.z);
    const float Fo = dielectric_reflectance(eta, lwi.z);
    if (reflection_constraint(lwo, lwi)) return mk(Fi, Fi, Fi);
    V3 brdf = ((1.0f - Fi) * (1.0f - Fo) * eta * eta * lwi.z * (1.f / kPi)) *
              (albedo / (mk(1.0f, 1.0f, 1.0f) - albedo * dfres));
    if (maxc(scaled) > 0.0f) brdf = brdf * absorb(lwi, lwo);
    return brdf;
  }
  float pdf(V3 wi, V3 wo) const {
    if (fr.causes(wo)) return fr.pdf(wi, wo);
    const V3 lwi = normalized(sf.to_local(wi));
    const V3 lwo = normalized(sf.to_local(wo));
    if (lwi.z <= 0.0f || lwo.z <= 0.0f) return 0.0f;
    const float Fi = dielectric_reflectance(1.0f / ior, lwo.z);
    const float substrate_weight = avg_t * (1.0f - Fi);
    const float specular_weight = Fi;
    const float sp = specular_weight / (specular_weight + substrate_weight);
    if (reflection_constraint(lwo, lwi)) return sp;
    return lwi.z * kInvPi * (1.0f - sp);
  }
};

struct Bsdf {
  int type;
  Lambert lam;
  Disney dis;
  V3 ng, ns;
  const Mat& m;
  Bsdf(const Mat& m_, V3 ng_, V3 ns_)
      : type(m_.type), lam(ng_, ns_, m_.base), dis(m_, ns_), ng(ng_), ns(ns_),
        m(m_) {}
  Sample sample(V3 wo, V3 s) const {
    switch (type) {
      case ORC_MAT_DIFFUSE: return lam.sample(wo, s);
      case ORC_MAT_DISNEY: return dis.sample(wo, s);
      case ORC_MAT_MIRROR: return MirrorB(ng, ns, m.base).sample(wo);
      case ORC_MAT_GLASS: return GlassB(ng, ns, m).sample(wo, s);
      case ORC_MAT_METAL: return MetalB(ng, ns, m).sample(wo, s);
      case ORC_MAT_PLASTIC: return PlasticB(ng, ns, m).sample(wo, s);
      default: /* NullBsdf (null.cpp:31-52): straight through */
        return Sample{-wo, mk(1.f, 1.f, 1.f), 1.f, true, true};
    }
  }
  V3 eval(V3 wi, V3 wo) const {
    switch (type) {
      case ORC_MAT_DIFFUSE: return lam.eval(wi, wo);
      case ORC_MAT_DISNEY: return dis.eval(wi, wo);
      case ORC_MAT_METAL: return MetalB(ng, ns, m).eval(wi, wo);
      case ORC_MAT_PLASTIC: return PlasticB(ng, ns, m).eval(wi, wo);
      default: return mk(0, 0, 0);
    }
  }
  float pdf(V3 wi, V3 wo) const {
    switch (type) {
      case ORC_MAT_DIFFUSE: return lam.pdf(wi, wo);
      case ORC_MAT_DISNEY: return dis.pdf(wi, wo);
      case ORC_MAT_METAL: return MetalB(ng, ns, m).pdf(wi, wo);
      case ORC_MAT_PLASTIC: return PlasticB(ng, ns, m).pdf(wi, wo);
      default: return 0.f;
    }
  }
};

/* ---------------------------------------------------------------- RNG --- */
/* Counter-based stand-in for RandomSampler (random_sampler.cpp:28-45), see
 * counter_rng.h. */
inline uint64_t path_key(uint64_t seed, uint32_t pixel, uint32_t sample) {
  return ajg_path_key(seed, pixel, sample);
}
inline float key_float(uint64_t key, uint32_t dim) {
  return ajg_key_float(key, dim);
}
struct Rng {
  uint64_t key;
  uint32_t dim = 0;
  float next() { return key_float(key, dim++); }
};

/* ------------------------------------------------------------- lights --- */
struct Light {
  int type;
  int area = -1; /* index into Scene::areas for ORC_LIGHT_AREA */
  V3 rgb;      /* directional radiance / env texel */
  V3 dir;      /* normalised toward-light direction */
  float cosmax;
  float scaler, rot;
  Frame frame;
  bool env_ok; /* luminance > 0: Distribution2D has mass */
  Light(const float* l)
      : type((int)l[0]),
        rgb(mk(l[1], l[2], l[3])),
        dir(normalized(mk(l[4], l[5], l[6]))),
        cosmax(l[7]),
        scaler(l[8]),
        rot(l[9]),
        frame(normalized(mk(l[4], l[5], l[6]))) {
    /* env_light.cpp:29-48 with a 1x1 texture: weight = lum * sin(pi/2) */
    float w = luminance(rgb) * std::sin(kPi * (0 + 0.5f) / float(1));
    env_ok = w * (1.f / float(1)) > 0.f;
  }
  Light(int area_index, V3 radiance)
      : type(ORC_LIGHT_AREA),
        area(area_index),
        rgb(radiance),
        dir(mk(0, 1, 0)),
        cosmax(1.f),
        scaler(1.f),
        rot(0.f),
        frame(mk(0, 1, 0)),
        env_ok(false) {}
};

/* AreaLight over an emissive primitive's geometry (area_light.cpp, with
 * the geometry's Sample / Pdf: quad.cpp:128-171, cube.cpp:145-191,
 * mesh.cpp:62-68,251-297, two_sided.cpp:65-114). */
struct AreaL {
  V3 rad;
  int kind = ORC_GEOM_QUAD;
  bool two_sided = false;
  /* quad: a, b, c, d; mesh: its corners in index-buffer order; cube: each
   * triangle's corners in the tuples' declared order */
  std::vector<V3> pts;
  int ntri = 0;
  float area = 0.f, sample_prob = 0.f;
  float pdf_const = 0.f; /* Geometry::Pdf (the same for every point) */
};

struct GeomSample {
  V3 pos, ng;
  float pdf;
};

GeomSample area_sample(const AreaL& A, float x, float y, float z) {
  V3 sam = mk(x, y, z);
  bool back = false;
  if (A.two_sided) { /* TwoSided::Sample splits x between the faces */
    back = sam.x < 0.5f;
    if (back)
      sam.x = 2 * x;
    else
      sam.x = 2 * (x - 0.5f);
  }
  V3 sn = sam;
  if (sn.x + sn.y > 1.f) {
    sn.x = 1.f - sn.x;
    sn.y = 1.f - sn.y;
  }
  GeomSample g;
  if (A.kind == ORC_GEOM_QUAD) {
    const V3 &a = A.pts[0], &b = A.pts[1], &c = A.pts[2], &d = A.pts[3];
    if (sam.z < A.sample_prob) {
      g.pos = (1 - sn.x - sn.y) * a + sn.x * b + sn.y * c;
      g.ng = normalized(cross(b - a, c - a));
    } else {
      g.pos = (1 - sn.x - sn.y) * a + sn.x * c + sn.y * d;
      g.ng = normalized(cross(c - a, d - a));
    }
    g.pdf = 1.f / A.area;
  } else if (A.kind == ORC_GEOM_MESH) {
    /* the triangle index addresses the index buffer without the factor
     * 3: corners idx, idx+1, idx+2 (mesh.cpp:260-262) */
    const int idx = std::min(int(sam.z * (float)A.ntri), A.ntri - 1);
    const V3 &pi = A.pts[idx], &pj = A.pts[idx + 1], &pk = A.pts[idx + 2];
    g.pos = (1 - sn.x - sn.y) * pi + sn.x * pj + sn.y * pk;
    g.ng = normalized(cross(pj - pi, pk - pi));
    g.pdf = 1.f / A.area;
  } else {
    const int idx = std::min(int(sam.z * (float)12), 11);
    const V3 &pa = A.pts[3 * idx], &pb = A.pts[3 * idx + 1],
             &pc = A.pts[3 * idx + 2];
    g.pos = (1 - sn.x - sn.y) * pa + sn.x * pb + sn.y * pc;
    g.ng = normalized(cross(pb - pa, pc - pa));
    g.pdf = 1.f / (12.f * length(cross(pb - pa, pc - pa)) * 0.5f);
  }
  if (A.two_sided) {
    g.pdf = (float)((double)g.pdf * 0.5);
    if (back) g.ng = g.ng * -1.f;
  }
  return g;
}

/* AreaLight::Pdf (area_light.cpp:68-79) */
float area_pdf(const AreaL& A, V3 ref, V3 pos, V3 normal) {
  if (dot(ref - pos, normal) <= 0.f) return 0.f;
  const V3 l2r = ref - pos;
  const float dist2 = dot(l2r, l2r);
  const float abscos = std::fabs(dot(l2r, normal));
  return A.pdf_const * (dist2 / abscos);
}

AreaL make_area(const float* tris, const float* rad, const int32_t* info) {
  AreaL A;
  A.rad = mk(rad[0], rad[1], rad[2]);
  const int64_t first = info[0];
  A.ntri = info[1];
  A.kind = info[2];
  A.two_sided = info[3] != 0;
  auto corner = [&](int64_t t, int k) { return ld3(tris + 9 * (first + t) + 3 * k); };
  if (A.kind == ORC_GEOM_QUAD) {
    const V3 a = corner(0, 0), b = corner(0, 1), c = corner(0, 2),
             d = corner(1, 2);
    A.pts = {a, b, c, d};
    const float abc = length(cross(b - a, c - a)) * 0.5f;
    const float acd = length(cross(c - a, d - a)) * 0.5f;
    A.area = abc + acd;
    A.sample_prob = abc / A.area;
    A.pdf_const = 1.f / A.area;
  } else if (A.kind == ORC_GEOM_MESH) {
    float area = 0.f;
    for (int t = 0; t < A.ntri; ++t) {
      const V3 pi = corner(t, 0), pj = corner(t, 1), pk = corner(t, 2);
      A.pts.push_back(pi);
      A.pts.push_back(pj);
      A.pts.push_back(pk);
      area = (float)((double)area +
                     0.5 * (double)length(cross(pj - pi, pk - pi)));
    }
    A.area = area;
    A.pdf_const = 1.f / area;
  } else {
    /* the MeshView sees each tuple reversed; Sample reads it as declared */
    for (int t = 0; t < A.ntri; ++t)
      for (int k = 2; k >= 0; --k) A.pts.push_back(corner(t, k));
    const V3 &pa = A.pts[0], &pb = A.pts[1], &pc = A.pts[2];
    A.pdf_const = 1.f / (12.f * length(cross(pb - pa, pc - pa)) * 0.5f);
  }
  if (A.two_sided) A.pdf_const = A.pdf_const * 0.5f;
  return A;
}

struct LightSample {
  V3 pos, radiance;
  float pdf;
};

/* --------------------------------------------------------- integrator --- */
struct Scene {
  Accel acc;
  const float* corner_n;
  const int32_t* tri_mat;
  const int32_t* tri_flags;
  std::vector<Mat> mats;
  std::vector<Light> lights;
  std::vector<AreaL> areas;
  std::vector<int> tri_light; /* light index of an emissive triangle, or -1 */
  int env = -1;
  float radius; /* (aabb.max - aabb.center).length() */
  Box world;     /* the primitives' joined bounds */
  int mode;
};

struct HitInfo {
  V3 pos, ng, ns, wr;
  int mat;
};

/* Triangle hit completion: Triangle::Intersect's normal plus the
 * geometry's PostIntersect (quad.cpp:73-90, cube.cpp:96-108,
 * mesh.cpp:183-204, two_sided.cpp:44-53). */
HitInfo complete_hit(const Scene& s, const Ray& r, const Hit& h) {
  HitInfo hi;
  const float* t = s.acc.tris + 9 * (int64_t)h.prim;
  V3 a = ld3(t), b = ld3(t + 3), c = ld3(t + 6);
  int fl = s.tri_flags[h.prim];
  hi.pos = r.o + h.t * r.d;
  if (fl & ORC_TRI_NG_REVERSED)
    hi.ng = normalized(cross(b - c, a - c));
  else
    hi.ng = normalized(cross(b - a, c - a));
  if (fl & ORC_TRI_HAS_NORMALS) {
    const float* cn = s.corner_n + 9 * (int64_t)h.prim;
    hi.ns = (1 - h.u - h.v) * ld3(cn) + h.u * ld3(cn + 3) + h.v * ld3(cn + 6);
  } else {
    hi.ns = hi.ng;
  }
  hi.wr = -r.d;
  if (fl & ORC_TRI_TWO_SIDED) {
    if (dot(hi.ng, hi.wr) < 0) {
      hi.ng = hi.ng * -1.f;
      hi.ns = hi.ns * -1.f;
    }
  }
  hi.mat = s.tri_mat[h.prim];
  return hi;
}

inline V3 eps_offset(const HitInfo& h, V3 dir) { /* intersection.h:42-47 */
  if (dot(dir, h.ng) > 0.f) return h.pos + h.ng * kEps;
  return h.pos - h.ng * kEps;
}

inline float power_heuristic(float a, float b) { /* helper.h:38-42 */
  a *= a;
  b *= b;
  return a / (a + b);
}

/* EnvLight::Pdf (env_light.cpp:152-170) for a 1x1 texture */
float env_pdf(const Light& L, V3 ref2light) {
  const V3 d = normalized(ref2light);
  float theta = std::acos(clampf(d.y, -1.f, 1.f));
  float st = std::sin(theta);
  float p2 = L.env_ok ? 1.f : 0.f;
  return p2 / (2.f * kPi * kPi * st);
}

/* MISSampleLight / MISSampleEnvLight (helper.h:73-133) */
V3 mis_light(const Scene& s, const Light& L, const HitInfo& h, const Bsdf& f,
             Rng& rng) {
  LightSample ls;
  if (L.type == ORC_LIGHT_AREA) { /* AreaLight::Sample (area_light.cpp:36-57) */
    const float x = rng.next(), y = rng.next(), z = rng.next(); /* Next3D */
    const AreaL& A = s.areas[L.area];
    const GeomSample g = area_sample(A, x, y, z);
    if (dot(g.ng, h.pos - g.pos) <= 0) return mk(0, 0, 0);
    const V3 i2r = h.pos - g.pos;
    const float dist2 = dot(i2r, i2r);
    ls.pdf = g.pdf * dist2 / std::fabs(dot(g.ng, i2r));
    ls.pos = g.pos;
    ls.radiance = A.rad;
  } else if (L.type == ORC_LIGHT_DIRECTIONAL) {
    float u0 = rng.next(), u1 = rng.next();
    V3 r2l = L.frame.to_world(uniform_cone(u0, u1, L.cosmax));
    ls.pdf = uniform_cone_pdf(L.cosmax);
    ls.pos = h.pos + 2.f * s.radius * r2l;
    ls.radiance = L.rgb;
  } else {
    /* the two Next1D() arguments of SampleContinuous are evaluated right to
     * left by g++: the first draw is v, the second u */
    float v = rng.next(), u = rng.next();
    if (!L.env_ok) return mk(0, 0, 0);
    float pdf = 1.f;
    constexpr float inv_2_pi = 1.f / (2.f * kPi);
    constexpr float two_pi = 2.f * kPi;
    u -= L.rot / 180 * kPi * inv_2_pi;
    if (u > 1.f) u -= 1.f;
    if (u < 0.f) u += 1.f;
    float phi = u * two_pi;
    float theta = v * kPi;
    float st = std::sin(theta);
    pdf = st != 0.f ? pdf / (2.f * kPi * kPi * st) : 0.f;
    V3 dir = mk(-std::sin(theta) * std::cos(phi), std::cos(theta),
                -std::sin(theta) * std::sin(phi));
    ls.pos = h.pos + 2.f * s.radius * dir;
    ls.radiance = L.rgb;
    ls.pdf = pdf;
  }
  if (is_black(ls.radiance) || ls.pdf <= 0.f) return mk(0, 0, 0);
  const float len = length(ls.pos - h.pos) - kEps;
  if (len < kEps) return mk(0, 0, 0);
  const V3 w = normalized(ls.pos - h.pos);
  Ray sr = make_ray(h.pos, w, kEps, 0.99f * len);
  if (trace_any(s.acc, sr, s.mode, true)) return mk(0, 0, 0);
  const V3 bf = f.eval(w, h.wr);
  if (is_black(bf)) return mk(0, 0, 0);
  /* MISSampleAreaLight takes the shading normal as it is; the others
   * normalise it (helper.h:64, 91, 120) */
  const V3 n = L.type == ORC_LIGHT_AREA ? h.ns : normalized(h.ns);
  V3 fv;
  if (L.type == ORC_LIGHT_DIRECTIONAL || L.type == ORC_LIGHT_AREA)
    fv = mk(1.f, 1.f, 1.f) * ls.radiance * bf * std::fabs(dot(w, n));
  else
    fv = ls.radiance * bf * std::fabs(dot(w, n));
  const float bp = f.pdf(w, h.wr);
  return fv / ls.pdf * power_heuristic(ls.pdf, bp);
}

/* MISSampleBsdf (helper.h:209-265): a ray that escapes sees the
 * environment, one that hits an emissive primitive its area light. */
V3 mis_bsdf(const Scene& s, const HitInfo& h, const Bsdf& f, Rng& rng) {
  float a = rng.next(), b = rng.next(), c = rng.next();
  Sample bs = f.sample(h.wr, mk(a, b, c));
  if (is_black(bs.f) || bs.pdf == 0.f) return mk(0, 0, 0);
  bs.dir = normalized(bs.dir);
  Ray r = make_ray(eps_offset(h, bs.dir), bs.dir);
  Hit hh = trace_closest(s.acc, r, s.mode, true);
  if (hh.prim >= 0) {
    const int li = s.tri_light.empty() ? -1 : s.tri_light[hh.prim];
    if (li < 0) return mk(0, 0, 0);
    const HitInfo lh = complete_hit(s, r, hh);
    const AreaL& A = s.areas[s.lights[li].area];
    const V3 le = dot(lh.ng, lh.wr) > 0 ? A.rad : mk(0, 0, 0);
    if (is_black(le)) return mk(0, 0, 0);
    const V3 fv = le * bs.f * std::fabs(dot(h.ns, r.d));
    if (bs.delta) return fv / bs.pdf;
    const float lp = area_pdf(A, r.o, lh.pos, lh.ng);
    return fv / bs.pdf * power_heuristic(bs.pdf, lp);
  }
  if (s.env < 0) return mk(0, 0, 0);
  const Light& L = s.lights[s.env];
  V3 rad = L.scaler * L.rgb;
  if (is_black(rad)) return mk(0, 0, 0);
  V3 fv = rad * bs.f * std::fabs(dot(h.ns, r.d));
  V3 out = mk(0, 0, 0);
  if (bs.delta) {
    out = out + fv / bs.pdf;
  } else {
    float lp = env_pdf(L, r.d);
    out = out + fv / bs.pdf * power_heuristic(bs.pdf, lp);
  }
  return out;
}

/* PathTracing::TraceMIS (pt.cpp:98-227) and Trace (pt.cpp:229-311) */
V3 trace_path(const Scene& s, Ray ray, Rng& rng, int min_b, int max_b,
              float cont, bool use_mis) {
  V3 L = mk(0, 0, 0);
  V3 T = mk(1.f, 1.f, 1.f);
  for (int bounce = 0; bounce < max_b; bounce++) {
    if (bounce > min_b) {
      if (rng.next() > cont) return L;
      T = T / cont;
    }
    Hit h = trace_closest(s.acc, ray, s.mode, true);
    if (h.prim < 0) {
      if ((bounce == 0 || !use_mis) && s.env >= 0) {
        const Light& E = s.lights[s.env];
        L = L + E.scaler * E.rgb;
      }
      return L;
    }
    HitInfo hi = complete_hit(s, ray, h);
    const Mat& m = s.mats[hi.mat];
    Bsdf f(m, hi.ng, hi.ns);
    T = T * mk(1.f, 1.f, 1.f); /* void medium: SampleScattering throughput */
    /* emission: on camera rays with MIS (pt.cpp:185-190), on every hit
     * without (pt.cpp:282-286); AreaLight::Radiance (area_light.cpp:30-34) */
    const int li = s.tri_light.empty() ? -1 : s.tri_light[h.prim];
    if (li >= 0 && (bounce == 0 || !use_mis)) {
      const AreaL& A = s.areas[s.lights[li].area];
      const V3 le = dot(hi.ng, hi.wr) > 0 ? A.rad : mk(0, 0, 0);
      L = L + T * le;
    }
    if (use_mis) {
      V3 direct = mk(0, 0, 0);
      for (const Light& lt : s.lights) direct = direct + T * mis_light(s, lt, hi, f, rng);
      direct = direct + T * mis_bsdf(s, hi, f, rng);
      L = L + 1.f / 1 * direct;
    }
    float a = rng.next(), b = rng.next(), c = rng.next();
    Sample bs = f.sample(hi.wr, mk(a, b, c));
    if (is_black(bs.f) || bs.pdf < 0.f) return L;
    T = T * (bs.f * std::fabs(dot(hi.ng, bs.dir)) / bs.pdf);
    ray = make_ray(eps_offset(hi, bs.dir), bs.dir);
  }
  return L;
}

/* ---------------------------------------------------------------- SPPM --- */
/* HasDiffuseComponent (sppm.cpp:77's visible-point rule): Lambert and
 * plastic yes, Disney when metallic < 1 (disney.cpp:79), mirror, glass and
 * null no.  Metal's AggregateBSDF::HasDiffuseComponent (aggregate_bsdf.cpp:
 * 37-41) runs off its end when no component is diffuse -- the reference's
 * Release build faults there; the loop's own verdict, no, is taken. */
bool has_diffuse(const Mat& m) {
  switch (m.type) {
    case ORC_MAT_DIFFUSE: return true;
    case ORC_MAT_DISNEY: return m.metallic < 1.f;
    case ORC_MAT_PLASTIC: return true;
    default: return false;
  }
}

struct VisPoint {
  bool valid = false;
  V3 pos, wr, thr, ng, ns;
  int mat = -1;
};

/* TracerVP (sppm.cpp:35-101) */
VisPoint tracer_vp(const Scene& s, Ray ray, Rng& rng, int fmd, V3& direct) {
  V3 T = mk(1.f, 1.f, 1.f);
  for (int depth = 0; depth < fmd; ++depth) {
    Hit h = trace_closest(s.acc, ray, s.mode, true);
    if (h.prim < 0) {
      if (depth == 0 && s.env >= 0) {
        const Light& E = s.lights[s.env];
        direct = direct + T * (E.scaler * E.rgb);
      }
      return VisPoint{};
    }
    HitInfo hi = complete_hit(s, ray, h);
    const Mat& m = s.mats[hi.mat];
    Bsdf f(m, hi.ng, hi.ns);
    if (depth == 0) {
      const int li = s.tri_light.empty() ? -1 : s.tri_light[h.prim];
      if (li >= 0) {
        const AreaL& A = s.areas[s.lights[li].area];
        const V3 le = dot(hi.ng, hi.wr) > 0 ? A.rad : mk(0, 0, 0);
        direct = direct + T * le;
      }
    }
    V3 sum = mk(0, 0, 0);
    for (const Light& lt : s.lights) sum = sum + T * mis_light(s, lt, hi, f, rng);
    sum = sum + T * mis_bsdf(s, hi, f, rng);
    direct = direct + 1.f / 1 * sum;
    if (has_diffuse(m) || depth == fmd - 1) {
      if (!(std::isfinite(T.x) && std::isfinite(T.y) && std::isfinite(T.z)))
        return VisPoint{};
      VisPoint vp;
      vp.valid = true;
      vp.pos = hi.pos;
      vp.thr = T;
      vp.wr = hi.wr;
      vp.ng = hi.ng;
      vp.ns = hi.ns;
      vp.mat = (int)hi.mat;
      return vp;
    }
    float a = rng.next(), b = rng.next(), c = rng.next();
    Sample bs = f.sample(hi.wr, mk(a, b, c));
    if (is_black(bs.f) || bs.pdf < 0.f) return VisPoint{};
    T = T * (bs.f * std::fabs(dot(hi.ng, bs.dir)) / bs.pdf);
    ray = make_ray(eps_offset(hi, bs.dir), bs.dir);
  }
  return VisPoint{};
}

/* sppm::Pixel (photon_mapping.h:54-67) */
struct SppmPixel {
  VisPoint vp;
  float radius = 0.1f;
  float phi[3] = {0.f, 0.f, 0.f};
  int M = 0;
  float N = 0;
  V3 tau = mk(0, 0, 0);
  V3 direct = mk(0, 0, 0);
};

/* VisiblePointSearcher (photon_mapping.h:69-148): 40960 hash entries of
 * pixel lists; a visible point joins the cells [lo, hi) of its radius box
 * (the last cell on each axis is left out). */
struct VpGrid {
  Box bound;
  float side;
  std::vector<std::vector<int>> entries;
  VpGrid(Box b, float s_) : bound(b), side(s_), entries(40960) {}
  void cell(V3 pos, int c[3]) const {
    const V3 hd = pos - bound.lo;
    c[0] = static_cast<int>(fmax_ref(hd.x, 0.f) / side);
    c[1] = static_cast<int>(fmax_ref(hd.y, 0.f) / side);
    c[2] = static_cast<int>(fmax_ref(hd.z, 0.f) / side);
  }
  static size_t hash_combine(size_t a, size_t b) {
    return a ^ (b + 0x9e3779b97f4a7c15ull + (a << 6) + (a >> 2));
  }
  size_t entry(int x, int y, int z) const {
    const size_t low3 = ((x & 1) << 0) | ((y & 1) << 1) | ((z & 2) << 0);
    size_t h = (size_t)x; /* std::hash<int> */
    h = hash_combine(h, (size_t)y);
    h = hash_combine(h, (size_t)z);
    return ((h << 3) % entries.size()) | low3;
  }
  void add_vp(int pix, V3 pos, float r) {
    int lo[3], hi[3];
    cell(pos - mk(r, r, r), lo);
    cell(pos + mk(r, r, r), hi);
    for (int z = lo[2]; z < hi[2]; ++z)
      for (int y = lo[1]; y < hi[1]; ++y)
        for (int x = lo[0]; x < hi[0]; ++x) entries[entry(x, y, z)].push_back(pix);
  }
};

/* AddPhoton (photon_mapping.h:101-120) */
void add_photon(const Scene& s, VpGrid& g, std::vector<SppmPixel>& px, V3 pos,
                V3 phi, V3 wr) {
  int c[3];
  g.cell(pos, c);
  const std::vector<int>& list = g.entries[g.entry(c[0], c[1], c[2])];
  for (auto it = list.rbegin(); it != list.rend(); ++it) {
    SppmPixel& p = px[*it];
    const V3 d = p.vp.pos - pos;
    if (dot(d, d) > p.radius * p.radius) continue;
    const Bsdf f(s.mats[p.vp.mat], p.vp.ng, p.vp.ns);
    const V3 dp = phi * f.eval(wr, p.vp.wr);
    if (!(std::isfinite(dp.x) && std::isfinite(dp.y) && std::isfinite(dp.z)))
      continue;
    p.phi[0] += dp.x;
    p.phi[1] += dp.y;
    p.phi[2] += dp.z;
    ++p.M;
  }
}

struct Emit {
  V3 pos, dir, normal, radiance;
  float pdf_pos = 0.f, pdf_dir = 0.f;
};

/* Light::SampleEmit: directional_light.cpp:60-79, env_light.cpp:105-150,
 * area_light.cpp:59-70 */
Emit sample_emit(const Scene& s, const Light& L, Rng& rng) {
  Emit e;
  const V3 center = box_center(s.world);
  if (L.type == ORC_LIGHT_AREA) {
    const float x = rng.next(), y = rng.next(), z = rng.next();
    const GeomSample g = area_sample(s.areas[L.area], x, y, z);
    const float u0 = rng.next(), u1 = rng.next();
    float pdf_dir;
    const V3 lwi = cosine_hemisphere(u0, u1, &pdf_dir);
    e.pos = g.pos;
    e.dir = Frame(g.ng).to_world(lwi);
    e.normal = g.ng;
    e.radiance = s.areas[L.area].rad;
    e.pdf_pos = g.pdf;
    e.pdf_dir = pdf_dir;
  } else if (L.type == ORC_LIGHT_DIRECTIONAL) {
    const float u0 = rng.next(), u1 = rng.next();
    const V3 r2l = L.frame.to_world(uniform_cone(u0, u1, L.cosmax));
    const float pdf_dir = uniform_cone_pdf(L.cosmax);
    const float radius = s.radius;
    const float d0 = rng.next(), d1 = rng.next();
    float dx, dy;
    concentric(d0, d1, &dx, &dy);
    const Frame dc(r2l);
    e.pos = center + (dx * dc.dx + dy * dc.dy + r2l) * radius;
    e.dir = -r2l;
    e.normal = normalized(-r2l);
    e.radiance = L.rgb;
    e.pdf_pos = 1.f / (kPi * radius * radius);
    e.pdf_dir = pdf_dir;
  } else {
    float v = rng.next(), u = rng.next(); /* g++: right to left */
    if (!L.env_ok) return Emit{};
    float pdf = 1.f;
    constexpr float inv_2_pi = 1.f / (2.f * kPi);
    constexpr float two_pi = 2.f * kPi;
    u -= L.rot / 180 * kPi * inv_2_pi;
    if (u > 1.f) u -= 1.f;
    if (u < 0.f) u += 1.f;
    const float phi = u * two_pi;
    const float theta = v * kPi;
    const float st = std::sin(theta);
    pdf = st != 0.f ? pdf / (2.f * kPi * kPi * st) : 0.f;
    V3 dir = mk(-std::sin(theta) * std::cos(phi), std::cos(theta),
                -std::sin(theta) * std::sin(phi));
    dir = -dir;
    const float radius = s.radius;
    const float d0 = rng.next(), d1 = rng.next();
    float dx, dy;
    concentric(d0, d1, &dx, &dy);
    const Frame dc(-dir);
    e.pos = center + (dx * dc.dx + dy * dc.dy - dir) * radius;
    e.dir = dir;
    e.normal = normalized(dir);
    e.radiance = L.rgb; /* the texel, without the scaler */
    e.pdf_pos = 1.f / (kPi * radius * radius);
    e.pdf_dir = pdf;
  }
  return e;
}

/* TracerPhoton (sppm.cpp:103-143); DefaultScene::SampleLight's uniform
 * Distribution (default_scene.cpp:48-53, 77-86) */
void tracer_photon(const Scene& s, const std::vector<float>& cdf, float lpdf,
                   int min_d, int max_d, float cont, VpGrid& g,
                   std::vector<SppmPixel>& px, Rng& rng) {
  const int n = (int)s.lights.size();
  if (n == 0) return;
  const float u = rng.next();
  int j = 0;
  while (j < (int)cdf.size() && !(u <= cdf[j])) ++j; /* upper_bound, <= */
  const int idx = std::min(std::max(j - 1, 0), n - 1);
  const Emit e = sample_emit(s, s.lights[idx], rng);
  if (is_black(e.radiance) || e.pdf_dir == 0.f || e.pdf_pos == 0.f) return;
  V3 coef = e.radiance * std::fabs(dot(e.normal, e.dir)) /
            (lpdf * e.pdf_pos * e.pdf_dir);
  Ray ray = make_ray(e.pos, e.dir);
  for (int depth = 1; depth <= max_d; ++depth) {
    if (depth > min_d) {
      if (rng.next() > cont) return;
      coef = coef / cont;
    }
    Hit h = trace_closest(s.acc, ray, s.mode, true);
    if (h.prim < 0) return;
    HitInfo hi = complete_hit(s, ray, h);
    if (depth > 1) add_photon(s, g, px, hi.pos, coef, hi.wr);
    Bsdf f(s.mats[hi.mat], hi.ng, hi.ns);
    float a = rng.next(), b = rng.next(), c = rng.next();
    Sample bs = f.sample(hi.wr, mk(a, b, c));
    if (is_black(bs.f) || bs.pdf < 0.f) return;
    coef = coef * (bs.f / bs.pdf * std::fabs(dot(hi.ng, bs.dir)));
    ray = make_ray(eps_offset(hi, bs.dir), bs.dir);
  }
}

/* UpdatePixel (sppm.cpp:145-169) */
void update_pixel(float alpha, SppmPixel& p) {
  if (p.M > 0) {
    const float new_N = p.N + alpha * p.M;
    const float new_R = p.radius * std::sqrt(new_N / (p.N + p.M));
    const V3 phi = mk(p.phi[0], p.phi[1], p.phi[2]);
    p.tau = (p.tau + p.vp.thr * phi) * (new_R * new_R) / (p.radius * p.radius);
    p.N = new_N;
    p.radius = new_R;
    p.M = 0;
    p.phi[0] = p.phi[1] = p.phi[2] = 0.f;
  }
  p.vp.thr = mk(0, 0, 0);
  p.vp.valid = false;
}

/* ThinLensCamera::GenerateRay (thin_lens.cpp:62-83) */
inline void mat_vec(const float* M, const float v[4], float out[4]) {
  for (int row = 0; row < 4; ++row) {
    float o = 0.f;
    for (int pos = 0; pos < 4; ++pos) o += M[pos * 4 + row] * v[pos];
    out[row] = o;
  }
}
inline V3 xform_point(const float* M, V3 p) {
  float v[4] = {p.x, p.y, p.z, 1.f}, o[4];
  mat_vec(M, v, o);
  return mk(o[0], o[1], o[2]) / o[3];
}
inline V3 xform_vec(const float* M, V3 p) {
  float v[4] = {p.x, p.y, p.z, 0.f}, o[4];
  mat_vec(M, v, o);
  return mk(o[0], o[1], o[2]);
}
Ray camera_ray(const float* cam, float rx, float ry, float lx, float ly) {
  const float* r2c = cam;
  const float* c2w = cam + 16;
  float lens_r = cam[32], focal = cam[33];
  V3 cc = xform_point(r2c, mk(rx, ry, 1.f));
  V3 o = mk(0.f, 0.f, 0.f);
  V3 d = normalized(cc);
  if (lens_r > 0 && focal > 0) {
    float px, py;
    concentric(lx, ly, &px, &py);
    float lxp = px * lens_r, lyp = py * lens_r;
    float ft = focal / d.z;
    V3 focus = o + ft * d;
    o = mk(lxp, lyp, 0.f);
    d = normalized(focus - o);
  }
  return make_ray(xform_point(c2w, o), xform_vec(c2w, d));
}

}  // namespace

/* ----------------------------------------------------------------- API --- */
extern "C" {

void orc_morton(const float* tris, int64_t n, const float* world,
                uint32_t* codes) {
  MortonEnc enc(world_box(world));
  for (int64_t i = 0; i < n; ++i)
    codes[i] = enc.enc(box_center(tri_box(tris + 9 * i)));
}

int orc_ploc_build(const float* tris, int64_t n, const float* world,
                   int64_t search_radius, int radix_compat, float* node_bounds,
                   int64_t* node_count_first, int64_t* perm) {
  if (n < 1) return -1;
  std::vector<Node> nodes;
  std::vector<int64_t> p;
  if (!ploc_build(tris, n, world, search_radius, radix_compat != 0, nodes, p))
    return -2;
  for (int64_t i = 0; i < 2 * n - 1; ++i) {
    const Node& x = nodes[i];
    float* b = node_bounds + 6 * i;
    b[0] = x.b.lo.x; b[1] = x.b.lo.y; b[2] = x.b.lo.z;
    b[3] = x.b.hi.x; b[4] = x.b.hi.y; b[5] = x.b.hi.z;
    node_count_first[2 * i] = x.count;
    node_count_first[2 * i + 1] = x.first;
  }
  for (int64_t i = 0; i < n; ++i) perm[i] = p[i];
  return 0;
}

static std::vector<Node> unpack_nodes(const float* nb, const int64_t* ncf,
                                      int64_t n) {
  std::vector<Node> nodes(2 * n - 1);
  for (int64_t i = 0; i < 2 * n - 1; ++i) {
    const float* b = nb + 6 * i;
    nodes[i].b = Box{mk(b[0], b[1], b[2]), mk(b[3], b[4], b[5])};
    nodes[i].count = ncf[2 * i];
    nodes[i].first = ncf[2 * i + 1];
  }
  return nodes;
}

int orc_trace(const float* tris, int64_t n_tris, const float* node_bounds,
              const int64_t* node_count_first, const int64_t* perm,
              int use_bvh, const float* rays, int64_t n_rays, int any_hit,
              int tri_test_mode, float* out_t, int32_t* out_prim,
              float* out_u, float* out_v, int threads) {
  std::vector<Node> nodes;
  if (use_bvh) nodes = unpack_nodes(node_bounds, node_count_first, n_tris);
  Accel acc{tris, n_tris, use_bvh ? nodes.data() : nullptr, perm};
  parallel_rows(n_rays, threads, [&](int64_t i) {
    const float* q = rays + 8 * i;
    Ray r{mk(q[0], q[1], q[2]), mk(q[3], q[4], q[5]), q[6], q[7]};
    if (any_hit) {
      bool o = trace_any(acc, r, tri_test_mode, use_bvh != 0);
      out_prim[i] = o ? 1 : -1;
      out_t[i] = 0.f;
      out_u[i] = 0.f;
      out_v[i] = 0.f;
    } else {
      Hit h = trace_closest(acc, r, tri_test_mode, use_bvh != 0);
      out_t[i] = h.t;
      out_prim[i] = h.prim;
      out_u[i] = h.u;
      out_v[i] = h.v;
    }
  });
  return 0;
}

void orc_bsdf(const float* material, const float* ng, const float* ns,
              const float* wo, const float* wi, const float* sam, int op,
              float* out) {
  Mat m = load_mat(material);
  Bsdf f(m, ld3(ng), ld3(ns));
  for (int k = 0; k < 8; ++k) out[k] = 0.f;
  if (op == 0) {
    V3 v = f.eval(ld3(wi), ld3(wo));
    out[0] = v.x; out[1] = v.y; out[2] = v.z;
    out[3] = f.pdf(ld3(wi), ld3(wo));
    out[7] = 1.f;
  } else {
    Sample s = f.sample(ld3(wo), ld3(sam));
    out[0] = s.f.x; out[1] = s.f.y; out[2] = s.f.z;
    out[3] = s.pdf;
    out[4] = s.dir.x; out[5] = s.dir.y; out[6] = s.dir.z;
    out[7] = (s.valid ? 1.f : 0.f) + (s.valid && s.delta ? 2.f : 0.f);
  }
}

void orc_camera_rays(const float* camera, const float* raster, int64_t n,
                     float* rays) {
  for (int64_t i = 0; i < n; ++i) {
    const float* q = raster + 4 * i;
    Ray r = camera_ray(camera, q[0], q[1], q[2], q[3]);
    float* o = rays + 6 * i;
    o[0] = r.o.x; o[1] = r.o.y; o[2] = r.o.z;
    o[3] = r.d.x; o[4] = r.d.y; o[5] = r.d.z;
  }
}

float orc_rng(uint64_t seed, uint32_t pixel, uint32_t sample, uint32_t dim) {
  return key_float(path_key(seed, pixel, sample), dim);
}

struct OrcScene {
  std::vector<Node> nodes;
  std::vector<int64_t> perm;
  Scene s;
  double build_seconds = 0;
};

void* orc_scene_create(const float* tris, const float* corner_n,
                       const int32_t* tri_mat, const int32_t* tri_flags,
                       int64_t n_tris, const float* materials,
                       int32_t n_materials, const float* lights,
                       int32_t n_lights, const float* world,
                       int64_t search_radius, int radix_compat, int tri_test,
                       const float* emit_rad, const int32_t* emit_info,
                       int32_t n_emit) {
  if (n_tris < 1) return nullptr;
  auto* o = new OrcScene();
  auto t0 = std::chrono::steady_clock::now();
  if (!ploc_build(tris, n_tris, world, search_radius, radix_compat != 0,
                  o->nodes, o->perm)) {
    delete o;
    return nullptr;
  }
  o->build_seconds = std::chrono::duration<double>(
                         std::chrono::steady_clock::now() - t0)
                         .count();
  Scene& s = o->s;
  s.acc = Accel{tris, n_tris, o->nodes.data(), o->perm.data()};
  s.corner_n = corner_n;
  s.tri_mat = tri_mat;
  s.tri_flags = tri_flags;
  for (int i = 0; i < n_materials; ++i)
    s.mats.push_back(load_mat(materials + 16 * i));
  /* the emissive primitives' area lights come first (default_scene.cpp) */
  if (n_emit > 0) s.tri_light.assign(n_tris, -1);
  for (int e = 0; e < n_emit; ++e) {
    s.areas.push_back(make_area(tris, emit_rad + 3 * e, emit_info + 4 * e));
    s.lights.emplace_back((int)e, s.areas.back().rad);
    for (int t = 0; t < emit_info[4 * e + 1]; ++t)
      s.tri_light[emit_info[4 * e] + t] = e;
  }
  for (int i = 0; i < n_lights; ++i) {
    s.lights.emplace_back(lights + 12 * i);
    if (s.lights.back().type == ORC_LIGHT_ENV) s.env = (int)s.lights.size() - 1;
  }
  Box wb = world_box(world);
  s.world = wb;
  s.radius = length(wb.hi - box_center(wb));
  s.mode = tri_test;
  return o;
}

void orc_scene_destroy(void* h) { delete static_cast<OrcScene*>(h); }

double orc_scene_build_seconds(void* h) {
  return static_cast<OrcScene*>(h)->build_seconds;
}

int orc_scene_render(void* h, const float* camera, const double* params,
                     uint64_t seed, int64_t pixel_begin, int64_t pixel_end,
                     float* out_li, double* out_film, int threads) {
  const Scene& s = static_cast<OrcScene*>(h)->s;
  const int spp = (int)params[0];
  const int min_b = (int)params[1], max_b = (int)params[2];
  const float cont = (float)params[3];
  const bool use_mis = params[4] != 0;
  const int W = (int)camera[34], H = (int)camera[35];
  const int64_t npix = (int64_t)W * H;
  if (pixel_end > npix) pixel_end = npix;
  const int64_t count = pixel_end - pixel_begin;
  std::vector<double> src(count > 0 ? 3 * count : 0, 0.0);
  parallel_rows(
      count, threads,
      [&](int64_t k) {
        int64_t p = pixel_begin + k;
        int x = (int)(p % W), y = (int)(p / W);
        double acc[3] = {0, 0, 0};
        for (int smp = 0; smp < spp; ++smp) {
          Rng rng{path_key(seed, (uint32_t)p, (uint32_t)smp)};
          const float u = x + rng.next();
          const float v = y + rng.next();
          float l0 = rng.next(), l1 = rng.next();
          Ray ray = camera_ray(camera, u, v, l0, l1);
          V3 L = trace_path(s, ray, rng, min_b, max_b, cont, use_mis);
          if (out_li) {
            float* o = out_li + 3 * ((p - pixel_begin) * (int64_t)spp + smp);
            o[0] = L.x; o[1] = L.y; o[2] = L.z;
          }
          acc[0] += L.x; acc[1] += L.y; acc[2] += L.z;
        }
        src[3 * k] = acc[0];
        src[3 * k + 1] = acc[1];
        src[3 * k + 2] = acc[2];
      },
      1);
  if (out_film) {
    /* Tile::AddSample's 2x2 footprint with the clamping merge: a sample at
     * (x, y) lands on (x-1..x, y-1..y), row/column -1 folding into 0. */
    for (int64_t i = 0; i < 4 * npix; ++i) out_film[i] = 0.0;
    for (int64_t k = 0; k < count; ++k) {
      int64_t p = pixel_begin + k;
      int x = (int)(p % W), y = (int)(p / W);
      for (int dy = -1; dy <= 0; ++dy)
        for (int dx = -1; dx <= 0; ++dx) {
          int tx = std::max(0, x + dx), ty = std::max(0, y + dy);
          double* o = out_film + 4 * ((int64_t)ty * W + tx);
          o[0] += src[3 * k];
          o[1] += src[3 * k + 1];
          o[2] += src[3 * k + 2];
          o[3] += spp;
        }
    }
  }
  return 0;
}

/* SPPMRenderer::Render (sppm.cpp:180-296) with the counter sampler: the
 * camera pass reseeds every pixel each iteration (the same visible points
 * every iteration, as in the reference), photon i of iteration k draws from
 * path_key(photon_seed(seed), i, k).  Serial.  params[8]: iterations,
 * photons per iteration, forward_max_depth, photon_min_depth,
 * photon_max_depth, photon_cont_prob, init_radius (< 0: the world
 * diagonal / 1000), update_alpha.  out_rad [H][W][3]; out_film [H][W][4]
 * the footprint sums (weight 1 per pixel). */
int orc_scene_sppm(void* h, const float* camera, const double* params,
                   uint64_t seed, float* out_rad, double* out_film) {
  const Scene& s = static_cast<OrcScene*>(h)->s;
  const int iters = (int)params[0], photons = (int)params[1];
  const int fmd = (int)params[2], pmin = (int)params[3], pmax = (int)params[4];
  const float cont = (float)params[5], alpha = (float)params[7];
  const int W = (int)camera[34], H = (int)camera[35];
  Box world = s.world;
  float init_radius = (float)params[6];
  if (init_radius < 0) init_radius = length(world.hi - world.lo) / 1000.f;
  world.lo = world.lo - mk(init_radius, init_radius, init_radius);
  world.hi = world.hi + mk(init_radius, init_radius, init_radius);
  std::vector<SppmPixel> px((size_t)W * H);
  for (auto& p : px) p.radius = init_radius;
  /* the scene's light selector */
  const int nl = (int)s.lights.size();
  std::vector<float> table(nl, 1.f), cdf(nl + 1, 0.f);
  float lpdf = 0.f;
  if (nl) {
    float sum = 0.f;
    for (float t : table) sum += t;
    const float ratio = 1.f / sum;
    for (float& t : table) t *= ratio;
    const float inv = 1.f / float(nl);
    for (int i = 1; i <= nl; ++i) cdf[i] = cdf[i - 1] + table[i - 1] * inv;
    const float fi = cdf[nl];
    if (fi > 0.f)
      for (float& c : cdf) c /= fi;
    else
      for (int i = 0; i <= nl; ++i) cdf[i] = float(i) / float(nl);
    lpdf = table[0];
  }
  const uint64_t pseed = ajg_photon_seed(seed);
  float max_radius = init_radius;
  for (int it = 0; it < iters; ++it) {
    VpGrid g(world, 1.05f * max_radius);
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < W; ++x) {
        const int p = y * W + x;
        Rng rng{path_key(seed, (uint32_t)p, 0)};
        const float u = x + rng.next();
        const float v = y + rng.next();
        const float l0 = rng.next(), l1 = rng.next();
        Ray ray = camera_ray(camera, u, v, l0, l1);
        px[p].vp = tracer_vp(s, ray, rng, fmd, px[p].direct);
        if (px[p].vp.valid) g.add_vp(p, px[p].vp.pos, px[p].radius);
      }
    for (int i = 0; i < photons; ++i) {
      Rng rng{path_key(pseed, (uint32_t)i, (uint32_t)it)};
      tracer_photon(s, cdf, lpdf, pmin, pmax, cont, g, px, rng);
    }
    max_radius = 0.f;
    for (auto& p : px)
      if (p.vp.valid) max_radius = fmax_ref(max_radius, p.radius);
    if (max_radius == 0.f) max_radius = init_radius;
    for (auto& p : px)
      if (p.vp.valid) update_pixel(alpha, p);
  }
  /* ComputePixelRadiance (sppm.cpp:171-180) */
  const uint64_t photon_n = uint64_t(iters) * uint64_t(photons);
  std::vector<V3> rad(px.size());
  for (size_t i = 0; i < px.size(); ++i) {
    const V3 d = px[i].direct / float(iters);
    const float dem = photon_n * kPi * px[i].radius * px[i].radius;
    rad[i] = d + px[i].tau / dem;
    if (out_rad) {
      out_rad[3 * i] = rad[i].x;
      out_rad[3 * i + 1] = rad[i].y;
      out_rad[3 * i + 2] = rad[i].z;
    }
  }
  if (out_film) {
    for (int64_t i = 0; i < 4 * (int64_t)W * H; ++i) out_film[i] = 0.0;
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < W; ++x)
        for (int dy = -1; dy <= 0; ++dy)
          for (int dx = -1; dx <= 0; ++dx) {
            const int tx = std::max(0, x + dx), ty = std::max(0, y + dy);
            double* o = out_film + 4 * ((int64_t)ty * W + tx);
            const V3& r = rad[(size_t)y * W + x];
            o[0] += r.x;
            o[1] += r.y;
            o[2] += r.z;
            o[3] += 1.0;
          }
  }
  return 0;
}

int orc_render(const float* tris, const float* corner_n,
               const int32_t* tri_mat, const int32_t* tri_flags, int64_t n_tris,
               const float* materials, int32_t n_materials,
               const float* lights, int32_t n_lights, const float* world,
               const float* camera, const double* params, uint64_t seed,
               int64_t pixel_begin, int64_t pixel_end, float* out_li,
               double* out_film, int threads, const float* emit_rad,
               const int32_t* emit_info, int32_t n_emit) {
  void* h = orc_scene_create(tris, corner_n, tri_mat, tri_flags, n_tris,
                             materials, n_materials, lights, n_lights, world,
                             (int64_t)params[6], params[7] != 0,
                             (int)params[5], emit_rad, emit_info, n_emit);
  if (!h) return -2;
  int rc = orc_scene_render(h, camera, params, seed, pixel_begin, pixel_end,
                            out_li, out_film, threads);
  orc_scene_destroy(h);
  return rc;
}

}  // extern "C"
