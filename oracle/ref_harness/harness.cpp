/*
 * Reference harness (TEST INFRASTRUCTURE ONLY).
 *
 * Drives the reference's own, unmodified PT-MIS / PLOC sources (compiled
 * where they lie by oracle/build.py) to produce golden vectors: PLOC trees,
 * ray hits, BSDF sample/eval/pdf values and per-sample radiance.  Scenes are
 * built through the reference's public Create* functions, as its YAML
 * factory would (factory/creator/*.cpp), because yaml-cpp is not available.
 * Triangle meshes use a harness geometry whose PostIntersect restates
 * MeshGeo's (core/geometry/mesh.cpp:183-204), since MeshGeo's constructor
 * needs Embree; it also records which triangle produced the final hit.
 *
 * Two reference classes keep the state the fixtures need in private members
 * (PLOCAggregate's tree, ThinLensCamera's matrices); their source files are
 * compiled into this translation unit with private access opened.
 */
#include <algorithm>
#include <array>
#include <atomic>
#include <cassert>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <execution>
#include <filesystem>
#include <functional>
#include <initializer_list>
#include <iostream>
#include <limits>
#include <map>
#include <memory>
#include <memory_resource>
#include <mutex>
#include <numeric>
#include <optional>
#include <queue>
#include <span>
#include <string>
#include <thread>
#include <tuple>
#include <type_traits>
#include <utility>
#include <variant>
#include <vector>

#include <ajisai/ajisai.h>
#include <ajisai/core/aggregate/aggregate.h>
#include <ajisai/core/bsdf/bsdf.h>
#include <ajisai/core/camera/camera.h>
#include <ajisai/core/film.h>
#include <ajisai/core/filter/filter.h>
#include <ajisai/core/geometry/geometry.h>
#include <ajisai/core/intersection.h>
#include <ajisai/core/light/env_light.h>
#include <ajisai/core/light/light.h>
#include <ajisai/core/material/material.h>
#include <ajisai/core/medium/medium.h>
#include <ajisai/core/primitive/primitive.h>
#include <ajisai/core/renderer/photon_mapping.h>
#include <ajisai/core/ray.h>
#include <ajisai/core/renderer/renderer.h>
#include <ajisai/core/sampler/sampler.h>
#include <ajisai/core/scene/scene.h>
#include <ajisai/core/texture2d/texture2d.h>
#include <ajisai/core/warp.h>
#include <ajisai/math/angle.h>
#include <ajisai/math/bounds.h>
#include <ajisai/math/matrix4.h>
#include <ajisai/math/spectrum.h>
#include <ajisai/utility/mem_arena.h>
#include <tbb/parallel_for.h>

#define private public
#define protected public
#include <ajisai/core/aggregate/ploc_aggregate.cpp>
#include <ajisai/core/camera/thin_lens.cpp>
#undef private
#undef protected

#include "../counter_rng.h"

using namespace aj;

namespace {

thread_local const void* g_last_geom = nullptr;
thread_local uint32_t g_last_id = 0;
thread_local float g_last_u = 0.f, g_last_v = 0.f;

/* Triangle mesh geometry for the harness.  PostIntersect follows MeshGeo
 * (mesh.cpp:183-204); when no vertex normals are given the shading normal is
 * the geometric one (as for Quad). */
class HarnessMesh : public Geometry {
 public:
  HarnessMesh(std::vector<Vector3f> p, std::vector<Vector3f> n,
              std::vector<uint32_t> idx)
      : p_(std::move(p)), n_(std::move(n)), idx_(std::move(idx)) {
    aabb_ = {Vector3f{std::numeric_limits<float>::max()},
             Vector3f{std::numeric_limits<float>::lowest()}};
    for (const auto& v : p_) {
      aabb_.min() = Min(aabb_.min(), v);
      aabb_.max() = Max(aabb_.max(), v);
    }
    /* MeshGeo's surface area (mesh.cpp:62-68) */
    surface_area_ = 0;
    for (size_t idx = 0; idx < idx_.size(); idx += 3) {
      int i = idx_[idx], j = idx_[idx + 1], k = idx_[idx + 2];
      auto e0 = p_[j] - p_[i];
      auto e1 = p_[k] - p_[i];
      surface_area_ += 0.5 * cross(e0, e1).length();
    }
  }
  bool Intersect(const Ray&, GeometryIntersection*) const noexcept override {
    return false;
  }
  void PostIntersect(const Ray& ray, GeometryIntersection* inct,
                     uint32_t id) const noexcept override {
    g_last_geom = this;
    g_last_id = id;
    g_last_u = inct->uv.x();
    g_last_v = inct->uv.y();
    int i = idx_[id * 3 + 0], j = idx_[id * 3 + 1], k = idx_[id * 3 + 2];
    inct->pos = ray.CalcPoint(inct->t);
    inct->geometry_normal = cross(p_[j] - p_[i], p_[k] - p_[i]).normalized();
    if (!n_.empty())
      inct->shading_normal = (1 - inct->uv.x() - inct->uv.y()) * n_[i] +
                             inct->uv.x() * n_[j] + inct->uv.y() * n_[k];
    else
      inct->shading_normal = inct->geometry_normal;
    inct->wr = -ray.d;
  }
  bool Occlude(const Ray&) const noexcept override { return false; }
  Bounds3f AABB() const noexcept override { return aabb_; }
  MeshView GetMeshView() const noexcept override {
    MeshView r{};
    r.position_buffer = p_.data();
    r.position_offset = 0;
    r.position_stride = sizeof(Vector3f);
    r.position_size = p_.size();
    r.index_buffer = idx_.data();
    r.index_offset = 0;
    r.index_stride = 3 * sizeof(uint32_t);
    r.index_size = idx_.size() / 3;
    return r;
  }
  /* MeshGeo::Sample / Pdf (mesh.cpp:251-297), restated: the triangle index
   * addresses the index buffer without the factor 3 */
  Intersection Sample(float* pdf, const Vector3f& sam) const noexcept override {
    Vector3f sam_new = sam;
    if (sam_new.x() + sam_new.y() > 1.f) {
      sam_new.x() = 1.f - sam_new.x();
      sam_new.y() = 1.f - sam_new.y();
    }
    Intersection inct;
    auto triangle_count = idx_.size() / 3;
    int idx = std::min(int(sam.z() * triangle_count), (int)triangle_count - 1);
    int i = idx_[idx], j = idx_[idx + 1], k = idx_[idx + 2];
    inct.pos = (1 - sam_new.x() - sam_new.y()) * p_[i] + sam_new.x() * p_[j] +
               sam_new.y() * p_[k];
    inct.geometry_normal = cross(p_[j] - p_[i], p_[k] - p_[i]).normalized();
    inct.shading_normal = inct.geometry_normal;
    *pdf = 1.f / surface_area_;
    return inct;
  }
  Intersection Sample(const Vector3f&, float* pdf,
                      const Vector3f& sam) const noexcept override {
    return Sample(pdf, sam);
  }
  float Pdf(const Vector3f&) const noexcept override {
    return 1.f / surface_area_;
  }
  float Pdf(const Vector3f&, const Vector3f& s) const noexcept override {
    return Pdf(s);
  }
  const std::vector<Vector3f>& normals() const { return n_; }
  const std::vector<uint32_t>& indices() const { return idx_; }

 private:
  std::vector<Vector3f> p_, n_;
  std::vector<uint32_t> idx_;
  Bounds3f aabb_;
  float surface_area_ = 0.f;
};

/* Counter sampler: the stand-in for RandomSampler keyed by
 * (seed, pixel = SetSeed's argument, sample, dimension). */
class CounterSampler : public Sampler {
 public:
  uint64_t seed = 0;
  uint32_t pixel = 0, sample = 0, dim = 0;
  uint64_t key = 0;
  void SetSeed(std::size_t s) override {
    pixel = (uint32_t)s;
    Begin(0);
  }
  void Begin(uint32_t smp) {
    sample = smp;
    dim = 0;
    key = ajg_path_key(seed, pixel, sample);
  }
  Rc<Sampler> Copy() const override { return RcNew<CounterSampler>(*this); }
  float Next1D() override { return ajg_key_float(key, dim++); }
  Vector2f Next2D() override { return {Next1D(), Next1D()}; }
  Vector3f Next3D() override { return {Next1D(), Next1D(), Next1D()}; }
};

Rc<Texture2D> constant(float v) { return CreateConstant2DTexture(Spectrum{v}); }
Rc<Texture2D> constant3(const float* v) {
  return CreateConstant2DTexture(Spectrum{v[0], v[1], v[2]});
}

Rc<Material> make_material(const float* m) {
  switch ((int)m[0]) {
    case 0: return CreateDiffuse(constant3(m + 1));
    case 2: return CreateMirror(constant3(m + 1));
    case 3: return CreateGlass(constant3(m + 1), constant3(m + 4), constant(m[7]));
    case 4:
      return CreateMetal(constant3(m + 1), constant3(m + 4), constant3(m + 7),
                         m[10], m[11]);
    case 5: return CreatePlastic(constant3(m + 1), m[4], m[5], m[6]);
    case 6: return CreateNull();
    default: break;
  }
  return CreateDisney(constant3(m + 1), constant(m[4]), constant(m[5]),
                      constant(m[6]), constant(m[7]), constant(m[8]),
                      constant(m[9]), constant(m[10]), constant(m[11]),
                      constant(m[12]), constant(m[13]));
}

struct HScene {
  std::vector<Rc<Primitive>> prims;
  std::vector<int> kind, two_sided;
  std::vector<Rc<Material>> mats;
  std::vector<Rc<Light>> lights;
  std::vector<const HarnessMesh*> meshes; /* per primitive, or null */
  std::vector<std::array<float, 12>> light_desc;
  Rc<Aggregate> agg;
  Rc<Scene> scene;
  Rc<Camera> camera;
  int width = 0, height = 0;
  PLOCAggregate* ploc() { return static_cast<PLOCAggregate*>(agg.get()); }
};

}  // namespace

// sppm.cpp's free functions (external linkage in the reference)
namespace aj {
sppm::VisiblePoint TracerVP(int forward_max_depth, const Scene* scene,
                            const Ray& r, Sampler* sampler,
                            Spectrum& direct_illum, MemoryArena& arena);
void TracerPhoton(int min_depth, int max_depth, float cont_prob,
                  sppm::VisiblePointSearcher& vp_searcher, const Scene* scene,
                  Sampler* sampler, MemoryArena& arena);
void UpdatePixel(float alpha, sppm::Pixel& pixel);
Spectrum ComputePixelRadiance(int iter_count, uint64_t photon_N,
                              const sppm::Pixel& pixel);
}  // namespace aj

extern "C" {

/* prims [np][8] int32: kind (0 quad, 1 cube, 2 mesh), two_sided, material,
 *   vertex offset, vertex count, index offset (in triangles), triangle
 *   count, has_normals.
 * prim_f [np][16]: quad a,b,c,d; cube transform as 16 row-major entries
 *   (the first 15 are read, as factory/creator/helper.h:86-91 does).
 * lights [nl][12]: type, rgb, direction (toward the light), angle (rad),
 *   scaler, rot (deg).
 * cam [12]: position, look_at, up, fov (deg), lens_radius, focal_distance.
 * emission [np][3]: per primitive radiance (0: not a light). */
void* ref_scene_create(const int32_t* prims, const float* prim_f, int32_t np,
                       const float* mesh_pos, const float* mesh_nrm,
                       const uint32_t* mesh_idx, const float* mats,
                       int32_t nm, const float* lights, int32_t nl,
                       const float* cam, int32_t width, int32_t height,
                       int64_t search_radius, const float* emission) {
  auto* s = new HScene();
  for (int i = 0; i < nm; ++i) s->mats.push_back(make_material(mats + 16 * i));
  MediumInterface med{};
  med.in = CreateVoidMedium();
  med.out = CreateVoidMedium();
  for (int i = 0; i < np; ++i) {
    const int32_t* p = prims + 8 * i;
    const float* f = prim_f + 16 * i;
    Rc<Geometry> g;
    const HarnessMesh* hm = nullptr;
    if (p[0] == 0) {
      g = CreateQuad(Vector3f{f[0], f[1], f[2]}, Vector3f{f[3], f[4], f[5]},
                     Vector3f{f[6], f[7], f[8]}, Vector3f{f[9], f[10], f[11]},
                     Vector2f{0.f, 0.f}, Vector2f{1.f, 0.f},
                     Vector2f{1.f, 1.f}, Vector2f{0.f, 1.f}, Matrix4f{});
    } else if (p[0] == 1) {
      Matrix4f m{};
      for (size_t k = 0; k != 15; ++k) m[k % 4][k / 4] = f[k];
      g = CreateCube(m);
    } else {
      std::vector<Vector3f> pos, nrm;
      for (int v = 0; v < p[4]; ++v) {
        const float* q = mesh_pos + 3 * (int64_t)(p[3] + v);
        pos.emplace_back(q[0], q[1], q[2]);
        if (p[7]) {
          const float* nn = mesh_nrm + 3 * (int64_t)(p[3] + v);
          nrm.emplace_back(nn[0], nn[1], nn[2]);
        }
      }
      std::vector<uint32_t> idx(mesh_idx + 3 * (int64_t)p[5],
                                mesh_idx + 3 * (int64_t)(p[5] + p[6]));
      auto m = RcNew<HarnessMesh>(std::move(pos), std::move(nrm),
                                  std::move(idx));
      hm = m.get();
      g = m;
    }
    if (p[1]) g = CreateTwoSided(g);
    const Spectrum e = emission ? Spectrum{emission[3 * i], emission[3 * i + 1],
                                           emission[3 * i + 2]}
                                : Spectrum{};
    s->prims.push_back(CreateGeometric(g, s->mats[p[2]], med, e, false, -1));
    s->kind.push_back(p[0]);
    s->two_sided.push_back(p[1]);
    s->meshes.push_back(hm);
  }
  for (int i = 0; i < nl; ++i) {
    const float* l = lights + 12 * i;
    std::array<float, 12> d{};
    for (int k = 0; k < 12; ++k) d[k] = l[k];
    if ((int)l[0] == 0) {
      s->lights.push_back(CreateDirectionalLight(
          Vector3f{l[4], l[5], l[6]}, Rad<float>(l[7]),
          Spectrum{l[1], l[2], l[3]}, -1));
      d[7] = std::cos(l[7]);
    } else {
      s->lights.push_back(CreateEnvLight(
          CreateConstant2DTexture(Spectrum{l[1], l[2], l[3]}), l[9], l[8]));
    }
    s->light_desc.push_back(d);
  }
  s->agg = CreatePLOCAggregate((size_t)search_radius);
  s->agg->Build(s->prims);
  SceneArgs args{s->prims, s->lights, s->agg};
  s->scene = CreateDefaultScene(args);
  s->width = width;
  s->height = height;
  if (cam) {
    auto fov = Deg<float>(cam[9]);
    s->camera = CreateThinLensCamera(
        CreateBoxFilter(0.5f, 0.5f),
        Vector2f{(float)width, (float)height},
        Vector3f{cam[0], cam[1], cam[2]}, Vector3f{cam[3], cam[4], cam[5]},
        Vector3f{cam[6], cam[7], cam[8]}, (float)Rad<float>(fov), cam[10],
        cam[11]);
  }
  return s;
}

void ref_scene_destroy(void* h) { delete static_cast<HScene*>(h); }

/* The scene's primitives (a std::vector<Rc<Primitive>>), for code that
 * drives the reference's interfaces with them (the adapters' tests). */
const void* ref_scene_primitives(void* h) {
  return &static_cast<HScene*>(h)->prims;
}

int64_t ref_scene_num_tris(void* h) {
  return (int64_t)static_cast<HScene*>(h)->ploc()->triangles_.size();
}

/* The scene as the PLOC aggregate gathered it, in the flat layout of
 * oracle/ajg_oracle.h. */
void ref_scene_dump(void* h, float* tris, float* corner_n, int32_t* tri_mat,
                    int32_t* tri_flags, float* world, float* camera,
                    float* lights_out, int32_t* mat_of_prim) {
  auto* s = static_cast<HScene*>(h);
  auto* pl = s->ploc();
  std::map<const Primitive*, int> pidx;
  for (size_t i = 0; i < s->prims.size(); ++i) pidx[s->prims[i].get()] = i;
  for (size_t t = 0; t < pl->triangles_.size(); ++t) {
    const auto& tr = pl->triangles_[t];
    const float v[9] = {tr.a[0], tr.a[1], tr.a[2], tr.b[0], tr.b[1],
                        tr.b[2], tr.c[0], tr.c[1], tr.c[2]};
    std::memcpy(tris + 9 * t, v, sizeof(v));
    int pi = pidx[tr.primitive];
    int flags = 0;
    if (s->two_sided[pi]) flags |= 1;
    if (s->kind[pi] == 1) flags |= 2;
    float cn[9] = {0};
    if (s->kind[pi] == 2 && !s->meshes[pi]->normals().empty()) {
      flags |= 4;
      const auto& idx = s->meshes[pi]->indices();
      const auto& nn = s->meshes[pi]->normals();
      for (int k = 0; k < 3; ++k) {
        const auto& n = nn[idx[tr.id * 3 + k]];
        cn[3 * k] = n[0];
        cn[3 * k + 1] = n[1];
        cn[3 * k + 2] = n[2];
      }
    }
    std::memcpy(corner_n + 9 * t, cn, sizeof(cn));
    tri_flags[t] = flags;
    tri_mat[t] = mat_of_prim ? mat_of_prim[pi] : 0;
  }
  Bounds3f wb = s->scene->WorldBound();
  for (int k = 0; k < 3; ++k) {
    world[k] = wb.min()[k];
    world[3 + k] = wb.max()[k];
  }
  if (camera && s->camera) {
    auto* c = static_cast<ThinLensCamera*>(s->camera.get());
    for (int col = 0; col < 4; ++col)
      for (int row = 0; row < 4; ++row) {
        camera[col * 4 + row] = c->raster2camera_[col][row];
        camera[16 + col * 4 + row] = c->camera2world_[col][row];
      }
    camera[32] = c->lens_radius_;
    camera[33] = c->focal_distance_;
    camera[34] = (float)s->width;
    camera[35] = (float)s->height;
  }
  if (lights_out)
    for (size_t i = 0; i < s->light_desc.size(); ++i)
      for (int k = 0; k < 12; ++k) lights_out[12 * i + k] = s->light_desc[i][k];
}

/* The reference's PLOC tree: nodes_ and primitive_indices_. */
void ref_scene_ploc(void* h, float* node_bounds, int64_t* node_count_first,
                    int64_t* perm) {
  auto* pl = static_cast<HScene*>(h)->ploc();
  const int64_t n = (int64_t)pl->triangles_.size();
  for (int64_t i = 0; i < 2 * n - 1; ++i) {
    const auto& nd = pl->nodes_[i];
    for (int k = 0; k < 3; ++k) {
      node_bounds[6 * i + k] = nd.bound.min()[k];
      node_bounds[6 * i + 3 + k] = nd.bound.max()[k];
    }
    node_count_first[2 * i] = (int64_t)nd.primitive_count;
    node_count_first[2 * i + 1] = (int64_t)nd.first_child_or_primitive;
  }
  for (int64_t i = 0; i < n; ++i) perm[i] = (int64_t)pl->primitive_indices_[i];
}

/* Scene::Intersect / Occlude on rays [n][8] (o, d, t_min, t_max, set
 * directly, without the Ray constructor's offset).  Closest hits report the
 * global triangle index (the aggregate's triangles_ order), t and the raw
 * barycentrics; only mesh primitives record the triangle. */
void ref_scene_trace(void* h, const float* rays, int64_t n, int any_hit,
                     float* out_t, int32_t* out_prim, float* out_u,
                     float* out_v) {
  auto* s = static_cast<HScene*>(h);
  auto* pl = s->ploc();
  std::map<std::pair<const void*, uint32_t>, int32_t> tri_index;
  for (size_t t = 0; t < pl->triangles_.size(); ++t) {
    const auto& tr = pl->triangles_[t];
    const Geometry* g = tr.primitive->AsGeometry();
    tri_index[{g, tr.id}] = (int32_t)t;
  }
  for (int64_t i = 0; i < n; ++i) {
    const float* q = rays + 8 * i;
    Ray r;
    r.o = Vector3f{q[0], q[1], q[2]};
    r.d = Vector3f{q[3], q[4], q[5]};
    r.t_min = q[6];
    r.t_max = q[7];
    if (any_hit) {
      out_prim[i] = s->scene->Occlude(r) ? 1 : -1;
      out_t[i] = out_u[i] = out_v[i] = 0.f;
      continue;
    }
    PrimitiveIntersection inct;
    g_last_geom = nullptr;
    bool hit = s->scene->Intersect(r, &inct);
    if (!hit) {
      out_prim[i] = -1;
      out_t[i] = std::numeric_limits<float>::infinity();
      out_u[i] = out_v[i] = 0.f;
      continue;
    }
    auto it = tri_index.find({g_last_geom, g_last_id});
    out_prim[i] = it == tri_index.end() ? -2 : it->second;
    out_t[i] = inct.t;
    out_u[i] = g_last_u;
    out_v[i] = g_last_v;
  }
}

/* One BSDF query through Material::Shade + BSDF::*All.  op 0: eval and
 * pdf; op 1: sample.  out[8]: f rgb, pdf, wi xyz, valid (1) + delta (2). */
void ref_bsdf(const float* mat, const float* ng, const float* ns,
              const float* wo, const float* wi, const float* sam, int op,
              float* out) {
  auto m = make_material(mat);
  MemoryArena arena;
  PrimitiveIntersection inct{};
  inct.geometry_normal = Vector3f{ng[0], ng[1], ng[2]};
  inct.shading_normal = Vector3f{ns[0], ns[1], ns[2]};
  inct.uv = Vector2f{0.f, 0.f};
  auto sp = m->Shade(inct, arena);
  for (int k = 0; k < 8; ++k) out[k] = 0.f;
  const Vector3f o{wo[0], wo[1], wo[2]};
  if (op == 0) {
    const Vector3f i{wi[0], wi[1], wi[2]};
    auto f = sp.bsdf->EvalAll(i, o, TransMode::Radiance);
    out[0] = f[0];
    out[1] = f[1];
    out[2] = f[2];
    out[3] = sp.bsdf->PdfAll(i, o);
    out[7] = 1.f;
  } else {
    auto r = sp.bsdf->SampleAll(o, TransMode::Radiance,
                                Vector3f{sam[0], sam[1], sam[2]});
    out[0] = r.f[0];
    out[1] = r.f[1];
    out[2] = r.f[2];
    out[3] = r.pdf;
    out[4] = r.dir[0];
    out[5] = r.dir[1];
    out[6] = r.dir[2];
    out[7] = (r.f.IsBlack() && r.pdf == 0.f && r.dir.max() <= 0.f &&
              r.dir.min() >= 0.f)
                 ? 0.f
                 : (r.is_delta ? 3.f : 1.f);
  }
}

/* TiledIntegrator::Render's per-pixel loop (pt.cpp:54-64) with the counter
 * sampler, calling the reference's own Li.  params[8]: spp, min_bounces,
 * max_bounces, cont_prob, use_mis.  out_li [W*H][spp][3]; out_film
 * [W*H][4] is Tile::AddSample accumulated over one full-image tile and
 * merged with Film::MergeTile's clamped indexing (film.h:119-129). */
int ref_scene_render(void* h, const double* params, uint64_t seed,
                     float* out_li, float* out_film) {
  auto* s = static_cast<HScene*>(h);
  PTRendererArgs a{(int)params[0], 16, (int)params[1], (int)params[2],
                   (float)params[3], params[4] != 0, 20};
  auto integ = std::dynamic_pointer_cast<Integrator>(CreatePTRenderer(a));
  if (!integ || !s->camera) return -1;
  const int W = s->width, H = s->height, spp = a.spp;
  auto film = s->camera->CreateFilm();
  auto tile = film->GetTile(Bounds2i{Vector2i{0, 0}, Vector2i{W, H}});
  MemoryArena arena;
  CounterSampler smp;
  smp.seed = seed;
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      smp.SetSeed(x + y * W);
      for (int k = 0; k < spp; ++k) {
        smp.Begin((uint32_t)k);
        const float u = x + smp.Next1D();
        const float v = y + smp.Next1D();
        auto ray = s->camera->GenerateRay(Vector2f{u, v}, smp.Next2D());
        auto li = integ->Li(ray, s->scene.get(), &smp, arena);
        float* o = out_li + 3 * (((int64_t)y * W + x) * spp + k);
        o[0] = li.value[0];
        o[1] = li.value[1];
        o[2] = li.value[2];
        tile.AddSample(Vector2i{x, y}, li.value, 1.f);
      }
    }
  for (int64_t i = 0; i < 4 * (int64_t)W * H; ++i) out_film[i] = 0.f;
  const auto lo = tile.bounds.min(), hi = tile.bounds.max();
  for (int y = lo.y(); y < hi.y(); ++y)
    for (int x = lo.x(); x < hi.x(); ++x) {
      auto pix = tile(Vector2i{x, y});
      int cx = std::clamp(x, 0, W - 1), cy = std::clamp(y, 0, H - 1);
      float* o = out_film + 4 * ((int64_t)cy * W + cx);
      o[0] += pix.radiance[0];
      o[1] += pix.radiance[1];
      o[2] += pix.radiance[2];
      o[3] += pix.weight;
    }
  return 0;
}

/* Per-sample radiance of a window [x0, x0+w) x [y0, y0+h) of the film, the
 * pixels keyed as in the full render (SetSeed(x + y * W)), so a window of a
 * large film gives exactly the full render's samples there without tracing
 * the rest.  out_li [h][w][spp][3]. */
int ref_scene_render_window(void* h, const double* params, uint64_t seed,
                            int x0, int y0, int w, int hh, float* out_li) {
  auto* s = static_cast<HScene*>(h);
  PTRendererArgs a{(int)params[0], 16, (int)params[1], (int)params[2],
                   (float)params[3], params[4] != 0, 20};
  auto integ = std::dynamic_pointer_cast<Integrator>(CreatePTRenderer(a));
  if (!integ || !s->camera) return -1;
  const int W = s->width, H = s->height, spp = a.spp;
  if (x0 < 0 || y0 < 0 || w < 0 || hh < 0 || x0 + w > W || y0 + hh > H) return -2;
  MemoryArena arena;
  CounterSampler smp;
  smp.seed = seed;
  for (int y = y0; y < y0 + hh; ++y)
    for (int x = x0; x < x0 + w; ++x) {
      smp.SetSeed(x + y * W);
      for (int k = 0; k < spp; ++k) {
        smp.Begin((uint32_t)k);
        const float u = x + smp.Next1D();
        const float v = y + smp.Next1D();
        auto ray = s->camera->GenerateRay(Vector2f{u, v}, smp.Next2D());
        auto li = integ->Li(ray, s->scene.get(), &smp, arena);
        float* o = out_li + 3 * (((int64_t)(y - y0) * w + (x - x0)) * spp + k);
        o[0] = li.value[0];
        o[1] = li.value[1];
        o[2] = li.value[2];
      }
      arena.Release();
    }
  return 0;
}

/* Camera rays straight from ThinLensCamera::GenerateRay, for the raygen
 * parity check: raster [n][4] (x, y, lens u, lens v) -> rays [n][6]. */
void ref_camera_rays(void* h, const float* raster, int64_t n, float* rays) {
  auto* s = static_cast<HScene*>(h);
  for (int64_t i = 0; i < n; ++i) {
    const float* q = raster + 4 * i;
    auto r = s->camera->GenerateRay(Vector2f{q[0], q[1]}, Vector2f{q[2], q[3]});
    for (int k = 0; k < 3; ++k) {
      rays[6 * i + k] = r.o[k];
      rays[6 * i + 3 + k] = r.d[k];
    }
  }
}

/* Material::Shade then BSDF::HasDiffuseComponent (SPPM's visible-point
 * rule, sppm.cpp:77). */
int ref_has_diffuse(const float* mat) {
  auto m = make_material(mat);
  MemoryArena arena;
  PrimitiveIntersection inct{};
  inct.geometry_normal = Vector3f{0.f, 0.f, 1.f};
  inct.shading_normal = Vector3f{0.f, 0.f, 1.f};
  auto sp = m->Shade(inct, arena);
  return sp.bsdf->HasDiffuseComponent() ? 1 : 0;
}

/* SPPMRenderer::Render (sppm.cpp:180-296) driven serially over the
 * reference's own TracerVP, TracerPhoton, VisiblePointSearcher, UpdatePixel
 * and ComputePixelRadiance, with the counter sampler: the camera pass
 * reseeds every pixel each iteration (SetSeed(x + y * W), as the reference
 * does, so every iteration sees the same visible points), and photon i of
 * iteration k draws from its own stream (ajg_path_key(ajg_photon_seed(seed),
 * i, k)) -- the reference hands every photon the render's one shared
 * sampler from all pool threads (sppm.cpp:275-279).
 * params[8]: iterations, photons per iteration, forward_max_depth,
 * photon_min_depth, photon_max_depth, photon_cont_prob, init_radius,
 * update_alpha.  out_rad [H][W][3]: ComputePixelRadiance; out_film
 * [H][W][4]: the one full-image tile merged as ref_scene_render does. */
int ref_sppm_render(void* h, const double* params, uint64_t seed,
                    float* out_rad, float* out_film) {
  auto* s = static_cast<HScene*>(h);
  if (!s->camera) return -1;
  const int iters = (int)params[0], photons = (int)params[1];
  const int fmd = (int)params[2], pmin = (int)params[3], pmax = (int)params[4];
  const float cont = (float)params[5], alpha = (float)params[7];
  const int W = s->width, H = s->height;
  const Scene* scene = s->scene.get();
  auto world = scene->WorldBound();
  float init_radius = (float)params[6];
  if (init_radius < 0)
    init_radius = (world.max() - world.min()).length() / 1000.f;
  world.min() -= Vector3f{init_radius};
  world.max() += Vector3f{init_radius};
  std::vector<sppm::Pixel> px((size_t)W * H);
  for (auto& p : px) p.radius = init_radius;
  float max_radius = init_radius;
  MemoryArena arena;
  for (int it = 0; it < iters; ++it) {
    const float side = 1.05f * max_radius;
    sppm::VisiblePointSearcher vps(world, side, 40960);
    arena.Release();
    for (int ty = 0; ty < (H + 63) / 64; ++ty)
      for (int tx = 0; tx < (W + 63) / 64; ++tx)
        for (int y = 64 * ty; y < std::min(H, 64 * ty + 64); ++y)
          for (int x = 64 * tx; x < std::min(W, 64 * tx + 64); ++x) {
            CounterSampler cs;
            cs.seed = seed;
            cs.SetSeed(x + y * W);
            const float u = x + cs.Next1D();
            const float v = y + cs.Next1D();
            auto ray = s->camera->GenerateRay(Vector2f{u, v}, cs.Next2D());
            sppm::Pixel& p = px[(size_t)y * W + x];
            p.vp = TracerVP(fmd, scene, ray, &cs, p.direct_illum, arena);
            if (p.vp.IsValid()) vps.AddVp(p, arena);
          }
    for (int i = 0; i < photons; ++i) {
      CounterSampler ps;
      ps.seed = ajg_photon_seed(seed);
      ps.pixel = (uint32_t)i;
      ps.Begin((uint32_t)it);
      TracerPhoton(pmin, pmax, cont, vps, scene, &ps, arena);
    }
    max_radius = 0.f;
    for (auto& p : px)
      if (p.vp.IsValid()) max_radius = std::max(max_radius, p.radius);
    if (max_radius == 0.f) max_radius = init_radius;
    for (auto& p : px)
      if (p.vp.IsValid()) UpdatePixel(alpha, p);
  }
  const uint64_t photon_count = uint64_t(iters) * uint64_t(photons);
  auto film = s->camera->CreateFilm();
  auto tile = film->GetTile(Bounds2i{Vector2i{0, 0}, Vector2i{W, H}});
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      const Spectrum r = ComputePixelRadiance(iters, photon_count,
                                              px[(size_t)y * W + x]);
      float* o = out_rad + 3 * ((int64_t)y * W + x);
      o[0] = r[0];
      o[1] = r[1];
      o[2] = r[2];
      tile.AddSample(Vector2i{x, y}, r, 1.f);
    }
  for (int64_t i = 0; i < 4 * (int64_t)W * H; ++i) out_film[i] = 0.f;
  const auto lo = tile.bounds.min(), hi = tile.bounds.max();
  for (int y = lo.y(); y < hi.y(); ++y)
    for (int x = lo.x(); x < hi.x(); ++x) {
      auto pix = tile(Vector2i{x, y});
      int cx = std::clamp(x, 0, W - 1), cy = std::clamp(y, 0, H - 1);
      float* o = out_film + 4 * ((int64_t)cy * W + cx);
      o[0] += pix.radiance[0];
      o[1] += pix.radiance[1];
      o[2] += pix.radiance[2];
      o[3] += pix.weight;
    }
  return 0;
}

}  // extern "C"
