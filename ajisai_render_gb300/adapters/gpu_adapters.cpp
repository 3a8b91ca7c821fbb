// Reference-side adapters around libajisai_gpu: the "pt_gpu" renderer and
// the "ploc_gpu" aggregate (declarations and conventions in
// gpu_adapters.h).  Compiled against the reference's headers, as a
// maintainer would add it next to factory/creator/renderer_creators.cpp and
// aggregate_creators.cpp.
#include "gpu_adapters.h"

#include <ajisai/core/film.h>
#include <ajisai/core/geometry/geometry.h>
#include <ajisai/core/intersection.h>
#include <ajisai/core/primitive/primitive.h>
#include <ajisai/core/ray.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <vector>

#include "ajisai_host.h"

namespace ajg_adapters {
namespace {

// The reference's convention for an unusable scene or device: report, then
// end the process.
[[noreturn]] void die(const std::string& what) {
  std::fprintf(stderr, "ajisai_gpu: %s\n", what.c_str());
  std::fflush(stderr);
  std::exit(1);
}

void check(int rc, ajg_ctx* ctx, const char* call) {
  if (rc != AJG_OK)
    die(std::string(call) + " failed (" + std::to_string(rc) + "): " +
        ajg_last_error(ctx));
}

class GpuPTRenderer : public aj::Renderer {
 public:
  GpuPTRenderer(const aj::PTRendererArgs& a, std::string file, int device,
                uint64_t seed)
      : args_(a), file_(std::move(file)), device_(device), seed_(seed) {}

  // The reference objects carry no geometry or matrices
  // (scene/scene.h:46-62, camera/camera.h:32-50), so the scene comes from
  // the scene file through ajisai_host's reader, which follows the same
  // creators; the film receives the footprint sums as one full-film tile.
  void Render(aj::Scene*, aj::Camera*, aj::Film* film, aj::Sampler*) override {
    char err[512] = {0};
    ajh_scene* hs = nullptr;
    if (ajh_load_scene(file_.c_str(), &hs, err, sizeof(err)) != 0)
      die(std::string("scene file: ") + err);
    ajh_scene_view v{};
    ajh_scene_view_get(hs, &v);
    ajg_ctx* ctx = nullptr;
    ajg_config cfg{};
    cfg.device = device_;
    check(ajg_create_context(&cfg, &ctx), ctx, "ajg_create_context");
    ajg_scene* scene = nullptr;
    check(ajg_scene_create_flat_ex(ctx, v.tris, v.corner_normals, v.tri_material,
                                   v.tri_flags, v.num_triangles, v.world,
                                   v.materials, v.num_materials, v.lights,
                                   v.num_lights, v.emitters, v.num_emitters,
                                   &v.opts, &scene),
          ctx, "ajg_scene_create_flat_ex");
    ajg_render_params p{};
    p.spp = (uint32_t)args_.spp;
    p.min_bounces = args_.min_bounces;
    p.max_bounces = args_.max_bounces;
    p.cont_prob = args_.cont_prob;
    p.use_mis = args_.use_mis ? 1u : 0u;
    p.seed = seed_;
    const auto dim = film->Dimension();
    if ((uint32_t)dim.x() != v.camera.width || (uint32_t)dim.y() != v.camera.height)
      die("the film and the scene file's camera differ in size");
    std::vector<float> rgbw(4ull * dim.x() * dim.y());
    check(ajg_render(scene, &v.camera, &p, rgbw.data()), ctx, "ajg_render");
    // rgbw holds the 2x2 box-footprint sums (row/column -1 folded into 0)
    aj::Tile tile{aj::Bounds2i{aj::Vector2i{0, 0}, dim}, nullptr};
    for (size_t i = 0; i < tile.pixels.size(); ++i) {
      tile.pixels[i].radiance =
          aj::Spectrum{rgbw[4 * i], rgbw[4 * i + 1], rgbw[4 * i + 2]};
      tile.pixels[i].weight = rgbw[4 * i + 3];
    }
    film->MergeTile(tile);
    ajg_scene_release(scene);
    ajg_destroy_context(ctx);
    ajh_scene_free(hs);
  }

 private:
  aj::PTRendererArgs args_;
  std::string file_;
  int device_;
  uint64_t seed_;
};

class GpuPLOCAggregate : public aj::Aggregate {
 public:
  GpuPLOCAggregate(size_t radius, int device) : radius_(radius), device_(device) {}
  ~GpuPLOCAggregate() override {
    if (scene_) ajg_scene_release(scene_);
    if (ctx_) ajg_destroy_context(ctx_);
  }

  void Build(const std::vector<aj::Rc<aj::Primitive>>& primitives) override {
    primitives_ = primitives;
    std::vector<float> tris;
    float world[6];
    GatherMeshViewTriangles(primitives_, &tris, &prim_, &id_, world);
    const uint64_t n = prim_.size();
    if (n == 0) return;  // nothing to intersect
    ajg_config cfg{};
    cfg.device = device_;
    check(ajg_create_context(&cfg, &ctx_), ctx_, "ajg_create_context");
    // geometry only: hits are completed on the host by the primitives
    std::vector<float> corner(tris.size(), 0.f);
    std::vector<int32_t> mat(n, 0), flags(n, 0);
    ajg_material m{};
    m.type = AJG_MAT_DIFFUSE;
    ajg_scene_opts opts{};
    opts.search_radius = (uint32_t)radius_;
    opts.tri_test = AJG_TRI_MOLLER_TRUMBORE;
    check(ajg_scene_create_flat(ctx_, tris.data(), corner.data(), mat.data(),
                                flags.data(), n, world, &m, 1, nullptr, 0,
                                &opts, &scene_),
          ctx_, "ajg_scene_create_flat");
    tris_ = std::move(tris);
  }

  bool Intersect(const aj::Ray& ray,
                 aj::PrimitiveIntersection* inct) const noexcept override {
    if (!scene_) return false;
    ajg_ray r = to_ray(ray);
    ajg_hit h{};
    if (ajg_trace_closest(scene_, &r, 1, &h) != AJG_OK || h.prim < 0) return false;
    // what Triangle::Intersect sets before PostIntersect
    const float* t = tris_.data() + 9 * (size_t)h.prim;
    const aj::Vector3f a{t[0], t[1], t[2]}, b{t[3], t[4], t[5]}, c{t[6], t[7], t[8]};
    inct->t = h.t;
    inct->geometry_normal = aj::cross(b - a, c - a).normalized();
    inct->uv = aj::Vector2f{h.u, h.v};
    prim_[h.prim]->PostIntersect(ray, inct, id_[h.prim]);
    return true;
  }

  bool Occlude(const aj::Ray& ray) const noexcept override {
    if (!scene_) return false;
    ajg_ray r = to_ray(ray);
    uint8_t occ = 0;
    return ajg_trace_any(scene_, &r, 1, &occ) == AJG_OK && occ != 0;
  }

 private:
  static ajg_ray to_ray(const aj::Ray& ray) {
    ajg_ray r{};
    for (int k = 0; k < 3; ++k) {
      r.o[k] = ray.o[k];
      r.d[k] = ray.d[k];
    }
    r.t_min = ray.t_min;
    r.t_max = ray.t_max;
    return r;
  }
  size_t radius_;
  int device_;
  ajg_ctx* ctx_ = nullptr;
  ajg_scene* scene_ = nullptr;
  std::vector<aj::Rc<aj::Primitive>> primitives_;
  std::vector<float> tris_;
  std::vector<const aj::Primitive*> prim_;
  std::vector<uint32_t> id_;
};

}  // namespace

void GatherMeshViewTriangles(const std::vector<aj::Rc<aj::Primitive>>& prims,
                             std::vector<float>* out_tris,
                             std::vector<const aj::Primitive*>* out_prim,
                             std::vector<uint32_t>* out_id, float world[6]) {
  out_tris->clear();
  out_prim->clear();
  out_id->clear();
  float lo[3], hi[3];
  for (int k = 0; k < 3; ++k) {
    lo[k] = std::numeric_limits<float>::max();
    hi[k] = std::numeric_limits<float>::lowest();
  }
  for (const auto& p : prims) {
    const aj::Bounds3f bb = p->AABB();
    for (int k = 0; k < 3; ++k) {
      lo[k] = bb.min()[k] < lo[k] ? bb.min()[k] : lo[k];
      hi[k] = hi[k] < bb.max()[k] ? bb.max()[k] : hi[k];
    }
    const aj::MeshView mv = p->AsGeometry()->GetMeshView();
    const char* ib = static_cast<const char*>(mv.index_buffer) + mv.index_offset;
    const char* pb = static_cast<const char*>(mv.position_buffer) + mv.position_offset;
    for (size_t i = 0; i < mv.index_size; ++i) {
      for (int k = 0; k < 3; ++k) {
        uint32_t idx;
        std::memcpy(&idx, ib + i * mv.index_stride + k * sizeof(uint32_t),
                    sizeof(idx));
        float v[3];
        std::memcpy(v, pb + (size_t)idx * mv.position_stride, sizeof(v));
        out_tris->insert(out_tris->end(), v, v + 3);
      }
      out_prim->push_back(p.get());
      out_id->push_back((uint32_t)i);
    }
  }
  for (int k = 0; k < 3; ++k) {
    world[k] = lo[k];
    world[3 + k] = hi[k];
  }
}

aj::Rc<aj::Renderer> CreateGpuPTRenderer(const aj::PTRendererArgs& args,
                                         const std::string& scene_file,
                                         int device, uint64_t seed) {
  return std::make_shared<GpuPTRenderer>(args, scene_file, device, seed);
}

aj::Rc<aj::Aggregate> CreateGpuPLOCAggregate(size_t search_radius, int device) {
  return std::make_shared<GpuPLOCAggregate>(search_radius, device);
}

}  // namespace ajg_adapters
