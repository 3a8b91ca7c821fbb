// ajisai_gpu: the reference's command line (app/main.cpp: `-s scene.yaml`)
// over the GPU path: read the scene file, build the scene (PLOC on the
// GPU), render with the file's renderer (pt or sppm), run its save_to_img
// post processors.
//
//   ajisai_gpu -s scene.yaml [--device N] [--out image.pfm] [--spp N]
//              [--seed N]
//
// --out also writes the float image (PFM); --spp / --seed override the
// renderer node.  A save_to_img output with the .jpg extension is written
// as PNG beside it (no JPEG encoder here).
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "../../include/ajisai_gpu.h"
#include "image_out.h"
#include "scene_file.h"

namespace {

int usage(const char* argv0) {
  std::fprintf(stderr,
               "usage: %s -s scene.yaml [--device N] [--out image.pfm] "
               "[--spp N] [--seed N]\n",
               argv0);
  return 2;
}

int check(int rc, ajg_ctx* ctx, const char* what) {
  if (rc != AJG_OK)
    std::fprintf(stderr, "ajisai_gpu: %s: %s\n", what, ajg_last_error(ctx));
  return rc;
}

}  // namespace

int main(int argc, char** argv) {
  std::string scene_path, out_path;
  int device = 0;
  long spp = -1, seed = -1;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    auto next = [&]() -> const char* { return i + 1 < argc ? argv[++i] : nullptr; };
    const char* v = nullptr;
    if (a == "-s" || a == "--scene") {
      if (!(v = next())) return usage(argv[0]);
      scene_path = v;
    } else if (a == "--out") {
      if (!(v = next())) return usage(argv[0]);
      out_path = v;
    } else if (a == "--device") {
      if (!(v = next())) return usage(argv[0]);
      device = std::atoi(v);
    } else if (a == "--spp") {
      if (!(v = next())) return usage(argv[0]);
      spp = std::atol(v);
    } else if (a == "--seed") {
      if (!(v = next())) return usage(argv[0]);
      seed = std::atol(v);
    } else if (a == "-h" || a == "--help") {
      usage(argv[0]);
      return 0;
    } else {
      return usage(argv[0]);
    }
  }
  if (scene_path.empty()) {
    std::fprintf(stderr, "ajisai_gpu: scene file is unspecified\n");
    return usage(argv[0]);
  }
  ajh::SceneFile f;
  try {
    f = ajh::LoadSceneFile(scene_path);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "ajisai_gpu: %s\n", e.what());
    return 1;
  }
  for (const std::string& n : f.notes) std::fprintf(stderr, "note: %s\n", n.c_str());
  if (spp > 0) f.params.spp = (uint32_t)spp;
  if (seed >= 0) f.params.seed = f.sppm.seed = (uint64_t)seed;

  ajg_config cfg{device, 0, 0};
  ajg_ctx* ctx = nullptr;
  if (check(ajg_create_context(&cfg, &ctx), nullptr, "context")) return 1;
  ajg_scene* scene = nullptr;
  const auto t0 = std::chrono::steady_clock::now();
  int rc = ajg_scene_create_flat_ex(
      ctx, f.tris.data(), f.corner_normals.data(), f.tri_material.data(),
      f.tri_flags.data(), f.tri_material.size(), f.world, f.materials.data(),
      (uint32_t)f.materials.size(), f.lights.data(), (uint32_t)f.lights.size(),
      f.emitters.data(), (uint32_t)f.emitters.size(), &f.opts, &scene);
  if (check(rc, ctx, "scene")) {
    ajg_destroy_context(ctx);
    return 1;
  }
  const auto t1 = std::chrono::steady_clock::now();
  std::vector<float> rgbw(4ull * f.camera.width * f.camera.height);
  rc = f.is_sppm ? ajg_render_sppm(scene, &f.camera, &f.sppm, rgbw.data(), nullptr)
                 : ajg_render(scene, &f.camera, &f.params, rgbw.data());
  const auto t2 = std::chrono::steady_clock::now();
  int status = check(rc, ctx, "render") ? 1 : 0;
  if (!status) {
    const double build_s = std::chrono::duration<double>(t1 - t0).count();
    const double render_s = std::chrono::duration<double>(t2 - t1).count();
    if (f.is_sppm) {
      const double photons =
          (double)f.sppm.iterations * f.sppm.photons_per_iteration;
      std::printf("%zu triangles, %ux%u, sppm %u x %u photons: scene %.3f s, "
                  "render %.3f s (%.1f Mphotons/s)\n",
                  f.tri_material.size(), f.camera.width, f.camera.height,
                  f.sppm.iterations, f.sppm.photons_per_iteration, build_s,
                  render_s, photons / render_s / 1e6);
    } else {
      const double samples =
          (double)f.camera.width * f.camera.height * f.params.spp;
      std::printf("%zu triangles, %ux%u, %u spp: scene %.3f s, render %.3f s "
                  "(%.1f Msamples/s)\n",
                  f.tri_material.size(), f.camera.width, f.camera.height,
                  f.params.spp, build_s, render_s, samples / render_s / 1e6);
    }
    std::vector<std::string> files = f.outputs;
    for (std::string& o : files)
      if (o.size() > 4 && o.compare(o.size() - 4, 4, ".jpg") == 0)
        o += ".png";
    if (!out_path.empty()) files.push_back(out_path);
    for (const std::string& o : files) {
      try {
        ajh::WriteImage(o, rgbw.data(), f.camera.width, f.camera.height);
        std::printf("wrote %s\n", o.c_str());
      } catch (const std::exception& e) {
        std::fprintf(stderr, "ajisai_gpu: %s\n", e.what());
        status = 1;
      }
    }
  }
  ajg_scene_release(scene);
  ajg_destroy_context(ctx);
  return status;
}
