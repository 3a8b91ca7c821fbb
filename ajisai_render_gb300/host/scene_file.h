// An Ajisai YAML scene file read into the C ABI's flat scene description,
// following the reference's factory (app/main.cpp:84-112,
// factory/creator/*.cpp) for the nodes the PT/PLOC path renders:
//   scene:    type default; primitives of type geometry with geometry quad,
//             cube, twosided, mesh (OBJ) and material diffuse or disney
//             (constant textures); lights directional and envmap (constant
//             texture); aggregate ploc (search_radius) -- native and embree
//             fall back to PLOC
//   camera:   thin_lens (resolution, position, look_at, up, fov,
//             lens_radius, focal_distance; box filter 0.5)
//   renderer: pt (or pt_gpu) with the PTRendererArgs keys and defaults
//   post_processors: save_to_img (filename [+ ext])
// Everything else on the reference's factory -- spheres (no triangles for
// the PLOC tree), emissive primitives, plastic/metal/mirror/glass, image
// textures, media, other filters and renderers -- is refused with a message
// naming the node.
#pragma once
#include <string>
#include <vector>

#include "../../include/ajisai_gpu.h"

namespace ajh {

struct SceneFile {
  // ajg_scene_create_flat_ex's arrays: triangles in MeshView order per
  // primitive, YAML order (ploc_aggregate.cpp:252-285)
  std::vector<float> tris;            // [n][9]
  std::vector<float> corner_normals;  // [n][9], meshes only
  std::vector<int32_t> tri_material;  // [n]
  std::vector<int32_t> tri_flags;     // [n] AJG_MESH_*
  float world[6];                     // Join of the primitives' bounds
  std::vector<ajg_material> materials;  // one per primitive
  std::vector<ajg_light> lights;        // YAML order
  std::vector<ajg_emitter> emitters;    // emissive primitives, YAML order
  ajg_scene_opts opts;
  ajg_camera camera;
  ajg_render_params params;
  ajg_sppm_params sppm;  // the sppm renderer's node
  bool is_sppm = false;
  std::string renderer;
  std::vector<std::string> outputs;  // files save_to_img would write
  std::vector<std::string> notes;    // fallbacks taken
};

// Throws std::runtime_error naming the file, node and reason.
SceneFile LoadSceneFile(const std::string& path);

// ThinLensCamera's two matrices (thin_lens.cpp:40-54), computed in double
// and rounded once, as the flat camera record.
ajg_camera ThinLensCamera(const float position[3], const float look_at[3],
                          const float up[3], float fov_deg, uint32_t width,
                          uint32_t height, float lens_radius,
                          float focal_distance);

}  // namespace ajh
