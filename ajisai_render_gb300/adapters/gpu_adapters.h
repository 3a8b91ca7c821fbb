// Reference-side adapters: what a maintainer adds to the reference
// (siyuanpan/ajisai_render) to render its PT path and answer its aggregate
// queries with libajisai_gpu.  They compile against the reference's own
// headers and link against libajisai_gpu (and libajisai_host for the scene
// file); nothing of the reference is compiled into the library.
//
//   "pt_gpu"   Renderer::Render (core/renderer/renderer.h:53-59) on the GPU,
//              the scene read from the YAML file the reference parsed
//   "ploc_gpu" Aggregate::Build / Intersect / Occlude
//              (core/aggregate/aggregate.h:32-42) over the GPU's PLOC tree
//
// Errors follow the reference's convention (a message, then exit(1), as its
// creators do on a bad scene, geometry_creators.cpp:118-123); the message
// carries ajg_last_error's text.
#pragma once

#include <ajisai/ajisai.h>
#include <ajisai/core/aggregate/aggregate.h>
#include <ajisai/core/renderer/renderer.h>

#include <string>

#include "ajisai_gpu.h"

namespace ajg_adapters {

// A renderer of type "pt_gpu" with the pt renderer's arguments
// (renderer_creators.cpp:33-39) and the scene file that holds the scene.
aj::Rc<aj::Renderer> CreateGpuPTRenderer(const aj::PTRendererArgs& args,
                                         const std::string& scene_file,
                                         int device = 0, uint64_t seed = 0);

// An aggregate of type "ploc_gpu": the PLOC tree built on the GPU with the
// given search radius; Intersect / Occlude trace one ray each on the GPU and
// complete the hit on the host with the primitive's PostIntersect, as
// PLOCAggregate's Triangle::Intersect does (ploc_aggregate.cpp:184-216).
aj::Rc<aj::Aggregate> CreateGpuPLOCAggregate(size_t search_radius, int device = 0);

// The triangles a PLOC aggregate gathers from primitives, in the order
// PLOCAggregate::Build gathers them (ploc_aggregate.cpp:252-285): each
// primitive's MeshView triangles in index order.  out_tris [n][9].
void GatherMeshViewTriangles(const std::vector<aj::Rc<aj::Primitive>>& prims,
                             std::vector<float>* out_tris,
                             std::vector<const aj::Primitive*>* out_prim,
                             std::vector<uint32_t>* out_id, float world[6]);

}  // namespace ajg_adapters
