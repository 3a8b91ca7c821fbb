// Wavefront OBJ reader for the "mesh" geometry (the reference reads it with
// tinyobjloader, factory/creator/geometry_creators.cpp:102-241): positions,
// normals and texture coordinates, faces "f v", "f v/t", "f v//n",
// "f v/t/n" with 1-based or negative (relative) indices, polygons split into
// a fan (0, i, i+1), every object / group in file order.  Materials (.mtl),
// lines and points are ignored.
#pragma once
#include <array>
#include <string>
#include <vector>

namespace ajh {

struct ObjIndex {
  int v, t, n;  // 0-based; -1 when absent
};

struct ObjData {
  std::vector<float> positions;  // [nv][3]
  std::vector<float> normals;    // [nn][3]
  std::vector<float> texcoords;  // [nt][2]
  std::vector<ObjIndex> corners;  // [ntri][3] face corners in file order
};

// Throws std::runtime_error (file name, line) on a malformed file.
ObjData LoadObj(const std::string& path);
ObjData ParseObj(const std::string& text, const std::string& name);

}  // namespace ajh
