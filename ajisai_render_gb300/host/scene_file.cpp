#include "scene_file.h"

#include <cfloat>
#include <cmath>
#include <cstring>
#include <map>
#include <stdexcept>
#include <tuple>

#include "obj_lite.h"
#include "yaml_lite.h"

namespace ajh {
namespace {

[[noreturn]] void fail(const std::string& file, const Node& n,
                       const std::string& what) {
  throw std::runtime_error(file + ":" + std::to_string(n.line) + ": " + what);
}

// ---- float math in the reference's operation order (math/vector.h,
// math/matrix4.h): dot products accumulate from 0, normalized is
// v * (1 / length), a matrix-vector product sums the columns in order.
struct V3 {
  float x, y, z;
};
V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
float dot(V3 a, V3 b) {
  float r = 0.f;
  r += a.x * b.x;
  r += a.y * b.y;
  r += a.z * b.z;
  return r;
}
V3 cross(V3 a, V3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z,
          a.x * b.y - a.y * b.x};
}
V3 normalized(V3 v) { return v * (1.f / std::sqrt(dot(v, v))); }

struct M4 {  // m[col][row], column-major like Matrix4f
  float m[4][4];
};
M4 identity() {
  M4 r{};
  for (int i = 0; i < 4; ++i) r.m[i][i] = 1.f;
  return r;
}
M4 mul(const M4& a, const M4& b) {
  M4 r{};
  for (int col = 0; col < 4; ++col)
    for (int row = 0; row < 4; ++row) {
      float acc = 0.f;
      for (int k = 0; k < 4; ++k) acc += a.m[k][row] * b.m[col][k];
      r.m[col][row] = acc;
    }
  return r;
}
void mat_vec(const M4& a, const float v[4], float out[4]) {
  for (int row = 0; row < 4; ++row) {
    float acc = 0.f;
    for (int pos = 0; pos < 4; ++pos) acc = acc + a.m[pos][row] * v[pos];
    out[row] = acc;
  }
}
V3 transform_point(const M4& a, V3 p) {  // matrix4.h:115-118
  const float h[4] = {p.x, p.y, p.z, 1.f};
  float o[4];
  mat_vec(a, h, o);
  return {o[0] / o[3], o[1] / o[3], o[2] / o[3]};
}
V3 transform_vector(const M4& a, V3 v) {  // matrix4.h:119-122
  const float h[4] = {v.x, v.y, v.z, 0.f};
  float o[4];
  mat_vec(a, h, o);
  return {o[0], o[1], o[2]};
}

// helper.h:83-130: {type: matrix, matrix: [16 row-major numbers]} (the
// decoder reads the first 15), or a sequence of them multiplied in order.
M4 get_transform(const std::string& file, const Node& n) {
  if (!n.IsDefined()) return identity();
  if (n.IsSequence()) {
    M4 r = identity();
    for (size_t i = 0; i < n.size(); ++i)
      r = mul(r, get_transform(file, n[i]));
    return r;
  }
  const std::string type = n["type"].AsString("");
  if (type != "matrix" || !n["matrix"].IsDefined())
    fail(file, n, "transform: expected {type: matrix, matrix: [16 numbers]}");
  const std::vector<float> v = n["matrix"].AsFloats(16);
  M4 r = identity();
  for (size_t i = 0; i < 15; ++i) r.m[i % 4][i / 4] = v[i];
  return r;
}

V3 vec3(const std::string& file, const Node& n) {
  const std::vector<float> v = n.AsFloats(3);
  (void)file;
  return {v[0], v[1], v[2]};
}

// A constant texture (texture2d_creators.cpp:34-45): texel as a vector or
// a scalar.
V3 constant_texel(const std::string& file, const Node& n,
                  const std::string& what) {
  if (!n.IsDefined()) fail(file, n, what + ": missing texture");
  const std::string type = n["type"].AsString("");
  if (type != "constant")
    fail(file, n, what + ": only constant textures are supported (got '" +
                      type + "')");
  const Node& t = n["texel"];
  if (t.IsSequence()) return vec3(file, t);
  const float s = t.AsFloat();
  return {s, s, s};
}

struct Bounds {
  V3 lo, hi;
};
bool is_point(const Bounds& b) {
  return b.lo.x == b.hi.x && b.lo.y == b.hi.y && b.lo.z == b.hi.z;
}
// Bounds::Join (math/bounds.h:108-113): a point box is absorbed.
Bounds join(const Bounds& a, const Bounds& b) {
  if (is_point(a)) return b;
  if (is_point(b)) return a;
  return {{std::fmin(a.lo.x, b.lo.x), std::fmin(a.lo.y, b.lo.y),
           std::fmin(a.lo.z, b.lo.z)},
          {std::fmax(a.hi.x, b.hi.x), std::fmax(a.hi.y, b.hi.y),
           std::fmax(a.hi.z, b.hi.z)}};
}
Bounds bounds_of(const std::vector<V3>& pts) {
  Bounds b{{FLT_MAX, FLT_MAX, FLT_MAX}, {-FLT_MAX, -FLT_MAX, -FLT_MAX}};
  for (const V3& p : pts) {
    b.lo = {std::fmin(b.lo.x, p.x), std::fmin(b.lo.y, p.y),
            std::fmin(b.lo.z, p.z)};
    b.hi = {std::fmax(b.hi.x, p.x), std::fmax(b.hi.y, p.y),
            std::fmax(b.hi.z, p.z)};
  }
  return b;
}

// Triangles of one geometry in MeshView order.
struct Geo {
  std::vector<V3> tri;     // 3 per triangle
  std::vector<V3> corner;  // 3 per triangle (meshes)
  int flags = 0;
  uint32_t kind = AJG_GEOM_MESH;  // how an AreaLight samples it
  Bounds bounds;
};

// Corner table of the unit cube, face by face (core/geometry/cube.cpp:36-61).
const float kCube[6][4][3] = {
    {{-.5f, -.5f, -.5f}, {-.5f, -.5f, .5f}, {.5f, -.5f, .5f}, {.5f, -.5f, -.5f}},
    {{-.5f, .5f, .5f}, {-.5f, .5f, -.5f}, {.5f, .5f, -.5f}, {.5f, .5f, .5f}},
    {{-.5f, .5f, -.5f}, {-.5f, -.5f, -.5f}, {.5f, -.5f, -.5f}, {.5f, .5f, -.5f}},
    {{.5f, .5f, .5f}, {.5f, -.5f, .5f}, {-.5f, -.5f, .5f}, {-.5f, .5f, .5f}},
    {{-.5f, .5f, .5f}, {-.5f, -.5f, .5f}, {-.5f, -.5f, -.5f}, {-.5f, .5f, -.5f}},
    {{.5f, .5f, -.5f}, {.5f, -.5f, -.5f}, {.5f, -.5f, .5f}, {.5f, .5f, .5f}},
};

std::string dir_of(const std::string& path) {
  const size_t s = path.find_last_of('/');
  return s == std::string::npos ? std::string() : path.substr(0, s + 1);
}

bool file_exists(const std::string& p) {
  FILE* f = std::fopen(p.c_str(), "rb");
  if (f) std::fclose(f);
  return f != nullptr;
}

// geometry_creators.cpp:102-241: vertices deduplicated by their
// (position, normal, texcoord) index triple in order of first use;
// positions through transformPoint; normals from the file, or -- when the
// file has none -- the normal of the first face that uses the vertex
// (from the untransformed positions), then transformVector + normalized.
Geo load_mesh(const std::string& file, const Node& n, const M4& xf,
              const std::string& scene_dir) {
  std::string fname = n["filename"].AsString();
  if (!file_exists(fname) && !scene_dir.empty() &&
      file_exists(scene_dir + fname))
    fname = scene_dir + fname;
  ObjData obj = LoadObj(fname);
  const bool file_normals = !obj.normals.empty();
  std::map<std::tuple<int, int, int>, uint32_t> index_of;
  std::vector<V3> pos, nrm;
  std::vector<uint32_t> idx;
  for (size_t i = 0; i < obj.corners.size(); ++i) {
    const ObjIndex c = obj.corners[i];
    const auto key = std::make_tuple(c.v, c.n, c.t);
    auto it = index_of.find(key);
    if (it != index_of.end()) {
      idx.push_back(it->second);
      continue;
    }
    const float* pv = &obj.positions[3 * (size_t)c.v];
    pos.push_back(transform_point(xf, {pv[0], pv[1], pv[2]}));
    V3 normal;
    if (file_normals && c.n >= 0) {
      const float* pn = &obj.normals[3 * (size_t)c.n];
      normal = {pn[0], pn[1], pn[2]};
    } else {
      const size_t f = (i / 3) * 3;
      V3 p[3];
      for (int k = 0; k < 3; ++k) {
        const float* q = &obj.positions[3 * (size_t)obj.corners[f + k].v];
        p[k] = {q[0], q[1], q[2]};
      }
      normal = normalized(cross(p[1] - p[0], p[2] - p[0]));
    }
    nrm.push_back(normalized(transform_vector(xf, normal)));
    const uint32_t id = (uint32_t)pos.size() - 1;
    index_of[key] = id;
    idx.push_back(id);
  }
  Geo g;
  g.flags = AJG_MESH_HAS_NORMALS;
  for (size_t i = 0; i < idx.size(); ++i) {
    g.tri.push_back(pos[idx[i]]);
    g.corner.push_back(nrm[idx[i]]);
  }
  g.bounds = bounds_of(pos);
  return g;
}

Geo load_geometry(const std::string& file, const Node& n,
                  const std::string& scene_dir) {
  const std::string type = n["type"].AsString("");
  Geo g;
  if (type == "quad") {  // geometry_creators.cpp:31-58, quad.cpp:36-50
    const M4 xf = get_transform(file, n["transform"]);
    auto corner = [&](const char* k, V3 def) {
      return n[k].IsDefined() ? vec3(file, n[k]) : def;
    };
    const V3 a = transform_point(xf, corner("a", {-1.f, -1.f, 0.f}));
    const V3 b = transform_point(xf, corner("b", {1.f, -1.f, 0.f}));
    const V3 c = transform_point(xf, corner("c", {1.f, 1.f, 0.f}));
    const V3 d = transform_point(xf, corner("d", {-1.f, 1.f, 0.f}));
    g.tri = {a, b, c, a, c, d};
    g.kind = AJG_GEOM_QUAD;
    g.bounds = bounds_of(g.tri);
  } else if (type == "cube") {  // cube.cpp:35-76
    const M4 xf = get_transform(file, n["transform"]);
    V3 pos[24];
    for (int f = 0; f < 6; ++f)
      for (int k = 0; k < 4; ++k)
        pos[4 * f + k] = transform_point(
            xf, {kCube[f][k][0], kCube[f][k][1], kCube[f][k][2]});
    for (int f = 0; f < 6; ++f) {
      const int i = 4 * f;
      // index tuples (i, i+2, i+1) and (i, i+3, i+2); libstdc++ keeps a
      // tuple's members in reverse, so the MeshView sees them reversed
      g.tri.insert(g.tri.end(), {pos[i + 1], pos[i + 2], pos[i]});
      g.tri.insert(g.tri.end(), {pos[i + 2], pos[i + 3], pos[i]});
    }
    g.flags = AJG_MESH_NG_REVERSED;
    g.kind = AJG_GEOM_CUBE;
    g.bounds = bounds_of(g.tri);
  } else if (type == "twosided") {  // two_sided.cpp
    g = load_geometry(file, n["internal"], scene_dir);
    g.flags |= AJG_MESH_TWO_SIDED;
  } else if (type == "mesh") {
    g = load_mesh(file, n, get_transform(file, n["transform"]), scene_dir);
  } else if (type == "sphere") {
    fail(file, n,
         "sphere: an analytic sphere has no triangles for the PLOC tree "
         "(the reference's PLOC aggregate leaves it out); use a mesh");
  } else {
    fail(file, n, "unknown geometry type '" + type + "'");
  }
  return g;
}

ajg_material load_material(const std::string& file, const Node& n) {
  ajg_material m;
  std::memset(&m, 0, sizeof(m));
  // no material node: CreateNull (primitive_creators.cpp:54-59)
  if (!n.IsDefined()) {
    m.type = AJG_MAT_NULL;
    return m;
  }
  const std::string type = n["type"].AsString("");
  auto color = [&](const char* key, float* out) {
    const V3 c = constant_texel(file, n[key], type + "." + key);
    out[0] = c.x;
    out[1] = c.y;
    out[2] = c.z;
  };
  if (type == "diffuse") {  // material_creators.cpp:28-39
    const V3 a = constant_texel(file, n["albedo"], "diffuse.albedo");
    m.type = AJG_MAT_DIFFUSE;
    m.base_color[0] = a.x;
    m.base_color[1] = a.y;
    m.base_color[2] = a.z;
  } else if (type == "disney") {  // material_creators.cpp:85-110
    const V3 bc = constant_texel(file, n["base_color"], "disney.base_color");
    m.type = AJG_MAT_DISNEY;
    m.base_color[0] = bc.x;
    m.base_color[1] = bc.y;
    m.base_color[2] = bc.z;
    // scalar parameters read SampleReal: the texel's first component
    auto real = [&](const char* k) {
      return constant_texel(file, n[k], std::string("disney.") + k).x;
    };
    m.subsurface = real("subsurface");
    m.metallic = real("metallic");
    m.specular = real("specular");
    m.specular_tint = real("specular_tint");
    m.roughness = real("roughness");
    m.anisotropic = real("anisotropic");
    m.sheen = real("sheen");
    m.sheen_tint = real("sheen_tint");
    m.clearcoat = real("clearcoat");
    m.clearcoat_gloss = real("clearcoat_gloss");
  } else if (type == "mirror") {  // material_creators.cpp:70-79
    m.type = AJG_MAT_MIRROR;
    color("kr", m.base_color);
  } else if (type == "glass") {  // material_creators.cpp:128-152
    m.type = AJG_MAT_GLASS;
    // absent colours are constant 1 textures
    if (n["color_reflection"].IsDefined())
      color("color_reflection", m.base_color);
    else
      m.base_color[0] = m.base_color[1] = m.base_color[2] = 1.f;
    if (n["color_refraction"].IsDefined())
      color("color_refraction", m.params);
    else
      m.params[0] = m.params[1] = m.params[2] = 1.f;
    // the ior texture is read with SampleReal: its first component
    m.params[3] = constant_texel(file, n["ior"], "glass.ior").x;
  } else if (type == "metal") {  // material_creators.cpp:54-68
    m.type = AJG_MAT_METAL;
    color("color", m.base_color);
    color("k", m.params);
    color("eta", m.params + 3);
    m.params[6] = n["uroughness"].AsFloat(0.1f);
    m.params[7] = n["vroughness"].AsFloat(0.1f);
  } else if (type == "plastic") {  // material_creators.cpp:40-52
    m.type = AJG_MAT_PLASTIC;
    color("albedo", m.base_color);
    m.params[0] = n["ior"].AsFloat(1.5f);
    m.params[1] = n["thickness"].AsFloat(1.f);
    m.params[2] = n["sigma_a"].AsFloat(0.f);
  } else {
    fail(file, n, "unknown material type '" + type + "'");
  }
  return m;
}

ajg_light load_light(const std::string& file, const Node& n) {
  ajg_light l;
  std::memset(&l, 0, sizeof(l));
  const std::string type = n["type"].AsString("");
  if (type == "directional") {  // light_creators.cpp:28-41
    const V3 dir = vec3(file, n["direction"]);
    const V3 e = vec3(file, n["emission"]);
    // Deg -> Rad in float, cos as the light's constructor takes it
    const float rad = n["angle"].AsFloat(0.f) * 3.141592654f / 180.f;
    l.type = AJG_LIGHT_DIRECTIONAL;
    l.rgb[0] = e.x;
    l.rgb[1] = e.y;
    l.rgb[2] = e.z;
    l.direction[0] = dir.x;
    l.direction[1] = dir.y;
    l.direction[2] = dir.z;
    l.cos_angle = std::cos(rad);
    l.scaler = 1.f;
  } else if (type == "envmap") {  // light_creators.cpp:43-54
    const V3 t = constant_texel(file, n["texture"], "envmap.texture");
    l.type = AJG_LIGHT_ENV;
    l.rgb[0] = t.x;
    l.rgb[1] = t.y;
    l.rgb[2] = t.z;
    l.direction[1] = 1.f;
    l.cos_angle = 1.f;
    l.scaler = n["scaler"].AsFloat(1.f);
    l.rot_deg = n["rot"].AsFloat(0.f);
  } else {
    fail(file, n, "unknown light type '" + type + "'");
  }
  return l;
}

}  // namespace

ajg_camera ThinLensCamera(const float position[3], const float look_at[3],
                          const float up[3], float fov_deg, uint32_t width,
                          uint32_t height, float lens_radius,
                          float focal_distance) {
  // Matrix4::lookAt, perspectiveProjection, the screen-to-raster scaling
  // (thin_lens.cpp:40-54, matrix4.h), in double, rounded once
  double eye[3], tgt[3], upv[3];
  for (int i = 0; i < 3; ++i) {
    eye[i] = position[i];
    tgt[i] = look_at[i];
    upv[i] = up[i];
  }
  auto norm = [](double v[3]) {
    const double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int i = 0; i < 3; ++i) v[i] /= l;
  };
  auto crs = [](const double a[3], const double b[3], double o[3]) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
  };
  double back[3] = {eye[0] - tgt[0], eye[1] - tgt[1], eye[2] - tgt[2]};
  norm(back);
  double right[3], rup[3];
  crs(upv, back, right);
  norm(right);
  crs(back, right, rup);
  norm(rup);
  const double W = width, H = height, near = 1.0, far = 1000.0;
  const double fov = (double)(fov_deg * 3.141592654f / 180.f);
  const double aspect = W / H;
  const double sx = 2.0 * near * std::tan(fov * 0.5) * aspect;
  const double sy = 2.0 * near * std::tan(fov * 0.5);
  const double xs = 2 * near / sx, ys = 2 * near / sy * -1.0;
  const double zs = 1.0 / (far - near);
  // raster -> screen: inverse of diag(W,H,1,1) diag(.5,-.5,1,1) T(1,-1,0)
  // screen -> camera: inverse of the projection
  // r2c = P^-1 S^-1, written out for these matrices
  double s2r[4][4] = {{W * 0.5, 0, 0, W * 0.5},
                      {0, -H * 0.5, 0, H * 0.5},
                      {0, 0, 1, 0},
                      {0, 0, 0, 1}};
  double proj[4][4] = {{xs, 0, 0, 0},
                       {0, ys, 0, 0},
                       {0, 0, near * zs, near * zs * far},
                       {0, 0, -1, 0}};
  auto inv4 = [](double a[4][4], double out[4][4]) {
    double m[4][8];
    for (int r = 0; r < 4; ++r)
      for (int c = 0; c < 8; ++c)
        m[r][c] = c < 4 ? a[r][c] : (c - 4 == r ? 1.0 : 0.0);
    for (int c = 0; c < 4; ++c) {
      int piv = c;
      for (int r = c + 1; r < 4; ++r)
        if (std::fabs(m[r][c]) > std::fabs(m[piv][c])) piv = r;
      for (int k = 0; k < 8; ++k) std::swap(m[c][k], m[piv][k]);
      const double d = m[c][c];
      for (int k = 0; k < 8; ++k) m[c][k] /= d;
      for (int r = 0; r < 4; ++r) {
        if (r == c) continue;
        const double f = m[r][c];
        for (int k = 0; k < 8; ++k) m[r][k] -= f * m[c][k];
      }
    }
    for (int r = 0; r < 4; ++r)
      for (int c = 0; c < 4; ++c) out[r][c] = m[r][c + 4];
  };
  double ip[4][4], is[4][4], r2c[4][4];
  inv4(proj, ip);
  inv4(s2r, is);
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) {
      double acc = 0;
      for (int k = 0; k < 4; ++k) acc += ip[r][k] * is[k][c];
      r2c[r][c] = acc;
    }
  ajg_camera cam;
  std::memset(&cam, 0, sizeof(cam));
  const double c2w[4][4] = {{right[0], rup[0], back[0], eye[0]},
                            {right[1], rup[1], back[1], eye[1]},
                            {right[2], rup[2], back[2], eye[2]},
                            {0, 0, 0, 1}};
  for (int col = 0; col < 4; ++col)
    for (int row = 0; row < 4; ++row) {
      cam.raster2camera[col * 4 + row] = (float)r2c[row][col];
      cam.camera2world[col * 4 + row] = (float)c2w[row][col];
    }
  cam.lens_radius = lens_radius;
  cam.focal_distance = focal_distance;
  cam.width = width;
  cam.height = height;
  return cam;
}

SceneFile LoadSceneFile(const std::string& path) {
  const Node root = LoadYamlFile(path);
  const std::string dir = dir_of(path);
  SceneFile out;
  std::memset(out.world, 0, sizeof(out.world));
  std::memset(&out.opts, 0, sizeof(out.opts));
  std::memset(&out.params, 0, sizeof(out.params));
  std::memset(&out.sppm, 0, sizeof(out.sppm));

  // ---- scene
  const Node& scene = root["scene"];
  if (!scene.IsDefined()) fail(path, root, "no 'scene' node");
  const std::string stype = scene["type"].AsString("default");
  if (stype != "default") fail(path, scene, "unknown scene type '" + stype + "'");
  Bounds world{{FLT_MAX, FLT_MAX, FLT_MAX}, {-FLT_MAX, -FLT_MAX, -FLT_MAX}};
  const Node& prims = scene["primitives"];
  for (size_t i = 0; i < prims.size(); ++i) {
    const Node& p = prims[i];
    const std::string ptype = p["type"].AsString("");
    if (ptype != "geometry")
      fail(path, p, "unknown primitive type '" + ptype + "'");
    for (const char* med : {"med_in", "med_out"})
      if (p[med].IsDefined() && p[med]["type"].AsString("void") != "void")
        fail(path, p, "participating media are not on this path");
    const Geo g = load_geometry(path, p["geometry"], dir);
    // `emission` makes the primitive an area light (primitive_creators.cpp:
    // 65-72, geometric.cpp:41-44); a black one makes none
    if (p["emission"].IsDefined()) {
      const V3 e = vec3(path, p["emission"]);
      if (e.x != 0.f || e.y != 0.f || e.z != 0.f) {
        ajg_emitter em{};
        em.radiance[0] = e.x;
        em.radiance[1] = e.y;
        em.radiance[2] = e.z;
        em.first_triangle = (uint32_t)out.tri_material.size();
        em.num_triangles = (uint32_t)(g.tri.size() / 3);
        em.geometry = g.kind;
        em.two_sided = (g.flags & AJG_MESH_TWO_SIDED) ? 1u : 0u;
        out.emitters.push_back(em);
      }
    }
    const ajg_material m = load_material(path, p["material"]);
    const int32_t mat = (int32_t)out.materials.size();
    out.materials.push_back(m);
    const size_t ntri = g.tri.size() / 3;
    for (size_t t = 0; t < ntri; ++t) {
      for (int k = 0; k < 3; ++k) {
        const V3 v = g.tri[3 * t + k];
        out.tris.insert(out.tris.end(), {v.x, v.y, v.z});
        const V3 c = g.corner.empty() ? V3{0.f, 0.f, 0.f} : g.corner[3 * t + k];
        out.corner_normals.insert(out.corner_normals.end(), {c.x, c.y, c.z});
      }
      out.tri_material.push_back(mat);
      out.tri_flags.push_back(g.flags);
    }
    world = join(world, g.bounds);
  }
  if (out.tri_material.empty()) fail(path, scene, "the scene has no triangles");
  out.world[0] = world.lo.x;
  out.world[1] = world.lo.y;
  out.world[2] = world.lo.z;
  out.world[3] = world.hi.x;
  out.world[4] = world.hi.y;
  out.world[5] = world.hi.z;
  const Node& lights = scene["lights"];
  for (size_t i = 0; i < lights.size(); ++i)
    out.lights.push_back(load_light(path, lights[i]));
  out.opts.search_radius = 14;
  out.opts.tri_test = AJG_TRI_MOLLER_TRUMBORE;
  if (const Node& ag = scene["aggregate"]) {
    const std::string at = ag["type"].AsString("");
    if (at == "ploc") {
      out.opts.search_radius = (uint32_t)ag["search_radius"].AsInt(14);
    } else if (at == "native" || at == "embree") {
      out.notes.push_back("aggregate '" + at + "' rendered over a PLOC tree "
                          "(search radius 14)");
    } else {
      fail(path, ag, "unknown aggregate type '" + at + "'");
    }
  } else {
    out.notes.push_back("no aggregate node (the reference's native "
                        "aggregate): rendered over a PLOC tree");
  }

  // ---- camera (camera_creators.cpp:28-56)
  const Node& cn = root["camera"];
  if (!cn.IsDefined()) fail(path, root, "no 'camera' node");
  if (cn["type"].AsString("") != "thin_lens")
    fail(path, cn, "camera type must be thin_lens");
  if (const Node& f = cn["filter"]) {
    if (f["type"].AsString("") != "box" || f["xwidth"].AsFloat(0.5f) != 0.5f ||
        f["ywidth"].AsFloat(0.5f) != 0.5f)
      fail(path, f, "only the 0.5-wide box filter is on this path");
  }
  const std::vector<float> res = cn["resolution"].AsFloats(2);
  const V3 pos = vec3(path, cn["position"]);
  const V3 at = vec3(path, cn["look_at"]);
  const V3 upv = vec3(path, cn["up"]);
  const float p3[3] = {pos.x, pos.y, pos.z}, a3[3] = {at.x, at.y, at.z},
              u3[3] = {upv.x, upv.y, upv.z};
  out.camera = ThinLensCamera(p3, a3, u3, cn["fov"].AsFloat(), (uint32_t)res[0],
                              (uint32_t)res[1], cn["lens_radius"].AsFloat(0.f),
                              cn["focal_distance"].AsFloat(1.f));

  // ---- renderer (renderer_creators.cpp:27-52)
  const Node& rn = root["renderer"];
  if (!rn.IsDefined()) fail(path, root, "no 'renderer' node");
  out.renderer = rn["type"].AsString("");
  if (out.renderer == "sppm" || out.renderer == "sppm_gpu") {
    // SPPMCreatorImpl (renderer_creators.cpp:55-76)
    ajg_sppm_params& q = out.sppm;
    q.forward_max_depth = (int32_t)rn["forward_max_depth"].AsInt(8);
    q.init_radius = rn["init_radius"].AsFloat(0.1f);
    q.iterations = (uint32_t)rn["iteration_count"].AsInt(100);
    q.photons_per_iteration = (uint32_t)rn["photons_per_iteration"].AsInt(100000);
    q.photon_min_depth = (int32_t)rn["photon_min_depth"].AsInt(5);
    q.photon_max_depth = (int32_t)rn["photon_max_depth"].AsInt(10);
    q.photon_cont_prob = rn["photon_cont_prob"].AsFloat(0.9f);
    q.update_alpha = rn["update_alpha"].AsFloat(2.f / 3);
    q.seed = (uint64_t)rn["seed"].AsInt(0);
    out.is_sppm = true;
  } else if (out.renderer != "pt" && out.renderer != "pt_gpu") {
    fail(path, rn, "renderer '" + out.renderer + "' is not on this path (pt, "
                   "pt_gpu, sppm and sppm_gpu are)");
  }
  out.params.spp = out.is_sppm ? 1u : (uint32_t)rn["spp"].AsInt();
  out.params.min_bounces = (int32_t)rn["min_bounces"].AsInt(5);
  out.params.max_bounces = (int32_t)rn["max_bounces"].AsInt(10);
  out.params.cont_prob = rn["cont_prob"].AsFloat(0.9f);
  out.params.use_mis = rn["use_mis"].AsBool(true) ? 1u : 0u;
  out.params.seed = (uint64_t)rn["seed"].AsInt(0);

  // ---- post processors (post_processor_creators.cpp:28-50): the file is
  // filename + "." + ext (post_processor.cpp:36), ext from the node or the
  // filename's suffix
  const Node& pp = root["post_processors"];
  auto add_output = [&](const Node& p) {
    if (p["type"].AsString("") != "save_to_img")
      fail(path, p, "unknown post processor");
    const std::string fn = p["filename"].AsString();
    std::string ext;
    if (p["ext"].IsDefined()) {
      ext = p["ext"].AsString();
    } else if (fn.size() > 4 && fn.compare(fn.size() - 4, 4, ".png") == 0) {
      ext = "png";
    } else if (fn.size() > 4 && fn.compare(fn.size() - 4, 4, ".jpg") == 0) {
      ext = "jpg";
    } else {
      fail(path, p, "unknown image file format: " + fn);
    }
    out.outputs.push_back(fn + "." + ext);
  };
  if (pp.IsSequence()) {
    for (size_t i = 0; i < pp.size(); ++i) add_output(pp[i]);
  } else if (pp.IsMap()) {
    add_output(pp);
  }
  return out;
}

}  // namespace ajh
