#include "obj_lite.h"

#include <cstdlib>
#include <fstream>
#include <sstream>
#include <stdexcept>

namespace ajh {
namespace {

[[noreturn]] void fail(const std::string& name, int line,
                       const std::string& what) {
  throw std::runtime_error(name + ":" + std::to_string(line) + ": " + what);
}

bool read_floats(std::istringstream& in, float* out, int n) {
  for (int i = 0; i < n; ++i)
    if (!(in >> out[i])) return false;
  return true;
}

// Resolves a 1-based or negative (relative to the end) OBJ index.
int resolve(long v, size_t count, const std::string& name, int line) {
  long r = v > 0 ? v - 1 : (long)count + v;
  if (v == 0 || r < 0 || r >= (long)count) fail(name, line, "index out of range");
  return (int)r;
}

}  // namespace

ObjData ParseObj(const std::string& text, const std::string& name) {
  ObjData d;
  std::istringstream in(text);
  std::string raw;
  int no = 0;
  while (std::getline(in, raw)) {
    ++no;
    if (!raw.empty() && raw.back() == '\r') raw.pop_back();
    // a trailing backslash joins the next line
    while (!raw.empty() && raw.back() == '\\') {
      raw.pop_back();
      std::string next;
      if (!std::getline(in, next)) break;
      ++no;
      raw += " " + next;
    }
    const size_t hash = raw.find('#');
    if (hash != std::string::npos) raw.resize(hash);
    std::istringstream ls(raw);
    std::string tag;
    if (!(ls >> tag)) continue;
    if (tag == "v") {
      float p[3];
      if (!read_floats(ls, p, 3)) fail(name, no, "bad vertex");
      d.positions.insert(d.positions.end(), p, p + 3);
    } else if (tag == "vn") {
      float p[3];
      if (!read_floats(ls, p, 3)) fail(name, no, "bad normal");
      d.normals.insert(d.normals.end(), p, p + 3);
    } else if (tag == "vt") {
      float p[2] = {0.f, 0.f};
      if (!(ls >> p[0])) fail(name, no, "bad texture coordinate");
      ls >> p[1];
      d.texcoords.insert(d.texcoords.end(), p, p + 2);
    } else if (tag == "f") {
      std::vector<ObjIndex> poly;
      std::string tok;
      while (ls >> tok) {
        ObjIndex ix{-1, -1, -1};
        long parts[3] = {0, 0, 0};
        bool have[3] = {false, false, false};
        size_t a = 0;
        for (int k = 0; k < 3 && a <= tok.size(); ++k) {
          const size_t b = tok.find('/', a);
          const std::string f = tok.substr(a, b == std::string::npos ? b : b - a);
          if (!f.empty()) {
            char* end = nullptr;
            parts[k] = std::strtol(f.c_str(), &end, 10);
            if (*end != '\0') fail(name, no, "bad face index '" + tok + "'");
            have[k] = true;
          }
          if (b == std::string::npos) break;
          a = b + 1;
        }
        if (!have[0]) fail(name, no, "face corner without a vertex");
        ix.v = resolve(parts[0], d.positions.size() / 3, name, no);
        if (have[1]) ix.t = resolve(parts[1], d.texcoords.size() / 2, name, no);
        if (have[2]) ix.n = resolve(parts[2], d.normals.size() / 3, name, no);
        poly.push_back(ix);
      }
      if (poly.size() < 3) fail(name, no, "face with fewer than 3 corners");
      for (size_t i = 1; i + 1 < poly.size(); ++i) {
        d.corners.push_back(poly[0]);
        d.corners.push_back(poly[i]);
        d.corners.push_back(poly[i + 1]);
      }
    }
    // o, g, s, usemtl, mtllib, l, p: ignored
  }
  return d;
}

ObjData LoadObj(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("cannot open " + path);
  std::stringstream ss;
  ss << f.rdbuf();
  return ParseObj(ss.str(), path);
}

}  // namespace ajh
