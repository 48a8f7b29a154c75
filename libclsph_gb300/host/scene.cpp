// scene::load (libclsph/scene.cpp:9-67) with an OBJ reader that gives the
// same arrays as the tinyobjloader 0.9.6 the reference vendors
// (util/tinyobj/tiny_obj_loader.cc:118-661):
//   * v / vn / vt records read with atof, f records of i, i/j, i//k, i/j/k
//     with 1-based or negative (relative) indices;
//   * polygons become the triangle fan (v0, v[k-1], v[k]);
//   * per shape, vertices are re-indexed in first-use order and shared when
//     the (position, normal, texcoord) index triple repeats;
//   * every `o` or `g` record after faces starts a new shape;
//   * an `mtllib` file that cannot be opened makes the load fail.
// Per shape, as the reference does: indices and vertices are replaced, one
// unit face normal per face is appended to face_normals.

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "scene.h"

namespace {

struct Corner {
  int v, vt, vn;
  bool operator<(const Corner& o) const {
    return std::tie(v, vn, vt) < std::tie(o.v, o.vn, o.vt);
  }
};

struct Shape {
  std::vector<float> positions;
  std::vector<unsigned int> indices;
};

int resolve_index(int idx, int count) {
  if (idx > 0) return idx - 1;
  if (idx == 0) return 0;
  return count + idx;  // negative: relative to the end
}

bool is_blank(char c) { return c == ' ' || c == '\t'; }
bool is_line_end(char c) { return c == '\r' || c == '\n' || c == '\0'; }

float read_float(const char*& p) {
  p += std::strspn(p, " \t");
  float f = (float)std::atof(p);
  p += std::strcspn(p, " \t\r");
  return f;
}

Corner read_corner(const char*& p, int nv, int nvn, int nvt) {
  Corner c{-1, -1, -1};
  c.v = resolve_index(std::atoi(p), nv);
  p += std::strcspn(p, "/ \t\r");
  if (*p != '/') return c;
  ++p;
  if (*p == '/') {  // i//k
    ++p;
    c.vn = resolve_index(std::atoi(p), nvn);
    p += std::strcspn(p, "/ \t\r");
    return c;
  }
  c.vt = resolve_index(std::atoi(p), nvt);  // i/j or i/j/k
  p += std::strcspn(p, "/ \t\r");
  if (*p != '/') return c;
  ++p;
  c.vn = resolve_index(std::atoi(p), nvn);
  p += std::strcspn(p, "/ \t\r");
  return c;
}

bool flush_group(std::vector<std::vector<Corner>>& group, const std::vector<float>& v,
                 std::vector<Shape>& shapes, std::string& err) {
  if (group.empty()) return true;
  Shape s;
  std::map<Corner, unsigned int> seen;
  auto vertex_of = [&](const Corner& c, unsigned int& out) {
    auto it = seen.find(c);
    if (it != seen.end()) {
      out = it->second;
      return true;
    }
    if (c.v < 0 || (size_t)(3 * (size_t)c.v + 2) >= v.size()) return false;
    s.positions.insert(s.positions.end(), v.begin() + 3 * c.v, v.begin() + 3 * c.v + 3);
    out = (unsigned int)(s.positions.size() / 3 - 1);
    seen[c] = out;
    return true;
  };
  for (const auto& face : group)
    for (size_t k = 2; k < face.size(); ++k) {
      unsigned int a, b, c;
      if (!vertex_of(face[0], a) || !vertex_of(face[k - 1], b) || !vertex_of(face[k], c)) {
        err = "vertex index out of range";
        return false;
      }
      s.indices.push_back(a);
      s.indices.push_back(b);
      s.indices.push_back(c);
    }
  shapes.push_back(std::move(s));
  group.clear();
  return true;
}

std::string read_obj(const std::string& path, const std::string& mtl_base, std::vector<Shape>& shapes) {
  std::ifstream in(path);
  if (!in) return "Cannot open file [" + path + "]";
  std::vector<float> v, vn, vt;
  std::vector<std::vector<Corner>> group;
  std::string line, err;
  while (std::getline(in, line)) {
    if (line.size() > 8191) line.resize(8191);
    const char* p = line.c_str();
    p += std::strspn(p, " \t");
    if (*p == '\0' || *p == '#') continue;
    if (p[0] == 'v' && is_blank(p[1])) {
      p += 2;
      for (int k = 0; k < 3; ++k) v.push_back(read_float(p));
    } else if (p[0] == 'v' && p[1] == 'n' && is_blank(p[2])) {
      p += 3;
      for (int k = 0; k < 3; ++k) vn.push_back(read_float(p));
    } else if (p[0] == 'v' && p[1] == 't' && is_blank(p[2])) {
      p += 3;
      for (int k = 0; k < 2; ++k) vt.push_back(read_float(p));
    } else if (p[0] == 'f' && is_blank(p[1])) {
      p += 2;
      p += std::strspn(p, " \t");
      std::vector<Corner> face;
      while (!is_line_end(*p)) {
        face.push_back(read_corner(p, (int)(v.size() / 3), (int)(vn.size() / 3), (int)(vt.size() / 2)));
        p += std::strspn(p, " \t\r");
      }
      group.push_back(std::move(face));
    } else if (std::strncmp(p, "mtllib", 6) == 0 && is_blank(p[6])) {
      p += 7;
      p += std::strspn(p, " \t");
      std::string name(p, std::strcspn(p, " \t\r"));
      std::ifstream mtl(mtl_base + name);
      if (!mtl) return "Cannot open file [" + mtl_base + name + "]";
    } else if ((p[0] == 'g' || p[0] == 'o') && is_blank(p[1])) {
      if (!flush_group(group, v, shapes, err)) return err;
    }
  }
  if (!flush_group(group, v, shapes, err)) return err;
  return "";
}

}  // namespace

bool scene::load(std::string filename) {
  std::vector<Shape> shapes;
  std::string err = read_obj("scenes/" + filename, "scenes/", shapes);
  if (!err.empty()) {
    std::cerr << err << std::endl;
    return false;
  }
  std::cout << "Scene Loading - number of shapes in file [" << filename << "]: " << shapes.size()
            << std::endl;
  if (fix_multi_shape && !shapes.empty()) {
    Shape all;
    for (const Shape& s : shapes) {
      const unsigned int base = (unsigned int)(all.positions.size() / 3);
      for (unsigned int i : s.indices) all.indices.push_back(i + base);
      all.positions.insert(all.positions.end(), s.positions.begin(), s.positions.end());
    }
    shapes.assign(1, all);
  }
  for (const Shape& s : shapes) {
    indices = s.indices;
    if (indices.size() % 3 != 0) {
      std::cerr << "Meshes must be made of triangles only" << std::endl;
      return false;
    }
    face_count = (unsigned int)(indices.size() / 3);
    vertices = s.positions;
    for (size_t f = 0; f < face_count; ++f) {
      const float* a = &vertices[3 * indices[3 * f]];
      const float* b = &vertices[3 * indices[3 * f + 1]];
      const float* c = &vertices[3 * indices[3 * f + 2]];
      const float ux = b[0] - a[0], uy = b[1] - a[1], uz = b[2] - a[2];
      const float vx = c[0] - a[0], vy = c[1] - a[1], vz = c[2] - a[2];
      const float nx = uy * vz - uz * vy;
      const float ny = uz * vx - ux * vz;
      const float nz = ux * vy - uy * vx;
      const float len = std::sqrt(nx * nx + ny * ny + nz * nz);
      face_normals.push_back(nx / len);
      face_normals.push_back(ny / len);
      face_normals.push_back(nz / len);
    }
  }
  return true;
}
