// Houdini geometry frame writers
// (libclsph/file_save_delegates/houdini_file_saver.cpp:25-92).
//
// ASCII .geo, the format of util/houdini_geo/HoudiniFileDumpHelper.cpp:19-90:
// a PGEOMETRY V5 file with one particle primitive, point attributes v
// (3 floats), color (3 floats, a ramp of the density) and mass, floats printed
// with the default ostream formatting (6 significant digits). Large frames are
// formatted in parallel: contiguous point ranges go to separate string buffers
// on host threads and are written in order, so the file is byte-identical to
// the serial output.
//
// Binary .bgeo, what the reference's USE_PARTIO build hands to Partio::write
// (houdini_file_saver.cpp:76-88, attributes of util/partio/PartioFunctions.h:
// 5-65). Partio itself is not part of the reference tree; this writer emits
// the classic (version 5) binary Houdini geometry layout that Partio's BGEO
// writer produces, restated from that published format:
//   header   "Bgeo" 'V' int32 5, then int32 counts: points, primitives (1),
//            point groups (0), primitive groups (0), point attributes (5),
//            vertex attributes (0), primitive attributes (1), detail
//            attributes (0);
//   point attribute table, one entry per attribute after the position:
//            uint16 name length, name, uint16 component count, int32 type
//            (0 float, 1 int, 5 vector), one zero default per component;
//   points   x y z w (w = 1) then velocity[3], color[3], id, mass, pscale;
//   primitive attribute table: "generator", 1 component, type 4 (index),
//            one string "papi";
//   the particle primitive: int32 0x8000, int32 point count, every point
//            index (uint16 when there are at most 65,535 points, else int32),
//            then its generator value (int32 0);
//   0x00 0xff (the empty extra block).
// Every multi-byte value is big-endian. Attribute values follow makeData()
// (PartioFunctions.h:19-61): pscale = h, mass = particle_mass, id = the
// particle's index in the array, color = the density ramp of the .geo file.
// Deliberate difference: makeData() stores velocity.x three times into
// component 0 and never sets components 1 and 2 (their bytes are whatever the
// attribute buffer held); this writer stores the full velocity.

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "file_save_delegates/houdini_file_saver.h"

namespace {

// Last 7 digits of the zero-padded counter (houdini_file_saver.cpp:15-23).
std::string frame_number(int num) {
  std::ostringstream ss;
  ss << std::setw(9) << std::setfill('0') << num;
  std::string s = ss.str();
  if (s.size() > 7) s.erase(0, s.size() - 7);
  return s;
}

// Density -> RGB ramp of houdini_file_saver.cpp:47-60.
void density_color(float d, float& r, float& g, float& b) {
  r = (d > 1000.f && d <= 2000.f) ? (d - 1000.f) / 1000.f : 0.f;
  g = (d >= 0.f && d < 1000.f) ? 1.f - d / 1000.f : 0.f;
  if (d >= 500.f && d <= 1000.f)
    b = (d - 500.f) / 500.f;
  else if (d >= 1000.f && d <= 1500.f)
    b = 1.f - (d - 1000.f) / 500.f;
  else
    b = 0.f;
}

// Point lines [begin, end): position, w, (velocity, color ramp, mass).
std::string format_points(const particle* particles, unsigned int begin, unsigned int end, float mass) {
  std::ostringstream out;
  for (unsigned int i = begin; i < end; ++i) {
    const particle& p = particles[i];
    float r, g, b;
    density_color(p.density, r, g, b);
    const float pw = 0.f;
    out << p.position.s[0] << " " << p.position.s[1] << " " << p.position.s[2] << " " << pw << " ";
    out << "(" << p.velocity.s[0] << " " << p.velocity.s[1] << " " << p.velocity.s[2] << "\t" << r
        << " " << g << " " << b << "\t" << mass << ")" << '\n';
  }
  return out.str();
}

// " i" for every point index of [begin, end) (the particle primitive's list).
std::string format_indices(unsigned int begin, unsigned int end) {
  std::ostringstream out;
  for (unsigned int i = begin; i < end; ++i) out << " " << (int)i;
  return out.str();
}

// f(begin, end) over [0, n) in contiguous chunks, on host threads when n is
// large; the pieces come back in order.
template <class F>
std::vector<std::string> chunked(unsigned int n, F f) {
  constexpr unsigned int kMinChunk = 1024;
  unsigned int threads = std::max(1u, std::thread::hardware_concurrency());
  threads = std::min(threads, std::max(1u, n / kMinChunk));
  std::vector<std::string> parts(threads);
  if (threads == 1) {
    parts[0] = f(0u, n);
    return parts;
  }
  std::vector<std::thread> pool;
  for (unsigned int t = 0; t < threads; ++t) {
    const unsigned int b = (unsigned int)((unsigned long long)n * t / threads);
    const unsigned int e = (unsigned int)((unsigned long long)n * (t + 1) / threads);
    pool.emplace_back([&parts, &f, t, b, e] { parts[t] = f(b, e); });
  }
  for (auto& th : pool) th.join();
  return parts;
}

// Big-endian stores into a byte buffer.
inline unsigned char* put_u32(unsigned char* p, uint32_t v) {
  p[0] = (unsigned char)(v >> 24);
  p[1] = (unsigned char)(v >> 16);
  p[2] = (unsigned char)(v >> 8);
  p[3] = (unsigned char)v;
  return p + 4;
}
inline unsigned char* put_f32(unsigned char* p, float f) {
  uint32_t v;
  std::memcpy(&v, &f, 4);
  return put_u32(p, v);
}
inline void put_u16(std::string& s, unsigned v) {
  s.push_back((char)(unsigned char)(v >> 8));
  s.push_back((char)(unsigned char)v);
}
inline void put_i32(std::string& s, int32_t v) {
  unsigned char b[4];
  put_u32(b, (uint32_t)v);
  s.append(reinterpret_cast<const char*>(b), 4);
}
inline void put_name(std::string& s, const char* name) {
  const size_t len = std::strlen(name);
  put_u16(s, (unsigned)len);
  s.append(name, len);
}

constexpr size_t kBgeoPointBytes = 13 * 4;  // x y z w, velocity, color, id, mass, pscale

// The whole .bgeo file of one frame.
std::vector<unsigned char> bgeo_bytes(const particle* particles, const simulation_parameters& parameters) {
  const unsigned int n = parameters.particles_count;
  std::string head;
  head.append("Bgeo", 4);
  head.push_back('V');
  put_i32(head, 5);
  for (int32_t c : {(int32_t)n, 1, 0, 0, 5, 0, 1, 0}) put_i32(head, c);
  struct Attr {
    const char* name;
    unsigned size;
    int32_t type;
  };
  for (const Attr& a : {Attr{"velocity", 3, 5}, Attr{"color", 3, 5}, Attr{"id", 1, 1},
                        Attr{"mass", 1, 0}, Attr{"pscale", 1, 0}}) {
    put_name(head, a.name);
    put_u16(head, a.size);
    put_i32(head, a.type);
    for (unsigned c = 0; c < a.size; ++c) put_i32(head, 0);  // 0 and 0.0f share their bytes
  }
  std::string prim_head;
  put_name(prim_head, "generator");
  put_u16(prim_head, 1);
  put_i32(prim_head, 4);
  put_i32(prim_head, 1);
  put_name(prim_head, "papi");
  put_i32(prim_head, 0x8000);
  put_i32(prim_head, (int32_t)n);
  const bool short_index = n <= 65535u;
  const size_t index_bytes = short_index ? 2 : 4;

  const size_t points_at = head.size();
  const size_t prim_at = points_at + kBgeoPointBytes * n;
  const size_t index_at = prim_at + prim_head.size();
  const size_t tail_at = index_at + index_bytes * n;
  std::vector<unsigned char> out(tail_at + 4 + 2);
  std::memcpy(out.data(), head.data(), head.size());
  std::memcpy(out.data() + prim_at, prim_head.data(), prim_head.size());
  const float mass = parameters.particle_mass;
  const float h = parameters.h;
  chunked(n, [&](unsigned int b, unsigned int e) {
    unsigned char* q = out.data() + points_at + kBgeoPointBytes * b;
    for (unsigned int i = b; i < e; ++i) {
      const particle& p = particles[i];
      float r, g, bl;
      density_color(p.density, r, g, bl);
      for (float f : {p.position.s[0], p.position.s[1], p.position.s[2], 1.f, p.velocity.s[0],
                      p.velocity.s[1], p.velocity.s[2], r, g, bl})
        q = put_f32(q, f);
      q = put_u32(q, (uint32_t)i);
      q = put_f32(q, mass);
      q = put_f32(q, h);
    }
    unsigned char* x = out.data() + index_at + index_bytes * b;
    for (unsigned int i = b; i < e; ++i) {
      if (short_index) {
        x[0] = (unsigned char)(i >> 8);
        x[1] = (unsigned char)i;
        x += 2;
      } else {
        x = put_u32(x, (uint32_t)i);
      }
    }
    return std::string();
  });
  unsigned char* t = put_u32(out.data() + tail_at, 0u);  // the primitive's generator index
  t[0] = 0x00;
  t[1] = 0xff;
  return out;
}

}  // namespace

int houdini_file_saver::writeFrameToFile(particle* particles, const simulation_parameters& parameters) {
  if (binary_bgeo) {
    std::string name = frames_folder_prefix + "frames/frame" + frame_number(++frame_count) + ".bgeo";
    std::ofstream out(name, std::ios::out | std::ios::trunc | std::ios::binary);
    if (!out.is_open()) {
      std::cerr << "Error while writing to " << name << std::endl;
      return 0;
    }
    const std::vector<unsigned char> bytes = bgeo_bytes(particles, parameters);
    out.write(reinterpret_cast<const char*>(bytes.data()), (std::streamsize)bytes.size());
    return 0;
  }
  std::string name = frames_folder_prefix + "frames/frame" + frame_number(++frame_count) + ".geo";
  std::ofstream out(name, std::ios::out | std::ios::trunc);
  if (!out.is_open()) {
    std::cerr << "Error while writing to " << name << std::endl;
    return 0;
  }
  const unsigned int n = parameters.particles_count;
  out << "PGEOMETRY V5" << std::endl;
  out << "NPoints " << (int)n << " NPrims 1" << std::endl;
  out << "NPointGroups 0 NPrimGroups 1" << std::endl;
  out << "NPointAttrib " << 3 << " NVertexAttrib 0 NPrimAttrib 2 NAttrib 0" << std::endl;
  out << "PointAttrib" << std::endl;
  out << "v 3 float 1 1 1" << std::endl;
  out << "color 3 float 1 1 1" << std::endl;
  out << "mass 1 float 1" << std::endl;
  const float mass = parameters.particle_mass;
  for (const std::string& part :
       chunked(n, [&](unsigned int b, unsigned int e) { return format_points(particles, b, e, mass); }))
    out << part;
  out << "PrimitiveAttrib" << std::endl;
  out << "generator 1 index 1 location1" << std::endl;
  out << "dopobject 1 index 1 /obj/AutoDopNetwork:1" << std::endl;
  out << "Part " << (int)n;
  for (const std::string& part : chunked(n, format_indices)) out << part;
  out << " [0\t0]" << std::endl;
  out << "box_object1 unordered" << std::endl;
  out << "1 1" << std::endl;
  out << "beginExtra" << std::endl;
  out << "endExtra" << std::endl;
  return 0;
}
