// Houdini ASCII geometry frame writer
// (libclsph/file_save_delegates/houdini_file_saver.cpp:25-92 with the format
// of util/houdini_geo/HoudiniFileDumpHelper.cpp:19-90): a PGEOMETRY V5 file
// with one particle primitive, point attributes v (3 floats), color (3 floats,
// a ramp of the density) and mass, floats printed with the default ostream
// formatting (6 significant digits). Large frames are formatted in parallel:
// contiguous point ranges go to separate string buffers on host threads and
// are written in order, so the file is byte-identical to the serial output.

#include <algorithm>
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

}  // namespace

int houdini_file_saver::writeFrameToFile(particle* particles, const simulation_parameters& parameters) {
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
