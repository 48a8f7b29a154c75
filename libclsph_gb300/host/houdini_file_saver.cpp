// Houdini ASCII geometry frame writer
// (libclsph/file_save_delegates/houdini_file_saver.cpp:25-92 with the format
// of util/houdini_geo/HoudiniFileDumpHelper.cpp:19-90): a PGEOMETRY V5 file
// with one particle primitive, point attributes v (3 floats), color (3 floats,
// a ramp of the density) and mass, floats printed with the default ostream
// formatting (6 significant digits).

#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <string>

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
  for (unsigned int i = 0; i < n; ++i) {
    const particle& p = particles[i];
    float r, g, b;
    density_color(p.density, r, g, b);
    const float pw = 0.f;
    out << p.position.s[0] << " " << p.position.s[1] << " " << p.position.s[2] << " " << pw << " ";
    out << "(" << p.velocity.s[0] << " " << p.velocity.s[1] << " " << p.velocity.s[2] << "\t" << r
        << " " << g << " " << b << "\t" << mass << ")" << std::endl;
  }
  out << "PrimitiveAttrib" << std::endl;
  out << "generator 1 index 1 location1" << std::endl;
  out << "dopobject 1 index 1 /obj/AutoDopNetwork:1" << std::endl;
  out << "Part " << (int)n;
  for (unsigned int i = 0; i < n; ++i) out << " " << (int)i;
  out << " [0\t0]" << std::endl;
  out << "box_object1 unordered" << std::endl;
  out << "1 1" << std::endl;
  out << "beginExtra" << std::endl;
  out << "endExtra" << std::endl;
  return 0;
}
