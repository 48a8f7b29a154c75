// TEST INFRASTRUCTURE (oracle/_ref/ref_geo): runs the reference's own Houdini
// .geo frame writer (libclsph/file_save_delegates/houdini_file_saver.cpp:25-72,
// the build without USE_PARTIO, and util/houdini_geo/HoudiniFileDumpHelper.cpp,
// both compiled unchanged by oracle/Makefile) on one frame:
//
//   ref_geo <params: 128-byte simulation_parameters> <particles: 80-byte records> <prefix>
//
// writes <prefix>frames/frame0000001.geo, exactly as
// houdini_file_saver(prefix).writeFrameToFile(particles, params) does in the
// reference. tests/golden/make_golden.py uses it to make the golden frame.
#include <cstdio>
#include <vector>

#include "file_save_delegates/houdini_file_saver.h"

static_assert(sizeof(particle) == 80, "particle record layout");
static_assert(sizeof(simulation_parameters) == 128, "parameter block layout");

int main(int argc, char** argv) {
  if (argc != 4) {
    std::fprintf(stderr, "usage: ref_geo params.bin particles.bin prefix\n");
    return 2;
  }
  simulation_parameters params;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f || std::fread(&params, sizeof(params), 1, f) != 1) return 3;
  std::fclose(f);
  f = std::fopen(argv[2], "rb");
  if (!f) return 4;
  std::vector<particle> parts(params.particles_count);
  if (!parts.empty() && std::fread(parts.data(), sizeof(particle), parts.size(), f) != parts.size()) return 5;
  std::fclose(f);
  houdini_file_saver saver(argv[3]);
  return saver.writeFrameToFile(parts.data(), params);
}
