// Exercises the host layer's parsers and writers (JSON settings, OBJ scenes,
// .geo and .bgeo frames) for a build with AddressSanitizer and
// UndefinedBehaviorSanitizer. Run from a directory holding scenes/<name>.obj.
//   host_sanitize <fluid.json> <sim.json> <frames prefix> <scene name>...
// Prints one line per input; exit status 0 unless the harness itself fails.
#include <cstdio>
#include <exception>
#include <string>
#include <vector>

#include "file_save_delegates/houdini_file_saver.h"
#include "scene.h"
#include "sph_simulation.h"

int main(int argc, char** argv) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: %s fluid.json sim.json prefix [scene...]\n", argv[0]);
    return 2;
  }
  simulation_parameters params{};
  {
    sph_simulation sim;
    try {
      sim.load_settings(argv[1], argv[2]);
      params = sim.parameters;
      std::printf("settings h=%g mass=%g\n", (double)params.h, (double)params.particle_mass);
    } catch (const std::exception& e) {
      std::printf("settings error: %s\n", e.what());
    }
  }
  for (int a = 4; a < argc; ++a) {
    scene sc;
    const bool ok = sc.load(argv[a]);
    std::printf("scene %s ok=%d faces=%u\n", argv[a], ok ? 1 : 0, sc.face_count);
  }
  // Frames of a small ragged particle set, both formats.
  const unsigned int n = 3001;
  std::vector<particle> parts(n);
  for (unsigned int i = 0; i < n; ++i) {
    particle& p = parts[i];
    p = particle{};
    for (int c = 0; c < 3; ++c) {
      p.position.s[c] = 0.001f * (float)((i * (c + 3)) % 997);
      p.velocity.s[c] = 0.01f * (float)((int)(i % 13) - 6);
    }
    p.density = 2.f * (float)(i % 1200);
  }
  params.particles_count = n;
  houdini_file_saver geo(argv[3]);
  houdini_file_saver bgeo(argv[3]);
  bgeo.binary_bgeo = true;
  for (int f = 0; f < 2; ++f) {
    geo.writeFrameToFile(parts.data(), params);
    bgeo.writeFrameToFile(parts.data(), params);
  }
  return 0;
}
