// A libclsph-style driver written against the drop-in headers: load the two
// property files and a scene, run `frames` frames with pre/post callbacks,
// write a Houdini frame and the final particle AoS (raw, like last_frame.bin).
//   dropin_example <fluid.json> <sim.json> <scene.obj> <frames> <out_prefix>
//                  [frames_only|raise_mesh|flip_gravity]
// raise_mesh: the 4th substep's pre_frame callback moves every vertex of the
// scene up by 0.4995 m, in place (the next substeps collide with the moved mesh).
// flip_gravity: the same callback negates the y gravity in sim.parameters.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <string>

#include "file_save_delegates/houdini_file_saver.h"
#include "sph_simulation.h"
#include "util/cereal/archives/binary.hpp"

int main(int argc, char** argv) {
  if (argc < 6) {
    std::cerr << "usage: dropin_example fluid.json sim.json scene.obj frames out_prefix [frames_only]\n";
    return 2;
  }
  sph_simulation sim;
  try {
    sim.load_settings(argv[1], argv[2]);
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
    return 1;
  }
  if (!sim.current_scene.load(argv[3])) return 1;
  if (argc > 6 && std::string(argv[6]) == "frames_only")
    sim.transfers = sph_simulation::transfer_policy::frames_only;
  const bool raise_mesh = argc > 6 && std::string(argv[6]) == "raise_mesh";
  const bool flip_gravity = argc > 6 && std::string(argv[6]) == "flip_gravity";
  int substep_calls = 0;
  const std::string prefix = argv[5];
  houdini_file_saver saver(prefix);
  int pre_calls = 0, post_calls = 0;
  sim.pre_frame = [&](particle* p, const simulation_parameters& prm, bool full) {
    ++pre_calls;
    if (full) saver.writeFrameToFile(p, prm);
    if (!full && ++substep_calls == 4) {
      if (raise_mesh)
        for (size_t v = 1; v < sim.current_scene.vertices.size(); v += 3) sim.current_scene.vertices[v] += 0.4995f;
      if (flip_gravity) sim.parameters.constant_acceleration.s[1] = -sim.parameters.constant_acceleration.s[1];
    }
  };
  sim.post_frame = [&](particle* p, const simulation_parameters& prm, bool full) {
    ++post_calls;
    if (!full) return;
    double ke = 0, rho = 0;
    for (unsigned i = 0; i < prm.particles_count; ++i) {
      const float* v = p[i].velocity.s;
      ke += 0.5 * prm.particle_mass * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
      rho += p[i].density;
    }
    std::printf("frame ke=%.9g mean_density=%.9g cells=%u\n", ke, rho / prm.particles_count,
                prm.grid_cell_count);
    std::ofstream out(prefix + "final.bin", std::ios::binary);
    cereal::BinaryOutputArchive ar(out);
    ar.saveBinary(p, sizeof(particle) * prm.particles_count);
  };
  sim.simulate(std::atoi(argv[4]));
  std::printf("calls pre=%d post=%d\n", pre_calls, post_calls);
  return 0;
}
