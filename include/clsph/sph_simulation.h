// sph_simulation of libclsph/sph_simulation.h:8-52, running its substeps on a
// GB300 through the C ABI of include/clsph_gpu.h.
//
// The public surface is the reference's: load_settings(fluid, parameters)
// reads the two JSON property files, simulate(frame_count) runs
// ceil(simulation_time * target_fps) frames (or frame_count) of
// 1/simulation_scale substeps each, calling pre_frame / post_frame with the
// host particle AoS (sorted order) around every substep (full_frame = false)
// and every frame (full_frame = true). Particles start from last_frame.bin
// when that file exists in the working directory, else from the reference's
// cube lattice. Callbacks may modify the particles; the change is seen by the
// next substep.
//
// Particles stay resident on the GPU between substeps. Host copies are made
// only when a callback is set: by default (transfer_policy::every_substep)
// the AoS is downloaded before and uploaded after every callback, which is
// the reference's visible behaviour; transfer_policy::frames_only limits the
// copies (and the substep callbacks' view) to frame boundaries.
#ifndef _SPH_SIMULATION_H_
#define _SPH_SIMULATION_H_

#include <cstring>
#include <functional>
#include <string>

#include "common/structures.h"
#include "scene.h"

struct clsph_gpu;

class sph_simulation {
 public:
  // Padding bytes of the parameter block are zeroed too, so that copies of it
  // (callbacks, the C ABI) are byte-for-byte reproducible.
  sph_simulation() : parameters(), write_intermediate_frames(false) {
    std::memset(&parameters, 0, sizeof(parameters));
  }
  ~sph_simulation();
  sph_simulation(const sph_simulation&) = delete;
  sph_simulation& operator=(const sph_simulation&) = delete;

  void simulate(int frame_count = 0);

  simulation_parameters parameters;
  precomputed_kernel_values precomputed_terms;

  std::function<void(particle*, const simulation_parameters&, bool)> pre_frame;
  std::function<void(particle*, const simulation_parameters&, bool)> post_frame;

  void load_settings(std::string fluid_file_name, std::string parameters_file_name);

  bool write_intermediate_frames;
  bool serialize;
  float initial_volume;
  scene current_scene;

  // Host-transfer policy (no counterpart in the reference, which copies the
  // whole AoS to and from the device several times per substep).
  enum class transfer_policy { every_substep, frames_only };
  transfer_policy transfers = transfer_policy::every_substep;

  // Cap of the advect/collide loop per particle and substep (the reference's
  // loop has none, kernels/sph.cl:82-101).
  unsigned int collision_iteration_cap = 1024;

 private:
  void init_particles(particle* buffer, const simulation_parameters&);
  clsph_gpu* gpu_ = nullptr;
};

#endif
