// C entry points of the C++ host layer, for callers that bind C (ctypes,
// cgo, JNI): property-file loading, scene loading, Houdini frame writing and
// a whole simulate() run with C callbacks. They wrap the same sph_simulation,
// scene and houdini_file_saver code that C++ callers use.

#include <cstdint>
#include <cstring>
#include <exception>
#include <string>

#include "file_save_delegates/houdini_file_saver.h"
#include "scene.h"
#include "sph_simulation.h"

namespace {
thread_local std::string g_host_error;

int host_fail(const std::exception& e) {
  g_host_error = e.what();
  return 1;
}
}  // namespace

extern "C" {

const char* clsph_host_last_error(void) { return g_host_error.c_str(); }

// sph_simulation::load_settings; params_out: 128-byte simulation_parameters,
// terms_out: 20-byte precomputed_kernel_values.
int clsph_host_load_settings(const char* fluid_file, const char* params_file, void* params_out,
                             void* terms_out, float* initial_volume, int* write_all_frames,
                             int* serialize) {
  try {
    sph_simulation sim;
    sim.load_settings(fluid_file, params_file);
    if (params_out) std::memcpy(params_out, &sim.parameters, sizeof(sim.parameters));
    if (terms_out) std::memcpy(terms_out, &sim.precomputed_terms, sizeof(sim.precomputed_terms));
    if (initial_volume) *initial_volume = sim.initial_volume;
    if (write_all_frames) *write_all_frames = sim.write_intermediate_frames ? 1 : 0;
    if (serialize) *serialize = sim.serialize ? 1 : 0;
    return 0;
  } catch (const std::exception& e) {
    return host_fail(e);
  }
}

void* clsph_host_scene_new(void) { return new scene(); }
void clsph_host_scene_free(void* s) { delete static_cast<scene*>(s); }

// scene::load("scenes/<filename>"); 1 on success, 0 on failure (as the reference).
int clsph_host_scene_load(void* s, const char* filename) {
  return static_cast<scene*>(s)->load(filename) ? 1 : 0;
}

// scene::fix_multi_shape (0: the reference's behaviour, 1: shapes concatenated).
void clsph_host_scene_set_fix_multi_shape(void* s, int on) {
  static_cast<scene*>(s)->fix_multi_shape = on != 0;
}

void clsph_host_scene_sizes(void* s, uint32_t* face_count, uint64_t* normals, uint64_t* vertices,
                            uint64_t* indices) {
  scene* sc = static_cast<scene*>(s);
  *face_count = sc->face_count;
  *normals = sc->face_normals.size();
  *vertices = sc->vertices.size();
  *indices = sc->indices.size();
}

void clsph_host_scene_copy(void* s, float* normals, float* vertices, uint32_t* indices) {
  scene* sc = static_cast<scene*>(s);
  if (normals && !sc->face_normals.empty())
    std::memcpy(normals, sc->face_normals.data(), sizeof(float) * sc->face_normals.size());
  if (vertices && !sc->vertices.empty())
    std::memcpy(vertices, sc->vertices.data(), sizeof(float) * sc->vertices.size());
  if (indices && !sc->indices.empty())
    std::memcpy(indices, sc->indices.data(), sizeof(uint32_t) * sc->indices.size());
}

// A new houdini_file_saver(prefix) writing its first frame:
// <prefix>frames/frame0000001.geo.
int clsph_host_write_houdini(const char* prefix, void* particles, const void* params) {
  try {
    houdini_file_saver saver{std::string(prefix)};
    simulation_parameters p;
    std::memcpy(&p, params, sizeof(p));
    return saver.writeFrameToFile(static_cast<particle*>(particles), p);
  } catch (const std::exception& e) {
    return host_fail(e);
  }
}

// The same with binary_bgeo set: <prefix>frames/frame0000001.bgeo.
int clsph_host_write_bgeo(const char* prefix, void* particles, const void* params) {
  try {
    houdini_file_saver saver{std::string(prefix)};
    saver.binary_bgeo = true;
    simulation_parameters p;
    std::memcpy(&p, params, sizeof(p));
    return saver.writeFrameToFile(static_cast<particle*>(particles), p);
  } catch (const std::exception& e) {
    return host_fail(e);
  }
}

typedef void (*clsph_frame_callback)(void* user, void* particles, const void* params, int full_frame);

// A whole sph_simulation run: load_settings(fluid, params), scene load,
// simulate(frame_count) with optional C callbacks. transfer_policy: 0 =
// every substep, 1 = frames only.
int clsph_host_simulate(const char* fluid_file, const char* params_file, const char* scene_name,
                        int frame_count, clsph_frame_callback pre, clsph_frame_callback post,
                        void* user, int transfer_policy) {
  try {
    sph_simulation sim;
    sim.load_settings(fluid_file, params_file);
    if (scene_name && *scene_name && !sim.current_scene.load(scene_name)) {
      g_host_error = std::string("cannot load scene ") + scene_name;
      return 1;
    }
    sim.transfers = transfer_policy ? sph_simulation::transfer_policy::frames_only
                                    : sph_simulation::transfer_policy::every_substep;
    if (pre)
      sim.pre_frame = [&](particle* p, const simulation_parameters& prm, bool full) {
        pre(user, p, &prm, full ? 1 : 0);
      };
    if (post)
      sim.post_frame = [&](particle* p, const simulation_parameters& prm, bool full) {
        post(user, p, &prm, full ? 1 : 0);
      };
    sim.simulate(frame_count);
    return 0;
  } catch (const std::exception& e) {
    return host_fail(e);
  }
}

}  // extern "C"
