// sph_simulation (libclsph/sph_simulation.h:8-52) on the GB300 engine.
//
//   load_settings  libclsph/sph_simulation.cpp:405-505 (JSON + derived values)
//   init_particles sph_simulation.cpp:48-94 (last_frame.bin or cube lattice)
//   simulate       sph_simulation.cpp:346-403 (frames x substeps + callbacks)
// Each substep is clsph_gpu_step(h, 1), the whole of simulate_single_frame
// (sph_simulation.cpp:173-344) on the device. Errors that the reference turns
// into exit(-1) or assert() are thrown as std::runtime_error.

#include <cmath>
#include <cstddef>
#include <cstring>
#include <fstream>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "clsph_gpu.h"
#include "json_reader.h"
#include "sph_simulation.h"

static_assert(sizeof(particle) == sizeof(clsph_particle), "particle layouts differ");
static_assert(sizeof(simulation_parameters) == sizeof(clsph_parameters), "parameter layouts differ");
static_assert(sizeof(precomputed_kernel_values) == sizeof(clsph_kernel_terms), "term layouts differ");

namespace {

void check(int rc, const char* what) {
  if (rc != CLSPH_OK)
    throw std::runtime_error(std::string(what) + " failed (status " + std::to_string(rc) +
                             "): " + clsph_gpu_last_error());
}

void check_flags(uint32_t flags) {
  if (flags & CLSPH_WARN_GRID_OVERFLOW)
    throw std::runtime_error("particle grid reached 1024 cells on an axis (Morton keys hold 10 bits)");
  if (flags & CLSPH_WARN_COLLISION_CAP)
    std::cerr << "warning: a particle's collision loop reached its iteration cap" << std::endl;
  if (flags & CLSPH_WARN_NONFINITE) std::cerr << "warning: non-finite particle position" << std::endl;
}

}  // namespace

sph_simulation::~sph_simulation() {
  if (gpu_) clsph_gpu_destroy(gpu_);
}

void sph_simulation::load_settings(std::string fluid_file_name, std::string parameters_file_name) {
  using clsph_host::JsonValue;
  int influence = 0;
  {
    JsonValue f = clsph_host::parse_json_file(fluid_file_name);
    parameters.fluid_density = (float)f.at("fluid_density").as_number("fluid_density");
    parameters.dynamic_viscosity = (float)f.at("dynamic_viscosity").as_number("dynamic_viscosity");
    parameters.restitution = (float)f.at("restitution").as_number("restitution");
    if (parameters.restitution < 0 || parameters.restitution > 1)
      throw std::runtime_error("Restitution has an invalid value!");
    parameters.K = (float)f.at("k").as_number("k");
    parameters.surface_tension_threshold =
        (float)f.at("surface_tension_threshold").as_number("surface_tension_threshold");
    parameters.surface_tension = (float)f.at("surface_tension").as_number("surface_tension");
    influence = (int)f.at("particles_inside_influence_radius").as_number("particles_inside_influence_radius");
  }
  {
    JsonValue s = clsph_host::parse_json_file(parameters_file_name);
    parameters.particles_count = (unsigned int)s.at("particles_count").as_number("particles_count");
    if (parameters.particles_count % 64 != 0) {
      std::cout << std::endl
                << "\033[1;31m You should choose a number of particles that is divisble by the "
                   "preferred work group size.\033[0m"
                << std::endl
                << "\033[1;31m Performances will be sub-optimal.\033[0m" << std::endl;
    }
    parameters.particle_mass = (float)s.at("particle_mass").as_number("particle_mass");
    parameters.simulation_time = (float)s.at("simulation_time").as_number("simulation_time");
    parameters.target_fps = (float)s.at("target_fps").as_number("target_fps");
    parameters.simulation_scale = (float)s.at("simulation_scale").as_number("simulation_scale");
    const JsonValue& g = s.at("constant_acceleration");
    parameters.constant_acceleration.s[0] = (float)g.at("x").as_number("constant_acceleration.x");
    parameters.constant_acceleration.s[1] = (float)g.at("y").as_number("constant_acceleration.y");
    parameters.constant_acceleration.s[2] = (float)g.at("z").as_number("constant_acceleration.z");
    parameters.constant_acceleration.s[3] = 0.f;
    write_intermediate_frames = s.at("write_all_frames").as_bool("write_all_frames");
    serialize = s.at("serialize").as_bool("serialize");
  }
  // derived values (sph_simulation.cpp:490-505): float arithmetic, except the
  // division by 4*pi and the kernel constants, which the reference evaluates
  // in double (M_PI and ::pow are double) before narrowing.
  parameters.total_mass = parameters.particles_count * parameters.particle_mass;
  initial_volume = parameters.total_mass / parameters.fluid_density;
  const double q = (3.f * (influence * (initial_volume / parameters.particles_count))) / (4.f * M_PI);
  parameters.h = std::cbrt((float)q);
  parameters.time_delta = 1.f / parameters.target_fps;
  parameters.max_velocity = 0.8f * parameters.h / parameters.time_delta;
  const double h = parameters.h;
  precomputed_terms.poly_6 = (float)(315.f / (64.f * M_PI * std::pow(h, 9.0)));
  precomputed_terms.poly_6_gradient = (float)(-945.f / (32.f * M_PI * std::pow(h, 9.0)));
  precomputed_terms.poly_6_laplacian = (float)(-945.f / (32.f * M_PI * std::pow(h, 9.0)));
  precomputed_terms.spiky = (float)(-45.f / (M_PI * std::pow(h, 6.0)));
  precomputed_terms.viscosity = (float)(45.f / (M_PI * std::pow(h, 6.0)));
}

void sph_simulation::init_particles(particle* buffer, const simulation_parameters& p) {
  const int side = (int)std::ceil(std::cbrt((float)p.particles_count));
  const float len = std::cbrt(initial_volume);
  const float gap = len / (float)side;
  std::cout << "volume: " << initial_volume << " side_length: " << len << " spacing: " << gap
            << std::endl;
  std::ifstream in("last_frame.bin", std::ios::in | std::ios::binary);
  if (in) {  // resume from the last serialized frame
    in.read(reinterpret_cast<char*>(buffer), (std::streamsize)(sizeof(particle) * p.particles_count));
    if ((size_t)in.gcount() != sizeof(particle) * p.particles_count)
      throw std::runtime_error("last_frame.bin is shorter than the particle count");
    return;
  }
  std::memset(buffer, 0, sizeof(particle) * p.particles_count);
  for (unsigned int i = 0; i < p.particles_count; ++i) {
    buffer[i].position.s[0] = (float)(i % side) * gap - len / 2.f;
    buffer[i].position.s[1] = (float)((i / side) % side) * gap;
    buffer[i].position.s[2] = (float)(i / (side * side)) * gap - len / 2.f;
  }
}

void sph_simulation::simulate(int frame_count) {
  if (frame_count == 0) frame_count = (int)std::ceil(parameters.simulation_time * parameters.target_fps);
  const unsigned int n = parameters.particles_count;
  if (gpu_) {
    clsph_gpu_destroy(gpu_);
    gpu_ = nullptr;
  }
  check(clsph_gpu_create(reinterpret_cast<const clsph_parameters*>(&parameters),
                         reinterpret_cast<const clsph_kernel_terms*>(&precomputed_terms), n, &gpu_),
        "clsph_gpu_create");
  check(clsph_gpu_set_collision_cap(gpu_, collision_iteration_cap), "clsph_gpu_set_collision_cap");
  // The reference hands current_scene to the kernels every substep
  // (sph_simulation.cpp:296-337: face_normals.data() with face_count faces,
  // the first face_count normals), so a callback may edit the scene in place
  // and the next substep collides with the edited mesh. The device keeps the
  // mesh; after a callback the scene is compared with the copy last uploaded
  // and uploaded again when it differs.
  unsigned int up_faces = 0;
  std::vector<float> up_normals, up_vertices;
  std::vector<unsigned int> up_indices;
  auto upload_scene = [&]() {
    const unsigned int faces = current_scene.face_count;
    if (faces > 0 && (current_scene.face_normals.size() < 3ull * faces ||
                      current_scene.indices.size() < 3ull * faces))
      throw std::runtime_error("scene arrays are shorter than face_count");
    check(clsph_gpu_set_mesh(gpu_, faces ? current_scene.face_normals.data() : nullptr,
                             faces ? current_scene.vertices.data() : nullptr,
                             (uint32_t)(current_scene.vertices.size() / 3),
                             faces ? current_scene.indices.data() : nullptr, faces),
          "clsph_gpu_set_mesh");
    up_faces = faces;
    up_normals = current_scene.face_normals;
    up_vertices = current_scene.vertices;
    up_indices = current_scene.indices;
  };
  if (current_scene.face_count > 0) upload_scene();
  // The same holds for `parameters` and `precomputed_terms`, which the
  // reference's kernels receive by value every substep: edits other than to
  // the grid fields (the engine's own) are handed to the device.
  auto inputs_of = [&]() {
    simulation_parameters p = parameters;
    p.min_point = p.max_point = cl_float3{};
    p.grid_size_x = p.grid_size_y = p.grid_size_z = p.grid_cell_count = 0;
    p.constant_acceleration.s[3] = 0.f;  // the padding lane of cl_float3
    std::vector<unsigned char> b(sizeof(p) + sizeof(precomputed_terms));
    std::memcpy(b.data(), &p, sizeof(p));
    std::memcpy(b.data() + sizeof(p), &precomputed_terms, sizeof(precomputed_terms));
    // the struct's padding before constant_acceleration holds no value
    const size_t pad0 = offsetof(simulation_parameters, K) + sizeof(p.K);
    std::memset(b.data() + pad0, 0, offsetof(simulation_parameters, constant_acceleration) - pad0);
    return b;
  };
  std::vector<unsigned char> up_inputs = inputs_of();
  bool scene_check = false;  // a callback ran since the last comparison
  auto refresh_scene = [&]() {
    if (!scene_check) return;
    scene_check = false;
    if (current_scene.face_count != up_faces || current_scene.face_normals != up_normals ||
        current_scene.vertices != up_vertices || current_scene.indices != up_indices)
      upload_scene();
    std::vector<unsigned char> now = inputs_of();
    if (now != up_inputs) {
      if (parameters.particles_count != n)
        throw std::runtime_error("the particle count cannot change during simulate()");
      check(clsph_gpu_set_parameters(gpu_, reinterpret_cast<const clsph_parameters*>(&parameters),
                                     reinterpret_cast<const clsph_kernel_terms*>(&precomputed_terms)),
            "clsph_gpu_set_parameters");
      up_inputs.swap(now);
    }
  };

  std::vector<particle> storage(n);
  particle* particles = storage.data();
  init_particles(particles, parameters);
  check(clsph_gpu_upload(gpu_, reinterpret_cast<const clsph_particle*>(particles)), "clsph_gpu_upload");

  bool device_newer = false;  // the device holds a state the host has not seen
  bool host_dirty = false;    // a callback may have changed the host copy
  auto refresh_host = [&]() {
    if (!device_newer) return;
    check(clsph_gpu_download(gpu_, reinterpret_cast<clsph_particle*>(particles)), "clsph_gpu_download");
    simulation_parameters grid;
    check(clsph_gpu_get_parameters(gpu_, reinterpret_cast<clsph_parameters*>(&grid)),
          "clsph_gpu_get_parameters");
    parameters.min_point = grid.min_point;
    parameters.max_point = grid.max_point;
    parameters.grid_size_x = grid.grid_size_x;
    parameters.grid_size_y = grid.grid_size_y;
    parameters.grid_size_z = grid.grid_size_z;
    parameters.grid_cell_count = grid.grid_cell_count;
    uint32_t flags = 0;
    check(clsph_gpu_sync(gpu_, &flags), "clsph_gpu_sync");
    check_flags(flags);
    device_newer = false;
  };
  auto callback = [&](const std::function<void(particle*, const simulation_parameters&, bool)>& cb,
                      bool full_frame) {
    if (!cb) return;
    scene_check = true;
    if (full_frame || transfers == transfer_policy::every_substep) {
      refresh_host();
      cb(particles, parameters, full_frame);
      host_dirty = true;
    } else {
      cb(particles, parameters, full_frame);  // frames_only: last frame's copy, not uploaded
    }
  };

  for (int i = 0; i < frame_count; ++i) {
    callback(pre_frame, true);
    for (int j = 0; (float)j < (1.f / parameters.simulation_scale); ++j) {
      callback(pre_frame, false);
      if (host_dirty) {
        check(clsph_gpu_upload(gpu_, reinterpret_cast<const clsph_particle*>(particles)),
              "clsph_gpu_upload");
        host_dirty = false;
      }
      refresh_scene();
      check(clsph_gpu_step(gpu_, 1), "clsph_gpu_step");
      device_newer = true;
      callback(post_frame, false);
    }
    callback(post_frame, true);
  }
  refresh_host();
  clsph_gpu_destroy(gpu_);
  gpu_ = nullptr;
}
