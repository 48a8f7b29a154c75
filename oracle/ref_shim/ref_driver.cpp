// oracle/_ref driver: one libclsph substep on the CPU, built from the
// reference's OWN kernel sources (compiled unchanged through cl_host_shim.hpp)
// plus a restatement of the parts that cannot compile as C++:
//   * the three kernel bodies of libclsph/kernels/sph.cl:9-112 (they use
//     OpenCL work-group built-ins), and
//   * the host orchestration of libclsph/sph_simulation.cpp:173-344
//     (it is written against cl.hpp), including the 4-pass / 128-chunk LSD
//     radix sort of sph_simulation.cpp:107-171 + kernels/sort.cl:1-59 with
//     32-bit offsets (the intended behaviour; sort.cl:42 reads the offsets
//     through a size_t pointer, which is a bug on 64-bit devices).
//
// Test infrastructure only: used in the development container to pin the
// oracle restatement (oracle/clsph_oracle.cpp) and to generate the golden
// fixtures under tests/golden/. It is never shipped or timed.
//
// Build recipe: oracle/Makefile (target `ref`), output oracle/_ref/.

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

namespace clref {
#include "cl_host_shim.hpp"

static thread_local size_t g_global_id = 0;
inline size_t get_global_id(int) { return g_global_id; }

// Reference sources, compiled as they are (include path points at
// libclsph/kernels). Order mirrors the #include list of sph.cl:1-7 minus
// sort.cl (OpenCL vector literals) and sph.cl itself (restated below).
#include "common.cl"
#include "smoothing.cl"
#include "forces.cl"
#include "collisions.cl"
#include "grid.cl"
#include "advection.cl"

// sph.cl:9-40 density_pressure. The async_work_group_copy into __local memory
// only re-reads the particle itself, so it is a plain copy here.
static void density_pressure_at(size_t i, const particle* in, particle* out,
                                const simulation_parameters& params,
                                const precomputed_kernel_values& terms,
                                const unsigned int* cell_table) {
  particle self = in[i];
  self.density = compute_density_with_grid(i, in, params, terms, cell_table);
  out[i] = self;
  out[i].pressure = params.K * (pown(self.density / params.fluid_density, 7) - 1.f);
}

// sph.cl:42-62 forces. The kernel stores a partly uninitialised private
// struct over the copied input; the intended result is "input particle with a
// new acceleration", which is what this does.
static void forces_at(size_t i, const particle* in, particle* out,
                      const simulation_parameters& params,
                      const precomputed_kernel_values& terms,
                      const unsigned int* cell_table) {
  out[i] = in[i];
  float3 a = compute_internal_forces_with_grid(i, in, params, terms, cell_table) /
             in[i].density;
  a += params.constant_acceleration;
  out[i].acceleration = a;
}

// sph.cl:64-112 advection_collision. The reference loop has no bound; this
// one stops after max_iters passes and reports it.
static bool advection_collision_at(size_t i, const particle* in, particle* out,
                                   const simulation_parameters& params,
                                   const float* normals, const float* vertices,
                                   const uint* indices, uint face_count,
                                   unsigned max_iters) {
  particle result = in[i];
  float remaining = params.time_delta * params.simulation_scale;
  float3 pos = in[i].position;
  float3 vel = in[i].intermediate_velocity;
  collision_response resp;
  unsigned iters = 0;
  bool capped = false;
  for (;;) {
    advection_result adv = advect(pos, vel, result.acceleration, params.max_velocity, remaining);
    resp = handle_collisions(adv.old_position, adv.new_position, adv.next_velocity,
                             params.restitution, remaining, normals, vertices, indices,
                             face_count);
    pos = resp.position;
    vel = resp.next_velocity;
    remaining -= resp.time_elapsed;
    result.acceleration = float3(0.f, 0.f, 0.f);
    ++iters;
    if (!resp.collision_happened) break;
    if (iters >= max_iters) { capped = true; break; }
  }
  result.velocity = (in[i].intermediate_velocity + resp.next_velocity) / 2.f;
  result.intermediate_velocity = resp.next_velocity;
  result.position = resp.position;
  out[i] = result;
  return capped;
}

}  // namespace clref

using clref::particle;
using clref::simulation_parameters;
using clref::precomputed_kernel_values;

static_assert(sizeof(particle) == 80, "particle must be the 80-byte host layout");
static_assert(sizeof(simulation_parameters) == 128, "parameter block must be 128 bytes");
static_assert(offsetof(particle, density) == 64, "density offset");
static_assert(offsetof(particle, grid_index) == 72, "grid_index offset");

// sph_simulation.cpp:107-156: 4 passes x 8-bit digits, 128 contiguous chunks,
// bucket-major exclusive scan -> stable LSD radix sort. Applied to an index
// array so that the permutation can be reported.
static void ref_radix_sort(const particle* in, particle* out, uint32_t* perm, uint32_t n) {
  const int kThreads = 128, kBuckets = 256, kWidth = 8;
  std::vector<uint32_t> cur(n), nxt(n);
  for (uint32_t i = 0; i < n; ++i) cur[i] = i;
  std::vector<uint32_t> counts((size_t)kThreads * kBuckets);
  for (int pass = 0; pass < 4; ++pass) {
    std::fill(counts.begin(), counts.end(), 0u);
    auto chunk = [&](int t, uint32_t& s, uint32_t& e) {  // sort.cl:9-20, end exclusive
      uint32_t per = n / kThreads;
      s = per * (uint32_t)t;
      e = (t == kThreads - 1) ? n : s + per;
    };
    for (int t = 0; t < kThreads; ++t) {
      uint32_t s, e;
      chunk(t, s, e);
      for (uint32_t i = s; i < e; ++i) {
        uint32_t b = (in[cur[i]].grid_index >> (pass * kWidth)) & 0xFFu;
        counts[(size_t)b * kThreads + t]++;
      }
    }
    uint32_t running = 0;
    for (size_t k = 0; k < counts.size(); ++k) {
      uint32_t c = counts[k];
      counts[k] = running;
      running += c;
    }
    for (int t = 0; t < kThreads; ++t) {
      uint32_t s, e;
      chunk(t, s, e);
      for (uint32_t i = s; i < e; ++i) {
        uint32_t b = (in[cur[i]].grid_index >> (pass * kWidth)) & 0xFFu;
        nxt[counts[(size_t)b * kThreads + t]++] = cur[i];
      }
    }
    cur.swap(nxt);
  }
  for (uint32_t i = 0; i < n; ++i) {
    out[i] = in[cur[i]];
    if (perm) perm[i] = cur[i];
  }
}

extern "C" {

// Return codes shared with the oracle: 0 ok, 1 bad argument, 2 grid >= 1024
// cells on an axis (sph_simulation.cpp:247-249 asserts), 3 cell table too
// small for the caller's buffer.
int clsph_ref_step(const void* params_in, void* params_out, const void* terms_in,
                   const float* normals, const float* vertices, const uint32_t* indices,
                   uint32_t face_count, void* particles_io, uint32_t n, uint32_t* perm_out,
                   uint32_t* cell_table_out, uint64_t cell_table_cap, void* snap_sorted,
                   void* snap_density, void* snap_forces, uint32_t max_collision_iters,
                   uint32_t* capped_out) {
  if (!params_in || !terms_in || !particles_io || n < 128) return 1;
  simulation_parameters params;
  std::memcpy(&params, params_in, sizeof(params));
  precomputed_kernel_values terms;
  std::memcpy(&terms, terms_in, sizeof(terms));
  params.particles_count = n;
  particle* host = static_cast<particle*>(particles_io);

  // sph_simulation.cpp:199-252 bounding box, padding, grid dimensions
  float cell = params.h * 2;
  float mnx, mny, mnz, mxx, mxy, mxz;
  mnx = mny = mnz = (float)std::numeric_limits<int>::max();
  mxx = mxy = mxz = (float)std::numeric_limits<int>::min();
  for (uint32_t i = 0; i < n; ++i) {
    const clref::float3 p = host[i].position;
    if (p.x < mnx) mnx = p.x;
    if (p.y < mny) mny = p.y;
    if (p.z < mnz) mnz = p.z;
    if (p.x > mxx) mxx = p.x;
    if (p.y > mxy) mxy = p.y;
    if (p.z > mxz) mxz = p.z;
  }
  mnx -= cell * 2; mny -= cell * 2; mnz -= cell * 2;
  mxx += cell * 2; mxy += cell * 2; mxz += cell * 2;
  params.min_point = clref::float3(mnx, mny, mnz);
  params.max_point = clref::float3(mxx, mxy, mxz);
  params.grid_size_x = (int)(uint32_t)((mxx - mnx) / cell);
  params.grid_size_y = (int)(uint32_t)((mxy - mny) / cell);
  params.grid_size_z = (int)(uint32_t)((mxz - mnz) / cell);
  if (params.grid_size_x >= 1024 || params.grid_size_y >= 1024 || params.grid_size_z >= 1024 ||
      params.grid_size_x < 0 || params.grid_size_y < 0 || params.grid_size_z < 0)
    return 2;
  params.grid_cell_count = clref::get_grid_index_z_curve(params.grid_size_x, params.grid_size_y,
                                                         params.grid_size_z);
  if (params_out) std::memcpy(params_out, &params, sizeof(params));

  std::vector<particle> front(host, host + n), back(n);
  // locate_in_grid (grid.cl:43-67), run once per global id
  for (uint32_t i = 0; i < n; ++i) {
    clref::g_global_id = i;
    clref::locate_in_grid(front.data(), back.data(), params);
  }
  ref_radix_sort(back.data(), front.data(), perm_out, n);
  if (snap_sorted) std::memcpy(snap_sorted, front.data(), sizeof(particle) * n);

  // sph_simulation.cpp:162-170 dense cell table
  std::vector<unsigned int> table(params.grid_cell_count);
  {
    unsigned int at = 0;
    for (unsigned int c = 0; c < params.grid_cell_count; ++c) {
      table[c] = at;
      while (at != n && front[at].grid_index == c) ++at;
    }
  }
  if (cell_table_out) {
    if (cell_table_cap < params.grid_cell_count) return 3;
    std::memcpy(cell_table_out, table.data(), sizeof(unsigned int) * params.grid_cell_count);
  }

#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i)
    clref::density_pressure_at((size_t)i, front.data(), back.data(), params, terms, table.data());
  if (snap_density) std::memcpy(snap_density, back.data(), sizeof(particle) * n);

#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i)
    clref::forces_at((size_t)i, back.data(), front.data(), params, terms, table.data());
  if (snap_forces) std::memcpy(snap_forces, front.data(), sizeof(particle) * n);

  uint32_t capped = 0;
  const unsigned iters = max_collision_iters ? max_collision_iters : 1000000u;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : capped)
  for (int64_t i = 0; i < (int64_t)n; ++i)
    capped += clref::advection_collision_at((size_t)i, front.data(), back.data(), params,
                                            normals, vertices, indices, face_count, iters)
                  ? 1u
                  : 0u;
  if (capped_out) *capped_out = capped;
  std::memcpy(host, back.data(), sizeof(particle) * n);
  return 0;
}

uint32_t clsph_ref_morton(uint32_t x, uint32_t y, uint32_t z) {
  return clref::get_grid_index_z_curve(x, y, z);
}

void clsph_ref_cell_coords(uint32_t key, uint32_t* xyz) {
  clref::uint3 c = clref::get_cell_coords_z_curve(key);
  xyz[0] = c.x; xyz[1] = c.y; xyz[2] = c.z;
}

// Smoothing kernels of smoothing.cl evaluated once, for unit tests.
void clsph_ref_smoothing(float rx, float ry, float rz, float h, const void* terms_in, float* out9) {
  precomputed_kernel_values t;
  std::memcpy(&t, terms_in, sizeof(t));
  clref::float3 r(rx, ry, rz);
  float len = clref::length(r);
  out9[0] = clref::poly_6(len, h, t);
  clref::float3 g = clref::poly_6_gradient(r, h, t);
  out9[1] = g.x; out9[2] = g.y; out9[3] = g.z;
  out9[4] = clref::poly_6_laplacian(len, h, t);
  clref::float3 s = clref::spiky_gradient(r, h, t);
  out9[5] = s.x; out9[6] = s.y; out9[7] = s.z;
  out9[8] = clref::viscosity_laplacian(len, h, t);
}

}  // extern "C"
