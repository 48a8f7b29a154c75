/* CPU oracle for the libclsph per-substep SPH path — TEST INFRASTRUCTURE.
 *
 * A from-scratch restatement (oracle/clsph_oracle.cpp) of the reference's
 * algorithm, used only by tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg as the oracle. Nothing in the product links or calls it.
 *
 * Parity is pinned two ways: (1) against oracle/_ref, the reference's own
 * kernel sources compiled as C++ (bit-exact, development container), and
 * (2) against golden fixtures generated from oracle/_ref and committed under
 * tests/golden/ (everywhere, including the GPU host).
 *
 * All particle buffers use the reference's 80-byte host AoS `particle`
 * (libclsph/common/structures.h:42-46 with 16-byte cl_float3). The parameter
 * block is the 128-byte `simulation_parameters` (structures.h:16-40) and the
 * kernel constants the 20-byte `precomputed_kernel_values` (structures.h:48-54).
 */
#ifndef CLSPH_ORACLE_H
#define CLSPH_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One substep (sph_simulation.cpp:173-344). Status: 0 ok, 1 bad argument,
 * 2 grid >= 1024 cells on an axis, 3 cell_table_out too small.
 * particles_io: in = host AoS, out = AoS after the substep (sorted order).
 * Optional outputs (NULL to skip): params_out (grid fields filled),
 * perm_out[n] (sorted slot -> input slot), cell_table_out[grid_cell_count],
 * snap_sorted / snap_density / snap_forces (AoS after each phase).
 * max_collision_iters: cap of the advect/collide loop (0 = 1e6).
 * threads: OpenMP threads (<= 0: runtime default). */
int clsph_oracle_step(const void* params_in, void* params_out, const void* terms,
                      const float* face_normals, const float* vertices, const uint32_t* indices,
                      uint32_t face_count, void* particles_io, uint32_t n, uint32_t* perm_out,
                      uint32_t* cell_table_out, uint64_t cell_table_cap, void* snap_sorted,
                      void* snap_density, void* snap_forces, uint32_t max_collision_iters,
                      uint32_t* capped_out, int threads);

/* `steps` substeps back to back on the same buffer (CPU baseline timing). */
int clsph_oracle_run(const void* params_in, const void* terms, const float* face_normals,
                     const float* vertices, const uint32_t* indices, uint32_t face_count,
                     void* particles_io, uint32_t n, uint32_t steps, int threads);

/* FP64 restatement of density, Tait pressure and acceleration on an already
 * sorted AoS (e.g. snap_sorted) with the FP32 grid of params (grid fields
 * filled) and its dense cell table. Kernel constants are re-derived in double
 * from h. Outputs: density[n], pressure[n], accel[3n]. */
int clsph_oracle_fields_f64(const void* params, const void* sorted_aos, uint32_t n,
                            const uint32_t* cell_table, double* density, double* pressure,
                            double* accel, int threads);

/* sph_simulation.cpp:490-505: derived parameters from the JSON numbers.
 * params_io has the JSON fields filled; h, time_delta, max_velocity,
 * total_mass are written, terms_out gets the 5 kernel constants. */
void clsph_oracle_derive(void* params_io, void* terms_out, int particles_inside_influence_radius,
                         float* initial_volume_out);

/* sph_simulation.cpp:48-94 cube lattice used when no last_frame.bin exists. */
void clsph_oracle_init_lattice(void* particles_out, uint32_t n, float initial_volume);

uint32_t clsph_oracle_morton(uint32_t x, uint32_t y, uint32_t z);
void clsph_oracle_cell_coords(uint32_t key, uint32_t* xyz);

#ifdef __cplusplus
}
#endif
#endif
