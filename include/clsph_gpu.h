/* clsph_gpu.h — C ABI of the GB300 (sm_103a) SPH substep engine.
 *
 * This is the boundary between the reference-compatible C++ host layer
 * (sph_simulation, scene, houdini_file_saver; include/clsph/) and the CUDA
 * kernels. Plain C: opaque handle, plain pointers and sizes, int status.
 * Every function returns 0 (CLSPH_OK) or a CLSPH_ERR_* code and never exits.
 *
 * Byte formats are the reference's own shared host/device structs:
 *   clsph_particle     = particle                    (libclsph/common/structures.h:42-46), 80 B
 *   clsph_parameters   = simulation_parameters       (structures.h:16-40), 128 B
 *   clsph_kernel_terms = precomputed_kernel_values   (structures.h:48-54), 20 B
 *
 * One call of clsph_gpu_step(h, 1) is one call of the reference's
 * sph_simulation::simulate_single_frame (libclsph/sph_simulation.cpp:173-344):
 * bounding box + grid, Morton keys, stable sort, cell offsets, density and
 * Tait pressure, internal forces, leapfrog + mesh collision. Particles stay
 * resident in device memory between substeps; host transfers happen only in
 * clsph_gpu_upload / clsph_gpu_download.
 */
#ifndef CLSPH_GPU_H
#define CLSPH_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  float s[4];
} clsph_float3; /* cl_float3: 16 bytes, .s[3] unused */

typedef struct {
  clsph_float3 position, velocity, intermediate_velocity, acceleration;
  float density, pressure;
  uint32_t grid_index;
  uint32_t padding_;
} clsph_particle;

typedef struct {
  uint32_t particles_count;
  float max_velocity, fluid_density, total_mass, particle_mass, dynamic_viscosity,
      simulation_time, target_fps, h, simulation_scale, time_delta, surface_tension_threshold,
      surface_tension, restitution, K;
  float padding_;
  clsph_float3 constant_acceleration;
  int32_t grid_size_x, grid_size_y, grid_size_z;
  uint32_t grid_cell_count;
  clsph_float3 min_point, max_point;
} clsph_parameters;

typedef struct {
  float poly_6, poly_6_gradient, poly_6_laplacian, spiky, viscosity;
} clsph_kernel_terms;

typedef struct clsph_gpu clsph_gpu;

/* Status codes. Values >= 256 are hard errors; the low bits are sticky
 * device-side conditions reported by clsph_gpu_sync (they may be OR-ed). */
enum {
  CLSPH_OK = 0,
  CLSPH_WARN_GRID_OVERFLOW = 1,  /* a grid axis reached 1024 cells: keys wrap
                                    (the reference asserts, sph_simulation.cpp:247-249) */
  CLSPH_WARN_COLLISION_CAP = 2,  /* an advect/collide loop hit its iteration cap
                                    (the reference loop is unbounded, sph.cl:82-101) */
  CLSPH_WARN_NONFINITE = 4,      /* a non-finite position was seen */
  CLSPH_ERR_ARGUMENT = 256,
  CLSPH_ERR_CUDA = 512,
  CLSPH_ERR_NO_DEVICE = 1024,
  CLSPH_ERR_STATE = 2048,        /* call out of order (e.g. step before upload) */
  CLSPH_ERR_TOO_LARGE = 4096
};

/* Stages for clsph_gpu_step_until (parity inspection). */
enum {
  CLSPH_STAGE_GRID = 1,    /* bbox, grid parameters, keys */
  CLSPH_STAGE_SORT = 2,    /* stable sort, gather, cell offsets */
  CLSPH_STAGE_DENSITY = 3, /* density + pressure */
  CLSPH_STAGE_FORCES = 4,  /* acceleration */
  CLSPH_STAGE_ADVECT = 5   /* leapfrog + collision = full substep */
};

/* Replaces the context/queue/program/buffer set-up of sph_simulation::simulate
 * (sph_simulation.cpp:346-380). Allocates all device memory for up to n
 * particles on the current CUDA device; no allocation happens per substep.
 * params: the derived parameter block of sph_simulation::load_settings
 * (sph_simulation.cpp:405-505); particles_count is replaced by n. */
int clsph_gpu_create(const clsph_parameters* params, const clsph_kernel_terms* terms, uint32_t n,
                     clsph_gpu** out);

/* S independent scenes in one handle (no counterpart in the reference, which
 * runs one scene per sph_simulation): params[s], terms[s] and counts[s] are
 * scene s's derived parameter block, kernel constants and particle count.
 * Every substep runs all scenes in the same kernel launches; scene s's
 * particles are slots [sum(counts[<s]), sum(counts[<=s])) of the AoS given to
 * upload/download, and each scene's result is the one a handle of its own
 * would produce (own grid, own sort order, own mesh). S <= 65535. */
int clsph_gpu_create_batched(const clsph_parameters* params, const clsph_kernel_terms* terms,
                             const uint32_t* counts, uint32_t nscenes, clsph_gpu** out);
int clsph_gpu_destroy(clsph_gpu* h);

/* Cap of the advect/collide loop per particle and substep (default 1024).
 * The reference loop is unbounded (kernels/sph.cl:82-101); a particle that
 * reaches the cap keeps its last position and CLSPH_WARN_COLLISION_CAP is
 * raised. */
int clsph_gpu_set_collision_cap(clsph_gpu* h, uint32_t max_iterations);

/* Launch stream (a cudaStream_t); NULL selects the handle's own stream. */
int clsph_gpu_set_stream(clsph_gpu* h, void* cuda_stream);

/* Replaces the per-substep mesh buffers of sph_simulation.cpp:296-319: the
 * scene (scene.h:11-14 arrays) stays on the device, indexed by a per-cell
 * triangle list, until it is set again (the host layers set it again when a
 * callback has changed current_scene). Face order is kept, so hit selection
 * equals the reference's brute-force loop (collisions.cl:21-87). Synchronises
 * the handle's stream. */
int clsph_gpu_set_mesh(clsph_gpu* h, const float* face_normals, const float* vertices,
                       uint32_t vertex_count, const uint32_t* indices, uint32_t face_count);
/* The mesh of one scene of a batched handle (clsph_gpu_set_mesh = scene 0). */
int clsph_gpu_set_scene_mesh(clsph_gpu* h, uint32_t scene, const float* face_normals,
                             const float* vertices, uint32_t vertex_count, const uint32_t* indices,
                             uint32_t face_count);

/* Replay substeps from a CUDA graph of two captured substeps (1) or launch
 * every kernel (0, default). The graph is captured on the first clsph_gpu_step
 * of at least two substeps and re-captured when the collision cap changes;
 * it is bypassed while profiling. */
int clsph_gpu_set_graph(clsph_gpu* h, int enabled);

/* Replaces the enqueueWriteBuffer of sph_simulation.cpp:195-197: host AoS ->
 * device. `particles` points to n clsph_particle (only position, velocity and
 * intermediate_velocity are read, as in the reference). Pageable memory is
 * copied before the call returns; pinned (page-locked, 16-byte aligned)
 * memory is read by a kernel on the handle's stream, so it must stay
 * unchanged until the stream gets there, as with any asynchronous copy. */
int clsph_gpu_upload(clsph_gpu* h, const clsph_particle* particles);

/* Replaces the enqueueReadBuffer of sph_simulation.cpp:339-341: device -> host
 * AoS in the current (sorted) order, with density, pressure and grid_index of
 * the last substep and acceleration = 0, as the reference leaves them.
 * Pinned destinations are written by the packing kernel in place, pageable
 * ones through a staging copy. Synchronises the stream. */
int clsph_gpu_download(clsph_gpu* h, clsph_particle* particles);

/* `substeps` calls of simulate_single_frame (sph_simulation.cpp:173-344) with
 * no host round trip in between. Asynchronous on the handle's stream. */
int clsph_gpu_step(clsph_gpu* h, uint32_t substeps);

/* One substep run up to and including `stage` (CLSPH_STAGE_*), for parity
 * inspection with the read functions below. */
int clsph_gpu_step_until(clsph_gpu* h, int stage);

/* Waits for the stream; *flags (may be NULL) receives the sticky
 * CLSPH_WARN_* bits accumulated since the last call, which are then cleared. */
int clsph_gpu_sync(clsph_gpu* h, uint32_t* flags);

/* Replaces the parameter block and kernel constants between substeps. The
 * reference hands `parameters` and `precomputed_terms` to its kernels by value
 * every substep (sph_simulation.cpp:282-337), so a program that edits them
 * between substeps (gravity, viscosity, restitution, time step, ...) sees the
 * change at the next substep; the host layers call this when a callback has
 * changed them. The particle count of a scene cannot change
 * (CLSPH_ERR_ARGUMENT: the reference's buffers have a fixed size too); the
 * grid fields are recomputed every substep and ignored here. The per-cell
 * triangle lists stay valid for any value (a segment longer than the lists'
 * reach, which follows from max_velocity and the time step at set_mesh,
 * tests every face). Synchronises the handle's stream. */
int clsph_gpu_set_parameters(clsph_gpu* h, const clsph_parameters* params, const clsph_kernel_terms* terms);
int clsph_gpu_set_scene_parameters(clsph_gpu* h, uint32_t scene, const clsph_parameters* params,
                                   const clsph_kernel_terms* terms);

/* The parameter block with the grid of the last substep (min_point,
 * max_point, grid_size_*, grid_cell_count), as sph_simulation keeps it. */
int clsph_gpu_get_parameters(clsph_gpu* h, clsph_parameters* out);
int clsph_gpu_get_scene_parameters(clsph_gpu* h, uint32_t scene, clsph_parameters* out);

/* Inspection (synchronising). keys: sorted grid_index (the scene's Morton
 * key) per slot; perm: sorted slot -> slot before the sort (may be NULL). */
int clsph_gpu_read_keys(clsph_gpu* h, uint32_t* keys, uint32_t* perm);

/* The reference's dense cell table (sph_simulation.cpp:162-170) rebuilt from
 * the device cell index: table[c] = first sorted slot with key >= c, for
 * c < grid_cell_count. Needs cap >= grid_cell_count. Debug path: allocates. */
int clsph_gpu_read_cell_table(clsph_gpu* h, uint32_t* table, uint64_t cap);
/* The same for one scene of a batched handle: slots relative to the scene's
 * first slot. */
int clsph_gpu_read_cell_table_scene(clsph_gpu* h, uint32_t scene, uint32_t* table, uint64_t cap);

/* density[n], pressure[n], accel[4n] (x, y, z, 0) of the last substep; any
 * pointer may be NULL. accel is valid after CLSPH_STAGE_FORCES. */
int clsph_gpu_read_fields(clsph_gpu* h, float* density, float* pressure, float* accel);

/* Persistent particle ids per slot (identity at the first upload; they follow
 * the particles through every sort). */
int clsph_gpu_read_ids(clsph_gpu* h, uint32_t* ids);

/* Per-kernel timing with CUDA events on the launch stream (0 = off). While
 * on, clsph_gpu_kernel_times fills ms[i] with the summed duration of kernel
 * class i and counts[i] with its launch count since the last reset. */
int clsph_gpu_set_profiling(clsph_gpu* h, int enabled);
int clsph_gpu_kernel_times(clsph_gpu* h, int max_classes, char* names, int name_stride,
                           float* ms, uint32_t* counts, int* n_classes);

/* Autotuner (no counterpart in the reference): times the density kernel in
 * every neighbour search mode and the density and forces kernels at
 * 64/128/256 threads per block, and the
 * advection grid at 4/8/16 blocks per SM, `substeps` substeps per trial, on
 * the handle's current
 * particles, keeps the fastest shapes and restores the particle state (the
 * trials leave the simulation where it was). `report` (may be NULL) receives
 * the timings as text. Requires an uploaded state. */
int clsph_gpu_autotune(clsph_gpu* h, uint32_t substeps, char* report, int report_len);

/* Sets the launch shapes directly (e.g. from a cached autotune result):
 * blocks of 64, 128 or 256 threads; 1..64 advection blocks per SM. */
int clsph_gpu_set_launch_shape(clsph_gpu* h, int density_block, int forces_block,
                               uint32_t advect_blocks_per_sm);

/* Neighbour search of the density kernel (no counterpart in the reference;
 * all modes give bit-identical results, they differ only in speed):
 *  WINDOW: one thread per particle walks its 2x2x2 window of cells and skips
 *    the particles in each neighbour cell's far half by their half-cell code;
 *  CELL_WARPS: one warp per occupied cell stages each neighbour cell's facing
 *    half in shared memory once for all of the cell's particles. The default;
 *  PARTICLE_WARPS: one warp per particle tests 32 candidates at a time (for
 *    scenes too small to fill the GPU otherwise).
 * The density block size of clsph_gpu_set_launch_shape sets WINDOW's block
 * (64 or 128 threads; 256 runs as 128) and CELL_WARPS' staging tiles per
 * block (64 / 128 / 256 threads = 2 / 4 / 8 warps, each staging 32
 * candidates at a time); clsph_gpu_autotune tries every combination. */
enum {
  CLSPH_SEARCH_WINDOW = 0,
  CLSPH_SEARCH_CELL_WARPS = 1,
  CLSPH_SEARCH_PARTICLE_WARPS = 2
};
int clsph_gpu_set_neighbour_search(clsph_gpu* h, int mode);

/* Runs whole substeps as one persistent launch (no counterpart in the
 * reference): every phase of the substep in one cooperative kernel of 256-
 * thread blocks, all resident at once, separated by grid-wide barriers,
 * up to 64 substeps per launch, for handles of any number of scenes. The
 * results equal the launched substeps' bit for bit (the same block-level
 * code); clsph_gpu_autotune keeps whichever form is faster. Neighbour search
 * is CELL_WARPS with 8 warps per block; per-kernel profiling and
 * clsph_gpu_step_until launch the kernels as usual. CLSPH_ERR_CUDA if the
 * device has no cooperative launch. */
int clsph_gpu_set_persistent(clsph_gpu* h, int enabled);

/* Bound of each grid-barrier wait of the persistent launch (default
 * CLSPH_DEFAULT_BARRIER_SPINS, about seconds) and a test hook of its failure
 * path: block `withheld_block` (CLSPH_NO_BLOCK in normal use) leaves at the
 * first barrier, as a block that never arrives, so every other block's wait
 * runs out; clsph_gpu_sync then returns CLSPH_ERR_CUDA and resets the
 * barrier. */
#define CLSPH_DEFAULT_BARRIER_SPINS (1u << 22)
#define CLSPH_NO_BLOCK 0xFFFFFFFFu
int clsph_gpu_set_barrier_limits(clsph_gpu* h, uint32_t barrier_spins, uint32_t withheld_block);

/* The per-cell triangle lists of a scene's mesh, as built on the device by
 * clsph_gpu_set_scene_mesh (an inspection call: the collision loop of
 * libclsph/kernels/collisions.cl:91-129 scans every face; the engine scans
 * the list of the cell a segment starts in, which holds, in ascending order,
 * every face whose box grown by the list reach and a tolerance meets the
 * cell). sizes[0] = cells + 1 (CSR starts), sizes[1] = list entries (both 0
 * without lists: an empty or non-finite mesh); plan (10 floats, may be NULL)
 * = grid origin xyz, cell edge, pad, tolerance, dims xyz, reach. A NULL
 * cell_start or cell_faces skips that copy. */
int clsph_gpu_read_face_lists(clsph_gpu* h, uint32_t scene, float* plan, uint32_t* cell_start,
                              uint64_t start_cap, uint32_t* cell_faces, uint64_t faces_cap, uint32_t* sizes);

/* Bounds of the engine's device-side waits; no counterpart in the reference,
 * whose OpenCL queue has no device-side waits. radix_lookback_spins bounds
 * each radix-sort look-back wait (default CLSPH_DEFAULT_LOOKBACK_SPINS): a
 * wait that runs out leaves that substep's order wrong, keeps every access in
 * bounds and makes the next clsph_gpu_sync return CLSPH_ERR_CUDA.
 * mlp_wait_polls bounds each mbarrier wait of the learned stepper's tcgen05
 * MLP kernel (default CLSPH_DEFAULT_MLP_WAIT_POLLS; 0 gives up at once): a wait
 * that runs out makes clsph_gpu_step_learned return CLSPH_ERR_CUDA.
 * radix_withheld_tile (CLSPH_NO_TILE in normal use) is a test hook of the
 * failure path: that tile of every radix pass never publishes its digit
 * counts, so the tile after it waits on a word nothing sets until its bound
 * runs out. Takes effect at the next launch (cached graphs are rebuilt). */
#define CLSPH_DEFAULT_LOOKBACK_SPINS (1u << 20)
#define CLSPH_DEFAULT_MLP_WAIT_POLLS (1u << 24)
#define CLSPH_NO_TILE 0xFFFFFFFFu
int clsph_gpu_set_wait_limits(clsph_gpu* h, uint32_t radix_lookback_spins, uint32_t mlp_wait_polls,
                              uint32_t radix_withheld_tile);

/* Counters since create: [0] substeps, [1] particles whose collision loop hit
 * the cap, [2] kernel launches. */
int clsph_gpu_counters(clsph_gpu* h, uint64_t* out3);

/* Stable sort of n device-resident 32-bit keys that allocates no memory.
 * No counterpart in the reference: it exists for callers that may not call
 * cudaMalloc themselves (a host application or framework that owns every
 * device allocation and forbids raw cudaMalloc/cudaFree, or a real-time loop
 * that must not allocate after start-up). It is the substep's stable sort
 * (the 4 x 8-bit LSD radix sort) on caller buffers: keys_out receives the
 * keys in ascending order, perm_out[s] the input index of sorted slot s
 * (equal keys keep input order). keys_in must not overlap the outputs.
 * Scratch comes from one 8.3 MB file-scope __device__ array held by every GPU
 * that loads the library until exit; n above 1,048,576 is rejected with
 * CLSPH_ERR_TOO_LARGE. All calls share that array (each clears what must
 * start at zero): calls whose GPU work overlaps race, so serialise them. The
 * first call on a device looks the array up (cudaGetSymbolAddress) with that
 * device current; make it before any stream capture. The address is kept for
 * the life of the process: after cudaDeviceReset the device's code is loaded
 * anew and that address is stale, so a process that resets a device must not
 * call this function on it again. Asynchronous on
 * `cuda_stream` (a cudaStream_t, NULL = legacy default stream). */
int clsph_gpu_sort_keys_noalloc(const uint32_t* keys_in, uint32_t* keys_out, uint32_t* perm_out,
                                uint32_t n, void* cuda_stream);

/* Text of the last error on this thread. */
const char* clsph_gpu_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* CLSPH_GPU_H */
