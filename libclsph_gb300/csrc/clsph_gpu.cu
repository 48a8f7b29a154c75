// C ABI of the GB300 SPH substep engine (include/clsph_gpu.h).
//
// One handle owns every device buffer for its particles (allocated once at
// create), the scene meshes with their per-cell triangle lists, and a
// stream. A handle runs S independent scenes (S = 1 for clsph_gpu_create):
// every kernel of a substep covers all scenes in one launch.
// clsph_gpu_step enqueues the substep kernels of clsph_kernels.cuh, replayed
// from a CUDA graph when enabled; no host round trip and no allocation
// happens between substeps.

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "clsph_gpu.h"
#include "clsph_handle.cuh"
#include "clsph_mesh.cuh"

static_assert(sizeof(clsph_particle) == 80, "particle layout");
static_assert(sizeof(clsph_parameters) == 128, "parameter layout");
static_assert(offsetof(clsph_parameters, constant_acceleration) == 64, "parameter layout");
static_assert(offsetof(clsph_parameters, grid_size_x) == 80, "parameter layout");
static_assert(offsetof(clsph_parameters, min_point) == 96, "parameter layout");
static_assert(sizeof(clsph_kernel_terms) == 20, "kernel constant layout");
static_assert(kRadixLookbackSpins == CLSPH_DEFAULT_LOOKBACK_SPINS, "default look-back bound");
static_assert(kNoTile == CLSPH_NO_TILE, "withheld-tile sentinel");
static_assert(kBarrierSpins == CLSPH_DEFAULT_BARRIER_SPINS, "default barrier bound");
static_assert(kNoBlock == CLSPH_NO_BLOCK, "withheld-block sentinel");

namespace clsph_host {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

const char* kKernelNames[K_NUM_CLASSES] = {
    "grid_setup", "keys",       "radix_hist",  "radix_sweep",    "gather",
    "density",    "forces",     "advect",      "unpack_aos",     "pack_aos",      "misc",
    "features",   "mlp",        "learned_advect", "gate"};

}  // namespace clsph_host

// Error text for clsph_gpu_last_error from the library's other translation units.
void clsph_set_last_error(const std::string& msg) { clsph_host::g_last_error = msg; }
namespace {

Consts derive_consts(const clsph_parameters& p, const clsph_kernel_terms& t, uint32_t n) {
  Consts c{};
  c.n = n;
  c.h = p.h;
  c.mass = p.particle_mass;
  c.rho0 = p.fluid_density;
  c.K = p.K;
  c.mu = p.dynamic_viscosity;
  c.sigma = p.surface_tension;
  c.sigma_threshold = p.surface_tension_threshold;
  c.restitution = p.restitution;
  c.time_delta = p.time_delta;
  c.scale = p.simulation_scale;
  c.vmax = p.max_velocity;
  c.gx = p.constant_acceleration.s[0];
  c.gy = p.constant_acceleration.s[1];
  c.gz = p.constant_acceleration.s[2];
  c.poly6 = t.poly_6;
  c.grad6 = t.poly_6_gradient;
  c.lap6 = t.poly_6_laplacian;
  c.spiky = t.spiky;
  c.visc = t.viscosity;
  // smoothing.cl:24: -45 / (float)(M_PI * pown(h, 6)) with M_PI in double
  c.spiky_zero = -45.f / (float)(M_PI * (double)pown_f(p.h, 6));
  // conservative h^2 of the FMA culls: 5e-4 above h^2, five times the largest
  // rounding of the cell-relative cull (k_density_cells) and far above that
  // of the direct differences; the exact test decides
  c.cull_r2 = p.h * p.h * 1.0005f;
  return c;
}

}  // namespace

int clsph_host::enqueue_substep(clsph_gpu* h, int until) {
  const uint32_t n = h->n;
  const uint32_t blocks = grid_blocks(n);
  const uint32_t* cctl = h->ctl;
  h->launch(K_GRID_SETUP, k_grid_setup, dim3(1), dim3(256), h->bbox, h->grids,
            (const float*)h->scene_h, h->nscenes, h->status, h->digit_total, h->step_counters,
            h->ctl);
  // k_keys also clears the cell index (slots is a power of two >= 1024)
  h->launch(K_KEYS, k_keys, dim3(blocks), dim3(kBlock), (const float4*)h->st[0].pos, n,
            (const DevGrid*)h->grids, (const uint16_t*)h->scene_of, h->ctl, h->keys,
            reinterpret_cast<uint4*>(h->ci.keys), h->slots / 4u);
  if (until <= CLSPH_STAGE_GRID) return 0;
  h->launch(K_RADIX_HIST, k_radix_hist, dim3(grid_blocks((n + 3) / 4, h->sm_count * 4)), dim3(kRadixThreads),
            (const uint32_t*)h->keys, n, cctl, h->digit_total, h->lookback, h->ntiles);
  for (int pass = 0; pass < 4; ++pass)
    h->launch(K_RADIX_SWEEP, k_radix_onesweep, dim3(h->ntiles), dim3(kRadixThreads), h->keys, h->vals, n,
              pass, cctl, (const uint32_t*)h->digit_total, h->lookback, h->ntiles,
              h->step_counters + kCntRadixTile + pass, h->status, h->radix_spin_limit,
              h->radix_withheld_tile);
  const int src_ids = h->ids_sel, dst_ids = h->ids_sel ^ 1;
  h->launch(K_GATHER, k_gather, dim3(blocks), dim3(kBlock), n, (const DevGrid*)h->grids,
            (const uint16_t*)h->scene_of, cctl, (const uint32_t*)h->keys,
            (const uint32_t*)h->vals, h->st[0], h->st[1], (const uint32_t*)h->ids[src_ids],
            h->ids[dst_ids], h->ci, h->cell_list, h->step_counters + kCntCells);
  h->ids_sel = dst_ids;
  if (until <= CLSPH_STAGE_SORT) return 0;
  {
    // the window mode's per-thread tables fit shared memory up to 128 threads
    const int b = h->density_block == 64 ? 64 : 128;
    const dim3 grid((n + b - 1) / b);
    auto args = [&](auto kernel) {
      h->launch(K_DENSITY, kernel, grid, dim3(b), n, (const DevGrid*)h->grids,
                (const uint16_t*)h->scene_of, cctl, (const uint32_t*)h->keys,
                (const float4*)h->st[1].pos, h->ci, (const Consts*)h->consts, h->aux, h->nlist,
                h->ncount, h->nlist_cap, (const float4*)h->st[1].vel, h->frec, h->nb_start);
    };
    // cell-warp mode: the block size sets the warps (cell staging tiles) per
    // block, 2, 4 or 8, each with its own 32-candidate tile and buffers
    auto cells = [&](auto kernel, int warps) {
      h->launch(K_DENSITY, kernel, dim3(h->sm_count * (64 / warps)), dim3(warps * 32),
                n, (const DevGrid*)h->grids, (const uint16_t*)h->scene_of, cctl,
                (const uint32_t*)h->keys, (const float4*)h->st[1].pos, h->ci,
                (const Consts*)h->consts, h->aux, h->nlist, h->ncount, h->nlist_cap,
                (const float4*)h->st[1].vel, h->frec, (const uint32_t*)h->cell_list,
                h->step_counters, h->nb_start);
    };
    if (h->search == CLSPH_SEARCH_CELL_WARPS) {
      if (h->density_block == 64) cells(k_density_cells<2>, 2);
      else if (h->density_block == 256) cells(k_density_cells<8>, 8);
      else cells(k_density_cells<kCellWarps>, kCellWarps);
    } else if (h->search == CLSPH_SEARCH_PARTICLE_WARPS) {
      h->launch(K_DENSITY, k_density_pwarp, dim3((n + kParticleWarps - 1) / kParticleWarps),
                dim3(kParticleWarps * 32), n, (const DevGrid*)h->grids, (const uint16_t*)h->scene_of,
                cctl, (const uint32_t*)h->keys, (const float4*)h->st[1].pos, h->ci,
                (const Consts*)h->consts, h->aux, h->nlist, h->ncount, h->nlist_cap,
                (const float4*)h->st[1].vel, h->frec, h->nb_start);
    } else {
      if (b == 64) args(k_density<64>);
      else args(k_density<128>);
    }
  }
  if (until <= CLSPH_STAGE_DENSITY) return 0;
  {
    const int b = h->forces_block;
    const dim3 grid((n + b - 1) / b);
    auto args = [&](auto kernel) {
      h->launch(K_FORCES, kernel, grid, dim3(b), n, (const DevGrid*)h->grids,
                (const uint16_t*)h->scene_of, cctl, (const uint32_t*)h->keys, h->st[1],
                (const float4*)h->aux, h->ci, (const Consts*)h->consts, (const uint16_t*)h->nlist,
                (const uint32_t*)h->ncount, h->nlist_cap, h->acc, NoForceHook{}, (const float4*)h->frec,
                (const uint32_t*)h->nb_start);
    };
    if (b == 64) args(k_forces<64>);
    else if (b == 256) args(k_forces<256>);
    else args(k_forces<128>);
  }
  if (until <= CLSPH_STAGE_FORCES) return 0;
  return enqueue_advect(h);
}

// Runs `substeps` substeps as one persistent cooperative launch per at most
// 64 substeps (clsph_persistent.cuh).
int clsph_host::launch_persistent(clsph_gpu* h, uint32_t substeps) {
  if (!h->persist_blocks) {
    int per_sm = 0, coop = 0;
    CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, h->device));
    if (!coop) return fail(CLSPH_ERR_CUDA, "persistent substeps: the device has no cooperative launch");
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_substeps_persistent, kPersistThreads, 0));
    if (per_sm < 1) return fail(CLSPH_ERR_CUDA, "persistent substeps: no resident block fits an SM");
    h->persist_blocks = (uint32_t)per_sm * h->sm_count;
  }
  PersistArgs a{};
  a.n = h->n;
  a.nscenes = h->nscenes;
  a.ntiles = h->ntiles;
  a.slots = h->slots;
  a.nlist_cap = h->nlist_cap;
  a.max_iters = h->max_iters;
  a.bbox = h->bbox;
  a.grids = h->grids;
  a.scene_h = h->scene_h;
  a.status = h->status;
  a.digit_total = h->digit_total;
  a.step_counters = h->step_counters;
  a.ctl = h->ctl;
  a.scene_of = h->scene_of;
  a.keys = h->keys;
  a.vals = h->vals;
  a.lookback = h->lookback;
  a.st[0] = h->st[0];
  a.st[1] = h->st[1];
  a.ids[0] = h->ids[0];
  a.ids[1] = h->ids[1];
  a.ci = h->ci;
  a.cell_list = h->cell_list;
  a.consts = h->consts;
  a.aux = h->aux;
  a.nlist = h->nlist;
  a.ncount = h->ncount;
  a.frec = h->frec;
  a.nb_start = h->nb_start;
  a.acc = h->acc;
  a.meshes = h->meshes;
  a.capped = h->capped;
  a.barrier = h->pbar;
  a.spin_limit = h->radix_spin_limit;
  a.withheld_tile = h->radix_withheld_tile;
  a.barrier_limit = h->barrier_limit;
  a.withheld_block = h->withheld_block;
  for (uint32_t done = 0; done < substeps;) {
    uint32_t count = std::min<uint32_t>(substeps - done, 64u);
    uint32_t sel = (uint32_t)h->ids_sel;
    void* args[] = {&a, &count, &sel};
    CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_substeps_persistent, dim3(h->persist_blocks),
                                         dim3(kPersistThreads), args, 0, h->stream));
    ++h->launches;
    h->ids_sel ^= (int)(count & 1u);
    done += count;
  }
  return 0;
}

int clsph_host::enqueue_advect(clsph_gpu* h) {
  const uint32_t n = h->n;
  h->launch(K_ADVECT, k_advect<false>, dim3(grid_blocks(n, h->sm_count * h->advect_blocks_per_sm)),
            dim3(kBlock), n, h->st[1],
            (const float4*)h->acc, h->st[0], (const DevMesh*)h->meshes, (const Consts*)h->consts,
            (const uint16_t*)h->scene_of, h->max_iters, h->bbox, h->status, h->capped,
            (const float4*)nullptr, 1.f, 1.f, (const float4*)nullptr, (const float*)nullptr);
  return 0;
}

int clsph_host::check_launch(clsph_gpu* h) {
  (void)h;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(CLSPH_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  return 0;
}

namespace {

// An even number of substeps (kGraphLen[kind]) captured once and replayed.
// The particle ids alternate between their two buffers, so an even count
// returns them to the buffer it started from; there is one graph per
// starting buffer.
int ensure_graph(clsph_gpu* h, int kind) {
  const int par = h->ids_sel;
  cudaGraphExec_t& ge = h->graph_exec[kind][par];
  if (ge && h->graph_max_iters[kind][par] == h->max_iters) return 0;
  if (ge) cudaGraphExecDestroy(ge);
  ge = nullptr;
  cudaGraph_t graph = nullptr;
  CUDA_TRY(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  const uint64_t launches = h->launches;
  int rc = 0;
  for (uint32_t k = 0; k < clsph_gpu::kGraphLen[kind] && !rc; ++k) rc = enqueue_substep(h, CLSPH_STAGE_ADVECT);
  h->graph_launches[kind][par] = h->launches - launches;
  h->launches = launches;
  cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
  if (rc) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (e != cudaSuccess) return fail(CLSPH_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(&ge, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    ge = nullptr;
    return fail(CLSPH_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  }
  h->graph_max_iters[kind][par] = h->max_iters;
  return 0;
}

int read_grid(clsph_gpu* h, uint32_t scene, DevGrid* g, uint32_t* ctl) {
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  if (g) CUDA_TRY(cudaMemcpy(g, h->grids + scene, sizeof(DevGrid), cudaMemcpyDeviceToHost));
  if (ctl) CUDA_TRY(cudaMemcpy(ctl, h->ctl, sizeof(uint32_t) * kCtlWords, cudaMemcpyDeviceToHost));
  return 0;
}

// Plan of the per-cell triangle lists (clsph_mesh.cuh): a uniform grid
// around the mesh's bounding box, padded by the list reach (the longest
// segment one list serves: 1.5 x the largest distance a particle moves in a
// substep, plus 2 mm) and a rounding tolerance, with at most 2^22 cells.
// Returns 1 for a non-finite mesh (then every face is scanned).
int plan_face_grid(const clsph_parameters& p, const float* vx, uint32_t nv, const uint32_t* ix,
                   uint32_t faces, FaceGridPlan& g, float& reach) {
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (uint32_t f = 0; f < faces; ++f)
    for (int k = 0; k < 3; ++k) {
      uint32_t v = ix[3 * f + k];
      if (v >= nv) return fail(CLSPH_ERR_ARGUMENT, "mesh index out of range");
      for (int a = 0; a < 3; ++a) {
        float c = vx[3 * v + a];
        if (!std::isfinite(c)) return 1;
        lo[a] = std::fmin(lo[a], c);
        hi[a] = std::fmax(hi[a], c);
      }
    }
  float extent = 0.f;
  for (int a = 0; a < 3; ++a) extent = std::fmax(extent, hi[a] - lo[a]);
  reach = std::fmax(p.max_velocity * p.time_delta * p.simulation_scale * 1.5f + 0.002f, 1e-4f);
  const float tol = 1e-4f * extent + 1e-5f;
  const float pad = reach + tol;
  float ghi[3];
  for (int a = 0; a < 3; ++a) {
    g.glo[a] = lo[a] - pad;
    ghi[a] = hi[a] + pad;
  }
  float cell = std::fmax((extent + 2 * pad) / 128.f, pad);
  for (;;) {
    double total = 1.0;
    for (int a = 0; a < 3; ++a) {
      g.dims[a] = (int)std::ceil((ghi[a] - g.glo[a]) / cell);
      if (g.dims[a] < 1) g.dims[a] = 1;
      total *= g.dims[a];
    }
    if (total <= (double)(1u << 22)) break;
    cell *= 1.25f;
  }
  g.cell = cell;
  g.pad = pad;
  g.tol = tol;
  g.cells = (uint32_t)g.dims[0] * (uint32_t)g.dims[1] * (uint32_t)g.dims[2];
  return 0;
}

// Builds the lists of an uploaded mesh on the device (clsph_mesh.cuh) into
// sm.cell_start / sm.cell_faces.
int build_face_lists(clsph_gpu* h, SceneMesh& sm, uint32_t faces, const FaceGridPlan& g) {
  const uint32_t cells = g.cells;
  if (faces > kScanBlock * kScanThreads) return fail(CLSPH_ERR_TOO_LARGE, "face lists: more than 2^22 faces");
  uint32_t *count = nullptr, *csums = nullptr, *fill = nullptr, *face_n = nullptr, *face_start = nullptr,
           *fsums = nullptr;
  unsigned long long* entries = nullptr;
  int rc = 0;
  auto done = [&](int code) {
    void* bufs[] = {count, csums, fill, face_n, face_start, fsums, entries};
    for (void* b : bufs) cudaFree(b);
    return code;
  };
  const uint32_t cblocks = (cells + kScanBlock - 1) / kScanBlock;
  const uint32_t fblocks_scan = (faces + kScanBlock - 1) / kScanBlock;
  if ((rc = dev_alloc(&count, cells)) || (rc = dev_alloc(&csums, cblocks + 1)) || (rc = dev_alloc(&fill, cells)) ||
      (rc = dev_alloc(&face_n, faces)) || (rc = dev_alloc(&face_start, (size_t)faces + 1)) ||
      (rc = dev_alloc(&fsums, fblocks_scan + 1)) || (rc = dev_alloc(&entries, 1)) ||
      (rc = dev_alloc(&sm.cell_start, (size_t)cells + 1)))
    return done(rc);
  cudaStream_t s = h->stream;
  cudaError_t e = cudaMemsetAsync(entries, 0, sizeof(unsigned long long), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(count, 0, sizeof(uint32_t) * cells, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(fill, 0, sizeof(uint32_t) * cells, s);
  if (e != cudaSuccess) return done(fail(CLSPH_ERR_CUDA, std::string("face lists: ") + cudaGetErrorString(e)));
  k_face_entries<<<grid_blocks(faces, h->sm_count * 8), kBlock, 0, s>>>(sm.vertices, sm.indices, faces, g, face_n,
                                                                         entries);
  unsigned long long total = 0;
  e = cudaMemcpyAsync(&total, entries, sizeof(total), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return done(fail(CLSPH_ERR_CUDA, std::string("face lists: ") + cudaGetErrorString(e)));
  if (total > 0x7FFFFFFFull) return done(fail(CLSPH_ERR_TOO_LARGE, "face lists too large"));
  const uint32_t n_entries = (uint32_t)total;
  if ((rc = dev_alloc(&sm.cell_faces, total ? total : 1))) return done(rc);
  // entry starts of the faces, then the cells' counts and CSR starts
  k_scan_sums<<<fblocks_scan, kScanThreads, 0, s>>>(face_n, faces, fsums);
  k_scan_top<<<1, kScanThreads, 0, s>>>(fsums, fblocks_scan, face_start + faces);
  k_scan_apply<<<fblocks_scan, kScanThreads, 0, s>>>(face_n, faces, fsums, face_start);
  const uint32_t eblocks = grid_blocks(n_entries, h->sm_count * 16);
  k_face_count<<<eblocks, kBlock, 0, s>>>(sm.vertices, sm.indices, faces, g, face_start, n_entries, count);
  k_scan_sums<<<cblocks, kScanThreads, 0, s>>>(count, cells, csums);
  k_scan_top<<<1, kScanThreads, 0, s>>>(csums, cblocks, sm.cell_start + cells);
  k_scan_apply<<<cblocks, kScanThreads, 0, s>>>(count, cells, csums, sm.cell_start);
  k_face_fill<<<eblocks, kBlock, 0, s>>>(sm.vertices, sm.indices, faces, g, face_start, n_entries, sm.cell_start,
                                         fill, sm.cell_faces);
  k_face_sort<<<grid_blocks(cells, h->sm_count * 8), kBlock, 0, s>>>(sm.cell_start, cells, sm.cell_faces);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return done(fail(CLSPH_ERR_CUDA, std::string("face lists: ") + cudaGetErrorString(e)));
  sm.plan = g;
  sm.list_len = n_entries;
  return done(0);
}

int sync_scene_tables(clsph_gpu* h) {
  CUDA_TRY(cudaMemcpy(h->consts, h->consts_host.data(), sizeof(Consts) * h->nscenes, cudaMemcpyHostToDevice));
  CUDA_TRY(cudaMemcpy(h->meshes, h->mesh_host.data(), sizeof(DevMesh) * h->nscenes, cudaMemcpyHostToDevice));
  return 0;
}

}  // namespace

extern "C" {

const char* clsph_gpu_last_error(void) { return clsph_host::g_last_error.c_str(); }

int clsph_gpu_destroy(clsph_gpu* h);

int clsph_gpu_create_batched(const clsph_parameters* params, const clsph_kernel_terms* terms,
                             const uint32_t* counts, uint32_t nscenes, clsph_gpu** out) {
  if (!params || !terms || !counts || !out || nscenes == 0)
    return fail(CLSPH_ERR_ARGUMENT, "create: bad argument");
  if (nscenes > 65535) return fail(CLSPH_ERR_TOO_LARGE, "create: more than 65535 scenes");
  uint64_t total = 0;
  for (uint32_t s = 0; s < nscenes; ++s) {
    if (counts[s] == 0) return fail(CLSPH_ERR_ARGUMENT, "create: a scene has no particles");
    if (!(params[s].h > 0.f)) return fail(CLSPH_ERR_ARGUMENT, "create: h must be positive");
    total += counts[s];
  }
  if (total > (1u << 28)) return fail(CLSPH_ERR_TOO_LARGE, "create: more than 2^28 particles");
  int devices = 0;
  if (cudaGetDeviceCount(&devices) != cudaSuccess || devices == 0)
    return fail(CLSPH_ERR_NO_DEVICE, "create: no CUDA device");
  clsph_gpu* h = new clsph_gpu();
  cudaGetDevice(&h->device);
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device) == cudaSuccess && sms > 0)
    h->sm_count = (uint32_t)sms;
  const uint32_t n = (uint32_t)total;
  h->n = n;
  h->nscenes = nscenes;
  h->scene_first.assign(nscenes + 1, 0u);
  for (uint32_t s = 0; s < nscenes; ++s) {
    h->scene_first[s + 1] = h->scene_first[s] + counts[s];
    clsph_parameters p = params[s];
    p.particles_count = counts[s];
    h->params.push_back(p);
    h->terms.push_back(terms[s]);
    h->consts_host.push_back(derive_consts(p, terms[s], counts[s]));
  }
  h->scene_mesh.resize(nscenes);
  h->mesh_host.assign(nscenes, DevMesh{});
  int rc = 0;
  auto bail = [&](int code) {
    clsph_gpu_destroy(h);
    return code;
  };
  if (cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(CLSPH_ERR_CUDA, "create: stream"));
  h->stream = h->own_stream;
  for (int s = 0; s < 2; ++s) {
    if ((rc = dev_alloc(&h->st[s].pos, n)) || (rc = dev_alloc(&h->st[s].vel, n)) ||
        (rc = dev_alloc(&h->st[s].ivel, n)) || (rc = dev_alloc(&h->ids[s], n)))
      return bail(rc);
  }
  h->ntiles = (n + kRadixTile - 1) / kRadixTile;
  uint32_t slots = 1024;
  while (slots < 2u * n) slots <<= 1;
  h->slots = slots;
  uint32_t log2s = 0;
  while ((1u << log2s) < slots) ++log2s;
  if ((rc = dev_alloc(&h->aux, n)) || (rc = dev_alloc(&h->acc, n)) || (rc = dev_alloc(&h->frec, 2 * (size_t)n)) ||
      (rc = dev_alloc(&h->nlist, (size_t)h->nlist_cap * n)) || (rc = dev_alloc(&h->ncount, n)) ||
      (rc = dev_alloc(&h->nb_start, 27 * (size_t)n + 32)) ||  // + 32: any 5-bit cell index stays inside
      (rc = dev_alloc(&h->cell_list, n)) || (rc = dev_alloc(&h->step_counters, kStepCounters)) ||
      (rc = dev_alloc(&h->keys, 2 * (size_t)n)) || (rc = dev_alloc(&h->vals, 2 * (size_t)n)) ||
      (rc = dev_alloc(&h->lookback, 4 * 256 * (size_t)h->ntiles)) ||
      (rc = dev_alloc(&h->digit_total, 4 * 256)) || (rc = dev_alloc(&h->ci.keys, slots)) ||
      (rc = dev_alloc(&h->ci.start, slots)) || (rc = dev_alloc(&h->ci.end, slots)) ||
      (rc = dev_alloc(&h->scene_of, n)) || (rc = dev_alloc(&h->grids, nscenes)) ||
      (rc = dev_alloc(&h->consts, nscenes)) || (rc = dev_alloc(&h->scene_h, nscenes)) ||
      (rc = dev_alloc(&h->meshes, nscenes)) || (rc = dev_alloc(&h->bbox, 6 * (size_t)nscenes)) ||
      (rc = dev_alloc(&h->ctl, kCtlWords)) || (rc = dev_alloc(&h->status, 1)) ||
      (rc = dev_alloc(&h->capped, 1)) || (rc = dev_alloc(&h->aos_stage, 5 * (size_t)n)) ||
      (rc = dev_alloc(&h->pbar, 2)))
    return bail(rc);
  h->ci.mask = slots - 1;
  h->ci.shift = 32 - log2s;
  uint32_t scene_bits = 0;
  while ((1u << scene_bits) < nscenes) ++scene_bits;
  uint32_t ctl_init[kCtlWords] = {};
  ctl_init[kCtlSceneBits] = scene_bits;
  ctl_init[kCtlShift] = 1;
  std::vector<uint16_t> scene_of(n);
  std::vector<float> hs(nscenes);
  for (uint32_t s = 0; s < nscenes; ++s) {
    hs[s] = h->params[s].h;
    for (uint32_t i = h->scene_first[s]; i < h->scene_first[s + 1]; ++i) scene_of[i] = (uint16_t)s;
  }
  std::vector<uint32_t> iota(n);
  for (uint32_t i = 0; i < n; ++i) iota[i] = i;
  if (cudaMemset(h->grids, 0, sizeof(DevGrid) * nscenes) != cudaSuccess ||
      cudaMemset(h->status, 0, sizeof(uint32_t)) != cudaSuccess ||
      cudaMemset(h->pbar, 0, 2 * sizeof(uint32_t)) != cudaSuccess ||
      cudaMemset(h->capped, 0, sizeof(unsigned long long)) != cudaSuccess ||
      cudaMemset(h->aux, 0, sizeof(float4) * n) != cudaSuccess ||
      cudaMemset(h->ncount, 0, sizeof(uint32_t) * n) != cudaSuccess ||
      cudaMemset(h->keys, 0, sizeof(uint32_t) * 2 * (size_t)n) != cudaSuccess ||
      cudaMemset(h->vals, 0, sizeof(uint32_t) * 2 * (size_t)n) != cudaSuccess ||
      cudaMemset(h->acc, 0, sizeof(float4) * n) != cudaSuccess ||
      cudaMemcpy(h->ctl, ctl_init, sizeof(ctl_init), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(h->scene_of, scene_of.data(), sizeof(uint16_t) * n, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(h->scene_h, hs.data(), sizeof(float) * nscenes, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(h->ids[0], iota.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice) != cudaSuccess)
    return bail(fail(CLSPH_ERR_CUDA, "create: initialisation copies"));
  if ((rc = sync_scene_tables(h))) return bail(rc);
  *out = h;
  return CLSPH_OK;
}

int clsph_gpu_create(const clsph_parameters* params, const clsph_kernel_terms* terms, uint32_t n,
                     clsph_gpu** out) {
  if (!params || !terms || !out || n == 0) return fail(CLSPH_ERR_ARGUMENT, "create: bad argument");
  return clsph_gpu_create_batched(params, terms, &n, 1, out);
}

int clsph_gpu_destroy(clsph_gpu* h) {
  if (!h) return CLSPH_OK;
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->free_learned) h->free_learned(h);
  h->drop_graph();
  for (auto& t : h->pending) {
    cudaEventDestroy(t.start);
    cudaEventDestroy(t.stop);
  }
  for (auto e : h->event_pool) cudaEventDestroy(e);
  for (int s = 0; s < 2; ++s) {
    cudaFree(h->st[s].pos);
    cudaFree(h->st[s].vel);
    cudaFree(h->st[s].ivel);
    cudaFree(h->ids[s]);
  }
  void* bufs[] = {h->aux,      h->acc,      h->frec,      h->nlist,     h->ncount,      h->cell_list,
                  h->nb_start,
                  h->step_counters, h->keys, h->vals,     h->lookback,    h->digit_total,
                  h->ci.keys,  h->ci.start, h->ci.end,    h->scene_of,    h->grids,
                  h->consts,   h->scene_h,  h->meshes,    h->bbox,        h->ctl,
                  h->status,   h->capped,   h->aos_stage, h->pbar};
  for (void* b : bufs) cudaFree(b);
  for (auto& m : h->scene_mesh) m.release();
  if (h->own_stream) cudaStreamDestroy(h->own_stream);
  delete h;
  return CLSPH_OK;
}

int clsph_gpu_set_collision_cap(clsph_gpu* h, uint32_t max_iterations) {
  if (!h || max_iterations == 0) return fail(CLSPH_ERR_ARGUMENT, "set_collision_cap: bad argument");
  h->max_iters = max_iterations;
  return CLSPH_OK;
}

int clsph_gpu_set_stream(clsph_gpu* h, void* stream) {
  if (!h) return fail(CLSPH_ERR_ARGUMENT, "set_stream: null handle");
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  h->stream = stream ? static_cast<cudaStream_t>(stream) : h->own_stream;
  return CLSPH_OK;
}

int clsph_gpu_set_graph(clsph_gpu* h, int enabled) {
  if (!h) return fail(CLSPH_ERR_ARGUMENT, "set_graph: null handle");
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  h->use_graph = enabled != 0;
  if (!h->use_graph) h->drop_graph();
  return CLSPH_OK;
}

int clsph_gpu_set_scene_mesh(clsph_gpu* h, uint32_t scene, const float* normals,
                             const float* vertices, uint32_t vertex_count, const uint32_t* indices,
                             uint32_t faces) {
  if (!h || scene >= h->nscenes) return fail(CLSPH_ERR_ARGUMENT, "set_mesh: bad handle or scene");
  if (faces && (!normals || !vertices || !indices))
    return fail(CLSPH_ERR_ARGUMENT, "set_mesh: null mesh array");
  for (uint64_t k = 0; k < 3ull * faces; ++k)
    if (indices[k] >= vertex_count) return fail(CLSPH_ERR_ARGUMENT, "set_mesh: vertex index out of range");
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  SceneMesh& sm = h->scene_mesh[scene];
  DevMesh& dm = h->mesh_host[scene];
  sm.release();
  dm = DevMesh{};
  if (faces) {
    int rc;
    if ((rc = dev_alloc(&sm.normals, 3 * (size_t)faces)) ||
        (rc = dev_alloc(&sm.vertices, 3 * (size_t)vertex_count)) ||
        (rc = dev_alloc(&sm.indices, 3 * (size_t)faces)))
      return rc;
    CUDA_TRY(cudaMemcpy(sm.normals, normals, sizeof(float) * 3 * faces, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(sm.vertices, vertices, sizeof(float) * 3 * vertex_count, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(sm.indices, indices, sizeof(uint32_t) * 3 * faces, cudaMemcpyHostToDevice));
    dm.normals = sm.normals;
    dm.vertices = sm.vertices;
    dm.indices = sm.indices;
    dm.faces = faces;
    FaceGridPlan plan{};
    float reach = 0.f;
    rc = plan_face_grid(h->params[scene], vertices, vertex_count, indices, faces, plan, reach);
    if (rc >= 256) return rc;
    if (rc == 0) {  // (a non-finite mesh keeps no lists: every face is scanned)
      if ((rc = build_face_lists(h, sm, faces, plan))) return rc;
      dm.cell_start = sm.cell_start;
      dm.cell_faces = sm.cell_faces;
      for (int a = 0; a < 3; ++a) {
        dm.lo[a] = plan.glo[a];
        dm.dims[a] = plan.dims[a];
      }
      dm.inv_cell = 1.f / plan.cell;
      dm.reach = reach;
    }
  }
  return sync_scene_tables(h);
}

int clsph_gpu_read_face_lists(clsph_gpu* h, uint32_t scene, float* plan, uint32_t* cell_start,
                              uint64_t start_cap, uint32_t* cell_faces, uint64_t faces_cap, uint32_t* sizes) {
  if (!h || scene >= h->nscenes || !sizes) return fail(CLSPH_ERR_ARGUMENT, "read_face_lists: bad argument");
  const SceneMesh& sm = h->scene_mesh[scene];
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  if (!sm.cell_start) {
    sizes[0] = sizes[1] = 0;
    return CLSPH_OK;
  }
  const FaceGridPlan& g = sm.plan;
  sizes[0] = g.cells + 1;
  sizes[1] = sm.list_len;
  if (plan) {
    const float v[10] = {g.glo[0], g.glo[1], g.glo[2], g.cell, g.pad, g.tol,
                         (float)g.dims[0], (float)g.dims[1], (float)g.dims[2], h->mesh_host[scene].reach};
    std::memcpy(plan, v, sizeof(v));
  }
  if (cell_start) {
    if (start_cap < sizes[0]) return fail(CLSPH_ERR_ARGUMENT, "read_face_lists: start buffer too small");
    CUDA_TRY(cudaMemcpy(cell_start, sm.cell_start, sizeof(uint32_t) * sizes[0], cudaMemcpyDeviceToHost));
  }
  if (cell_faces) {
    if (faces_cap < sizes[1]) return fail(CLSPH_ERR_ARGUMENT, "read_face_lists: face buffer too small");
    CUDA_TRY(cudaMemcpy(cell_faces, sm.cell_faces, sizeof(uint32_t) * sizes[1], cudaMemcpyDeviceToHost));
  }
  return CLSPH_OK;
}

int clsph_gpu_set_mesh(clsph_gpu* h, const float* normals, const float* vertices,
                       uint32_t vertex_count, const uint32_t* indices, uint32_t faces) {
  return clsph_gpu_set_scene_mesh(h, 0, normals, vertices, vertex_count, indices, faces);
}

// Device view of `p` when it is pinned host memory that kernels can read and
// write in place (16-byte aligned for float4 access), else nullptr.
static void* mapped_host_records(const void* p) {
  if (reinterpret_cast<uintptr_t>(p) % 16) return nullptr;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // not a pointer CUDA knows: take the copy path
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

static dim3 aos_grid(const clsph_gpu* h) {
  return dim3(grid_blocks((uint32_t)std::min<size_t>((size_t)h->n * 5, 0xFFFFFFFFu), h->sm_count * 8));
}

// Pageable records are copied into the staging buffer and unpacked there;
// pinned records are read by the unpack kernel directly (the host link is
// the bound either way, and this saves the staging pass).
int clsph_gpu_upload(clsph_gpu* h, const clsph_particle* particles) {
  if (!h || !particles) return fail(CLSPH_ERR_ARGUMENT, "upload: bad argument");
  const float4* src = static_cast<const float4*>(mapped_host_records(particles));
  if (!src) {
    CUDA_TRY(cudaMemcpyAsync(h->aos_stage, particles, sizeof(clsph_particle) * h->n,
                             cudaMemcpyHostToDevice, h->stream));
    src = h->aos_stage;
  }
  h->launch(K_MISC, k_bbox_reset, dim3(grid_blocks(6 * h->nscenes, 64)), dim3(kBlock), h->bbox,
            h->nscenes);
  h->launch(K_UNPACK, k_unpack_aos, aos_grid(h), dim3(kBlock), src, h->n, h->st[0],
            (const uint16_t*)h->scene_of, h->bbox, h->status);
  h->uploaded = true;
  h->partial = false;
  h->have_fields = false;
  return check_launch(h);
}

int clsph_gpu_download(clsph_gpu* h, clsph_particle* particles) {
  if (!h || !particles) return fail(CLSPH_ERR_ARGUMENT, "download: bad argument");
  if (!h->uploaded || h->partial) return fail(CLSPH_ERR_STATE, "download: no complete state");
  float4* dst = static_cast<float4*>(mapped_host_records(particles));
  h->launch(K_PACK, k_pack_aos, aos_grid(h), dim3(kBlock), dst ? dst : h->aos_stage, h->n, h->st[0],
            (const float4*)h->aux, (const uint32_t*)h->keys, (const uint32_t*)h->ctl,
            h->have_fields ? 1 : 0);
  if (!dst)
    CUDA_TRY(cudaMemcpyAsync(particles, h->aos_stage, sizeof(clsph_particle) * h->n,
                             cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  return check_launch(h);
}

int clsph_gpu_step(clsph_gpu* h, uint32_t substeps) {
  if (!h) return fail(CLSPH_ERR_ARGUMENT, "step: null handle");
  if (!h->uploaded || h->partial) return fail(CLSPH_ERR_STATE, "step: upload particles first");
  uint32_t done = 0;
  if (h->persistent && !h->profiling) {
    int rc = launch_persistent(h, substeps);
    if (rc) return rc;
    h->substeps += substeps;
    done = substeps;
  }
  if (h->use_graph && !h->profiling && substeps - done >= 2) {
    for (int kind = 1; kind >= 0; --kind) {  // the long graph first
      const uint32_t len = clsph_gpu::kGraphLen[kind];
      if (substeps - done < len) continue;
      int rc = ensure_graph(h, kind);
      if (rc) return rc;
      for (; done + len <= substeps; done += len) {
        CUDA_TRY(cudaGraphLaunch(h->graph_exec[kind][h->ids_sel], h->stream));
        h->launches += h->graph_launches[kind][h->ids_sel];
        h->substeps += len;
      }
    }
  }
  for (; done < substeps; ++done) {
    int rc = enqueue_substep(h, CLSPH_STAGE_ADVECT);
    if (rc) return rc;
    ++h->substeps;
  }
  if (substeps) h->have_fields = true;
  return check_launch(h);
}

int clsph_gpu_step_until(clsph_gpu* h, int stage) {
  if (!h || stage < CLSPH_STAGE_GRID || stage > CLSPH_STAGE_ADVECT)
    return fail(CLSPH_ERR_ARGUMENT, "step_until: bad argument");
  if (!h->uploaded || h->partial) return fail(CLSPH_ERR_STATE, "step_until: upload particles first");
  int rc = enqueue_substep(h, stage);
  if (rc) return rc;
  ++h->substeps;
  if (stage < CLSPH_STAGE_ADVECT) h->partial = true;
  h->have_fields = stage >= CLSPH_STAGE_DENSITY;
  return check_launch(h);
}

int clsph_gpu_sync(clsph_gpu* h, uint32_t* flags) {
  if (!h) return fail(CLSPH_ERR_ARGUMENT, "sync: null handle");
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  uint32_t f = 0;
  CUDA_TRY(cudaMemcpy(&f, h->status, sizeof(uint32_t), cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemset(h->status, 0, sizeof(uint32_t)));
  if (f & kFlagBarrierStall) {
    // the barrier words may be left mid-count: start the next launch afresh
    CUDA_TRY(cudaMemset(h->pbar, 0, 2 * sizeof(uint32_t)));
    return fail(CLSPH_ERR_CUDA, "sync: a grid barrier wait of the persistent substep kernel ran out "
                                "(the substeps of that launch are incomplete)");
  }
  if (f & kFlagSortStall)
    return fail(CLSPH_ERR_CUDA, "sync: a radix sort look-back wait ran out (that substep's order is wrong)");
  if (flags) *flags = f;
  if (h->profiling) h->harvest();
  return CLSPH_OK;
}

int clsph_gpu_set_scene_parameters(clsph_gpu* h, uint32_t scene, const clsph_parameters* params,
                                   const clsph_kernel_terms* terms) {
  if (!h || !params || !terms || scene >= h->nscenes)
    return fail(CLSPH_ERR_ARGUMENT, "set_parameters: bad argument");
  const uint32_t count = h->scene_first[scene + 1] - h->scene_first[scene];
  if (params->particles_count != count)
    return fail(CLSPH_ERR_ARGUMENT, "set_parameters: the particle count of a scene cannot change");
  if (!(params->h > 0.f)) return fail(CLSPH_ERR_ARGUMENT, "set_parameters: h must be positive");
  // kernels of queued substeps read the constants: replace them between substeps
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  clsph_parameters p = *params;
  const clsph_parameters& old = h->params[scene];
  // the grid fields are the engine's own, recomputed every substep
  p.min_point = old.min_point;
  p.max_point = old.max_point;
  p.grid_size_x = old.grid_size_x;
  p.grid_size_y = old.grid_size_y;
  p.grid_size_z = old.grid_size_z;
  p.grid_cell_count = old.grid_cell_count;
  h->params[scene] = p;
  h->terms[scene] = *terms;
  h->consts_host[scene] = derive_consts(p, *terms, count);
  const float hs = p.h;
  CUDA_TRY(cudaMemcpy(h->scene_h + scene, &hs, sizeof(float), cudaMemcpyHostToDevice));
  return sync_scene_tables(h);
}

int clsph_gpu_set_parameters(clsph_gpu* h, const clsph_parameters* params, const clsph_kernel_terms* terms) {
  return clsph_gpu_set_scene_parameters(h, 0, params, terms);
}

int clsph_gpu_get_scene_parameters(clsph_gpu* h, uint32_t scene, clsph_parameters* out) {
  if (!h || !out || scene >= h->nscenes) return fail(CLSPH_ERR_ARGUMENT, "get_parameters: bad argument");
  DevGrid g;
  int rc = read_grid(h, scene, &g, nullptr);
  if (rc) return rc;
  *out = h->params[scene];
  for (int a = 0; a < 3; ++a) {
    out->min_point.s[a] = g.lo[a];
    out->max_point.s[a] = g.hi[a];
  }
  out->min_point.s[3] = out->max_point.s[3] = 0.f;
  out->grid_size_x = g.size[0];
  out->grid_size_y = g.size[1];
  out->grid_size_z = g.size[2];
  out->grid_cell_count = g.cells;
  return CLSPH_OK;
}

int clsph_gpu_get_parameters(clsph_gpu* h, clsph_parameters* out) {
  return clsph_gpu_get_scene_parameters(h, 0, out);
}

int clsph_gpu_read_keys(clsph_gpu* h, uint32_t* keys, uint32_t* perm) {
  if (!h || !keys) return fail(CLSPH_ERR_ARGUMENT, "read_keys: bad argument");
  uint32_t ctl[kCtlWords];
  int rc = read_grid(h, 0, nullptr, ctl);
  if (rc) return rc;
  const size_t off = (size_t)sorted_sel(ctl[kCtlMaxKey]) * h->n;
  CUDA_TRY(cudaMemcpy(keys, h->keys + off, sizeof(uint32_t) * h->n, cudaMemcpyDeviceToHost));
  const KeySplit split{ctl[kCtlShift]};
  for (uint32_t i = 0; i < h->n; ++i) keys[i] = split.morton(keys[i]);
  if (perm) CUDA_TRY(cudaMemcpy(perm, h->vals + off, sizeof(uint32_t) * h->n, cudaMemcpyDeviceToHost));
  return CLSPH_OK;
}

int clsph_gpu_read_cell_table_scene(clsph_gpu* h, uint32_t scene, uint32_t* table, uint64_t cap) {
  if (!h || !table || scene >= h->nscenes) return fail(CLSPH_ERR_ARGUMENT, "read_cell_table: bad argument");
  DevGrid g;
  int rc = read_grid(h, scene, &g, nullptr);
  if (rc) return rc;
  if (cap < g.cells) return fail(CLSPH_ERR_ARGUMENT, "read_cell_table: buffer too small");
  if (g.cells == 0) return CLSPH_OK;
  uint32_t* d = nullptr;
  if ((rc = dev_alloc(&d, g.cells))) return rc;
  k_dense_table<<<(g.cells + 255) / 256, 256, 0, h->stream>>>(
      h->keys, h->n, h->ctl, h->grids + scene, scene, h->scene_first[scene], h->scene_first[scene + 1], d);
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e == cudaSuccess) e = cudaMemcpy(table, d, sizeof(uint32_t) * g.cells, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return fail(CLSPH_ERR_CUDA, std::string("read_cell_table: ") + cudaGetErrorString(e));
  return CLSPH_OK;
}

int clsph_gpu_read_cell_table(clsph_gpu* h, uint32_t* table, uint64_t cap) {
  return clsph_gpu_read_cell_table_scene(h, 0, table, cap);
}

int clsph_gpu_read_fields(clsph_gpu* h, float* density, float* pressure, float* accel) {
  if (!h) return fail(CLSPH_ERR_ARGUMENT, "read_fields: null handle");
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  if (density || pressure) {
    std::vector<float4> a(h->n);
    CUDA_TRY(cudaMemcpy(a.data(), h->aux, sizeof(float4) * h->n, cudaMemcpyDeviceToHost));
    for (uint32_t i = 0; i < h->n; ++i) {
      if (density) density[i] = a[i].x;
      if (pressure) pressure[i] = a[i].y;
    }
  }
  if (accel) CUDA_TRY(cudaMemcpy(accel, h->acc, sizeof(float4) * h->n, cudaMemcpyDeviceToHost));
  return CLSPH_OK;
}

int clsph_gpu_read_ids(clsph_gpu* h, uint32_t* ids) {
  if (!h || !ids) return fail(CLSPH_ERR_ARGUMENT, "read_ids: bad argument");
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  CUDA_TRY(cudaMemcpy(ids, h->ids[h->ids_sel], sizeof(uint32_t) * h->n, cudaMemcpyDeviceToHost));
  return CLSPH_OK;
}

int clsph_gpu_set_profiling(clsph_gpu* h, int enabled) {
  if (!h) return fail(CLSPH_ERR_ARGUMENT, "set_profiling: null handle");
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  h->harvest();
  h->profiling = enabled != 0;
  for (int k = 0; k < K_NUM_CLASSES; ++k) {
    h->class_ms[k] = 0.0;
    h->class_count[k] = 0;
  }
  return CLSPH_OK;
}

int clsph_gpu_kernel_times(clsph_gpu* h, int max_classes, char* names, int name_stride, float* ms,
                           uint32_t* counts, int* n_classes) {
  if (!h) return fail(CLSPH_ERR_ARGUMENT, "kernel_times: null handle");
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  h->harvest();
  int k_out = max_classes < K_NUM_CLASSES ? max_classes : K_NUM_CLASSES;
  for (int k = 0; k < k_out; ++k) {
    if (names && name_stride > 0) std::snprintf(names + (size_t)k * name_stride, name_stride, "%s", kKernelNames[k]);
    if (ms) ms[k] = (float)h->class_ms[k];
    if (counts) counts[k] = h->class_count[k];
  }
  if (n_classes) *n_classes = K_NUM_CLASSES;
  return CLSPH_OK;
}

static cudaEvent_t take_event_of(clsph_gpu* h) { return h->take_event(); }

int clsph_gpu_autotune(clsph_gpu* h, uint32_t substeps, char* report, int report_len) {
  if (!h || substeps == 0) return fail(CLSPH_ERR_ARGUMENT, "autotune: bad argument");
  if (!h->uploaded || h->partial) return fail(CLSPH_ERR_STATE, "autotune: upload particles first");
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  // snapshot of the state the trials advance, restored afterwards
  const size_t n = h->n;
  float4* snap = nullptr;
  uint32_t* snap_ids = nullptr;
  uint32_t* snap_bbox = nullptr;
  int rc;
  if ((rc = dev_alloc(&snap, 3 * n)) || (rc = dev_alloc(&snap_ids, n)) ||
      (rc = dev_alloc(&snap_bbox, 6 * (size_t)h->nscenes))) {
    cudaFree(snap);
    cudaFree(snap_ids);
    return rc;
  }
  auto save = [&](bool back) {
    float4* dst[3] = {h->st[0].pos, h->st[0].vel, h->st[0].ivel};
    for (int k = 0; k < 3; ++k) {
      if (back)
        cudaMemcpyAsync(dst[k], snap + k * n, sizeof(float4) * n, cudaMemcpyDeviceToDevice, h->stream);
      else
        cudaMemcpyAsync(snap + k * n, dst[k], sizeof(float4) * n, cudaMemcpyDeviceToDevice, h->stream);
    }
    if (back) {
      cudaMemcpyAsync(h->ids[h->ids_sel], snap_ids, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, h->stream);
      cudaMemcpyAsync(h->bbox, snap_bbox, sizeof(uint32_t) * 6 * h->nscenes, cudaMemcpyDeviceToDevice, h->stream);
    } else {
      cudaMemcpyAsync(snap_ids, h->ids[h->ids_sel], sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, h->stream);
      cudaMemcpyAsync(snap_bbox, h->bbox, sizeof(uint32_t) * 6 * h->nscenes, cudaMemcpyDeviceToDevice, h->stream);
    }
  };
  save(false);
  const int ids_sel0 = h->ids_sel;
  const bool prof0 = h->profiling;
  const uint64_t substeps0 = h->substeps, launches0 = h->launches;
  h->harvest();
  h->profiling = true;
  auto trial = [&](int cls) -> double {
    h->harvest();
    double before = h->class_ms[cls];
    uint32_t cnt0 = h->class_count[cls];
    for (uint32_t k = 0; k < substeps; ++k) enqueue_substep(h, CLSPH_STAGE_ADVECT);
    cudaStreamSynchronize(h->stream);
    h->harvest();
    save(true);
    h->ids_sel = ids_sel0;
    uint32_t c = h->class_count[cls] - cnt0;
    return c ? (h->class_ms[cls] - before) / c : 1e30;
  };
  std::string out;
  const int blocks[3] = {64, 128, 256};
  const int searches[3] = {CLSPH_SEARCH_WINDOW, CLSPH_SEARCH_CELL_WARPS, CLSPH_SEARCH_PARTICLE_WARPS};
  int best_d = h->density_block, best_f = h->forces_block, best_s = h->search;
  double td = 1e30, tf = 1e30;
  for (int b : blocks) {
    h->density_block = b;
    h->forces_block = b;
    for (int sm : searches) {
      h->search = sm;
      trial(K_DENSITY);  // warm-up of this shape
      double d = trial(K_DENSITY);
      out += "density block " + std::to_string(b) + " search " + std::to_string(sm) + ": " +
             std::to_string(d) + " ms\n";
      if (d < td) { td = d; best_d = b; best_s = sm; }
    }
    double f = trial(K_FORCES);
    out += "forces block " + std::to_string(b) + ": " + std::to_string(f) + " ms\n";
    if (f < tf) { tf = f; best_f = b; }
  }
  h->density_block = best_d;
  h->forces_block = best_f;
  h->search = best_s;
  const uint32_t advect_opts[3] = {4, 8, 16};
  uint32_t best_a = h->advect_blocks_per_sm;
  double ta = 1e30;
  for (uint32_t a : advect_opts) {
    h->advect_blocks_per_sm = a;
    double t = trial(K_ADVECT);
    out += "advect blocks/SM " + std::to_string(a) + ": " + std::to_string(t) + " ms\n";
    if (t < ta) { ta = t; best_a = a; }
  }
  h->advect_blocks_per_sm = best_a;
  // whole substeps: CUDA-graph replays of the tuned launches against the
  // persistent cooperative kernel; the faster form is kept
  h->drop_graph();
  int coop = 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, h->device);
  bool use_persistent = false;
  if (coop) {
    const uint32_t even = std::max<uint32_t>(2u, substeps & ~1u);
    const bool graph0 = h->use_graph;
    cudaEvent_t e0 = take_event_of(h), e1 = take_event_of(h);
    auto whole = [&](bool pers) -> double {
      h->persistent = pers;
      h->use_graph = true;
      h->profiling = false;
      cudaEventRecord(e0, h->stream);
      const int rc = clsph_gpu_step(h, even);
      cudaEventRecord(e1, h->stream);
      cudaStreamSynchronize(h->stream);
      float ms = 0.f;
      const bool ok = rc == 0 && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess;
      save(true);
      h->ids_sel = ids_sel0;
      h->profiling = true;
      return ok ? ms / even : 1e30;
    };
    whole(false);  // warm-up (graph capture)
    const double tg = whole(false);
    whole(true);
    const double tp = whole(true);
    use_persistent = tp < tg;
    out += "whole substep: graph " + std::to_string(tg) + " ms, persistent " + std::to_string(tp) + " ms\n";
    h->use_graph = graph0;
    h->event_pool.push_back(e0);
    h->event_pool.push_back(e1);
    cudaGetLastError();
  }
  h->persistent = use_persistent;
  out += "chosen: density block " + std::to_string(best_d) + ", search " + std::to_string(best_s) +
         ", forces block " + std::to_string(best_f) +
         ", advect blocks/SM " + std::to_string(best_a) +
         (use_persistent ? ", persistent substeps" : ", launched substeps") + "\n";
  h->profiling = prof0;
  for (int k = 0; k < K_NUM_CLASSES; ++k) {
    h->class_ms[k] = 0.0;
    h->class_count[k] = 0;
  }
  h->substeps = substeps0;
  h->launches = launches0;
  h->drop_graph();  // launch shapes changed
  cudaStreamSynchronize(h->stream);
  cudaFree(snap);
  cudaFree(snap_ids);
  cudaFree(snap_bbox);
  if (report && report_len > 0) std::snprintf(report, report_len, "%s", out.c_str());
  return check_launch(h);
}

int clsph_gpu_set_launch_shape(clsph_gpu* h, int density_block, int forces_block,
                               uint32_t advect_blocks_per_sm) {
  if (!h) return fail(CLSPH_ERR_ARGUMENT, "set_launch_shape: null handle");
  auto ok = [](int b) { return b == 64 || b == 128 || b == 256; };
  if (!ok(density_block) || !ok(forces_block) || advect_blocks_per_sm == 0 || advect_blocks_per_sm > 64)
    return fail(CLSPH_ERR_ARGUMENT, "set_launch_shape: unsupported shape");
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  h->density_block = density_block;
  h->forces_block = forces_block;
  h->advect_blocks_per_sm = advect_blocks_per_sm;
  h->drop_graph();
  return CLSPH_OK;
}

int clsph_gpu_set_neighbour_search(clsph_gpu* h, int mode) {
  if (!h) return fail(CLSPH_ERR_ARGUMENT, "set_neighbour_search: null handle");
  if (mode != CLSPH_SEARCH_WINDOW && mode != CLSPH_SEARCH_CELL_WARPS && mode != CLSPH_SEARCH_PARTICLE_WARPS)
    return fail(CLSPH_ERR_ARGUMENT, "set_neighbour_search: unknown mode");
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  h->search = mode;
  h->drop_graph();
  return CLSPH_OK;
}

int clsph_gpu_set_wait_limits(clsph_gpu* h, uint32_t radix_lookback_spins, uint32_t mlp_wait_polls,
                              uint32_t radix_withheld_tile) {
  if (!h) return fail(CLSPH_ERR_ARGUMENT, "set_wait_limits: null handle");
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  h->radix_spin_limit = radix_lookback_spins;
  h->mlp_wait_limit = mlp_wait_polls;
  h->radix_withheld_tile = radix_withheld_tile;
  h->drop_graph();  // the limits are kernel arguments of the captured launches
  return CLSPH_OK;
}

int clsph_gpu_set_persistent(clsph_gpu* h, int enabled) {
  if (!h) return fail(CLSPH_ERR_ARGUMENT, "set_persistent: null handle");
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  if (enabled) {
    int coop = 0;
    CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, h->device));
    if (!coop) return fail(CLSPH_ERR_CUDA, "set_persistent: the device has no cooperative launch");
  }
  h->persistent = enabled != 0;
  return CLSPH_OK;
}

int clsph_gpu_set_barrier_limits(clsph_gpu* h, uint32_t barrier_spins, uint32_t withheld_block) {
  if (!h) return fail(CLSPH_ERR_ARGUMENT, "set_barrier_limits: null handle");
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  h->barrier_limit = barrier_spins;
  h->withheld_block = withheld_block;
  return CLSPH_OK;
}

int clsph_gpu_counters(clsph_gpu* h, uint64_t* out3) {
  if (!h || !out3) return fail(CLSPH_ERR_ARGUMENT, "counters: bad argument");
  unsigned long long capped = 0;
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  CUDA_TRY(cudaMemcpy(&capped, h->capped, sizeof(capped), cudaMemcpyDeviceToHost));
  out3[0] = h->substeps;
  out3[1] = capped;
  out3[2] = h->launches;
  return CLSPH_OK;
}

}  // extern "C"
