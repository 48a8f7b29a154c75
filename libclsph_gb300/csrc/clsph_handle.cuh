// Internal: the engine handle shared by the library's translation units
// (clsph_gpu.cu: substep engine and C ABI; clsph_learned.cu: learned stepper).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "clsph_gpu.h"
#include "clsph_kernels.cuh"
#include "clsph_mesh.cuh"
#include "clsph_persistent.cuh"

using namespace clsph;

namespace clsph_host {

// Records `msg` as the thread's last error (clsph_gpu_last_error) and returns code.
int fail(int code, const std::string& msg);


#define CUDA_TRY(expr)                                                                  \
  do {                                                                                  \
    cudaError_t err_ = (expr);                                                          \
    if (err_ != cudaSuccess)                                                            \
      return fail(CLSPH_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(err_)); \
  } while (0)

enum KernelClass {
  K_GRID_SETUP,
  K_KEYS,
  K_RADIX_HIST,
  K_RADIX_SWEEP,
  K_GATHER,
  K_DENSITY,
  K_FORCES,
  K_ADVECT,
  K_UNPACK,
  K_PACK,
  K_MISC,
  K_FEATURES,
  K_MLP,
  K_LEARNED_ADVECT,
  K_GATE,
  K_NUM_CLASSES
};

extern const char* kKernelNames[K_NUM_CLASSES];


struct PendingTiming {
  int cls;
  cudaEvent_t start, stop;
};

template <typename T>
int dev_alloc(T** p, size_t count) {
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * (count ? count : 1));
  if (e != cudaSuccess) return fail(CLSPH_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  return 0;
}

inline uint32_t grid_blocks(uint32_t n, uint32_t cap = 0) {
  uint32_t b = (n + kBlock - 1) / kBlock;
  if (b == 0) b = 1;
  if (cap && b > cap) b = cap;
  return b;
}

inline float pown_f(float x, int k) {
  float r = x;
  for (int i = 1; i < k; ++i) r = r * x;
  return r;
}

// Device buffers of one scene's mesh.
struct SceneMesh {
  float* normals = nullptr;
  float* vertices = nullptr;
  uint32_t* indices = nullptr;
  uint32_t* cell_start = nullptr;
  uint32_t* cell_faces = nullptr;
  FaceGridPlan plan{};    // grid of the per-cell triangle lists
  uint32_t list_len = 0;  // entries in cell_faces
  void release() {
    cudaFree(normals);
    cudaFree(vertices);
    cudaFree(indices);
    cudaFree(cell_start);
    cudaFree(cell_faces);
    *this = SceneMesh{};
  }
};

}  // namespace clsph_host

using namespace clsph_host;

struct clsph_gpu {
  int device = 0;
  uint32_t sm_count = 152;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  uint32_t n = 0;

  // scenes
  uint32_t nscenes = 1;
  std::vector<uint32_t> scene_first;  // nscenes + 1 slot offsets
  std::vector<clsph_parameters> params;
  std::vector<clsph_kernel_terms> terms;
  std::vector<Consts> consts_host;
  std::vector<SceneMesh> scene_mesh;
  std::vector<DevMesh> mesh_host;
  uint16_t* scene_of = nullptr;
  DevGrid* grids = nullptr;
  Consts* consts = nullptr;
  float* scene_h = nullptr;
  DevMesh* meshes = nullptr;
  uint32_t* bbox = nullptr;  // 6 per scene
  uint32_t* ctl = nullptr;   // kCtlWords

  State st[2]{};
  uint32_t* ids[2]{};
  int ids_sel = 0;
  float4* aux = nullptr;  // (rho, p, m/rho, p/rho^2)
  float4* acc = nullptr;
  float4* frec = nullptr;  // [2n] forces records: (pos, m/rho), (vel, p/rho^2)
  uint16_t* nlist = nullptr;      // [nlist_cap][n] neighbour tags (visiting order)
  uint32_t* nb_start = nullptr;   // [n][27] rows of the cells' neighbour starts (by first slot)
  uint32_t* ncount = nullptr;
  uint32_t nlist_cap = 64;
  uint32_t* cell_list = nullptr;      // first sorted slot of every occupied cell
  uint32_t* step_counters = nullptr;  // kStepCounters, zeroed every substep
  uint32_t* keys = nullptr;           // [2n]
  uint32_t* vals = nullptr;           // [2n]
  uint32_t* lookback = nullptr;  // [4 passes][ntiles][256] radix look-back words
  uint32_t ntiles = 0;
  uint32_t* digit_total = nullptr;
  CellIndex ci{};
  uint32_t slots = 0;
  uint32_t* status = nullptr;
  unsigned long long* capped = nullptr;
  float4* aos_stage = nullptr;

  // launch shapes chosen by clsph_gpu_autotune
  int density_block = 128;
  int search = CLSPH_SEARCH_CELL_WARPS;  // neighbour search of the density kernel
  int forces_block = 128;
  uint32_t advect_blocks_per_sm = 8;

  // the substep loop as one persistent cooperative launch (clsph_persistent.cuh)
  bool persistent = false;
  uint32_t* pbar = nullptr;         // grid barrier words
  uint32_t persist_blocks = 0;      // co-resident blocks (0: not yet measured)
  uint32_t barrier_limit = kBarrierSpins;
  uint32_t withheld_block = kNoBlock;

  // bounds of the device waits (clsph_gpu_set_wait_limits)
  uint32_t radix_spin_limit = CLSPH_DEFAULT_LOOKBACK_SPINS;
  uint32_t radix_withheld_tile = CLSPH_NO_TILE;
  uint32_t mlp_wait_limit = CLSPH_DEFAULT_MLP_WAIT_POLLS;

  bool uploaded = false;
  bool partial = false;
  bool have_fields = false;
  uint32_t max_iters = 1024;

  // CUDA graphs of a few substeps, one per buffer the particle ids start in
  bool use_graph = false;
  // [length kind][particle-id buffer]: kind 0 replays 2 substeps, kind 1 16
  // (long runs of small scenes are otherwise bound by the host's graph
  // launches)
  static constexpr uint32_t kGraphLen[2] = {2, 16};
  cudaGraphExec_t graph_exec[2][2] = {};
  uint32_t graph_max_iters[2][2] = {};
  uint64_t graph_launches[2][2] = {};  // kernels in one replay of each graph
  uint32_t graph_epoch = 0;  // counts drop_graph(): other cached graphs compare it

  // buffers of the learned stepper (clsph_learned.cu), made on first use
  void* learned = nullptr;
  void (*free_learned)(clsph_gpu*) = nullptr;

  bool profiling = false;
  std::vector<PendingTiming> pending;
  std::vector<cudaEvent_t> event_pool;
  double class_ms[K_NUM_CLASSES] = {};
  uint32_t class_count[K_NUM_CLASSES] = {};
  uint64_t substeps = 0;
  uint64_t launches = 0;

  cudaEvent_t take_event() {
    if (!event_pool.empty()) {
      cudaEvent_t e = event_pool.back();
      event_pool.pop_back();
      return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
  }

  template <typename Kernel, typename... Args>
  void launch(int cls, Kernel k, dim3 g, dim3 b, Args... args) {
    launch_smem(cls, k, g, b, 0, args...);
  }

  template <typename Kernel, typename... Args>
  void launch_smem(int cls, Kernel k, dim3 g, dim3 b, size_t smem, Args... args) {
    PendingTiming t{cls, nullptr, nullptr};
    if (profiling) {
      t.start = take_event();
      cudaEventRecord(t.start, stream);
    }
    k<<<g, b, smem, stream>>>(args...);
    ++launches;
    if (profiling) {
      t.stop = take_event();
      cudaEventRecord(t.stop, stream);
      pending.push_back(t);
    }
  }

  void harvest() {
    for (auto& t : pending) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, t.start, t.stop) == cudaSuccess) {
        class_ms[t.cls] += ms;
        class_count[t.cls] += 1;
      }
      event_pool.push_back(t.start);
      event_pool.push_back(t.stop);
    }
    pending.clear();
  }

  void drop_graph() {
    ++graph_epoch;
    for (auto& row : graph_exec)
      for (auto& g : row) {
        if (g) cudaGraphExecDestroy(g);
        g = nullptr;
      }
  }
};


namespace clsph_host {

// Enqueues one substep up to and including `until` (CLSPH_STAGE_*).
int enqueue_substep(clsph_gpu* h, int until);
// Enqueues `substeps` whole substeps as persistent cooperative launches.
int launch_persistent(clsph_gpu* h, uint32_t substeps);
// Enqueues the advection of the sorted state (the CLSPH_STAGE_ADVECT part of
// a substep) back into the resident buffers.
int enqueue_advect(clsph_gpu* h);
// Reports a failed kernel launch as CLSPH_ERR_CUDA.
int check_launch(clsph_gpu* h);

}  // namespace clsph_host
