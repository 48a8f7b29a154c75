// The whole substep loop as one persistent, cooperative launch (for batched
// scenes of uneven sizes; no counterpart in the reference).
//
// One block of 256 threads per resident slot on every SM (all co-resident,
// which the cooperative launch guarantees) runs every phase of a substep in
// turn, S substeps per launch, with a grid-wide barrier between phases:
//   grid set-up (block 0) + cell-index clear | keys | digit counts |
//   radix passes (tiles by ticket, decoupled look-back) | gather |
//   density (one warp per occupied cell, 8 per block) | forces | advection
// Each phase is the block-level body of the corresponding kernel of
// clsph_kernels.cuh, so the results are those of the launched substeps bit
// for bit. The barrier is a counter and a generation word in device memory;
// every wait on it is bounded (a wait that runs out sets kFlagBarrierStall,
// its block leaves the kernel, and clsph_gpu_sync reports the error and
// resets the words).
#pragma once

#include "clsph_kernels.cuh"

namespace clsph {

constexpr uint32_t kFlagBarrierStall = 1u << 17;  // internal: a grid barrier wait ran out
constexpr uint32_t kPersistThreads = 256;
constexpr uint32_t kBarrierSpins = 1u << 22;  // ~ seconds: longer than any phase
constexpr uint32_t kNoBlock = 0xFFFFFFFFu;

struct PersistArgs {
  uint32_t n, nscenes, ntiles, slots, nlist_cap, max_iters;
  uint32_t* bbox;
  DevGrid* grids;
  const float* scene_h;
  uint32_t* status;
  uint32_t* digit_total;
  uint32_t* step_counters;
  uint32_t* ctl;
  const uint16_t* scene_of;
  uint32_t* keys;
  uint32_t* vals;
  uint32_t* lookback;
  State st[2];
  uint32_t* ids[2];
  CellIndex ci;
  uint32_t* cell_list;
  const Consts* consts;
  float4* aux;
  uint16_t* nlist;
  uint32_t* ncount;
  float4* frec;
  uint32_t* nb_start;
  float4* acc;
  const DevMesh* meshes;
  unsigned long long* capped;
  uint32_t* barrier;  // [0] arrivals, [1] generation
  uint32_t spin_limit, withheld_tile;  // radix look-back bound and test hook
  uint32_t barrier_limit, withheld_block;  // grid barrier bound and test hook
};

union PersistSmem {
  RadixSmem radix;
  uint32_t hist[4][256];
  DensitySmem<8> dens;
  GatherSmem gather;
  BboxSmem bbox;
  uint32_t word;
};
static_assert(sizeof(PersistSmem) <= 48 * 1024, "static shared memory of the persistent kernel");

__device__ __forceinline__ uint32_t ld_acquire_gpu(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Grid-wide barrier; false (for the whole block) when this block's wait ran
// out or when it is the test hook's withheld block (which leaves at once,
// as a block that never arrives).
__device__ __forceinline__ bool grid_barrier(const PersistArgs& a, uint32_t& ok_s) {
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t good = 1u;
    if (blockIdx.x == a.withheld_block) {
      good = 0u;
    } else {
      const uint32_t gen = ld_acquire_gpu(&a.barrier[1]);
      __threadfence();  // the block's writes (ordered by the barrier above) before the arrival
      if (atomicAdd(&a.barrier[0], 1u) == gridDim.x - 1u) {
        atomicExch(&a.barrier[0], 0u);
        __threadfence();
        atomicAdd(&a.barrier[1], 1u);
      } else {
        uint32_t spins = 0;
        while (ld_acquire_gpu(&a.barrier[1]) == gen) {
          if (++spins > a.barrier_limit) {
            atomicOr(a.status, kFlagBarrierStall);
            good = 0u;
            break;
          }
          __nanosleep(64);
        }
      }
      __threadfence();
    }
    ok_s = good;
  }
  __syncthreads();
  return ok_s != 0u;
}

// three resident blocks per SM (24 warps): at most 85 registers per thread
static __global__ void __launch_bounds__(kPersistThreads, 3)
    k_substeps_persistent(PersistArgs a, uint32_t substeps, uint32_t ids_sel0) {
  __shared__ PersistSmem sm;
  __shared__ uint32_t ok_s;
  const uint32_t n = a.n;
  const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t gstride = gridDim.x * blockDim.x;
  const uint32_t nblk = (n + kPersistThreads - 1) / kPersistThreads;
  for (uint32_t s = 0; s < substeps; ++s) {
    const uint32_t src_ids = (ids_sel0 + s) & 1u;
    // grid set-up of every scene, and an empty cell index
    if (blockIdx.x == 0)
      grid_setup_block(a.bbox, a.grids, a.scene_h, a.nscenes, a.status, a.digit_total, a.step_counters, a.ctl,
                       sm.word);
    for (uint32_t k = gtid; k < a.slots; k += gstride) a.ci.keys[k] = 0u;
    if (!grid_barrier(a, ok_s)) return;
    for (uint32_t vb = blockIdx.x; vb < nblk; vb += gridDim.x)
      keys_block(vb, a.st[0].pos, n, a.grids, a.scene_of, a.ctl, a.keys, sm.word);
    if (!grid_barrier(a, ok_s)) return;
    radix_hist_blocks(blockIdx.x, gridDim.x, a.keys, n, a.ctl, a.digit_total, a.lookback, a.ntiles, sm.hist);
    if (!grid_barrier(a, ok_s)) return;
    const uint32_t passes = radix_passes(a.ctl[kCtlMaxKey]);
    for (int pass = 0; pass < 4; ++pass) {
      if ((uint32_t)pass >= passes) break;  // the same for every block
      while (radix_sweep_tile(a.keys, a.vals, n, pass, a.digit_total, a.lookback, a.ntiles,
                              a.step_counters + kCntRadixTile + pass, a.status, a.spin_limit, a.withheld_tile,
                              sm.radix)) {
      }
      if (!grid_barrier(a, ok_s)) return;
    }
    for (uint32_t vb = blockIdx.x; vb < nblk; vb += gridDim.x)
      gather_block(vb, n, a.grids, a.scene_of, a.ctl, a.keys, a.vals, a.st[0], a.st[1], a.ids[src_ids],
                   a.ids[src_ids ^ 1u], a.ci, a.cell_list, a.step_counters + kCntCells, sm.gather);
    if (!grid_barrier(a, ok_s)) return;
    density_cells_warps<8>(n, a.grids, a.scene_of, a.ctl, a.keys, a.st[1].pos, a.ci, a.consts, a.aux, a.nlist,
                           a.ncount, a.nlist_cap, a.st[1].vel, a.frec, a.cell_list, a.step_counters, a.nb_start,
                           sm.dens);
    if (!grid_barrier(a, ok_s)) return;
    for (uint32_t i = gtid; i < n; i += gstride)
      forces_particle(i, n, a.grids, a.scene_of, a.ctl, a.keys, a.st[1], a.aux, a.ci, a.consts, a.nlist, a.ncount,
                      a.nlist_cap, a.acc, NoForceHook{}, a.frec, a.nb_start);
    if (!grid_barrier(a, ok_s)) return;
    advect_blocks<false>(blockIdx.x, gridDim.x, n, a.st[1], a.acc, a.st[0], a.meshes, a.consts, a.scene_of,
                         a.max_iters, a.bbox, a.status, a.capped, nullptr, 1.f, 1.f, nullptr, nullptr, sm.bbox);
    if (!grid_barrier(a, ok_s)) return;
  }
}

}  // namespace clsph
