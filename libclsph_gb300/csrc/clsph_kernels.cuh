// Device kernels of one SPH substep (sm_103a).
//
// Data layout in HBM (SoA, sorted order, 16-byte float4 rows):
//   pos[n], vel[n], ivel[n]   position, velocity, intermediate (half-step) velocity
//   aux[n]                    (rho, p, own cell's first slot (bits), p/rho^2) of the substep
//   nlist[cap][n], ncount[n]  contributing neighbours of each particle, in visiting order,
//                             as 16-bit tags (neighbour cell k of 27 << 11 | offset in it)
//   nb_start[n][27]           first slot of each of the 27 cells around a cell, in the
//                             row of the cell's first slot (resolves the tags)
//   acc[n]                    acceleration (forces -> advection)
//   keys[2][n], vals[2][n]    radix-sort ping-pong (Morton key, source slot)
//   ids[2][n]                 persistent particle ids (the reference has none)
//   hkeys[S], hstart[S], hend[S]  cell index: Morton key -> [start, end)
// A handle holds S independent scenes (S = 1 for a single simulation): the
// particles of scene s occupy one contiguous slot range, scene_of[slot] = s.
// The sort key is (s << scene_shift) | Morton key, so the one stable sort
// keeps every scene in its range and orders it exactly like a sort of that
// scene alone. Per-scene grids (bounding box, cell size, dense cell count),
// constants and meshes live in device arrays; the sort control (largest key,
// hence the number of radix passes) is shared. Nothing needs a host round
// trip between kernels.
#pragma once

#include "clsph_common.cuh"

namespace clsph {

constexpr int kBlock = 256;
// 2048-key tiles: 512 blocks per pass at 1M keys (4096-key tiles gave 256
// blocks, 20 % warp occupancy and an 80-register scatter; 9-14 % slower)
constexpr int kRadixThreads = 256;
constexpr int kRadixItems = 8;
constexpr int kRadixTile = kRadixThreads * kRadixItems;  // 2048 keys per tile
constexpr int kRadixWarps = kRadixThreads / 32;
constexpr int kRadixWarpSpan = kRadixTile / kRadixWarps;  // 256 keys per warp

// per-substep counters, zeroed by k_grid_setup
constexpr int kStepCounters = 8;
// [kCntCells] occupied cells listed by k_gather, [kCntWorkDensity] cells
// taken by the cell-warp density search, [kCntRadixTile + p] tiles taken by
// radix pass p
enum : int { kCntCells = 0, kCntWorkDensity = 1, kCntRadixTile = 4 };

enum : uint32_t {
  kFlagGridOverflow = 1u,
  kFlagCollisionCap = 2u,
  kFlagNonFinite = 4u,
  kFlagSortStall = 1u << 16,  // internal: a radix look-back wait ran out
};

struct DevGrid {         // one scene's grid of the current substep
  float lo[3];
  float hi[3];
  float cell;           // 2h
  int32_t size[3];      // grid_size_x/y/z
  uint32_t cells;       // grid_cell_count (dense Morton range)
  float half_margin;    // rounding margin of the half-cell tests, in cells
  uint32_t pad_[4];
};

// 8-bit radix passes that cover every key of the substep.
__host__ __device__ __forceinline__ uint32_t radix_passes(uint32_t maxkey) {
  uint32_t k = maxkey | 1u, bits = 0;
  while (k) { ++bits; k >>= 1; }
  return (bits + 7u) / 8u;
}
// Ping-pong buffer that holds the sorted keys and slots after all passes.
__host__ __device__ __forceinline__ uint32_t sorted_sel(uint32_t maxkey) {
  return radix_passes(maxkey) & 1u;
}

// Sort control block of a substep (device memory): [0] largest key,
// [1] Morton bits (widest grid of all scenes), [2] scene bits.
enum : int { kCtlMaxKey = 0, kCtlShift = 1, kCtlSceneBits = 2, kCtlWords = 8 };

// Scene bits of a sort key and its Morton part.
struct KeySplit {
  uint32_t shift;  // Morton keys use bits [0, shift)
  __host__ __device__ __forceinline__ uint32_t morton(uint32_t key) const {
    return shift >= 32u ? key : (key & ((1u << shift) - 1u));
  }
  __host__ __device__ __forceinline__ uint32_t scene_bits(uint32_t scene) const {
    return shift >= 32u ? 0u : (scene << shift);
  }
};

// Per-substep constants (kernel argument).
struct Consts {
  uint32_t n;
  float h, mass, rho0, K, mu, sigma, sigma_threshold, restitution;
  float time_delta, scale, vmax;
  float gx, gy, gz;
  float poly6, grad6, lap6, spiky, visc, spiky_zero;
  float cull_r2;  // conservative h^2 for the FMA cull test
};

struct State {
  float4* pos;
  float4* vel;
  float4* ivel;
};

struct CellIndex {
  uint32_t* keys;   // key + 1, 0 = empty
  uint32_t* start;
  uint32_t* end;
  uint32_t mask;    // slots - 1 (power of two)
  uint32_t shift;   // 32 - log2(slots)
};

struct DevMesh {
  const float* normals;     // 3 per face
  const float* vertices;    // 3 per vertex
  const uint32_t* indices;  // 3 per face
  uint32_t faces;
  // per-cell triangle lists (CSR over a uniform grid covering the mesh)
  const uint32_t* cell_start;  // dims product + 1
  const uint32_t* cell_faces;
  float lo[3];
  float inv_cell;
  int32_t dims[3];
  float reach;  // longest segment a cell list covers
};

// ------------------------------------------------------------ cell index
__device__ __forceinline__ uint32_t cell_slot_insert(const CellIndex& ci, uint32_t key) {
  const uint32_t tag = key + 1u;
  uint32_t slot = cell_hash(key) >> ci.shift;
  for (uint32_t probe = 0; probe <= ci.mask; ++probe) {
    uint32_t prev = atomicCAS(&ci.keys[slot], 0u, tag);
    if (prev == 0u || prev == tag) return slot;
    slot = (slot + 1u) & ci.mask;
  }
  return 0xFFFFFFFFu;  // unreachable: at most n keys in >= 2n slots
}

__device__ __forceinline__ uint2 cell_lookup(const CellIndex& ci, uint32_t key) {
  const uint32_t tag = key + 1u;
  uint32_t slot = cell_hash(key) >> ci.shift;
  for (uint32_t probe = 0; probe <= ci.mask; ++probe) {
    uint32_t k = __ldg(&ci.keys[slot]);
    if (k == tag) return make_uint2(__ldg(&ci.start[slot]), __ldg(&ci.end[slot]));
    if (k == 0u) break;
    slot = (slot + 1u) & ci.mask;
  }
  return make_uint2(0u, 0u);
}

// ---------------------------------------------------- neighbour cell window
// The support radius is h but cells are 2h wide (grid.cl:56-61 vs
// smoothing.cl:2). Each particle carries, per axis, whether it may lie in the
// lower half of its cell (bit 2a) and whether it may lie in the upper half
// (bit 2a+1), decided with a rounding margin so that a particle near the
// middle has both bits. A particle with only the lower bit cannot be within
// h of anything in the next cell up (the distance is > half a cell = h), and
// symmetrically; cells and particles so excluded contribute exact zeros in
// the reference, so skipping them keeps the reference's summation sequence.
// The code is computed after the sort and kept in pos.w of the sorted state.
__device__ __forceinline__ uint32_t half_code(float4 p, uint32_t key, const DevGrid& g) {
  const uint32_t c[3] = {compact_bits3(key), compact_bits3(key >> 1), compact_bits3(key >> 2)};
  const float pc[3] = {p.x, p.y, p.z};
  uint32_t code = 0;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float frac = XDIV(XSUB(pc[a], g.lo[a]), g.cell) - (float)c[a];
    code |= (frac < 0.5f + g.half_margin ? 1u : 0u) << (2 * a);
    code |= (frac > 0.5f - g.half_margin ? 1u : 0u) << (2 * a + 1);
  }
  return code;
}

struct Window {
  uint32_t lo[3], hi[3];
};

__device__ __forceinline__ Window neighbour_window(float4 p, uint32_t key, const DevGrid& g) {
  const uint32_t c[3] = {compact_bits3(key), compact_bits3(key >> 1), compact_bits3(key >> 2)};
  const uint32_t code = __float_as_uint(p.w);
  Window w;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    w.lo[a] = ((code >> (2 * a)) & 1u) ? c[a] - 1u : c[a];
    w.hi[a] = ((code >> (2 * a + 1)) & 1u) ? c[a] + 1u : c[a];
  }
  return w;
}

// --------------------------------------------------------------- kernels

// Grid set-up of every scene (sph_simulation.cpp:199-252), one thread per
// scene, from the bounding boxes accumulated by the previous kernel; resets
// the boxes, the radix digit totals and the sort control for this substep.
// (The kernels of this file are thin wrappers around block-level bodies with
// their shared memory passed in, so the persistent substep kernel of
// clsph_persistent.cuh runs the same code on its own blocks.)
__device__ __forceinline__ void grid_setup_block(uint32_t* __restrict__ bbox_all, DevGrid* __restrict__ grids,
                                                 const float* __restrict__ scene_h, uint32_t nscenes,
                                                 uint32_t* __restrict__ status, uint32_t* __restrict__ digit_total,
                                                 uint32_t* __restrict__ step_counters, uint32_t* __restrict__ ctl,
                                                 uint32_t& shift_s) {
  for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x) digit_total[i] = 0u;
  if (threadIdx.x < kStepCounters) step_counters[threadIdx.x] = 0u;
  if (threadIdx.x == 0) shift_s = 1u;
  __syncthreads();
  for (uint32_t sc = threadIdx.x; sc < nscenes; sc += blockDim.x) {
  uint32_t* bbox = bbox_all + 6 * (size_t)sc;
  DevGrid* grid = grids + sc;
  const float cell = XMUL(scene_h[sc], 2.f);
  DevGrid g;
  bool overflow = false;
  for (int a = 0; a < 3; ++a) {
    float mn = ord2f(bbox[a]);
    float mx = ord2f(bbox[3 + a]);
    mn = XSUB(mn, XMUL(cell, 2.f));
    mx = XADD(mx, XMUL(cell, 2.f));
    g.lo[a] = mn;
    g.hi[a] = mx;
    uint32_t sz = __float2uint_rz(XDIV(XSUB(mx, mn), cell));
    g.size[a] = (int32_t)sz;
    if (g.size[a] < 0 || g.size[a] >= 1024) overflow = true;
  }
  g.cell = cell;
  g.cells = morton3((uint32_t)g.size[0], (uint32_t)g.size[1], (uint32_t)g.size[2]);
  atomicMax(&shift_s, 32u - __clz(g.cells | 1u));  // keys of this scene are < cells
  // The cell coordinate t = fl(fl(p - lo) / 2h) is within ~2^-22 * t of the
  // exact value and t < grid size G, so 2^-20 * (G + 2) covers its rounding
  // and that of the distance test twice over.
  const int gmax = max(g.size[0], max(g.size[1], g.size[2]));
  g.half_margin = (float)(gmax + 2) * 0x1p-20f;
  for (int i = 0; i < 4; ++i) g.pad_[i] = 0u;
  *grid = g;
  if (overflow) atomicOr(status, kFlagGridOverflow);
  // sentinels of sph_simulation.cpp:204-205 for the next accumulation
  for (int a = 0; a < 3; ++a) {
    bbox[a] = f2ord(2147483648.0f);
    bbox[3 + a] = f2ord(-2147483648.0f);
  }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    ctl[kCtlMaxKey] = 0u;
    ctl[kCtlShift] = shift_s;
    // scene bits above the Morton bits must fit in 32 (batched scenes)
    if (shift_s + ctl[kCtlSceneBits] > 32u) atomicOr(status, kFlagGridOverflow);
  }
}

static __global__ void k_grid_setup(uint32_t* __restrict__ bbox_all, DevGrid* __restrict__ grids,
                                    const float* __restrict__ scene_h, uint32_t nscenes,
                                    uint32_t* __restrict__ status, uint32_t* __restrict__ digit_total,
                                    uint32_t* __restrict__ step_counters, uint32_t* __restrict__ ctl) {
  __shared__ uint32_t shift_s;
  grid_setup_block(bbox_all, grids, scene_h, nscenes, status, digit_total, step_counters, ctl, shift_s);
}

static __global__ void k_bbox_reset(uint32_t* __restrict__ bbox, uint32_t nscenes) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < 6 * nscenes; k += gridDim.x * blockDim.x)
    bbox[k] = (k % 6) < 3 ? f2ord(2147483648.0f) : f2ord(-2147483648.0f);
}

// Per-scene min/max of positions: a block whose threads all saw one scene
// reduces to one atomic per axis; otherwise every warp (or, across a scene
// boundary, every thread) adds its own. NaN coordinates are ignored, as the
// reference's `<` / `>` tests do. A thread with no particle passes scene = -1.
__device__ __forceinline__ void bbox_atomics(const float v[6], uint32_t* bbox) {
  if (v[0] == v[0]) atomicMin(&bbox[0], f2ord(v[0]));
  if (v[1] == v[1]) atomicMin(&bbox[1], f2ord(v[1]));
  if (v[2] == v[2]) atomicMin(&bbox[2], f2ord(v[2]));
  if (v[3] == v[3]) atomicMax(&bbox[3], f2ord(v[3]));
  if (v[4] == v[4]) atomicMax(&bbox[4], f2ord(v[4]));
  if (v[5] == v[5]) atomicMax(&bbox[5], f2ord(v[5]));
}

struct BboxSmem {
  int block_scene;
  float red[6][kBlock / 32];
};

__device__ __forceinline__ void bbox_accumulate(float3 lo, float3 hi, int scene, uint32_t* bbox_all,
                                                BboxSmem& sm) {
  int& block_scene = sm.block_scene;
  auto& red = sm.red;
  if (threadIdx.x == 0) block_scene = -2;
  __syncthreads();
  if (scene >= 0) atomicCAS(&block_scene, -2, scene);
  __syncthreads();
  const int s0 = block_scene;
  const bool uniform = __syncthreads_and(scene < 0 || scene == s0);
  if (!uniform) {
    const float v[6] = {lo.x, lo.y, lo.z, hi.x, hi.y, hi.z};
    if (scene >= 0) bbox_atomics(v, bbox_all + 6 * (size_t)scene);
    return;
  }
  if (s0 < 0) return;
  uint32_t* bbox = bbox_all + 6 * (size_t)s0;
  float v[6] = {lo.x, lo.y, lo.z, hi.x, hi.y, hi.z};
#pragma unroll
  for (int k = 0; k < 6; ++k) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      float o = __shfl_xor_sync(0xFFFFFFFFu, v[k], off);
      v[k] = k < 3 ? fminf(v[k], o) : fmaxf(v[k], o);
    }
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0)
    for (int k = 0; k < 6; ++k) red[k][warp] = v[k];
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      float x = lane < nw ? red[k][lane] : __int_as_float(0x7FC00000);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        float o = __shfl_xor_sync(0xFFFFFFFFu, x, off);
        x = k < 3 ? fminf(x, o) : fmaxf(x, o);
      }
      if (lane == 0 && x == x) {
        if (k < 3)
          atomicMin(&bbox[k], f2ord(x));
        else
          atomicMax(&bbox[k], f2ord(x));
      }
    }
  }
}

__device__ __forceinline__ void bbox_accumulate(float3 lo, float3 hi, int scene, uint32_t* bbox_all) {
  __shared__ BboxSmem sm;
  bbox_accumulate(lo, hi, scene, bbox_all, sm);
}

// Host AoS (80-byte particle records, 5 float4 each) -> SoA state, with
// bounding box. One thread per float4 of the record array, so a warp reads
// 512 contiguous bytes: `aos` is the device staging copy or, for pinned host
// memory, the caller's records themselves, read over the host link.
static __global__ void k_unpack_aos(const float4* __restrict__ aos, uint32_t n, State st,
                             const uint16_t* __restrict__ scene_of, uint32_t* __restrict__ bbox,
                             uint32_t* __restrict__ status) {
  const float qnan = __int_as_float(0x7FC00000);
  const size_t words = (size_t)n * 5;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t base = (size_t)blockIdx.x * blockDim.x; base < words; base += stride) {
    const size_t q = base + threadIdx.x;
    float3 lo = make_float3(qnan, qnan, qnan), hi = lo;
    int scene = -1;
    if (q < words) {
      const uint32_t i = (uint32_t)(q / 5), f = (uint32_t)(q - (size_t)i * 5);
      if (f < 3) {  // position, velocity, intermediate velocity; the rest is output only
        float4 v = aos[q];
        v.w = 0.f;
        if (f == 0) {
          st.pos[i] = v;
          lo = make_float3(v.x, v.y, v.z);
          hi = lo;
          scene = scene_of[i];
          if (!(isfinite(v.x) && isfinite(v.y) && isfinite(v.z))) atomicOr(status, kFlagNonFinite);
        } else if (f == 1) {
          st.vel[i] = v;
        } else {
          st.ivel[i] = v;
        }
      }
    }
    bbox_accumulate(lo, hi, scene, bbox);
  }
}

// SoA -> host AoS: acceleration is 0 after the advection loop (sph.cl:97-99).
// One thread per float4 of the record array (contiguous stores), into the
// staging copy or straight into pinned host memory.
static __global__ void k_pack_aos(float4* __restrict__ aos, uint32_t n, State st,
                           const float4* __restrict__ aux, const uint32_t* __restrict__ keys_base,
                           const uint32_t* __restrict__ ctl, int have_fields) {
  const KeySplit split{ctl[kCtlShift]};
  const uint32_t sel = have_fields ? sorted_sel(ctl[kCtlMaxKey]) : 0u;
  const uint32_t* keys = keys_base + (size_t)sel * n;
  const size_t words = (size_t)n * 5;
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < words; q += (size_t)gridDim.x * blockDim.x) {
    const uint32_t i = (uint32_t)(q / 5), f = (uint32_t)(q - (size_t)i * 5);
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (f == 0) {
      v = st.pos[i];
    } else if (f == 1) {
      v = st.vel[i];
    } else if (f == 2) {
      v = st.ivel[i];
    } else if (f == 4 && have_fields) {  // density, pressure, grid cell code, 0
      const float4 a = aux[i];
      v.x = a.x;
      v.y = a.y;
      v.z = __uint_as_float(split.morton(keys[i]));
    }
    aos[q] = v;
  }
}

// Morton key per particle (grid.cl:56-66) and the largest key.
__device__ __forceinline__ void keys_block(uint32_t vb, const float4* __restrict__ pos, uint32_t n,
                                           const DevGrid* __restrict__ grids,
                                           const uint16_t* __restrict__ scene_of, uint32_t* __restrict__ ctl,
                                           uint32_t* __restrict__ keys, uint32_t& block_max) {
  const KeySplit split{ctl[kCtlShift]};
  if (threadIdx.x == 0) block_max = 0u;
  __syncthreads();
  const uint32_t i = vb * blockDim.x + threadIdx.x;
  uint32_t key = 0u;
  if (i < n) {
    const uint32_t sc = scene_of[i];
    const DevGrid& g = grids[sc];
    const float4 p = pos[i];
    uint32_t cx = __float2uint_rz(XDIV(XSUB(p.x, g.lo[0]), g.cell));
    uint32_t cy = __float2uint_rz(XDIV(XSUB(p.y, g.lo[1]), g.cell));
    uint32_t cz = __float2uint_rz(XDIV(XSUB(p.z, g.lo[2]), g.cell));
    key = morton3(cx, cy, cz) | split.scene_bits(sc);
    keys[i] = key;
  }
  key = __reduce_max_sync(0xFFFFFFFFu, key);
  if ((threadIdx.x & 31) == 0) atomicMax(&block_max, key);
  __syncthreads();
  if (threadIdx.x == 0) atomicMax(&ctl[kCtlMaxKey], block_max);
}

// Also clears the cell index for this substep's k_gather (16 bytes a thread,
// grid-stride), which no kernel between the two reads.
static __global__ void __launch_bounds__(kBlock)
    k_keys(const float4* __restrict__ pos, uint32_t n, const DevGrid* __restrict__ grids,
           const uint16_t* __restrict__ scene_of, uint32_t* __restrict__ ctl,
           uint32_t* __restrict__ keys, uint4* __restrict__ index_keys, uint32_t index_quads) {
  __shared__ uint32_t block_max;
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < index_quads; q += gridDim.x * blockDim.x)
    index_keys[q] = make_uint4(0u, 0u, 0u, 0u);
  keys_block(blockIdx.x, pos, n, grids, scene_of, ctl, keys, block_max);
}

// ---------------------------------------------------------------- radix sort
// Stable LSD radix sort of (key, slot) with 8-bit digits in one-sweep form:
// k_radix_hist reads the keys once and counts the digits of every pass;
// k_radix_onesweep (one launch per pass) ranks a 2048-key tile in shared
// memory, publishes the tile's per-digit counts, finds the counts of all
// earlier tiles by decoupled look-back (each digit's thread walks back over
// the published words until it meets an inclusive prefix) and scatters.
// Passes beyond radix_passes return at once, so the launch sequence is fixed
// (graph-capturable) while the work follows the key width. Ping-pong: pass p
// reads buffer p&1 and writes (p+1)&1.
//
// Look-back words (one per tile and digit, per pass): bits 30-31 the state
// (0 not yet published, 1 the tile's own count, 2 the inclusive prefix of
// all tiles up to it), bits 0-29 the value (n < 2^28). Tiles are numbered in
// the order blocks start (an atomic ticket), so every tile a block waits for
// belongs to a block that is already running and publishes without waiting
// itself; the wait is bounded all the same (spin_limit, by default
// kRadixLookbackSpins), and a wait that runs out raises kFlagSortStall, which
// clsph_gpu_sync reports as an error. After a stall the offsets of the tiles
// behind it are wrong, but every store stays in bounds (destinations >= n are
// skipped, and the slots a pass leaves unwritten keep earlier in-range
// values), so the context stays usable.
//
// withheld_tile (a test hook of clsph_gpu_set_wait_limits; kNoTile in normal
// use): that tile never publishes its words, so the tile after it waits on a
// word that nothing sets until its spin limit runs out.
constexpr uint32_t kRadixLookbackSpins = 1u << 20;
constexpr uint32_t kNoTile = 0xFFFFFFFFu;
constexpr uint32_t kLbAggregate = 1u << 30, kLbInclusive = 2u << 30, kLbValue = (1u << 30) - 1u;

__device__ __forceinline__ uint32_t ld_relaxed_gpu(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_gpu(uint32_t* p, uint32_t v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;\n" ::"l"(p), "r"(v) : "memory");
}

// Digit counts of every pass in one read of the keys (16-byte loads), and the
// look-back words of this substep's passes cleared.
__device__ __forceinline__ void radix_hist_blocks(uint32_t blk, uint32_t nblk, const uint32_t* __restrict__ keys,
                                                  uint32_t n, const uint32_t* __restrict__ ctl,
                                                  uint32_t* __restrict__ digit_total,
                                                  uint32_t* __restrict__ lookback, uint32_t ntiles,
                                                  uint32_t (&hist)[4][256]) {
  const uint32_t passes = radix_passes(ctl[kCtlMaxKey]);
  for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x) hist[i >> 8][i & 255] = 0u;
  const size_t gtid = (size_t)blk * blockDim.x + threadIdx.x;
  const size_t gstride = (size_t)nblk * blockDim.x;
  const size_t words = (size_t)passes * ntiles * 256u;
  for (size_t i = gtid; i < words; i += gstride) lookback[i] = 0u;
  __syncthreads();
  auto count = [&](uint32_t key) {
    for (uint32_t p = 0; p < passes; ++p) atomicAdd(&hist[p][(key >> (8 * p)) & 0xFFu], 1u);
  };
  const uint32_t n4 = n / 4u;
  for (size_t q = gtid; q < n4; q += gstride) {
    const uint4 k = __ldg(reinterpret_cast<const uint4*>(keys) + q);
    count(k.x);
    count(k.y);
    count(k.z);
    count(k.w);
  }
  if (gtid < (n & 3u)) count(__ldg(&keys[4u * n4 + gtid]));
  __syncthreads();
  for (uint32_t p = 0; p < passes; ++p) {
    const uint32_t c = hist[p][threadIdx.x];
    if (c) atomicAdd(&digit_total[p * 256 + threadIdx.x], c);
  }
}

static __global__ void __launch_bounds__(kRadixThreads)
    k_radix_hist(const uint32_t* __restrict__ keys, uint32_t n, const uint32_t* __restrict__ ctl,
                 uint32_t* __restrict__ digit_total, uint32_t* __restrict__ lookback, uint32_t ntiles) {
  __shared__ uint32_t hist[4][256];
  radix_hist_blocks(blockIdx.x, gridDim.x, keys, n, ctl, digit_total, lookback, ntiles, hist);
}

struct RadixSmem {
  uint32_t cnt[kRadixWarps][256];
  uint32_t hist[256];
  uint32_t tile_off[256];
  uint32_t warp_sums[kRadixWarps];
  uint32_t tile_s;
};

// One tile of one radix pass: takes the next tile number from the ticket;
// returns false (the whole block) once every tile of the pass is taken.
__device__ __forceinline__ bool radix_sweep_tile(uint32_t* __restrict__ keys_base, uint32_t* __restrict__ vals_base,
                                                 uint32_t n, int pass, const uint32_t* __restrict__ digit_total,
                                                 uint32_t* __restrict__ lookback, uint32_t ntiles,
                                                 uint32_t* __restrict__ tile_ticket, uint32_t* __restrict__ status,
                                                 uint32_t spin_limit, uint32_t withheld_tile, RadixSmem& sm) {
  auto& cnt = sm.cnt;
  auto& hist = sm.hist;
  auto& tile_off = sm.tile_off;
  auto& warp_sums = sm.warp_sums;
  uint32_t& tile_s = sm.tile_s;
  __syncthreads();  // the block's previous tile is done with the shared arrays
  const uint32_t* keys_in = keys_base + (size_t)(pass & 1) * n;
  uint32_t* keys_out = keys_base + (size_t)((pass + 1) & 1) * n;
  const uint32_t* vals_in = vals_base + (size_t)(pass & 1) * n;
  uint32_t* vals_out = vals_base + (size_t)((pass + 1) & 1) * n;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) tile_s = atomicAdd(tile_ticket, 1u);
  for (int w = 0; w < kRadixWarps; ++w) cnt[w][threadIdx.x] = 0u;
  hist[threadIdx.x] = 0u;
  __syncthreads();
  const uint32_t tile = tile_s;
  if (tile >= ntiles) return false;
  const int shift = 8 * pass;
  const uint32_t lt_mask = (1u << lane) - 1u;
  const uint32_t base = tile * kRadixTile + warp * kRadixWarpSpan;
  uint32_t key[kRadixItems], val[kRadixItems], rank[kRadixItems];
  // the tile's keys and its digit counts, published before the ranking so
  // that later tiles' look-back finds them as early as possible
#pragma unroll
  for (int r = 0; r < kRadixItems; ++r) {
    const uint32_t idx = base + r * 32 + lane;
    const bool valid = idx < n;
    key[r] = valid ? keys_in[idx] : 0u;
    val[r] = valid ? (pass == 0 ? idx : vals_in[idx]) : 0u;
    if (valid) atomicAdd(&hist[(key[r] >> shift) & 0xFFu], 1u);
  }
  __syncthreads();
  const uint32_t d = threadIdx.x;  // this thread's digit in the look-back and the offsets
  const uint32_t local = hist[d];  // the tile's count of digit d
  uint32_t* lb = lookback + (size_t)pass * ntiles * 256u;
  const bool publish = tile != withheld_tile;
  if (publish) st_relaxed_gpu(&lb[(size_t)tile * 256u + d], (tile == 0 ? kLbInclusive : kLbAggregate) | local);
  // ranks within the tile: per warp in key order (rows of 32), then warps in order
#pragma unroll
  for (int r = 0; r < kRadixItems; ++r) {
    const uint32_t idx = base + r * 32 + lane;
    const bool valid = idx < n;
    const uint32_t dr = valid ? ((key[r] >> shift) & 0xFFu) : 256u;
    const uint32_t peers = __match_any_sync(0xFFFFFFFFu, dr);
    uint32_t rk = 0;
    if (valid) rk = cnt[warp][dr] + __popc(peers & lt_mask);
    __syncwarp();
    if (valid && (peers & lt_mask) == 0u) cnt[warp][dr] += __popc(peers);
    __syncwarp();
    rank[r] = valid ? ((rk << 8) | dr) : 0xFFFFFFFFu;
  }
  uint32_t excl = 0;  // digit d in all earlier tiles
  if (tile > 0) {
    // walk back kLookbackWindow tiles per round (independent loads), adding
    // published counts until an inclusive prefix (tile 0 always has one)
    constexpr int kLookbackWindow = 4;
    int64_t t = (int64_t)tile - 1;
    uint32_t spins = 0;
    bool done = false;
    while (!done) {
      uint32_t w[kLookbackWindow];
#pragma unroll
      for (int k = 0; k < kLookbackWindow; ++k)
        w[k] = t - k >= 0 ? ld_relaxed_gpu(&lb[(size_t)(t - k) * 256u + d]) : kLbInclusive;
      int used = 0;
#pragma unroll
      for (int k = 0; k < kLookbackWindow; ++k) {
        if (done || used < k) break;       // stopped at an earlier word of this round
        if ((w[k] & ~kLbValue) == 0u) break;  // not published yet: load it again
        excl += w[k] & kLbValue;
        ++used;
        if (w[k] & kLbInclusive) done = true;
      }
      t -= used;
      if (!done && used == 0) {
        if (++spins > spin_limit) {
          atomicOr(status, kFlagSortStall);
          break;
        }
        __nanosleep(32);
      }
    }
    if (publish) st_relaxed_gpu(&lb[(size_t)tile * 256u + d], kLbInclusive | (excl + local));
  }
  __syncthreads();
  {  // per digit: exclusive prefix over warps
    uint32_t run = 0;
    for (int w = 0; w < kRadixWarps; ++w) {
      const uint32_t c = cnt[w][d];
      cnt[w][d] = run;
      run += c;
    }
  }
  // keys with a smaller digit: exclusive scan of the pass's digit totals
  const uint32_t tot = digit_total[pass * 256 + d];
  uint32_t x = tot;
  for (int off = 1; off < 32; off <<= 1) {
    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, off);
    if (lane >= off) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  uint32_t below = x - tot;
  for (int w = 0; w < warp; ++w) below += warp_sums[w];
  tile_off[d] = below + excl;
  __syncthreads();
#pragma unroll
  for (int r = 0; r < kRadixItems; ++r) {
    if (rank[r] == 0xFFFFFFFFu) continue;
    const uint32_t dd = rank[r] & 0xFFu;
    const uint32_t dst = tile_off[dd] + cnt[warp][dd] + (rank[r] >> 8);
    if (dst >= n) continue;  // only after a look-back wait ran out (flagged)
    keys_out[dst] = key[r];
    vals_out[dst] = val[r];
  }
  return true;
}

static __global__ void __launch_bounds__(kRadixThreads)
    k_radix_onesweep(uint32_t* __restrict__ keys_base, uint32_t* __restrict__ vals_base, uint32_t n,
                     int pass, const uint32_t* __restrict__ ctl, const uint32_t* __restrict__ digit_total,
                     uint32_t* __restrict__ lookback, uint32_t ntiles, uint32_t* __restrict__ tile_ticket,
                     uint32_t* __restrict__ status, uint32_t spin_limit, uint32_t withheld_tile) {
  if ((uint32_t)pass >= radix_passes(ctl[kCtlMaxKey])) return;
  __shared__ RadixSmem sm;
  radix_sweep_tile(keys_base, vals_base, n, pass, digit_total, lookback, ntiles, tile_ticket, status,
                   spin_limit, withheld_tile, sm);
}

// Gathers the state into sorted order (the stable scatter of sort.cl:41-59)
// and records every cell's [start, end) in the cell index (the dense cell
// table of sph_simulation.cpp:162-170 in compact form).
// Cell starts join the cell list with one atomic per block (slot order is
// kept within the block, so the list stays close to sorted order).
struct GatherSmem {
  uint32_t warp_base[kBlock / 32];
  uint32_t block_base;
};

__device__ __forceinline__ void gather_block(uint32_t vb, uint32_t n, const DevGrid* __restrict__ grids,
                                             const uint16_t* __restrict__ scene_of,
                                             const uint32_t* __restrict__ ctl,
                                             const uint32_t* __restrict__ keys_base,
                                             const uint32_t* __restrict__ vals_base, State src, State dst,
                                             const uint32_t* __restrict__ ids_src, uint32_t* __restrict__ ids_dst,
                                             CellIndex ci, uint32_t* __restrict__ cell_list,
                                             uint32_t* __restrict__ cell_count, GatherSmem& sm) {
  auto& warp_base = sm.warp_base;
  uint32_t& block_base = sm.block_base;
  const uint32_t s = vb * blockDim.x + threadIdx.x;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const KeySplit split{ctl[kCtlShift]};
  const uint32_t sel = sorted_sel(ctl[kCtlMaxKey]);
  const uint32_t* keys = keys_base + (size_t)sel * n;
  const uint32_t* perm = vals_base + (size_t)sel * n;
  bool first = false;
  if (s < n) {
    const uint32_t from = min(perm[s], n - 1u);  // in range even after a flagged sort stall
    const uint32_t key = keys[s];
    float4 p = src.pos[from];
    p.w = __uint_as_float(half_code(p, split.morton(key), grids[scene_of[s]]));
    dst.pos[s] = p;
    dst.vel[s] = src.vel[from];
    dst.ivel[s] = src.ivel[from];
    ids_dst[s] = ids_src[from];
    first = s == 0 || keys[s - 1] != key;
    if (first) {
      uint32_t slot = cell_slot_insert(ci, key);
      if (slot != 0xFFFFFFFFu) ci.start[slot] = s;
    }
    if (s + 1 == n || keys[s + 1] != key) {
      uint32_t slot = cell_slot_insert(ci, key);
      if (slot != 0xFFFFFFFFu) ci.end[slot] = s + 1;
    }
  }
  const uint32_t bal = __ballot_sync(0xFFFFFFFFu, first);
  if (lane == 0) warp_base[warp] = __popc(bal);
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t run = 0;
    for (int w = 0; w < kBlock / 32; ++w) {
      const uint32_t c = warp_base[w];
      warp_base[w] = run;
      run += c;
    }
    block_base = run ? atomicAdd(cell_count, run) : 0u;
  }
  __syncthreads();
  if (first) cell_list[block_base + warp_base[warp] + __popc(bal & ((1u << lane) - 1u))] = s;
  __syncthreads();  // the shared counts are read before the block's next use
}

static __global__ void __launch_bounds__(kBlock)
    k_gather(uint32_t n, const DevGrid* __restrict__ grids,
             const uint16_t* __restrict__ scene_of, const uint32_t* __restrict__ ctl,
             const uint32_t* __restrict__ keys_base,
             const uint32_t* __restrict__ vals_base, State src, State dst,
             const uint32_t* __restrict__ ids_src, uint32_t* __restrict__ ids_dst,
             CellIndex ci, uint32_t* __restrict__ cell_list,
             uint32_t* __restrict__ cell_count) {
  __shared__ GatherSmem sm;
  gather_block(blockIdx.x, n, grids, scene_of, ctl, keys_base, vals_base, src, dst, ids_src, ids_dst, ci,
               cell_list, cell_count, sm);
}

// ------------------------------------------------- density and forces
// Both gathers visit neighbours in the reference's order (27 cells in z, y, x
// order, each cell's particles in sorted order; only the window cells can
// contribute, the others add exact zeros) and evaluate every contributing
// pair with IEEE round-to-nearest operations in the reference's expression
// order, so the sums are bit-identical to the reference's.
//
// A candidate j contributes iff fl(r/h) < 1 (the (1 - clamp(floor(r/h),0,1))
// factor of smoothing.cl). For floats r >= 0 and h > 0 that is exactly r < h:
// fl(r/h) < 1 iff r/h < 1 - 2^-25, i.e. r < h(1 - 2^-25), and no float lies in
// [h(1 - 2^-25), h) because the float below h is at most h(1 - 2^-24).
//
// Per particle the density kernel also stores (rho, p, m/rho, p/rho^2) -- the
// same IEEE quotients the reference forms per pair -- and the list of its
// contributing neighbours in visiting order (column-major, nlist[k*n + i]),
// which the forces kernel walks without a second search. The list is stored
// and read with evict-first (streaming) hints: it is read once, and at 1M
// particles it is larger than L2, where the neighbour records should stay.

constexpr int kGatherBlock = 128;

// Tait pressure (sph.cl:36-39): K * (pown(rho / rho0, 7) - 1).
__device__ __forceinline__ float tait_pressure(float rho, const Consts& c) {
  const float x = XDIV(rho, c.rho0);
  float p7 = x;
#pragma unroll
  for (int k = 1; k < 7; ++k) p7 = XMUL(p7, x);
  return XMUL(c.K, XSUB(p7, 1.f));
}

__device__ __forceinline__ float4 density_aux(float rho, const Consts& c) {
  const float p = tait_pressure(rho, c);
  return make_float4(rho, p, XDIV(c.mass, rho), XDIV(p, XMUL(rho, rho)));
}

// m * W_poly6(r) for a contributing pair (forces.cl:33-36, smoothing.cl:1-4).
__device__ __forceinline__ float poly6_term(float rr, float hh, const Consts& c) {
  const float q = XSUB(hh, XMUL(rr, rr));
  return XMUL(c.mass, XMUL(c.poly6, XMUL(XMUL(q, q), q)));
}

struct ForceSums {
  V3 P, Vs, Nm;
  float lap;
};

// One contributing pair of forces.cl:67-97. aux_j = (rho_j, p_j, m/rho_j, p_j/rho_j^2).
__device__ __forceinline__ void force_pair(ForceSums& f, bool self, V3 d, float rr, float4 vi,
                                           float4 vj, float4 aux_j, float own, float hh,
                                           float lap_b, const Consts& c) {
  const float mj = aux_j.z;
  if (!self) {
    const float coef = XMUL(XADD(aux_j.w, own), c.mass);
    V3 sg;
    if (XSUB(rr, 0.0000001f) < 0.f) {  // smoothing.cl:23-25
      sg = {c.spiky_zero, c.spiky_zero, c.spiky_zero};
    } else {
      const float q = XSUB(c.h, rr);
      const float q2 = XMUL(q, q);
      sg = {XMUL(XMUL(c.spiky, XDIV(d.x, rr)), q2), XMUL(XMUL(c.spiky, XDIV(d.y, rr)), q2),
            XMUL(XMUL(c.spiky, XDIV(d.z, rr)), q2)};
    }
    f.P.x = XADD(f.P.x, XMUL(coef, sg.x));
    f.P.y = XADD(f.P.y, XMUL(coef, sg.y));
    f.P.z = XADD(f.P.z, XMUL(coef, sg.z));
    const float vl = XMUL(c.visc, XSUB(c.h, rr));
    f.Vs.x = XADD(f.Vs.x, XMUL(XMUL(XSUB(vj.x, vi.x), mj), vl));
    f.Vs.y = XADD(f.Vs.y, XMUL(XMUL(XSUB(vj.y, vi.y), mj), vl));
    f.Vs.z = XADD(f.Vs.z, XMUL(XMUL(XSUB(vj.z, vi.z), mj), vl));
  }
  const float q = XSUB(hh, XMUL(rr, rr));
  const float q2 = XMUL(q, q);
  f.Nm.x = XADD(f.Nm.x, XMUL(mj, XMUL(XMUL(c.grad6, d.x), q2)));
  f.Nm.y = XADD(f.Nm.y, XMUL(mj, XMUL(XMUL(c.grad6, d.y), q2)));
  f.Nm.z = XADD(f.Nm.z, XMUL(mj, XMUL(XMUL(c.grad6, d.z), q2)));
  f.lap = XADD(f.lap, XMUL(mj, XMUL(XMUL(c.lap6, q), XSUB(lap_b, XMUL(7.f, XMUL(rr, rr))))));
}

// forces.cl:103-109 then sph.cl:53-58.
__device__ __forceinline__ float4 finish_accel(const ForceSums& f, float rho_i, const Consts& c) {
  const float nr = -rho_i;
  V3 sum = {XADD(XMUL(nr, f.P.x), XMUL(f.Vs.x, c.mu)), XADD(XMUL(nr, f.P.y), XMUL(f.Vs.y, c.mu)),
            XADD(XMUL(nr, f.P.z), XMUL(f.Vs.z, c.mu))};
  const float nl = xnorm(f.Nm);
  if (nl > c.sigma_threshold) {
    const float s = XMUL(-c.sigma, f.lap);
    sum.x = XADD(sum.x, XDIV(XMUL(s, f.Nm.x), nl));
    sum.y = XADD(sum.y, XDIV(XMUL(s, f.Nm.y), nl));
    sum.z = XADD(sum.z, XDIV(XMUL(s, f.Nm.z), nl));
  }
  return make_float4(XADD(XDIV(sum.x, rho_i), c.gx), XADD(XDIV(sum.y, rho_i), c.gy),
                     XADD(XDIV(sum.z, rho_i), c.gz), 0.f);
}

// Calls f(j) for every candidate of particle i's window in the reference's order.
template <class F>
__device__ __forceinline__ void for_each_candidate(const Window& w, uint32_t sbits,
                                                   const CellIndex& ci, F&& f) {
  for (uint32_t z = w.lo[2]; z <= w.hi[2]; ++z)
    for (uint32_t y = w.lo[1]; y <= w.hi[1]; ++y)
      for (uint32_t x = w.lo[0]; x <= w.hi[0]; ++x) {
        const uint2 r = cell_lookup(ci, morton3(x, y, z) | sbits);
        for (uint32_t j = r.x; j < r.y; ++j) f(j);
      }
}

// Density (forces.cl:15-43) + Tait pressure (sph.cl:36-39) + neighbour list.
// One thread per particle, two phases:
//  1. walk the window cells (z, y, x order; each cell's particles in sorted
//     order). A particle in a neighbour cell that lies in the half facing
//     away from this particle's cell (per its half code in pos.w) is more
//     than h away: skipped with one bit test. The others get an FMA distance
//     cull; survivors are buffered per thread in shared memory;
//  2. evaluate the survivors with exact arithmetic, in the same order, in
//     lock-step across the warp (the expensive part is no longer divergent).
// A thread with more survivors than its buffer repeats phase 1 inline.
constexpr int kScanCap = 48;

// Bits of a neighbour's half code that must be set for it to face cell
// offset (ox, oy, oz): its upper half when it is below, lower half when above.
__device__ __forceinline__ uint32_t facing_mask(int ox, int oy, int oz) {
  uint32_t m = 0;
  if (ox < 0) m |= 2u;
  if (ox > 0) m |= 1u;
  if (oy < 0) m |= 8u;
  if (oy > 0) m |= 4u;
  if (oz < 0) m |= 32u;
  if (oz > 0) m |= 16u;
  return m;
}

// Neighbour-list tags: the neighbour's cell as its index k < 27 among the 27
// cells around the particle's own cell (z, y, x order, 13 = own) in bits
// 11-15 and its offset in that cell in bits 0-10; a cell of 2048 or more
// particles cannot be tagged (kNoTag) and sends its particles to the rescan.
constexpr uint32_t kTagOffBits = 11;
constexpr uint32_t kNoTag = 0xFFFFu;
__device__ __forceinline__ uint32_t nb_tag(uint32_t k, uint32_t off) {
  return off < (1u << kTagOffBits) ? (k << kTagOffBits) | off : kNoTag;
}

// Calls f(j, pj, tag) for every candidate of the window that faces the
// particle's cell, in the reference's order, and g(k, start) once per window
// cell before its candidates.
template <class F, class G>
__device__ __forceinline__ void for_each_facing_candidate(const Window& w, uint32_t key,
                                                          uint32_t sbits, const CellIndex& ci,
                                                          const float4* __restrict__ pos, F&& f,
                                                          G&& g) {
  const int c[3] = {(int)compact_bits3(key), (int)compact_bits3(key >> 1), (int)compact_bits3(key >> 2)};
  for (uint32_t z = w.lo[2]; z <= w.hi[2]; ++z)
    for (uint32_t y = w.lo[1]; y <= w.hi[1]; ++y)
      for (uint32_t x = w.lo[0]; x <= w.hi[0]; ++x) {
        const int ox = (int)x - c[0], oy = (int)y - c[1], oz = (int)z - c[2];
        const uint32_t need = facing_mask(ox, oy, oz);
        const uint32_t k = (uint32_t)((oz + 1) * 9 + (oy + 1) * 3 + (ox + 1));
        const uint2 r = cell_lookup(ci, morton3(x, y, z) | sbits);
        g(k, r.x);
        for (uint32_t j = r.x; j < r.y; ++j) {
          const float4 pj = __ldg(&pos[j]);
          if ((__float_as_uint(pj.w) & need) == need) f(j, pj, nb_tag(k, j - r.x));
        }
      }
}
template <class F>
__device__ __forceinline__ void for_each_facing_candidate(const Window& w, uint32_t key,
                                                          uint32_t sbits, const CellIndex& ci,
                                                          const float4* __restrict__ pos, F&& f) {
  for_each_facing_candidate(w, key, sbits, ci, pos, f, [](uint32_t, uint32_t) {});
}

// Per-particle outputs of the density pass: aux = (rho, p, first slot of the
// particle's own cell as bits, p/rho^2) (the forces kernel resolves the
// neighbour tags through that cell's nb_start row), the forces kernel's two
// 16-byte neighbour records (position, m/rho) and (velocity, p/rho^2), and the
// neighbour count (> nlist_cap: the list is incomplete or holds an untaggable
// neighbour, so the forces kernel searches again).
__device__ __forceinline__ void density_outputs(uint32_t i, uint32_t n, float rho, const Consts& c,
                                                uint32_t own_start, float4 pi, const float4* __restrict__ vel,
                                                float4* __restrict__ aux_out, float4* __restrict__ frec,
                                                uint32_t* __restrict__ ncount, uint32_t count) {
  const float4 a = density_aux(rho, c);
  aux_out[i] = make_float4(a.x, a.y, __uint_as_float(own_start), a.w);
  const float4 v = vel[i];
  frec[i] = make_float4(pi.x, pi.y, pi.z, a.z);
  frec[(size_t)n + i] = make_float4(v.x, v.y, v.z, a.w);
  ncount[i] = count;
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK)
    k_density(uint32_t n, const DevGrid* __restrict__ grids, const uint16_t* __restrict__ scene_of,
              const uint32_t* __restrict__ ctl,
              const uint32_t* __restrict__ keys_base, const float4* __restrict__ pos, CellIndex ci,
              const Consts* __restrict__ consts, float4* __restrict__ aux_out,
              uint16_t* __restrict__ nlist, uint32_t* __restrict__ ncount, uint32_t nlist_cap,
              const float4* __restrict__ vel, float4* __restrict__ frec, uint32_t* __restrict__ nb_start) {
  __shared__ uint16_t cand[kScanCap][BLOCK];  // tags of the cull's survivors
  __shared__ uint32_t cstart[27][BLOCK];      // first slot of each window cell
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const KeySplit split{ctl[kCtlShift]};
  const uint32_t sc = scene_of[i];
  const Consts c = consts[sc];
  const uint32_t sbits = split.scene_bits(sc);
  const uint32_t* keys = keys_base + (size_t)sorted_sel(ctl[kCtlMaxKey]) * n;
  const uint32_t key = split.morton(keys[i]);
  const float4 pi = pos[i];
  const Window w = neighbour_window(pi, key, grids[sc]);
  const float hh = XMUL(c.h, c.h);
  uint32_t found = 0;
  for_each_facing_candidate(
      w, key, sbits, ci, pos,
      [&](uint32_t, float4 pj, uint32_t tag) {
        const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
        if (fmaf(dx, dx, fmaf(dy, dy, dz * dz)) <= c.cull_r2) {
          if (found < kScanCap) cand[found][threadIdx.x] = (uint16_t)tag;
          found = tag == kNoTag ? kScanCap + 1u : found + 1u;  // untaggable: rescan
        }
      },
      [&](uint32_t k, uint32_t start) { cstart[k][threadIdx.x] = start; });
  const uint32_t own_start = cstart[13][threadIdx.x];
  float rho = 0.f;
  uint32_t kept = 0;
  bool untagged = false;
  auto visit = [&](uint32_t j, float4 pj, uint32_t tag) {
    const V3 d = {XSUB(pi.x, pj.x), XSUB(pi.y, pj.y), XSUB(pi.z, pj.z)};
    const float rr = xnorm(d);
    if (rr < c.h) {
      rho = XADD(rho, poly6_term(rr, hh, c));
      if (tag == kNoTag) untagged = true;
      else if (kept < nlist_cap) __stcs(&nlist[(size_t)kept * n + i], (uint16_t)tag);
      ++kept;
    }
  };
  if (found <= (uint32_t)kScanCap) {
    for (uint32_t k = 0; k < found; ++k) {
      const uint32_t tag = cand[k][threadIdx.x];
      const uint32_t j = cstart[tag >> kTagOffBits][threadIdx.x] + (tag & ((1u << kTagOffBits) - 1u));
      visit(j, __ldg(&pos[j]), tag);
    }
  } else {
    for_each_facing_candidate(w, key, sbits, ci, pos, [&](uint32_t j, float4 pj, uint32_t tag) {
      const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
      if (fmaf(dx, dx, fmaf(dy, dy, dz * dz)) <= c.cull_r2) visit(j, pj, tag);
    });
  }
  // the own cell's row of the neighbour-start table (every particle of the
  // cell writes the same values for the cells of its window)
  const int cc[3] = {(int)compact_bits3(key), (int)compact_bits3(key >> 1), (int)compact_bits3(key >> 2)};
  for (uint32_t z = w.lo[2]; z <= w.hi[2]; ++z)
    for (uint32_t y = w.lo[1]; y <= w.hi[1]; ++y)
      for (uint32_t x = w.lo[0]; x <= w.hi[0]; ++x) {
        const uint32_t k = (uint32_t)(((int)z - cc[2] + 1) * 9 + ((int)y - cc[1] + 1) * 3 + ((int)x - cc[0] + 1));
        nb_start[(size_t)own_start * 27u + k] = cstart[k][threadIdx.x];
      }
  density_outputs(i, n, rho, c, own_start, pi, vel, aux_out, frec, ncount,
                  untagged ? max(kept, nlist_cap + 1u) : kept);
}

// ------------------------------------------------- density, one warp per cell
// The warp takes one occupied cell at a time (dynamic work counter), looks up
// the 27 cells around it once (lane k < 27: offset k in the reference's z, y,
// x loop order; also stored as the cell's nb_start row) and holds the cell's
// particles, two per lane. For each neighbour cell, in that order, that lies
// in at least one particle's window (the union of the windows as a 27-bit
// mask), it walks the cell's slots 32 at a time and stages the candidates
// that face the own cell (the far half is skipped by half code), compacted by
// ballot, which keeps their sorted order, into a tile in shared memory, with
// coordinates relative to the own cell's centre and their negated squared
// norm. A tile holds up to 32 candidates, of one cell or of consecutive
// cells: it is tested before a block would overflow it and at the end of the
// pass. A lane tests both its particles against every staged candidate with
// three FMAs, 2 p'.q' - |q'|^2 >= |p'|^2 - R^2 (the squared distance with the
// particle's part precomputed), sets the candidate's bit in the tile's hit
// mask, and after the tile appends the hits' tags to the particle's buffer in
// bit order, so each buffer holds the reference's visiting order. A particle
// also tests candidates of cells outside its own window (those of the other
// particles' windows); the exact test rejects them, as the reference's walk
// over all 27 cells does. The survivors are then evaluated exactly per
// particle, as in k_density.
// (Packing the candidates into tiles, instead of testing each 32-slot block
// on its own, cut the kernel's instructions by 8.5 % and its time by 6-8 %
// on the 1M dam break; letting tiles span cells, without skipping a half of
// the lanes whose particles' windows miss the tile's cell, cut another 5 %
// of the instructions and 4-7 % of the time.)
//
// Rounding of the cull: cell-relative coordinates are within 3h of the
// centre, so every intermediate of the test is below 50 h^2 and the four
// roundings of each side stay below 3e-5 h^2, a fifth of the cull's margin
// (R^2 = 1.0005 h^2); the test is conservative, and the exact evaluation
// decides.
// A buffer entry is a neighbour tag; cells of 2048 or more particles and full
// buffers send the particle to the in-order rescan.
constexpr int kCellWarps = 4;
constexpr uint32_t kCellOffBits = kTagOffBits;

// Per neighbour offset k (z, y, x order): the half-code bits a candidate of
// that cell needs to face the own cell, facing_mask(o).
struct OffsetMasks {
  uint8_t m[27];
};
constexpr OffsetMasks make_offset_masks() {
  OffsetMasks t{};
  for (int k = 0; k < 27; ++k) {
    const int o[3] = {k % 3 - 1, (k / 3) % 3 - 1, k / 9 - 1};
    uint32_t cand = 0;
    for (int a = 0; a < 3; ++a) {
      if (o[a] < 0) cand |= 2u << (2 * a);
      if (o[a] > 0) cand |= 1u << (2 * a);
    }
    t.m[k] = (uint8_t)cand;
  }
  return t;
}
__constant__ OffsetMasks kOffsetMasks = make_offset_masks();

__device__ __forceinline__ bool near_cull(const float4& p, const float4& q, float r2) {
  const float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
  return fmaf(dx, dx, fmaf(dy, dy, dz * dz)) <= r2;
}

// The cells of a particle's window as bits k < 27 (z, y, x order): on every
// axis offset 0, and -1 / +1 where its half code has the lower / upper bit.
// Bit k is set exactly when (code & facing_mask(-o)) == facing_mask(-o) for
// the cell's offset o.
__device__ __forceinline__ uint32_t window_cells(uint32_t code) {
  const uint32_t ax = 2u | (code & 1u) | ((code << 1) & 4u);
  const uint32_t ay = 2u | ((code >> 2) & 1u) | ((code >> 1) & 4u);
  const uint32_t az = 2u | ((code >> 4) & 1u) | ((code >> 3) & 4u);
  const uint32_t yx = ((ay & 1u) ? ax : 0u) | (ax << 3) | ((ay & 4u) ? ax << 6 : 0u);
  return ((az & 1u) ? yx : 0u) | (yx << 9) | ((az & 4u) ? yx << 18 : 0u);
}

// survivor buffer per particle: 48 tags (40 with 8 warps, which keeps the
// block within 48 KB of shared memory); fuller ones rescan
template <int WARPS>
struct DensitySmem {
  static constexpr uint32_t kCap = WARPS >= 8 ? 40u : (uint32_t)kScanCap;
  float4 stage[WARPS][32];
  uint32_t stag[WARPS][32];
  uint32_t starts[WARPS][32];
  uint16_t cand[WARPS][kCap][64];
};

template <int WARPS>
__device__ __forceinline__ void density_cells_warps(
    uint32_t n, const DevGrid* __restrict__ grids, const uint16_t* __restrict__ scene_of,
    const uint32_t* __restrict__ ctl, const uint32_t* __restrict__ keys_base, const float4* __restrict__ pos,
    CellIndex ci, const Consts* __restrict__ consts, float4* __restrict__ aux_out, uint16_t* __restrict__ nlist,
    uint32_t* __restrict__ ncount, uint32_t nlist_cap, const float4* __restrict__ vel,
    float4* __restrict__ frec, const uint32_t* __restrict__ cell_list, uint32_t* __restrict__ counters,
    uint32_t* __restrict__ nb_start, DensitySmem<WARPS>& sm) {
  constexpr uint32_t kCap = DensitySmem<WARPS>::kCap;
  auto& stage = sm.stage;
  auto& stag = sm.stag;
  auto& starts = sm.starts;
  auto& cand = sm.cand;
  const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
  const uint32_t lt = (1u << lane) - 1u;
  const uint32_t ncells = counters[kCntCells];
  const KeySplit split{ctl[kCtlShift]};
  const uint32_t* keys = keys_base + (size_t)sorted_sel(ctl[kCtlMaxKey]) * n;
  for (;;) {
    uint32_t cell = 0;
    if (lane == 0) cell = atomicAdd(&counters[kCntWorkDensity], 1u);
    cell = __shfl_sync(0xFFFFFFFFu, cell, 0);
    if (cell >= ncells) break;
    const uint32_t s0 = cell_list[cell];
    const uint32_t key = split.morton(keys[s0]);
    const uint32_t sc = scene_of[s0];
    const uint32_t sbits = split.scene_bits(sc);
    const uint32_t cx = compact_bits3(key), cy = compact_bits3(key >> 1), cz = compact_bits3(key >> 2);
    const float cull_r2 = consts[sc].cull_r2;
    const DevGrid& gr = grids[sc];
    // the own cell's centre: the origin of the cull's coordinates
    const float ox = gr.lo[0] + ((float)cx + 0.5f) * gr.cell, oy = gr.lo[1] + ((float)cy + 0.5f) * gr.cell,
                oz = gr.lo[2] + ((float)cz + 0.5f) * gr.cell;
    uint32_t nb_s = 0, nb_e = 0;
    if (lane < 27u) {
      const uint32_t x = cx + lane % 3u - 1u, y = cy + (lane / 3u) % 3u - 1u, z = cz + lane / 9u - 1u;
      const uint2 r = cell_lookup(ci, morton3(x, y, z) | sbits);
      nb_s = r.x;
      nb_e = r.y;
      nb_start[(size_t)s0 * 27u + lane] = nb_s;
    }
    starts[wid][lane] = nb_s;
    __syncwarp();
    const uint32_t own_e = __shfl_sync(0xFFFFFFFFu, nb_e, 13);
    const bool wide = __any_sync(0xFFFFFFFFu, nb_e - nb_s >= (1u << kCellOffBits));
    for (uint32_t base = s0; base < own_e; base += 64u) {
      const uint32_t ia = base + lane, ib = base + 32u + lane;
      const bool va = ia < own_e, vb = ib < own_e;
      const float4 pa = va ? pos[ia] : make_float4(0.f, 0.f, 0.f, 0.f);
      const float4 pb = vb ? pos[ib] : make_float4(0.f, 0.f, 0.f, 0.f);
      const uint32_t code_a = __float_as_uint(pa.w), code_b = __float_as_uint(pb.w);
      // 2 p' and |p'|^2 - R^2 of both particles
      const float ax = pa.x - ox, ay = pa.y - oy, az = pa.z - oz;
      const float bx = pb.x - ox, by = pb.y - oy, bz = pb.z - oz;
      const float a2x = 2.f * ax, a2y = 2.f * ay, a2z = 2.f * az;
      const float b2x = 2.f * bx, b2y = 2.f * by, b2z = 2.f * bz;
      const float ta = fmaf(ax, ax, fmaf(ay, ay, az * az)) - cull_r2;
      const float tb = fmaf(bx, bx, fmaf(by, by, bz * bz)) - cull_r2;
      uint32_t fa = wide ? kCap + 1u : 0u, fb = fa;
      // the cells of the pass's windows (the union over its particles) in z,
      // y, x order, each walked in 32-slot blocks; their facing candidates are
      // packed into tiles of up to 32 (a tile is tested before a block would
      // overflow it and at the end of the pass)
      uint32_t rem = 0;
      if (!wide)
        rem = __reduce_or_sync(0xFFFFFFFFu, (va ? window_cells(code_a) : 0u) | (vb ? window_cells(code_b) : 0u));
      uint32_t nt = 0;  // candidates in the tile
      auto test_tile = [&]() {
        const uint32_t m = nt;
        // slots [m, 8 * ceil(m / 8)) hold a candidate no test accepts
        if (m + lane < ((m + 7u) & ~7u)) stage[wid][m + lane] = make_float4(0.f, 0.f, 0.f, -INFINITY);
        __syncwarp();
        const float tak = va ? ta : INFINITY, tbk = vb ? tb : INFINITY;
        // the a or b half of the lanes skips the tile when it holds no particle
        const bool one = __any_sync(0xFFFFFFFFu, va), two = __any_sync(0xFFFFFFFFu, vb);
        uint32_t ma = 0, mb = 0;
        // eight candidates per step, each with its own constant bit
        for (uint32_t t0 = 0; t0 < m; t0 += 8u) {
          uint32_t ga = 0, gb = 0;
#pragma unroll
          for (uint32_t u = 0; u < 8u; ++u) {
            const float4 r = stage[wid][t0 + u];
            if (one && fmaf(a2x, r.x, fmaf(a2y, r.y, fmaf(a2z, r.z, r.w))) >= tak) ga |= 1u << u;
            if (two && fmaf(b2x, r.x, fmaf(b2y, r.y, fmaf(b2z, r.z, r.w))) >= tbk) gb |= 1u << u;
          }
          ma |= ga << t0;
          mb |= gb << t0;
        }
        // hits in candidate order
        while (ma) {
          const uint32_t t = __ffs(ma) - 1u;
          ma &= ma - 1u;
          if (fa < kCap) cand[wid][fa][lane] = (uint16_t)stag[wid][t];
          ++fa;
        }
        while (mb) {
          const uint32_t t = __ffs(mb) - 1u;
          mb &= mb - 1u;
          if (fb < kCap) cand[wid][fb][lane + 32u] = (uint16_t)stag[wid][t];
          ++fb;
        }
        __syncwarp();
        nt = 0;
      };
      while (rem) {
        const uint32_t k = __ffs(rem) - 1u;
        rem &= rem - 1u;
        const uint32_t fm = kOffsetMasks.m[k];  // a candidate's half toward the own cell
        const uint32_t s = __shfl_sync(0xFFFFFFFFu, nb_s, k), e = __shfl_sync(0xFFFFFFFFu, nb_e, k);
        for (uint32_t cb = s; cb < e; cb += 32u) {
          const uint32_t j = cb + lane;
          float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
          bool f = false;
          if (j < e) {
            q = __ldg(&pos[j]);
            f = (__float_as_uint(q.w) & fm) == fm;
          }
          const uint32_t bal = __ballot_sync(0xFFFFFFFFu, f);
          const uint32_t cnt = __popc(bal);
          if (nt + cnt > 32u) test_tile();  // the block would overflow the tile
          if (f) {
            const uint32_t at = nt + __popc(bal & lt);
            const float qx = q.x - ox, qy = q.y - oy, qz = q.z - oz;
            stage[wid][at] = make_float4(qx, qy, qz, -fmaf(qx, qx, fmaf(qy, qy, qz * qz)));
            stag[wid][at] = (k << kCellOffBits) | (j - s);
          }
          nt += cnt;
          if (nt == 32u) test_tile();
        }
      }
      if (nt) test_tile();  // the end of the pass
      auto finish = [&](uint32_t i, const float4& pi, uint32_t found, uint32_t col) {
        const Consts& c = consts[sc];
        const float hh = XMUL(c.h, c.h);
        float rho = 0.f;
        uint32_t kept = 0;
        bool untagged = false;
        auto visit = [&](uint32_t j, float4 pj, uint32_t tag) {
          const V3 d = {XSUB(pi.x, pj.x), XSUB(pi.y, pj.y), XSUB(pi.z, pj.z)};
          const float rr = xnorm(d);
          if (rr < c.h) {
            rho = XADD(rho, poly6_term(rr, hh, c));
            if (tag == kNoTag) untagged = true;
            else if (kept < nlist_cap) __stcs(&nlist[(size_t)kept * n + i], (uint16_t)tag);
            ++kept;
          }
        };
        if (found <= kCap) {
          // each survivor's position is loaded one survivor ahead
          auto slot_at = [&](uint32_t k) {
            const uint32_t tag = cand[wid][k][col];
            return starts[wid][tag >> kCellOffBits] + (tag & ((1u << kCellOffBits) - 1u));
          };
          uint32_t tag = found ? (uint32_t)cand[wid][0][col] : 0u;
          float4 pj = found ? __ldg(&pos[slot_at(0)]) : make_float4(0.f, 0.f, 0.f, 0.f);
          for (uint32_t k = 0; k < found; ++k) {
            const uint32_t kn = k + 1 < found ? k + 1 : k;
            const uint32_t tagn = cand[wid][kn][col];
            const float4 pn = __ldg(&pos[slot_at(kn)]);
            visit(0u, pj, tag);
            tag = tagn;
            pj = pn;
          }
        } else {
          const Window w = neighbour_window(pi, key, grids[sc]);
          for_each_facing_candidate(w, key, sbits, ci, pos, [&](uint32_t j, float4 pj, uint32_t tag) {
            if (near_cull(pi, pj, c.cull_r2)) visit(j, pj, tag);
          });
        }
        density_outputs(i, n, rho, c, s0, pi, vel, aux_out, frec, ncount,
                        untagged ? max(kept, nlist_cap + 1u) : kept);
      };
      if (va) finish(ia, pa, fa, lane);
      if (vb) finish(ib, pb, fb, lane + 32u);
      __syncwarp();
    }
    __syncwarp();
  }
}

template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
    k_density_cells(uint32_t n, const DevGrid* __restrict__ grids,
                    const uint16_t* __restrict__ scene_of, const uint32_t* __restrict__ ctl,
                    const uint32_t* __restrict__ keys_base, const float4* __restrict__ pos,
                    CellIndex ci, const Consts* __restrict__ consts, float4* __restrict__ aux_out,
                    uint16_t* __restrict__ nlist, uint32_t* __restrict__ ncount,
                    uint32_t nlist_cap, const float4* __restrict__ vel,
                    float4* __restrict__ frec, const uint32_t* __restrict__ cell_list,
                    uint32_t* __restrict__ counters, uint32_t* __restrict__ nb_start) {
  __shared__ DensitySmem<WARPS> sm;
  density_cells_warps<WARPS>(n, grids, scene_of, ctl, keys_base, pos, ci, consts, aux_out, nlist, ncount,
                             nlist_cap, vel, frec, cell_list, counters, nb_start, sm);
}


// Density + pressure + neighbour list with one warp per particle, for scenes
// too small to fill the GPU with one thread per particle or one warp per
// cell. The warp walks the particle's window cells in the reference's order,
// 32 candidates at a time (far halves skipped by half code, FMA cull), every
// lane evaluates its candidate exactly, and the contributing terms are added
// to the density one after another in lane order (ballot + shuffle), which is
// the reference's visiting order; survivors append to the neighbour list in
// the same order.
constexpr int kParticleWarps = 8;

static __global__ void __launch_bounds__(kParticleWarps * 32)
    k_density_pwarp(uint32_t n, const DevGrid* __restrict__ grids, const uint16_t* __restrict__ scene_of,
                    const uint32_t* __restrict__ ctl, const uint32_t* __restrict__ keys_base,
                    const float4* __restrict__ pos, CellIndex ci, const Consts* __restrict__ consts,
                    float4* __restrict__ aux_out, uint16_t* __restrict__ nlist,
                    uint32_t* __restrict__ ncount, uint32_t nlist_cap, const float4* __restrict__ vel,
                    float4* __restrict__ frec, uint32_t* __restrict__ nb_start) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t lt = (1u << lane) - 1u;
  const uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= n) return;  // whole warps
  const KeySplit split{ctl[kCtlShift]};
  const uint32_t sc = scene_of[i];
  const Consts& c = consts[sc];
  const uint32_t sbits = split.scene_bits(sc);
  const uint32_t* keys = keys_base + (size_t)sorted_sel(ctl[kCtlMaxKey]) * n;
  const uint32_t key = split.morton(keys[i]);
  const float4 pi = pos[i];
  const Window w = neighbour_window(pi, key, grids[sc]);
  const int cc[3] = {(int)compact_bits3(key), (int)compact_bits3(key >> 1), (int)compact_bits3(key >> 2)};
  const float hh = XMUL(c.h, c.h);
  const float h = c.h, cull_r2 = c.cull_r2;
  float rho = 0.f;
  uint32_t kept = 0;
  bool untagged = false;
  // lane k < 27 looks up window cell k (z, y, x order) in parallel
  uint32_t cs = 0, ce = 0;
  bool inw = false;
  if (lane < 27u) {
    const uint32_t x = (uint32_t)cc[0] + lane % 3u - 1u, y = (uint32_t)cc[1] + (lane / 3u) % 3u - 1u,
                   z = (uint32_t)cc[2] + lane / 9u - 1u;
    inw = x >= w.lo[0] && x <= w.hi[0] && y >= w.lo[1] && y <= w.hi[1] && z >= w.lo[2] && z <= w.hi[2];
    if (inw) {
      const uint2 r = cell_lookup(ci, morton3(x, y, z) | sbits);
      cs = r.x;
      ce = r.y;
    }
  }
  const uint32_t own_start = __shfl_sync(0xFFFFFFFFu, cs, 13);
  if (inw) nb_start[(size_t)own_start * 27u + lane] = cs;  // the same values from every particle of the cell
  uint32_t cells = __ballot_sync(0xFFFFFFFFu, inw && ce > cs);
  while (cells) {
    const uint32_t k = __ffs(cells) - 1u;
    cells &= cells - 1u;
    const uint32_t need = facing_mask((int)(k % 3u) - 1, (int)((k / 3u) % 3u) - 1, (int)(k / 9u) - 1);
    const uint2 r = make_uint2(__shfl_sync(0xFFFFFFFFu, cs, k), __shfl_sync(0xFFFFFFFFu, ce, k));
    for (uint32_t cb = r.x; cb < r.y; cb += 32u) {
      const uint32_t j = cb + lane;
      bool hit = false;
      float term = 0.f;
      if (j < r.y) {
        const float4 pj = __ldg(&pos[j]);
        if ((__float_as_uint(pj.w) & need) == need && near_cull(pi, pj, cull_r2)) {
          const V3 d = {XSUB(pi.x, pj.x), XSUB(pi.y, pj.y), XSUB(pi.z, pj.z)};
          const float rr = xnorm(d);
          if (rr < h) {
            hit = true;
            term = poly6_term(rr, hh, c);
          }
        }
      }
      uint32_t bal = __ballot_sync(0xFFFFFFFFu, hit);
      const uint32_t tag = nb_tag(k, j - r.x);
      untagged |= __any_sync(0xFFFFFFFFu, hit && tag == kNoTag);
      const uint32_t at = kept + __popc(bal & lt);
      if (hit && at < nlist_cap) __stcs(&nlist[(size_t)at * n + i], (uint16_t)tag);
      kept += __popc(bal);
      while (bal) {  // in lane order: the reference's summation sequence
        const int l = __ffs(bal) - 1;
        rho = XADD(rho, __shfl_sync(0xFFFFFFFFu, term, l));
        bal &= bal - 1u;
      }
    }
  }
  if (lane == 0)
    density_outputs(i, n, rho, c, own_start, pi, vel, aux_out, frec, ncount,
                    untagged ? max(kept, nlist_cap + 1u) : kept);
}

// Per-pair hook of k_forces (the learned stepper gathers its neighbour
// features in the same walk); the plain substep uses this empty one.
struct NoForceHook {
  struct Acc {};
  __device__ __forceinline__ Acc begin(uint32_t) const { return {}; }
  __device__ __forceinline__ void pair(Acc&, uint32_t, uint32_t, const V3&, const V3&) const {}
  __device__ __forceinline__ void end(Acc&, uint32_t, const float4&) const {}
};

// Internal forces (forces.cl:45-112) -> acceleration (sph.cl:53-58), walking
// the neighbour list of k_density (or the window, for overflowing lists).
template <class Hook>
__device__ __forceinline__ void forces_particle(
    uint32_t i, uint32_t n, const DevGrid* __restrict__ grids, const uint16_t* __restrict__ scene_of,
    const uint32_t* __restrict__ ctl, const uint32_t* __restrict__ keys_base, State st,
    const float4* __restrict__ aux, CellIndex ci, const Consts* __restrict__ consts,
    const uint16_t* __restrict__ nlist, const uint32_t* __restrict__ ncount, uint32_t nlist_cap,
    float4* __restrict__ acc_out, const Hook& hook, const float4* __restrict__ frec,
    const uint32_t* __restrict__ nb_start) {
  typename Hook::Acc ha = hook.begin(i);
  const uint32_t sc = scene_of[i];
  const Consts c = consts[sc];
  const float4 pi = st.pos[i];
  const float4 vi = st.vel[i];
  const float4 ai = aux[i];
  const float own = ai.w;
  const float hh = XMUL(c.h, c.h);
  const float lap_b = XMUL(3.f, hh);
  ForceSums f = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, 0.f};
  // neighbour data from the density kernel's 32-byte records
  auto pair_with = [&](uint32_t j, const float4& pj, const float4& sj) {
    const V3 d = {XSUB(pi.x, pj.x), XSUB(pi.y, pj.y), XSUB(pi.z, pj.z)};
    const float rr = xnorm(d);
    const float4 vj = make_float4(sj.x, sj.y, sj.z, 0.f);
    force_pair(f, j == i, d, rr, vi, vj, make_float4(0.f, 0.f, pj.w, sj.w), own, hh, lap_b, c);
    // the same differences force_pair forms (the compiler shares them); dead
    // code for the plain substep's empty hook
    const V3 dv = {XSUB(vj.x, vi.x), XSUB(vj.y, vi.y), XSUB(vj.z, vi.z)};
    hook.pair(ha, i, j, d, dv);
  };
  auto pair = [&](uint32_t j) { pair_with(j, __ldg(&frec[j]), __ldg(&frec[(size_t)n + j])); };
  const uint32_t cnt = ncount[i];
  if (cnt <= nlist_cap) {
    // a tag names the neighbour's cell among the 27 around the own cell and
    // its offset there; the own cell's nb_start row holds their first slots
    const uint32_t* nbs = nb_start + (size_t)__float_as_uint(ai.z) * 27u;
    auto slot = [&](uint32_t tag) {
      return __ldg(&nbs[tag >> kTagOffBits]) + (tag & ((1u << kTagOffBits) - 1u));
    };
    // software pipeline: while a pair is evaluated, the tag three pairs
    // ahead is loaded, the tag two ahead is resolved to its slot and the
    // records of the next pair are loaded
    if (cnt > 0) {
      auto tag_at = [&](uint32_t k) { return (uint32_t)__ldcs(&nlist[(size_t)k * n + i]); };
      const uint32_t t0 = tag_at(0);
      const uint32_t t1 = cnt > 1 ? tag_at(1) : t0;
      uint32_t tnn = cnt > 2 ? tag_at(2) : t1;
      uint32_t j = slot(t0);
      uint32_t jn = slot(t1);
      float4 pj = __ldg(&frec[j]), sj = __ldg(&frec[(size_t)n + j]);
      for (uint32_t k = 0; k < cnt; ++k) {
        const uint32_t t3 = k + 3 < cnt ? tag_at(k + 3) : tnn;
        const uint32_t jnn = slot(tnn);
        const float4 pn = __ldg(&frec[jn]), sn = __ldg(&frec[(size_t)n + jn]);
        pair_with(j, pj, sj);
        j = jn;
        jn = jnn;
        pj = pn;
        sj = sn;
        tnn = t3;
      }
    }
  } else {
    const KeySplit split{ctl[kCtlShift]};
    const uint32_t* keys = keys_base + (size_t)sorted_sel(ctl[kCtlMaxKey]) * n;
    const Window w = neighbour_window(pi, split.morton(keys[i]), grids[sc]);
    for_each_candidate(w, split.scene_bits(sc), ci, [&](uint32_t j) {
      const float4 pj = __ldg(&frec[j]);
      const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
      if (fmaf(dx, dx, fmaf(dy, dy, dz * dz)) > c.cull_r2) return;
      const V3 d = {XSUB(pi.x, pj.x), XSUB(pi.y, pj.y), XSUB(pi.z, pj.z)};
      if (xnorm(d) < c.h) pair(j);
    });
  }
  const float4 a = finish_accel(f, ai.x, c);
  acc_out[i] = a;
  hook.end(ha, i, a);
}

template <int BLOCK, class Hook = NoForceHook>
__global__ void __launch_bounds__(BLOCK)
    k_forces(uint32_t n, const DevGrid* __restrict__ grids, const uint16_t* __restrict__ scene_of,
             const uint32_t* __restrict__ ctl,
             const uint32_t* __restrict__ keys_base, State st, const float4* __restrict__ aux,
             CellIndex ci, const Consts* __restrict__ consts, const uint16_t* __restrict__ nlist,
             const uint32_t* __restrict__ ncount, uint32_t nlist_cap,
             float4* __restrict__ acc_out, Hook hook, const float4* __restrict__ frec,
             const uint32_t* __restrict__ nb_start) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  forces_particle(i, n, grids, scene_of, ctl, keys_base, st, aux, ci, consts, nlist, ncount, nlist_cap,
                  acc_out, hook, frec, nb_start);
}

// ------------------------------------------------------- mesh collision
struct Hit {
  V3 point, normal;
  float depth;
  bool any;
};

// One face of collisions.cl:21-87 (nearest hit; an equal distance replaces).
__device__ __forceinline__ void test_face(const DevMesh& m, uint32_t f, V3 p0, V3 p1, V3 d,
                                          float dlen, Hit& h) {
  V3 nrm = {__ldg(&m.normals[3 * f]), __ldg(&m.normals[3 * f + 1]), __ldg(&m.normals[3 * f + 2])};
  if (XDIV(xdot(nrm, d), XMUL(xnorm(nrm), dlen)) <= 0.f) nrm = {-nrm.x, -nrm.y, -nrm.z};
  const uint32_t ia = __ldg(&m.indices[3 * f]), ib = __ldg(&m.indices[3 * f + 1]),
                 ic = __ldg(&m.indices[3 * f + 2]);
  const V3 v0 = {__ldg(&m.vertices[3 * ia]), __ldg(&m.vertices[3 * ia + 1]), __ldg(&m.vertices[3 * ia + 2])};
  const V3 v1 = {__ldg(&m.vertices[3 * ib]), __ldg(&m.vertices[3 * ib + 1]), __ldg(&m.vertices[3 * ib + 2])};
  const V3 v2 = {__ldg(&m.vertices[3 * ic]), __ldg(&m.vertices[3 * ic + 1]), __ldg(&m.vertices[3 * ic + 2])};
  const V3 u = xsub3(v1, v0), v = xsub3(v2, v0);
  const float den = xdot(nrm, d);
  if (den == 0.f) return;
  const float r = XDIV(xdot(nrm, xsub3(v0, p0)), den);
  if (!(0.f <= r && r <= 1.f)) return;
  const V3 at = {XADD(p0.x, XMUL(r, d.x)), XADD(p0.y, XMUL(r, d.y)), XADD(p0.z, XMUL(r, d.z))};
  const V3 w = xsub3(at, v0);
  const float uv = xdot(u, v), wv = xdot(w, v), vv = xdot(v, v), wu = xdot(w, u), uu = xdot(u, u);
  const float den2 = XSUB(XMUL(uv, uv), XMUL(uu, vv));
  const float s = XDIV(XSUB(XMUL(uv, wv), XMUL(vv, wu)), den2);
  const float t = XDIV(XSUB(XMUL(uv, wu), XMUL(uu, wv)), den2);
  if (s >= 0.f && t >= 0.f && XADD(s, t) <= 1.f) {
    if (h.any && xnorm(xsub3(p0, at)) > xnorm(xsub3(p0, h.point))) return;
    h.normal = nrm;
    h.point = at;
    h.depth = xnorm(xsub3(p1, at));
    h.any = true;
  }
}

// Faces that can meet the segment, in ascending face order: the list of
// the cell holding p0 when the segment is short enough for that list, no
// face when p0 lies outside the list grid (nothing within reach), else all.
__device__ __forceinline__ bool nearest_hit(const DevMesh& m, V3 p0, V3 p1, Hit& h) {
  h.any = false;
  if (m.faces == 0) return false;
  const V3 d = xsub3(p1, p0);
  const float dlen = xnorm(d);
  uint32_t first = 0, last = m.faces;
  const uint32_t* list = nullptr;
  if (m.cell_start != nullptr && dlen <= m.reach) {
    const float t[3] = {(p0.x - m.lo[0]) * m.inv_cell, (p0.y - m.lo[1]) * m.inv_cell,
                        (p0.z - m.lo[2]) * m.inv_cell};
    bool inside = true;
    int ci[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      inside = inside && (t[a] >= 0.f) && (t[a] < (float)m.dims[a]);
      ci[a] = inside ? (int)t[a] : 0;
      if (ci[a] >= m.dims[a]) ci[a] = m.dims[a] - 1;
    }
    if (!inside) return false;
    const uint32_t cell = ((uint32_t)ci[2] * (uint32_t)m.dims[1] + (uint32_t)ci[1]) * (uint32_t)m.dims[0] + (uint32_t)ci[0];
    first = __ldg(&m.cell_start[cell]);
    last = __ldg(&m.cell_start[cell + 1]);
    list = m.cell_faces;
  }
  for (uint32_t k = first; k < last; ++k) {
    const uint32_t f = list ? __ldg(&list[k]) : k;
    test_face(m, f, p0, p1, d, dlen, h);
  }
  return h.any;
}

// Leapfrog + collision loop of sph.cl:64-112 (advection.cl:6-23,
// collisions.cl:91-129), capped at max_iters passes; writes the new state
// into `out` (same slots) and accumulates the next bounding box.
// kLearned (the learned stepper, no counterpart in the reference): the step
// spans dt_mult plain time steps, corr[i].xyz is added to the acceleration,
// corr[i].w (the predicted density) is stored in out.vel.w, and positions
// advance with (1 - pos_w) v + pos_w v' instead of v' (pos_w = (m + 1) / 2m
// for m = dt_mult reproduces m leapfrog substeps exactly under constant
// acceleration; m = 1 is the plain update).
// (4 resident blocks of 256 threads: 64 registers, against 90 and 2 blocks
// unconstrained; 23 % faster on the 1M dam break)
// With y_stats (the network's output means and standard deviations, 4 + 4),
// corr holds the MLP's de-standardised outputs and learned_correction turns
// them into the correction here.

// Each output clamped to its training mean +- kLearnedOutputClamp standard
// deviations (which bounds the correction one step can apply); outputs 0..2
// are accelerations in units of h / dt^2, output 3 the relative density
// change: (correction xyz, predicted density).
constexpr float kLearnedOutputClamp = 4.f;
__device__ __forceinline__ float4 learned_correction(float4 y, const float* y_stats, const Consts& c,
                                                     float rho) {
  auto clamp_out = [&](float v, int k) {
    const float mu = y_stats[k], sigma = y_stats[4 + k];
    return fminf(fmaxf(v, mu - kLearnedOutputClamp * sigma), mu + kLearnedOutputClamp * sigma);
  };
  const float dt = c.time_delta * c.scale;
  const float s = c.h / (dt * dt);
  return make_float4(clamp_out(y.x, 0) * s, clamp_out(y.y, 1) * s, clamp_out(y.z, 2) * s,
                     rho * (1.f + clamp_out(y.w, 3)));
}

template <bool kLearned>
__device__ __forceinline__ void advect_blocks(
    uint32_t blk, uint32_t nblk, uint32_t n, State in, const float4* __restrict__ acc, State out,
    const DevMesh* __restrict__ meshes, const Consts* __restrict__ consts,
    const uint16_t* __restrict__ scene_of, uint32_t max_iters, uint32_t* __restrict__ bbox,
    uint32_t* __restrict__ status, unsigned long long* __restrict__ capped_count,
    const float4* __restrict__ corr, float dt_mult, float pos_w, const float4* __restrict__ aux,
    const float* __restrict__ y_stats, BboxSmem& bsm) {
  const float qnan = __int_as_float(0x7FC00000);
  const uint32_t stride = nblk * blockDim.x;
  for (uint32_t base = blk * blockDim.x; base < n; base += stride) {
    const uint32_t i = base + threadIdx.x;
    float3 lo = make_float3(qnan, qnan, qnan), hi = lo;
    int scene = -1;
    if (i < n) {
    scene = scene_of[i];
    const Consts& c = consts[scene];
    const DevMesh m = meshes[scene];
    float remaining = XMUL(c.time_delta, c.scale);
    V3 pos = v3(in.pos[i]);
    const V3 vh_old = v3(in.ivel[i]);
    V3 v = vh_old;
    V3 a = v3(acc[i]);
    float predicted_rho = 0.f;
    if constexpr (kLearned) {
      remaining = XMUL(remaining, dt_mult);
      float4 d = corr[i];
      if (y_stats) d = learned_correction(d, y_stats, c, aux[i].x);
      a = {XADD(a.x, d.x), XADD(a.y, d.y), XADD(a.z, d.z)};
      predicted_rho = d.w;
    }
    bool capped = false;
    for (uint32_t it = 0;; ++it) {
      V3 nv = {XADD(v.x, XMUL(a.x, remaining)), XADD(v.y, XMUL(a.y, remaining)),
               XADD(v.z, XMUL(a.z, remaining))};
      const float sp = xnorm(nv);
      if (sp > c.vmax)
        nv = {XMUL(XDIV(nv.x, sp), c.vmax), XMUL(XDIV(nv.y, sp), c.vmax), XMUL(XDIV(nv.z, sp), c.vmax)};
      V3 vp = nv;
      if constexpr (kLearned) {
        const float w0 = XSUB(1.f, pos_w);
        vp = {XADD(XMUL(v.x, w0), XMUL(nv.x, pos_w)), XADD(XMUL(v.y, w0), XMUL(nv.y, pos_w)),
              XADD(XMUL(v.z, w0), XMUL(nv.z, pos_w))};
      }
      const V3 np = {XADD(pos.x, XMUL(vp.x, remaining)), XADD(pos.y, XMUL(vp.y, remaining)),
                     XADD(pos.z, XMUL(vp.z, remaining))};
      Hit h;
      const bool hit = nearest_hit(m, pos, np, h);
      float elapsed = remaining;
      V3 opos = np, ov = nv;
      if (hit) {
        opos = {XSUB(h.point.x, XMUL(h.normal.x, 0.001f)), XSUB(h.point.y, XMUL(h.normal.y, 0.001f)),
                XSUB(h.point.z, XMUL(h.normal.z, 0.001f))};
        const float k = XMUL(XADD(1.f, XDIV(XMUL(c.restitution, h.depth), XMUL(remaining, xnorm(nv)))),
                             xdot(nv, h.normal));
        ov = {XSUB(nv.x, XMUL(k, h.normal.x)), XSUB(nv.y, XMUL(k, h.normal.y)),
              XSUB(nv.z, XMUL(k, h.normal.z))};
        elapsed = XMUL(remaining, XDIV(xnorm(xsub3(opos, pos)), xnorm(xsub3(np, pos))));
      }
      pos = opos;
      v = ov;
      remaining = XSUB(remaining, elapsed);
      a = {0.f, 0.f, 0.f};
      if (!hit) break;
      if (it + 1 >= max_iters) {
        capped = true;
        break;
      }
    }
    if (capped) {
      atomicOr(status, kFlagCollisionCap);
      atomicAdd(capped_count, 1ull);
    }
    out.pos[i] = make_float4(pos.x, pos.y, pos.z, 0.f);
    out.ivel[i] = make_float4(v.x, v.y, v.z, 0.f);
    out.vel[i] = make_float4(XDIV(XADD(vh_old.x, v.x), 2.f), XDIV(XADD(vh_old.y, v.y), 2.f),
                             XDIV(XADD(vh_old.z, v.z), 2.f), predicted_rho);
    if (!(isfinite(pos.x) && isfinite(pos.y) && isfinite(pos.z))) atomicOr(status, kFlagNonFinite);
    lo = make_float3(pos.x, pos.y, pos.z);
    hi = lo;
    }
    bbox_accumulate(lo, hi, scene, bbox, bsm);
    __syncthreads();  // the shared reduction is read before the next chunk reuses it
  }
}

template <bool kLearned>
__global__ void __launch_bounds__(kBlock, 4)
    k_advect(uint32_t n, State in, const float4* __restrict__ acc, State out,
             const DevMesh* __restrict__ meshes, const Consts* __restrict__ consts,
             const uint16_t* __restrict__ scene_of, uint32_t max_iters, uint32_t* __restrict__ bbox,
             uint32_t* __restrict__ status, unsigned long long* __restrict__ capped_count,
             const float4* __restrict__ corr, float dt_mult, float pos_w, const float4* __restrict__ aux,
             const float* __restrict__ y_stats) {
  __shared__ BboxSmem bsm;
  advect_blocks<kLearned>(blockIdx.x, gridDim.x, n, in, acc, out, meshes, consts, scene_of, max_iters, bbox,
                          status, capped_count, corr, dt_mult, pos_w, aux, y_stats, bsm);
}

// Dense reference cell table of one scene from the sorted keys of its slot
// range [first, last): table[c] = lower_bound(c) - first, c < cells.
static __global__ void k_dense_table(const uint32_t* __restrict__ keys_base, uint32_t n,
                              const uint32_t* __restrict__ ctl, const DevGrid* __restrict__ grid,
                              uint32_t scene, uint32_t first, uint32_t last,
                              uint32_t* __restrict__ table) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t cells = grid->cells;
  if (c >= cells) return;
  const KeySplit split{ctl[kCtlShift]};
  const uint32_t* keys = keys_base + (size_t)sorted_sel(ctl[kCtlMaxKey]) * n;
  const uint32_t want = c | split.scene_bits(scene);
  uint32_t lo = first, hi = last;
  while (lo < hi) {
    uint32_t mid = lo + (hi - lo) / 2;
    if (keys[mid] < want) lo = mid + 1; else hi = mid;
  }
  table[c] = lo - first;
}

}  // namespace clsph
