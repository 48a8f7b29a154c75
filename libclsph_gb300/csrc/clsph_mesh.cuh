// Per-cell triangle lists of a scene mesh, built on the GPU (scene ingestion
// of libclsph/scene.cpp:9-67 feeds the collision loop of
// libclsph/kernels/collisions.cl:91-129, which scans every face).
//
// The lists cover a uniform grid around the mesh (planned on the host from
// the mesh's bounding box, FaceGridPlan). A face is listed in every cell that
// its bounding box, grown by the list reach plus a tolerance, overlaps, and
// each list holds its faces in ascending order, so scanning one list is the
// reference's scan over all faces for any segment that starts in the cell and
// is no longer than the reach (DevMesh::reach). The kernels:
//   k_face_entries  one thread per face: the size of its cell range
//   k_scan_*      exclusive scans: face entries into entry starts, cell
//                 counts into the CSR starts
//   k_face_count  one thread per (face, cell) entry: one atomic per cell
//   k_face_fill   one thread per entry: an atomic slot in the cell's list
//   k_face_sort   one thread per cell: its list into ascending face order
// (the atomic fill leaves each list in arbitrary order; the sort restores the
// order the reference's loop visits faces in).
#pragma once

#include "clsph_common.cuh"

namespace clsph {

struct FaceGridPlan {
  float glo[3];  // grid origin (mesh box minus pad)
  float cell;    // cell edge
  float pad;     // reach + tol
  float tol;     // rounding tolerance
  int32_t dims[3];
  uint32_t cells;  // dims product
};

// Cells [c0, c1] (inclusive, clamped to the grid) that face f's box, grown by
// pad + tol, overlaps; the float operations are those of the plan's
// restatement in the tests: (min - pad) - tol, floor((x - glo) / cell).
__device__ __forceinline__ void face_cell_range(const float* __restrict__ vx, const uint32_t* __restrict__ ix,
                                                uint32_t f, const FaceGridPlan& g, int c0[3], int c1[3]) {
  const uint32_t i0 = ix[3 * f], i1 = ix[3 * f + 1], i2 = ix[3 * f + 2];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float v0 = vx[3 * i0 + a], v1 = vx[3 * i1 + a], v2 = vx[3 * i2 + a];
    const float mn = __fsub_rn(__fsub_rn(fminf(v0, fminf(v1, v2)), g.pad), g.tol);
    const float mx = __fadd_rn(__fadd_rn(fmaxf(v0, fmaxf(v1, v2)), g.pad), g.tol);
    const int a0 = (int)floorf(__fdiv_rn(__fsub_rn(mn, g.glo[a]), g.cell));
    const int a1 = (int)floorf(__fdiv_rn(__fsub_rn(mx, g.glo[a]), g.cell));
    c0[a] = a0 < 0 ? 0 : (a0 >= g.dims[a] ? g.dims[a] - 1 : a0);
    c1[a] = a1 < 0 ? 0 : (a1 >= g.dims[a] ? g.dims[a] - 1 : a1);
  }
}

// Number of (face, cell) entries of every face (face_n) and their total in
// 64 bits (a size check before the 32-bit counts and starts are built).
static __global__ void k_face_entries(const float* __restrict__ vx, const uint32_t* __restrict__ ix,
                                      uint32_t faces, FaceGridPlan g, uint32_t* __restrict__ face_n,
                                      unsigned long long* __restrict__ total) {
  unsigned long long mine = 0;
  for (uint32_t f = blockIdx.x * blockDim.x + threadIdx.x; f < faces; f += gridDim.x * blockDim.x) {
    int c0[3], c1[3];
    face_cell_range(vx, ix, f, g, c0, c1);
    const unsigned long long e = (unsigned long long)(c1[0] - c0[0] + 1) *
                                 (unsigned long long)(c1[1] - c0[1] + 1) * (unsigned long long)(c1[2] - c0[2] + 1);
    face_n[f] = e > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)e;
    mine += e;
  }
  if (mine) atomicAdd(total, mine);
}

// The (face, cell) entries spread over all threads, whatever the faces' sizes
// (a wall of a box meets thousands of cells, a heightfield triangle a few):
// entry e belongs to the face f with face_start[f] <= e < face_start[f + 1]
// (binary search) and is cell number e - face_start[f] of f's range, x
// fastest. Calls fn(f, cell).
template <class F>
__device__ __forceinline__ void for_entries(const float* __restrict__ vx, const uint32_t* __restrict__ ix,
                                            uint32_t faces, const FaceGridPlan& g,
                                            const uint32_t* __restrict__ face_start, uint32_t entries, F&& fn) {
  for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < entries; e += gridDim.x * blockDim.x) {
    uint32_t lo = 0, hi = faces;  // last f with face_start[f] <= e
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (face_start[mid] <= e) lo = mid; else hi = mid;
    }
    const uint32_t f = lo;
    int c0[3], c1[3];
    face_cell_range(vx, ix, f, g, c0, c1);
    const uint32_t local = e - face_start[f];
    const uint32_t nx = (uint32_t)(c1[0] - c0[0] + 1), ny = (uint32_t)(c1[1] - c0[1] + 1);
    const uint32_t x = (uint32_t)c0[0] + local % nx, y = (uint32_t)c0[1] + (local / nx) % ny,
                   z = (uint32_t)c0[2] + local / (nx * ny);
    fn(f, (z * (uint32_t)g.dims[1] + y) * (uint32_t)g.dims[0] + x);
  }
}

static __global__ void k_face_count(const float* __restrict__ vx, const uint32_t* __restrict__ ix,
                                    uint32_t faces, FaceGridPlan g, const uint32_t* __restrict__ face_start,
                                    uint32_t entries, uint32_t* __restrict__ count) {
  for_entries(vx, ix, faces, g, face_start, entries, [&](uint32_t, uint32_t c) { atomicAdd(&count[c], 1u); });
}

static __global__ void k_face_fill(const float* __restrict__ vx, const uint32_t* __restrict__ ix,
                                   uint32_t faces, FaceGridPlan g, const uint32_t* __restrict__ face_start,
                                   uint32_t entries, const uint32_t* __restrict__ start,
                                   uint32_t* __restrict__ fill, uint32_t* __restrict__ list) {
  for_entries(vx, ix, faces, g, face_start, entries,
              [&](uint32_t f, uint32_t c) { list[start[c] + atomicAdd(&fill[c], 1u)] = f; });
}

static __global__ void k_face_sort(const uint32_t* __restrict__ start, uint32_t cells, uint32_t* __restrict__ list) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < cells; c += gridDim.x * blockDim.x) {
    const uint32_t b = start[c], e = start[c + 1];
    for (uint32_t k = b + 1; k < e; ++k) {  // insertion sort: lists are short and nearly all small
      const uint32_t v = list[k];
      uint32_t m = k;
      while (m > b && list[m - 1] > v) {
        list[m] = list[m - 1];
        --m;
      }
      list[m] = v;
    }
  }
}

// Exclusive scan of n counts into out[0..n] (out[n] = total) in three
// kernels: per-block sums of 4096 counts, one block scanning the sums, and
// the per-block scans with their offsets. n <= 2^22 (1024 blocks).
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr uint32_t kScanBlock = kScanThreads * kScanItems;

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* warp_tot, uint32_t* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    uint32_t t = lane < nw ? warp_tot[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < nw) warp_tot[lane] = t;  // inclusive over warps
    if (lane == nw - 1) *total = t;
  }
  __syncthreads();
  return x - v + (warp > 0 ? warp_tot[warp - 1] : 0u);
}

static __global__ void __launch_bounds__(kScanThreads)
    k_scan_sums(const uint32_t* __restrict__ in, uint32_t n, uint32_t* __restrict__ sums) {
  __shared__ uint32_t warp_tot[kScanThreads / 32];
  __shared__ uint32_t total;
  const uint32_t base = blockIdx.x * kScanBlock + threadIdx.x * kScanItems;
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) s += base + k < n ? in[base + k] : 0u;
  block_exclusive_scan(s, warp_tot, &total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

static __global__ void __launch_bounds__(kScanThreads)
    k_scan_top(uint32_t* __restrict__ sums, uint32_t blocks, uint32_t* __restrict__ grand_total) {
  __shared__ uint32_t warp_tot[kScanThreads / 32];
  __shared__ uint32_t total;
  const uint32_t v = threadIdx.x < blocks ? sums[threadIdx.x] : 0u;
  const uint32_t x = block_exclusive_scan(v, warp_tot, &total);
  if (threadIdx.x < blocks) sums[threadIdx.x] = x;
  if (threadIdx.x == 0) *grand_total = total;
}

static __global__ void __launch_bounds__(kScanThreads)
    k_scan_apply(const uint32_t* __restrict__ in, uint32_t n, const uint32_t* __restrict__ sums,
                 uint32_t* __restrict__ out) {
  __shared__ uint32_t warp_tot[kScanThreads / 32];
  __shared__ uint32_t total;
  const uint32_t base = blockIdx.x * kScanBlock + threadIdx.x * kScanItems;
  uint32_t v[kScanItems], s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = base + k < n ? in[base + k] : 0u;
    s += v[k];
  }
  uint32_t run = block_exclusive_scan(s, warp_tot, &total) + sums[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < n) out[base + k] = run;
    run += v[k];
  }
}

}  // namespace clsph
