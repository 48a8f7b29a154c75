// Shared device helpers of the GB300 SPH substep engine.
//
// "Exact" helpers use the round-to-nearest intrinsics, which the compiler
// never contracts into FMAs, so the pair arithmetic reproduces the
// reference's single-precision expression order operation by operation
// (libclsph/kernels/smoothing.cl, forces.cl, advection.cl, collisions.cl).
// Fast paths (candidate culling) may use FMAs; they only decide whether the
// exact path runs and carry a conservative margin.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace clsph {

#define XADD __fadd_rn
#define XSUB __fsub_rn
#define XMUL __fmul_rn
#define XDIV __fdiv_rn
#define XSQRT __fsqrt_rn

struct V3 {
  float x, y, z;
};

__device__ __forceinline__ V3 xsub3(V3 a, V3 b) { return {XSUB(a.x, b.x), XSUB(a.y, b.y), XSUB(a.z, b.z)}; }
// OpenCL length(): sqrt((x*x + y*y) + z*z)
__device__ __forceinline__ float xnorm(V3 v) {
  return XSQRT(XADD(XADD(XMUL(v.x, v.x), XMUL(v.y, v.y)), XMUL(v.z, v.z)));
}
__device__ __forceinline__ float xdot(V3 a, V3 b) {
  return XADD(XADD(XMUL(a.x, b.x), XMUL(a.y, b.y)), XMUL(a.z, b.z));
}
__device__ __forceinline__ V3 v3(float4 f) { return {f.x, f.y, f.z}; }

// ---------------------------------------------------------------- Morton
// 10 bits per axis; x -> bit 3k, y -> 3k+1, z -> 3k+2 (libclsph/common/util.h:41-62).
// Bit spreading by the standard shift-and-mask sequence ("Part1By2").
__host__ __device__ __forceinline__ uint32_t spread_bits3(uint32_t v) {
  v &= 0x3FFu;
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}
__host__ __device__ __forceinline__ uint32_t compact_bits3(uint32_t v) {
  v &= 0x09249249u;
  v = (v | (v >> 2)) & 0x030C30C3u;
  v = (v | (v >> 4)) & 0x0300F00Fu;
  v = (v | (v >> 8)) & 0x030000FFu;
  v = (v | (v >> 16)) & 0x000003FFu;
  return v;
}
__host__ __device__ __forceinline__ uint32_t morton3(uint32_t x, uint32_t y, uint32_t z) {
  return spread_bits3(x) | (spread_bits3(y) << 1) | (spread_bits3(z) << 2);
}

// float -> orderable uint for atomicMin/atomicMax bounding boxes
__host__ __device__ __forceinline__ uint32_t f2ord(float f) {
#ifdef __CUDA_ARCH__
  uint32_t u = __float_as_uint(f);
#else
  uint32_t u;
  memcpy(&u, &f, 4);
#endif
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ __forceinline__ float ord2f(uint32_t o) {
  uint32_t u = (o & 0x80000000u) ? (o & 0x7FFFFFFFu) : ~o;
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}

// Open-addressing cell index: key -> slot, linear probing, 0 = empty.
__device__ __forceinline__ uint32_t cell_hash(uint32_t key) { return key * 0x9E3779B1u; }

}  // namespace clsph
