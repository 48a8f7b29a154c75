// Fused MLP inference on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// One persistent CTA per SM, 128-row tiles. Both weight matrices live in
// shared memory for the whole launch (W2 128 KB, W1 16 KB, canonical
// no-swizzle K-major core-matrix layout); accumulators live in tensor memory
// (layer 1 in columns 0..255, layer 2 in columns 256..511 of a 512-column
// allocation). Per tile:
//   all threads   X rows -> shared memory (A operand of layer 1)
//   thread 0      2 x tcgen05.mma M128 N256 K16 -> TMEM, tcgen05.commit -> mbarrier
//   8 warps       tcgen05.ld, + b1, GELU, BF16 -> shared memory (A operand of layer 2)
//   thread 0      16 x tcgen05.mma M128 N256 K16 -> TMEM, commit
//   8 warps       tcgen05.ld, + b2, GELU, layer 3 (256 -> 4, FP32 W3) on the CUDA
//                 cores, the two column halves summed through shared memory,
//                 de-standardised and handed to the Store hook.
// Every mbarrier wait is bounded; a wait that runs out sets *err, the CTA
// leaves its tile loop, waits (bounded) for its own MMAs and frees TMEM.
//
// Encodings (PTX ISA, tcgen05): shared-memory descriptor = start address >> 4
// in bits 0-13, leading-dimension byte offset >> 4 in 16-29 (distance between
// the two core matrices of a K=16 slice), stride-dimension byte offset >> 4 in
// 32-45 (distance between 8-row groups), descriptor version 1 in 46-47,
// layout type 0 (no swizzle) in 61-63. Instruction descriptor for kind::f16:
// D format F32 (bits 4-5 = 1), A and B BF16 (7-9 = 1, 10-12 = 1), both
// K-major (15, 16 = 0), N >> 3 in 17-22, M >> 4 in 24-28.
#pragma once

#include "clsph_mlp.cuh"

namespace clsph_nn {

constexpr int kTcRows = 128;
constexpr int kTcThreads = 256;
constexpr uint32_t kTcCols = 512;
// shared-memory map (bytes)
constexpr uint32_t kTcW2 = 0;                            // 256 x 256 bf16, SBO 4096
constexpr uint32_t kTcH = kTcW2 + kHid * kHid * 2;       // 128 x 256 bf16, SBO 4096
constexpr uint32_t kTcW1 = kTcH + kTcRows * kHid * 2;    // 256 x 32 bf16, SBO 512
constexpr uint32_t kTcX = kTcW1 + kHid * kIn * 2;        // 128 x 32 bf16, SBO 512
constexpr uint32_t kTcW3 = kTcX + kTcRows * kIn * 2;     // fp32 [256][4]
constexpr uint32_t kTcB1 = kTcW3 + kHid * kOut * 4;      // fp32 [256]
constexpr uint32_t kTcB2 = kTcB1 + kHid * 4;             // fp32 [256]
constexpr uint32_t kTcRed = kTcB2 + kHid * 4;            // fp32 [128][4]
constexpr uint32_t kTcMisc = kTcRed + kTcRows * kOut * 4;  // b3, y_mu, y_sigma [4 each]
constexpr uint32_t kTcBar = kTcMisc + 48;                // mbarrier (8 B)
constexpr uint32_t kTcSlot = kTcBar + 8;                 // TMEM base address (4 B)
constexpr uint32_t kTcSmem = kTcSlot + 8;
static_assert(kTcSmem <= 232448, "shared memory of the tcgen05 MLP");

constexpr uint32_t kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kHid >> 3) << 17) |
                              ((uint32_t)(kTcRows >> 4) << 24);
constexpr uint32_t kTcWaitLimit = 1u << 24;

struct TcWeights {
  const bf16* w1t;  // [256][32]  (W1 transposed: output-major, K contiguous)
  const bf16* w2t;  // [256][256] (W2 transposed)
  const float* w3;  // [256][4]
  const float* b1;
  const float* b2;
  const float* b3;
  const float* y_mu;
  const float* y_sigma;
};

__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                       uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void tc_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar)
               : "memory");
}

__device__ __forceinline__ bool tc_wait(uint32_t bar, uint32_t parity) {
  for (uint32_t i = 0; i < kTcWaitLimit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

// 32 consecutive 32-bit TMEM columns of this thread's lane
__device__ __forceinline__ void tc_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
      "%12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, "
      "%30, %31}, [%32];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
        "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
        "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int k = 0; k < 32; ++k) v[k] = __uint_as_float(r[k]);
}

__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint4 v) {
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};\n" ::"r"(addr), "r"(v.x), "r"(v.y), "r"(v.z),
               "r"(v.w)
               : "memory");
}

template <class Store>
__global__ void __launch_bounds__(kTcThreads, 1)
    k_mlp_tc(const bf16* __restrict__ x, uint32_t rows, TcWeights w, Store store, uint32_t* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  const uint32_t sb = smem_addr(smem);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  float* s_w3 = reinterpret_cast<float*>(smem + kTcW3);
  float* s_b1 = reinterpret_cast<float*>(smem + kTcB1);
  float* s_b2 = reinterpret_cast<float*>(smem + kTcB2);
  float* s_red = reinterpret_cast<float*>(smem + kTcRed);
  float* s_misc = reinterpret_cast<float*>(smem + kTcMisc);
  const uint32_t bar = sb + kTcBar;

  // weights -> canonical K-major core-matrix layout: element (row, k) at
  // (row / 8) * SBO + (k / 8) * 128 + (row % 8) * 16 + (k % 8) * 2
  for (int q = tid; q < kHid * (kHid / 8); q += kTcThreads) {
    const int n = q >> 5, c = q & 31;
    const uint4 v = reinterpret_cast<const uint4*>(w.w2t)[q];
    st_shared_v4(sb + kTcW2 + (n >> 3) * 4096 + c * 128 + (n & 7) * 16, v);
  }
  for (int q = tid; q < kHid * (kIn / 8); q += kTcThreads) {
    const int n = q >> 2, c = q & 3;
    const uint4 v = reinterpret_cast<const uint4*>(w.w1t)[q];
    st_shared_v4(sb + kTcW1 + (n >> 3) * 512 + c * 128 + (n & 7) * 16, v);
  }
  for (int q = tid; q < kHid * kOut; q += kTcThreads) s_w3[q] = w.w3[q];
  for (int q = tid; q < kHid; q += kTcThreads) {
    s_b1[q] = w.b1[q];
    s_b2[q] = w.b2[q];
  }
  if (tid < kOut) {
    s_misc[tid] = w.b3[tid];
    s_misc[4 + tid] = w.y_mu[tid];
    s_misc[8 + tid] = w.y_sigma[tid];
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(sb + kTcSlot),
                 "r"(kTcCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(smem + kTcSlot);

  const int lg = warp & 3, half = warp >> 2;
  const int r = lg * 32 + lane;                                  // tile row = TMEM lane
  const uint32_t t_row = tmem + ((uint32_t)(lg * 32) << 16);     // this warp's lane quarter
  const uint32_t k0 = pack_bf16(0.7978845608028654f, 0.7978845608028654f);
  const uint32_t k01 = pack_bf16(0.7978845608028654f * 0.044715f, 0.7978845608028654f * 0.044715f);
  const uint32_t hf = pack_bf16(0.5f, 0.5f);
  uint32_t phase = 0;
  bool ok = true;
  uint32_t issued = 0;  // commits made by thread 0 and not yet waited for
  const uint32_t tiles = (rows + kTcRows - 1) / kTcRows;
  for (uint32_t tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
    const uint32_t row0 = tile * kTcRows;
    for (int q = tid; q < kTcRows * (kIn / 8); q += kTcThreads) {
      const int rr = q >> 2, c = q & 3;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (row0 + rr < rows) v = reinterpret_cast<const uint4*>(x)[(size_t)(row0 + rr) * (kIn / 8) + c];
      st_shared_v4(sb + kTcX + (rr >> 3) * 512 + c * 128 + (rr & 7) * 16, v);
    }
    fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
#pragma unroll
      for (int ks = 0; ks < kIn / 16; ++ks)
        tc_mma(tmem, tc_desc(sb + kTcX + ks * 256, 128, 512), tc_desc(sb + kTcW1 + ks * 256, 128, 512),
               kTcIdesc, ks > 0);
      tc_commit(bar);
      ++issued;
    }
    bool got = tc_wait(bar, phase);
    phase ^= 1;
    if (tid == 0 && got) --issued;
    ok = __syncthreads_and(got);
    if (!ok) break;
    tc_fence_after();
    // layer-1 epilogue: 128 columns of this thread's row
#pragma unroll 1
    for (int c = 0; c < 4; ++c) {
      const int col0 = half * 128 + c * 32;
      float v[32];
      tc_ld32(t_row + col0, v);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        uint32_t p[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int k = e * 8 + 2 * q;
          p[q] = gelu2_bf16(v[k] + s_b1[col0 + k], v[k + 1] + s_b1[col0 + k + 1], k0, k01, hf);
        }
        st_shared_v4(sb + kTcH + (r >> 3) * 4096 + ((col0 + e * 8) >> 3) * 128 + (r & 7) * 16,
                     make_uint4(p[0], p[1], p[2], p[3]));
      }
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
#pragma unroll
      for (int ks = 0; ks < kHid / 16; ++ks)
        tc_mma(tmem + 256, tc_desc(sb + kTcH + ks * 256, 128, 4096),
               tc_desc(sb + kTcW2 + ks * 256, 128, 4096), kTcIdesc, ks > 0);
      tc_commit(bar);
      ++issued;
    }
    got = tc_wait(bar, phase);
    phase ^= 1;
    if (tid == 0 && got) --issued;
    ok = __syncthreads_and(got);
    if (!ok) break;
    tc_fence_after();
    // layer-2 epilogue and layer 3
    float y[kOut] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 1
    for (int c = 0; c < 4; ++c) {
      const int col0 = half * 128 + c * 32;
      float v[32];
      tc_ld32(t_row + 256 + col0, v);
#pragma unroll
      for (int k = 0; k < 32; k += 2) {
        const uint32_t g = gelu2_bf16(v[k] + s_b2[col0 + k], v[k + 1] + s_b2[col0 + k + 1], k0, k01, hf);
        const float g0 = __uint_as_float(g << 16), g1 = __uint_as_float(g & 0xFFFF0000u);
        const float4 wa = reinterpret_cast<const float4*>(s_w3)[col0 + k];
        const float4 wb = reinterpret_cast<const float4*>(s_w3)[col0 + k + 1];
        y[0] += g0 * wa.x + g1 * wb.x;
        y[1] += g0 * wa.y + g1 * wb.y;
        y[2] += g0 * wa.z + g1 * wb.z;
        y[3] += g0 * wa.w + g1 * wb.w;
      }
    }
    if (half == 1) reinterpret_cast<float4*>(s_red)[r] = make_float4(y[0], y[1], y[2], y[3]);
    tc_fence_before();
    __syncthreads();
    if (half == 0 && row0 + r < rows) {
      const float4 o = reinterpret_cast<const float4*>(s_red)[r];
      store(row0 + r, make_float4((y[0] + o.x + s_misc[0]) * s_misc[8] + s_misc[4],
                                  (y[1] + o.y + s_misc[1]) * s_misc[9] + s_misc[5],
                                  (y[2] + o.z + s_misc[2]) * s_misc[10] + s_misc[6],
                                  (y[3] + o.w + s_misc[3]) * s_misc[11] + s_misc[7]));
    }
  }
  // teardown: MMAs of this CTA must be complete before TMEM is freed
  if (tid == 0 && issued) {
    if (!tc_wait(bar, phase)) atomicOr(err, 2u);
  }
  if (!ok && tid == 0) atomicOr(err, 1u);
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTcCols)
                 : "memory");
  }
}

}  // namespace clsph_nn
