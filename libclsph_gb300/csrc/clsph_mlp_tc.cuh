// Fused MLP inference on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// One persistent CTA of 16 warps per SM, 128-row tiles. All three weight
// matrices live in shared memory for the whole launch (W2 128 KB, W1 16 KB,
// W3 padded to 16 outputs 8 KB; canonical no-swizzle K-major core-matrix
// layout). A tile needs one 256-column region of tensor memory for its whole
// life: the layer-1 accumulator, then the layer-2 accumulator over it, then
// the layer-2 activations packed as BF16 over that (the A operand of layer 3,
// read by the MMA straight from tensor memory) and the layer-3 accumulator in
// columns the packing leaves free. Two regions (512 columns) hold two tiles,
// so the CTA runs a two-tile pipeline; per step u (tile c = u-th tile of the
// CTA, region u % 2):
//   16 warps   wait L3(u-2); outputs of tile u-2 (+ b3, de-standardised,
//              Store hook; 4 warps); X rows of c -> shared memory
//   thread 0   L1(c): 2 x tcgen05.mma M128 N256 K16 -> region, commit -> bar_l1
//   16 warps   wait L2(u-1) (frees the shared activation tile); wait L1(c);
//              tcgen05.ld, + b1, GELU, BF16 -> shared memory (A of layer 2)
//   thread 0   L2(c): 16 x M128 N256 K16 -> region, commit -> bar_l2
//   16 warps   tile u-1: tcgen05.ld, + b2, GELU, BF16, tcgen05.st in place
//              (while L2(c) runs on the tensor pipe)
//   thread 0   L3(u-1): 16 x M128 N16 K16, A from tensor memory, commit -> bar_l3
// so layer 2 of one tile runs under the epilogue of the other. Each mbarrier
// gets one commit and one wait per tile, so a wait never meets a phase that
// completed twice. Every wait is bounded; a wait that runs out sets *err, the
// CTA leaves its tile loop, waits (bounded) for its own MMAs and frees TMEM.
// The waits of the tile loop give up after `wait_limit` polls (by default
// kTcWaitLimit; a test hook sets 0 to make one run out); the teardown's waits
// for MMAs still in flight always allow kTcWaitLimit polls, so tensor memory
// is never freed under a running MMA.
//
// Encodings (PTX ISA, tcgen05): shared-memory descriptor = start address >> 4
// in bits 0-13, leading-dimension byte offset >> 4 in 16-29 (distance between
// the two core matrices of a K=16 slice), stride-dimension byte offset >> 4 in
// 32-45 (distance between 8-row groups), descriptor version 1 in 46-47,
// layout type 0 (no swizzle) in 61-63. Instruction descriptor for kind::f16:
// D format F32 (bits 4-5 = 1), A and B BF16 (7-9 = 1, 10-12 = 1), both
// K-major (15, 16 = 0), N >> 3 in 17-22, M >> 4 in 24-28. An A operand in
// tensor memory holds row r in lane r and two BF16 of consecutive K per
// 32-bit column (a K = 16 slice is 8 columns).
#pragma once

#include "clsph_mlp.cuh"

namespace clsph_nn {

constexpr int kTcRows = 128;
constexpr int kTcThreads = 512;
constexpr uint32_t kTcCols = 512;
constexpr int kOut3 = 16;  // layer-3 MMA width (4 outputs, 12 zero columns)
// shared-memory map (bytes)
constexpr uint32_t kTcW2 = 0;                            // 256 x 256 bf16, SBO 4096
constexpr uint32_t kTcH = kTcW2 + kHid * kHid * 2;       // 128 x 256 bf16, SBO 4096 (H1, then H2)
constexpr uint32_t kTcW1 = kTcH + kTcRows * kHid * 2;    // 256 x 32 bf16, SBO 512
constexpr uint32_t kTcX = kTcW1 + kHid * kIn * 2;        // 128 x 32 bf16, SBO 512
constexpr uint32_t kTcW3 = kTcX + kTcRows * kIn * 2;     // 16 x 256 bf16, SBO 4096
constexpr uint32_t kTcB1 = kTcW3 + kOut3 * kHid * 2;     // fp32 [256]
constexpr uint32_t kTcB2 = kTcB1 + kHid * 4;             // fp32 [256]
constexpr uint32_t kTcMisc = kTcB2 + kHid * 4;           // b3, y_mu, y_sigma [4 each]
constexpr uint32_t kTcBar = kTcMisc + 48;                // mbarriers bar_l1, bar_l2, bar_l3 (8 B each)
constexpr uint32_t kTcSlot = kTcBar + 24;                // TMEM base address (4 B)
constexpr uint32_t kTcSmem = kTcSlot + 8;
static_assert(kTcSmem <= 232448, "shared memory of the tcgen05 MLP");

constexpr uint32_t tc_idesc(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}
constexpr uint32_t kTcIdesc = tc_idesc(kTcRows, kHid);
constexpr uint32_t kTcIdesc3 = tc_idesc(kTcRows, kOut3);
// tensor-memory columns within a tile's 256-column region
constexpr uint32_t kTcRegion = 256;
constexpr uint32_t kTcAcc3 = 32;  // layer-3 accumulator: columns the packing leaves free
constexpr uint32_t kTcWaitLimit = 1u << 24;  // = CLSPH_DEFAULT_MLP_WAIT_POLLS

struct TcWeights {
  const bf16* w1t;  // [256][32]  (W1 transposed: output-major, K contiguous)
  const bf16* w2t;  // [256][256] (W2 transposed)
  const bf16* w3t;  // [16][256]  (W3 transposed, rows 4..15 zero)
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

// the same with the A operand in tensor memory at column address tmem_a
__device__ __forceinline__ void tc_mma_tmem_a(uint32_t tmem_d, uint32_t tmem_a, uint64_t bdesc, uint32_t idesc,
                                              uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "r"(tmem_a), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void tc_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar)
               : "memory");
}

__device__ __forceinline__ bool tc_wait(uint32_t bar, uint32_t parity, uint32_t limit) {
  for (uint32_t i = 0; i < limit; ++i) {
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

// 64 consecutive 32-bit TMEM columns of this thread's lane: one load and one
// wait in a single asm statement, so no use of the values can move above the
// wait and the load latency is paid once per 64 columns
__device__ __forceinline__ void tc_ld64(uint32_t taddr, float (&v)[64]) {
  uint32_t r[64];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x64.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, %32, %33, %34, %35, %36, %37, %38, %39, %40, %41, %42, %43, %44, %45, %46, %47, %48, %49, %50, %51, %52, %53, %54, %55, %56, %57, %58, %59, %60, %61, %62, %63}, [%64];\n\t"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]), "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int k = 0; k < 64; ++k) v[k] = __uint_as_float(r[k]);
}

// 4 consecutive 32-bit TMEM columns of this thread's lane
__device__ __forceinline__ void tc_ld4(uint32_t taddr, float (&v)[4]) {
  uint32_t r[4];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int k = 0; k < 4; ++k) v[k] = __uint_as_float(r[k]);
}

// 16 consecutive 32-bit TMEM columns of this thread's lane <- v
__device__ __forceinline__ void tc_st16(uint32_t taddr, const uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
      "%13, %14, %15, %16};\n" ::"r"(taddr),
      "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]), "r"(v[8]),
      "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15])
      : "memory");
  asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory");
}

__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint4 v) {
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};\n" ::"r"(addr), "r"(v.x), "r"(v.y), "r"(v.z),
               "r"(v.w)
               : "memory");
}

// TMEM columns [col0, col0 + 64) of this thread's row -> + bias, GELU, BF16
// -> the row's K slice of the canonical A-operand tile at `tile` (K = 256)
__device__ __forceinline__ void tc_hidden_epilogue(uint32_t taddr, int col0, const float* bias, uint32_t tile,
                                                   int r, const GeluTwiceConsts& gelu) {
  const float2* bias2 = reinterpret_cast<const float2*>(bias);
  float v[64];
  tc_ld64(taddr + col0, v);
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    uint32_t p[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int k = e * 8 + 2 * q;
      p[q] = gelu(make_float2(v[k], v[k + 1]), bias2[(col0 + k) >> 1]);
    }
    st_shared_v4(tile + (r >> 3) * 4096 + ((col0 + e * 8) >> 3) * 128 + (r & 7) * 16,
                 make_uint4(p[0], p[1], p[2], p[3]));
  }
}

// TMEM columns [taddr, taddr + 64) of this thread's row -> + bias, GELU, BF16
// pairs -> back into columns [taddr, taddr + 32) once all 64 are read, which
// makes the activations of these 64 K an A operand in tensor memory
__device__ __forceinline__ void tc_hidden_in_place(uint32_t taddr, const float* bias,
                                                   const GeluTwiceConsts& gelu) {
  const float2* bias2 = reinterpret_cast<const float2*>(bias);
  float v[64];
  tc_ld64(taddr, v);
  uint32_t p[32];
#pragma unroll
  for (int q = 0; q < 32; ++q) p[q] = gelu(make_float2(v[2 * q], v[2 * q + 1]), bias2[q]);
  tc_st16(taddr, reinterpret_cast<const uint32_t(&)[16]>(p[0]));
  tc_st16(taddr + 16u, reinterpret_cast<const uint32_t(&)[16]>(p[16]));
}

// column of the K = 16 slice `ks` of the packed layer-2 activations within a
// region: the 64-column chunk of warp column quarter ks / 4, whose first 32
// columns hold its 64 values
__device__ __forceinline__ uint32_t tc_h2_col(int ks) {
  return 64u * (uint32_t)(ks >> 2) + 8u * (uint32_t)(ks & 3);
}

template <class Store>
__global__ void __launch_bounds__(kTcThreads, 1)
    k_mlp_tc(const bf16* __restrict__ x, uint32_t rows, TcWeights w, Store store, uint32_t* __restrict__ err,
             uint32_t wait_limit) {
  extern __shared__ __align__(1024) unsigned char smem[];
  const uint32_t sb = smem_addr(smem);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  float* s_b1 = reinterpret_cast<float*>(smem + kTcB1);
  float* s_b2 = reinterpret_cast<float*>(smem + kTcB2);
  float* s_misc = reinterpret_cast<float*>(smem + kTcMisc);
  const uint32_t bar_l1 = sb + kTcBar, bar_l2 = bar_l1 + 8, bar_l3 = bar_l1 + 16;

  // weights -> canonical K-major core-matrix layout: element (row, k) at
  // (row / 8) * SBO + (k / 8) * 128 + (row % 8) * 16 + (k % 8) * 2
  for (int q = tid; q < kHid * (kHid / 8); q += kTcThreads) {
    const int n = q >> 5, c = q & 31;
    st_shared_v4(sb + kTcW2 + (n >> 3) * 4096 + c * 128 + (n & 7) * 16, reinterpret_cast<const uint4*>(w.w2t)[q]);
  }
  for (int q = tid; q < kHid * (kIn / 8); q += kTcThreads) {
    const int n = q >> 2, c = q & 3;
    st_shared_v4(sb + kTcW1 + (n >> 3) * 512 + c * 128 + (n & 7) * 16, reinterpret_cast<const uint4*>(w.w1t)[q]);
  }
  for (int q = tid; q < kOut3 * (kHid / 8); q += kTcThreads) {
    const int n = q >> 5, c = q & 31;
    st_shared_v4(sb + kTcW3 + (n >> 3) * 4096 + c * 128 + (n & 7) * 16, reinterpret_cast<const uint4*>(w.w3t)[q]);
  }
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
    for (uint32_t b = bar_l1; b <= bar_l3; b += 8)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(b) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(smem + kTcSlot);

  const int lg = warp & 3, cq = warp >> 2;                      // lane quarter, column quarter
  const int r = lg * 32 + lane;                                  // tile row = TMEM lane
  const uint32_t t_row = tmem + ((uint32_t)(lg * 32) << 16);
  const GeluTwiceConsts gelu;  // twice GELU: W2 and W3 are stored halved
  // one phase bit and one count of unwaited commits (thread 0) per barrier
  uint32_t ph1 = 0, ph2 = 0, ph3 = 0, n1 = 0, n2 = 0, n3 = 0;
  bool ok = true;
  const uint32_t tiles = (rows + kTcRows - 1) / kTcRows;
  const uint32_t mine = blockIdx.x < tiles ? (tiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;  // tiles of this CTA
  auto tile_of = [&](uint32_t u) { return blockIdx.x + u * gridDim.x; };
  auto region = [&](uint32_t u) { return (u & 1u) * kTcRegion; };
  // this thread's 16-byte chunk of a tile's X rows: row tid / 4, chunk tid % 4
  const int xr = tid >> 2, xc = tid & 3;
  const uint32_t x_dst = sb + kTcX + (xr >> 3) * 512 + xc * 128 + (xr & 7) * 16;
  auto load_x = [&](uint32_t u) {
    const uint32_t row = tile_of(u) * kTcRows + xr;
    return (u < mine && row < rows) ? reinterpret_cast<const uint4*>(x)[(size_t)row * (kIn / 8) + xc]
                                    : make_uint4(0u, 0u, 0u, 0u);
  };
  // a wait that runs out keeps its phase, so the teardown waits for the same one
  auto wait_on = [&](uint32_t b, uint32_t& ph, uint32_t& pending) {
    const bool got = tc_wait(b, ph, wait_limit);
    if (got) {
      ph ^= 1;
      if (tid == 0) --pending;
    }
    return __syncthreads_and(got);
  };
  uint4 xv = load_x(0);
  for (uint32_t u = 0; u < mine + 2 && ok; ++u) {
    const bool cur = u < mine;  // tile u gets layers 1 and 2 in this step
    if (u >= 2) {               // tile u - 2: outputs
      if (!(ok = wait_on(bar_l3, ph3, n3))) break;
      tc_fence_after();
      if (cq == 0) {
        float o[4];
        tc_ld4(t_row + region(u) + kTcAcc3, o);
        const uint32_t row = tile_of(u - 2) * kTcRows + r;
        if (row < rows)
          store(row, make_float4((o[0] + s_misc[0]) * s_misc[8] + s_misc[4],
                                 (o[1] + s_misc[1]) * s_misc[9] + s_misc[5],
                                 (o[2] + s_misc[2]) * s_misc[10] + s_misc[6],
                                 (o[3] + s_misc[3]) * s_misc[11] + s_misc[7]));
      }
    }
    if (cur) {
      st_shared_v4(x_dst, xv);
      fence_async_smem();
    }
    tc_fence_before();
    __syncthreads();
    if (cur && tid == 0) {  // L1(u) into the region tile u - 2 has just left
      tc_fence_after();
#pragma unroll
      for (int ks = 0; ks < kIn / 16; ++ks)
        tc_mma(tmem + region(u), tc_desc(sb + kTcX + ks * 256, 128, 512),
               tc_desc(sb + kTcW1 + ks * 256, 128, 512), kTcIdesc, ks > 0);
      tc_commit(bar_l1);
      ++n1;
    }
    if (cur) xv = load_x(u + 1);  // next tile's rows, in flight during this step
    if (u >= 1 && u <= mine) {    // L2(u - 1) done: the shared activation tile is free
      if (!(ok = wait_on(bar_l2, ph2, n2))) break;
    }
    if (cur) {
      if (!(ok = wait_on(bar_l1, ph1, n1))) break;
      tc_fence_after();
      tc_hidden_epilogue(t_row + region(u), cq * 64, s_b1, sb + kTcH, r, gelu);
      fence_async_smem();
      tc_fence_before();
      __syncthreads();
      if (tid == 0) {  // L2(u) over layer 1's accumulator, which the epilogue has read
        tc_fence_after();
#pragma unroll
        for (int ks = 0; ks < kHid / 16; ++ks)
          tc_mma(tmem + region(u), tc_desc(sb + kTcH + ks * 256, 128, 4096),
                 tc_desc(sb + kTcW2 + ks * 256, 128, 4096), kTcIdesc, ks > 0);
        tc_commit(bar_l2);
        ++n2;
      }
    }
    if (u >= 1 && u <= mine) {  // tile u - 1: layer-2 epilogue under L2(u), then L3(u - 1)
      const uint32_t reg = region(u - 1);
      tc_fence_after();
      tc_hidden_in_place(t_row + reg + 64u * cq, s_b2 + 64 * cq, gelu);
      tc_fence_before();
      __syncthreads();
      if (tid == 0) {
        tc_fence_after();
#pragma unroll
        for (int ks = 0; ks < kHid / 16; ++ks)
          tc_mma_tmem_a(tmem + reg + kTcAcc3, tmem + reg + tc_h2_col(ks),
                        tc_desc(sb + kTcW3 + ks * 256, 128, 4096), kTcIdesc3, ks > 0);
        tc_commit(bar_l3);
        ++n3;
      }
    }
  }
  // teardown: MMAs of this CTA must be complete before TMEM is freed (a
  // commit tracks every MMA issued before it; each barrier's oldest unwaited
  // commit is the phase to wait for)
  if (tid == 0) {
    if (n1 && !tc_wait(bar_l1, ph1, kTcWaitLimit)) atomicOr(err, 2u);
    if (n2 && !tc_wait(bar_l2, ph2, kTcWaitLimit)) atomicOr(err, 2u);
    if (n3 && !tc_wait(bar_l3, ph3, kTcWaitLimit)) atomicOr(err, 2u);
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

// ---------------------------------------------------------------------------
// Training GEMM on the tensor cores: C[M x N] = A[M x K] B[K x N] with BF16
// operands and FP32 accumulation in tensor memory; one CTA of 4 warps per
// 128-row tile of C and all N <= 256 columns, split-K over blockIdx.z, and
// the epilogue functors of k_gemm on every (row, even column) pair.
// A_K: A is stored with K contiguous (row m at A + m lda), else with M
// contiguous (A^T in memory: row k at A + k lda). B_K: B is stored with K
// contiguous per column n (B + n ldb), else with N contiguous (row k at
// B + k ldb). Operands are staged 32 K at a time, double-buffered, into the
// canonical no-swizzle K-major core-matrix layout of the inference kernel
// (element (r, k) at (r / 8) * 512 + (k / 8) * 128 + (r % 8) * 16 +
// (k % 8) * 2): 16-byte vectors when K is contiguous in memory, else 8
// two-byte stores per 16-byte vector (the transpose). Thread 0 issues two
// M128 x N x K16 MMAs per chunk and commits them to the chunk buffer's
// mbarrier; a buffer is restaged once the MMAs that read it have completed.
// Every wait is bounded: one that runs out sets *err, the CTA stops issuing,
// waits (bounded) for its last commit and frees tensor memory.
constexpr int kGtRows = 128;
constexpr int kGtBK = 32;
constexpr int kGtThreads = 128;
constexpr uint32_t kGtSmem = 100 * 1024;  // also keeps two CTAs per SM (512 TMEM columns)

template <int BN>
struct GemmTcLayout {
  static_assert(BN % 16 == 0 && BN >= 32 && BN <= 256, "N of an M128 MMA");
  static constexpr uint32_t kA = kGtRows * kGtBK * 2;
  static constexpr uint32_t kB = BN * kGtBK * 2;
  static constexpr uint32_t kStage = kA + kB;
  static constexpr uint32_t kBar = 2 * kStage;  // two mbarriers
  static constexpr uint32_t kSlot = kBar + 16;  // tensor-memory address
  static constexpr uint32_t kBytes = kSlot + 16;
  static constexpr uint32_t kCols = BN <= 32 ? 32 : (BN <= 64 ? 64 : (BN <= 128 ? 128 : 256));
  static constexpr uint32_t kIdesc = tc_idesc(kGtRows, BN);
  static_assert(kBytes <= kGtSmem, "shared memory of the tensor-core GEMM");
};

__device__ __forceinline__ void st_shared_u16(uint32_t addr, uint16_t v) {
  asm volatile("st.shared.u16 [%0], %1;\n" ::"r"(addr), "h"(v) : "memory");
}

// 32 consecutive 32-bit TMEM columns of this thread's lane
__device__ __forceinline__ void tc_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
      "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n\t"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int k = 0; k < 32; ++k) v[k] = __uint_as_float(r[k]);
}

// `rows` x 32 K of an operand into the canonical layout at `dst`: K-major in
// memory (row r at src + r ld, K contiguous) or MN-major (K row k at
// src + k ld, the rows contiguous)
template <bool KMAJOR>
__device__ __forceinline__ void gt_stage(uint32_t dst, const bf16* __restrict__ src, int ld, int rows) {
  if constexpr (KMAJOR) {
    for (int c = threadIdx.x; c < rows * 4; c += kGtThreads) {
      const int r = c >> 2, q = c & 3;
      const uint4 v = *reinterpret_cast<const uint4*>(src + (size_t)r * ld + q * 8);
      st_shared_v4(dst + (r >> 3) * 512 + q * 128 + (r & 7) * 16, v);
    }
  } else {
    const int vecs = rows / 8;
    for (int c = threadIdx.x; c < kGtBK * vecs; c += kGtThreads) {
      const int k = c / vecs, mq = c % vecs;
      const uint4 v = *reinterpret_cast<const uint4*>(src + (size_t)k * ld + mq * 8);
      const uint32_t w[4] = {v.x, v.y, v.z, v.w};
      const uint32_t base = dst + mq * 512 + (k >> 3) * 128 + (k & 7) * 2;
#pragma unroll
      for (int e = 0; e < 8; ++e)
        st_shared_u16(base + e * 16, (uint16_t)(e & 1 ? w[e >> 1] >> 16 : w[e >> 1] & 0xFFFFu));
    }
  }
}

template <int BN, bool A_K, bool B_K, class Epi>
__global__ void __launch_bounds__(kGtThreads, 1)
    k_gemm_tc(const bf16* __restrict__ A, int lda, const bf16* __restrict__ B, int ldb, int K, int k_split,
              Epi epi, uint32_t* __restrict__ err) {
  using L = GemmTcLayout<BN>;
  extern __shared__ __align__(1024) unsigned char smem[];
  const uint32_t sb = smem_addr(smem);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.y * kGtRows;
  const int k_begin = blockIdx.z * k_split;
  const int k_end = min(K, k_begin + k_split);
  const int chunks = (k_end - k_begin) / kGtBK;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(sb + L::kSlot),
                 "r"(L::kCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(sb + L::kBar) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(sb + L::kBar + 8) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  auto stage = [&](int buf, int k0) {
    const uint32_t a = sb + buf * L::kStage, b = a + L::kA;
    if constexpr (A_K) gt_stage<true>(a, A + (size_t)m0 * lda + k0, lda, kGtRows);
    else gt_stage<false>(a, A + (size_t)k0 * lda + m0, lda, kGtRows);
    if constexpr (B_K) gt_stage<true>(b, B + k0, ldb, BN);
    else gt_stage<false>(b, B + (size_t)k0 * ldb, ldb, BN);
    fence_async_smem();
  };
  if (chunks > 0) stage(0, k_begin);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(smem + L::kSlot);
  uint32_t ph[2] = {0u, 0u};
  bool ok = true;
  int issued = 0;  // chunks whose MMAs have been issued
  for (int c = 0; c < chunks && ok; ++c) {
    const int buf = c & 1;
    if (tid == 0) {
      tc_fence_after();
      const uint32_t a = sb + buf * L::kStage, b = a + L::kA;
#pragma unroll
      for (int ks = 0; ks < kGtBK / 16; ++ks)
        tc_mma(tmem, tc_desc(a + ks * 256, 128, 512), tc_desc(b + ks * 256, 128, 512), L::kIdesc,
               (c > 0 || ks > 0) ? 1u : 0u);
      tc_commit(sb + L::kBar + 8 * buf);
    }
    issued = c + 1;
    if (c + 1 < chunks) {
      const int nb = buf ^ 1;
      if (c >= 1) {  // the MMAs of chunk c - 1 read buffer nb
        const bool got = tc_wait(sb + L::kBar + 8 * nb, ph[nb], kTcWaitLimit);
        if (got) ph[nb] ^= 1u;
        ok = __syncthreads_and(got);
        if (!ok) break;
      }
      stage(nb, k_begin + (c + 1) * kGtBK);
      tc_fence_before();
      __syncthreads();
    }
  }
  // the last commit covers every MMA issued before it
  bool done = issued == 0;
  if (issued > 0) {
    const int lb = (issued - 1) & 1;
    // a barrier whose earlier commit was not waited for completes twice
    // before the last phase: wait for that one first
    if (issued >= 2 && ok) {
      const int ob = lb ^ 1;
      if (tc_wait(sb + L::kBar + 8 * ob, ph[ob], kTcWaitLimit)) ph[ob] ^= 1u;
    }
    done = tc_wait(sb + L::kBar + 8 * lb, ph[lb], kTcWaitLimit);
  }
  if (!__syncthreads_and(done && ok) && tid == 0) atomicOr(err, 1u);
  tc_fence_after();
  if (done && ok) {
    const int row = m0 + warp * 32 + lane;
    const uint32_t t_row = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += 32) {
      float v[32];
      tc_ld32(t_row + c0, v);
#pragma unroll
      for (int j = 0; j < 16; ++j) epi(row, c0 + 2 * j, v[2 * j], v[2 * j + 1]);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(L::kCols)
                 : "memory");
  }
}

}  // namespace clsph_nn
