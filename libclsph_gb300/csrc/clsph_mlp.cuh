// BF16 tensor-core kernels of the learned stepper's per-particle MLP
// (32 -> 256 -> 256 -> 4, GELU, BF16 weights and activations, FP32
// accumulation). No counterpart in the reference.
//
//   k_mlp_infer   fused inference: one warp carries a 16-row tile through all
//                 three layers; layer-1 outputs are re-packed from the
//                 accumulator fragments straight into the A fragments of
//                 layer 2, layer-2 outputs are consumed 64 columns at a time
//                 by layer 3, so nothing but the 64-byte feature row is read
//                 and one float4 written per particle.
//   Epi*          epilogue functors of the training GEMMs (bias + GELU,
//                 GELU', split partials), which run on the tcgen05 tensor
//                 cores (k_gemm_tc, clsph_mlp_tc.cuh).
//   k_head_*, k_colsum, k_reduce_splits, k_adam, k_gather_batch: the
//                 elementwise and reduction parts of one training iteration.
//
// Fragment layouts follow the PTX ISA description of
// mma.sync.m16n8k16.row.col.f32.bf16.bf16.f32 and ldmatrix.m8n8.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace clsph_nn {

constexpr int kIn = 32;
constexpr int kHid = 256;
constexpr int kOut = 4;
constexpr int kOutPad = 8;  // layer-3 weights padded to one n8 tile

// fp32 parameter blob: W1[32][256] b1[256] W2[256][256] b2[256] W3[256][4] b3[4]
// followed by the standardisation x_mu[32] x_sigma[32] y_mu[4] y_sigma[4].
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kIn * kHid;
constexpr int kOffW2 = kOffB1 + kHid;
constexpr int kOffB2 = kOffW2 + kHid * kHid;
constexpr int kOffW3 = kOffB2 + kHid;
constexpr int kOffB3 = kOffW3 + kHid * kOut;
constexpr int kParams = kOffB3 + kOut;  // trainable
constexpr int kOffXMu = kParams;
constexpr int kOffXSigma = kOffXMu + kIn;
constexpr int kOffYMu = kOffXSigma + kIn;
constexpr int kOffYSigma = kOffYMu + kOut;
constexpr int kBlob = kOffYSigma + kOut;

using bf16 = __nv_bfloat16;

// ---------------------------------------------------------------------------
// PTX wrappers

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void ldsm_x4_t(uint32_t (&r)[4], uint32_t addr) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0, %1, %2, %3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(addr));
}

__device__ __forceinline__ void ldsm_x2_t(uint32_t& r0, uint32_t& r1, uint32_t addr) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0, %1}, [%2];\n"
               : "=r"(r0), "=r"(r1)
               : "r"(addr));
}

// d += a * b, one m16n8k16 tile
__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, "
      "{%8, %9}, {%0, %1, %2, %3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}


// Standardised inputs are clamped to +-kInputClamp (training and inference
// alike): states outside the training distribution cannot drive the network
// into extrapolation.
constexpr float kInputClamp = 6.f;
__device__ __forceinline__ float standardise(float v, float mu, float sigma) {
  return fminf(fmaxf((v - mu) / sigma, -kInputClamp), kInputClamp);
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}

// hardware tanh (tanh.approx.f32: one special-function-unit operation,
// absolute error about 2^-11, below the BF16 rounding of the activations)
__device__ __forceinline__ float tanh_hw(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;\n" : "=f"(y) : "f"(x));
  return y;
}

// Derivative of the tanh form of GELU (the form of
// torch.nn.functional.gelu(x, approximate="tanh")), with the hardware tanh.
__device__ __forceinline__ float gelu_grad(float x) {
  const float k0 = 0.7978845608028654f, k1 = 0.044715f;
  const float x2 = x * x;
  const float t = tanh_hw(k0 * x * (1.f + k1 * x2));
  return 0.5f * (1.f + t) + 0.5f * x * (1.f - t * t) * k0 * (1.f + 3.f * k1 * x2);
}

// GELU of two values, evaluated in packed BF16 (inputs rounded to BF16, the
// tanh form with BF16 constants, tanh.approx.bf16x2): two activations per
// special-function operation. The network is trained and run with this
// function; the backward pass uses gelu_grad of the FP32 input.
// k0 = bf16x2(sqrt(2/pi)), k01 = bf16x2(sqrt(2/pi) * 0.044715), hf = bf16x2(0.5).
__device__ __forceinline__ uint32_t gelu2_bf16(float a, float b, uint32_t k0, uint32_t k01, uint32_t hf) {
  const uint32_t x = pack_bf16(a, b);
  uint32_t x2, c, u, t, hx, r;
  asm("mul.rn.bf16x2 %0, %1, %1;\n" : "=r"(x2) : "r"(x));
  asm("fma.rn.bf16x2 %0, %1, %2, %3;\n" : "=r"(c) : "r"(x2), "r"(k01), "r"(k0));
  asm("mul.rn.bf16x2 %0, %1, %2;\n" : "=r"(u) : "r"(x), "r"(c));
  asm("tanh.approx.bf16x2 %0, %1;\n" : "=r"(t) : "r"(u));
  asm("mul.rn.bf16x2 %0, %1, %2;\n" : "=r"(hx) : "r"(x), "r"(hf));
  asm("fma.rn.bf16x2 %0, %1, %2, %1;\n" : "=r"(r) : "r"(hx), "r"(t));
  return r;
}

struct GeluConsts {
  uint32_t k0, k01, hf;
  __device__ GeluConsts()
      : k0(pack_bf16(0.7978845608028654f, 0.7978845608028654f)),
        k01(pack_bf16(0.7978845608028654f * 0.044715f, 0.7978845608028654f * 0.044715f)),
        hf(pack_bf16(0.5f, 0.5f)) {}
  __device__ uint32_t operator()(float a, float b) const { return gelu2_bf16(a, b, k0, k01, hf); }
};

// Twice gelu2_bf16, exactly: x (1 + tanh u) = fma(x, t, x) is the same
// rounding of twice 0.5 x (1 + tanh u) (a power-of-two factor commutes with
// rounding), one multiplication fewer. The tcgen05 kernel uses it with the
// next layer's BF16 weights halved (Bf16Weights::w2t, w3t), so every product
// of the layer is unchanged.
__device__ __forceinline__ uint32_t gelu2x2_bf16(float2 v, uint32_t k0, uint32_t k01) {
  const uint32_t x = pack_bf16(v.x, v.y);
  uint32_t x2, c, u, t, r;
  asm("mul.rn.bf16x2 %0, %1, %1;\n" : "=r"(x2) : "r"(x));
  asm("fma.rn.bf16x2 %0, %1, %2, %3;\n" : "=r"(c) : "r"(x2), "r"(k01), "r"(k0));
  asm("mul.rn.bf16x2 %0, %1, %2;\n" : "=r"(u) : "r"(x), "r"(c));
  asm("tanh.approx.bf16x2 %0, %1;\n" : "=r"(t) : "r"(u));
  asm("fma.rn.bf16x2 %0, %1, %2, %1;\n" : "=r"(r) : "r"(x), "r"(t));
  return r;
}

struct GeluTwiceConsts {
  uint32_t k0, k01;
  __device__ GeluTwiceConsts()
      : k0(pack_bf16(0.7978845608028654f, 0.7978845608028654f)),
        k01(pack_bf16(0.7978845608028654f * 0.044715f, 0.7978845608028654f * 0.044715f)) {}
  // two accumulator values + their biases (one packed FP32 addition)
  __device__ uint32_t operator()(float2 acc, float2 bias) const {
    return gelu2x2_bf16(__fadd2_rn(acc, bias), k0, k01);
  }
};

// ---------------------------------------------------------------------------
// Fused inference on the warp-level mma.sync path (cross-check of the
// tcgen05 kernel in clsph_mlp_tc.cuh)

constexpr int kInferWarps = 8;
constexpr int kW1Stride = kHid + 8;  // bf16 per smem row, 528 B: ldmatrix rows hit distinct banks
constexpr int kW2Stride = kHid + 8;
constexpr size_t kInferSmem =
    sizeof(bf16) * ((size_t)kIn * kW1Stride + (size_t)kHid * kW2Stride + (size_t)kHid * kOutPad) +
    sizeof(float) * (2 * kHid + kOutPad);

struct InferWeights {
  const bf16* w1;  // [32][256]
  const bf16* w2;  // [256][256]
  const bf16* w3;  // [256][8], columns 4..7 zero
  const float* b1;
  const float* b2;
  const float* b3;  // [4]
  const float* y_mu;
  const float* y_sigma;
};

// Per-row output hook: receives the de-standardised outputs of row `row`.
struct StoreRaw {
  float4* out;
  __device__ void operator()(uint32_t row, float4 y) const { out[row] = y; }
};

template <class Store>
__global__ void __launch_bounds__(kInferWarps * 32, 1)
    k_mlp_infer(const bf16* __restrict__ x, uint32_t rows, InferWeights w, Store store) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  bf16* s_w1 = reinterpret_cast<bf16*>(smem_raw);
  bf16* s_w2 = s_w1 + kIn * kW1Stride;
  bf16* s_w3 = s_w2 + kHid * kW2Stride;
  float* s_b1 = reinterpret_cast<float*>(s_w3 + kHid * kOutPad);
  float* s_b2 = s_b1 + kHid;
  float* s_b3 = s_b2 + kHid;  // b3 padded to 8

  // stage the weights (16-byte chunks)
  for (int c = threadIdx.x; c < kIn * kHid / 8; c += blockDim.x) {
    const int r = c / (kHid / 8), q = c % (kHid / 8);
    *reinterpret_cast<uint4*>(s_w1 + r * kW1Stride + q * 8) =
        reinterpret_cast<const uint4*>(w.w1)[c];
  }
  for (int c = threadIdx.x; c < kHid * kHid / 8; c += blockDim.x) {
    const int r = c / (kHid / 8), q = c % (kHid / 8);
    *reinterpret_cast<uint4*>(s_w2 + r * kW2Stride + q * 8) =
        reinterpret_cast<const uint4*>(w.w2)[c];
  }
  for (int c = threadIdx.x; c < kHid * kOutPad / 8; c += blockDim.x)
    reinterpret_cast<uint4*>(s_w3)[c] = reinterpret_cast<const uint4*>(w.w3)[c];
  for (int c = threadIdx.x; c < kHid; c += blockDim.x) {
    s_b1[c] = w.b1[c];
    s_b2[c] = w.b2[c];
  }
  if (threadIdx.x < kOutPad) s_b3[threadIdx.x] = threadIdx.x < kOut ? w.b3[threadIdx.x] : 0.f;
  __syncthreads();

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, tig = lane & 3;
  const int lr = lane & 7, lj = lane >> 3;  // ldmatrix row and matrix index of this lane
  float ymu[kOut], ysig[kOut];
#pragma unroll
  for (int k = 0; k < kOut; ++k) {
    ymu[k] = w.y_mu[k];
    ysig[k] = w.y_sigma[k];
  }
  const uint32_t w1_base = smem_addr(s_w1), w2_base = smem_addr(s_w2), w3_base = smem_addr(s_w3);
  const GeluConsts gelu;
  const uint32_t tiles = (rows + 15) / 16;
  for (uint32_t tile = blockIdx.x * kInferWarps + warp; tile < tiles; tile += gridDim.x * kInferWarps) {
    const uint32_t rb = tile * 16;
    const uint32_t r0 = rb + g, r1 = rb + g + 8;
    // layer-1 A fragments straight from the feature rows (64 B each)
    uint32_t xa[2][4];
    {
      const uint32_t* x0 = reinterpret_cast<const uint32_t*>(x + (size_t)r0 * kIn);
      const uint32_t* x1 = reinterpret_cast<const uint32_t*>(x + (size_t)r1 * kIn);
#pragma unroll
      for (int ks = 0; ks < 2; ++ks) {
        xa[ks][0] = r0 < rows ? x0[ks * 8 + tig] : 0u;
        xa[ks][1] = r1 < rows ? x1[ks * 8 + tig] : 0u;
        xa[ks][2] = r0 < rows ? x0[ks * 8 + 4 + tig] : 0u;
        xa[ks][3] = r1 < rows ? x1[ks * 8 + 4 + tig] : 0u;
      }
    }
    // layer 1 -> GELU -> A fragments of layer 2 (16 k-steps of 16 columns)
    uint32_t ha[16][4];
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      float acc[2][4] = {};
#pragma unroll
      for (int ks = 0; ks < 2; ++ks) {
        uint32_t b[4];
        // rows k = ks*16 + lr + (lj&1)*8, columns c*16 + (lj>>1)*8
        ldsm_x4_t(b, w1_base + 2u * ((ks * 16 + lr + (lj & 1) * 8) * kW1Stride + c * 16 + (lj >> 1) * 8));
        mma16816(acc[0], xa[ks], b[0], b[1]);
        mma16816(acc[1], xa[ks], b[2], b[3]);
      }
#pragma unroll
      for (int t = 0; t < 2; ++t) {
        const int col = c * 16 + t * 8 + tig * 2;
        const float bb0 = s_b1[col], bb1 = s_b1[col + 1];
        ha[c][2 * t + 0] = gelu(acc[t][0] + bb0, acc[t][1] + bb1);
        ha[c][2 * t + 1] = gelu(acc[t][2] + bb0, acc[t][3] + bb1);
      }
    }
    // layers 2 and 3, 64 hidden columns at a time
    float o[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 1
    for (int q = 0; q < 4; ++q) {
      float acc[8][4] = {};
#pragma unroll
      for (int ks = 0; ks < 16; ++ks) {
#pragma unroll
        for (int np = 0; np < 4; ++np) {
          uint32_t b[4];
          ldsm_x4_t(b, w2_base + 2u * ((ks * 16 + lr + (lj & 1) * 8) * kW2Stride + q * 64 + np * 16 +
                                       (lj >> 1) * 8));
          mma16816(acc[2 * np], ha[ks], b[0], b[1]);
          mma16816(acc[2 * np + 1], ha[ks], b[2], b[3]);
        }
      }
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        uint32_t h2[4];
#pragma unroll
        for (int t = 0; t < 2; ++t) {
          const int nt = 2 * kk + t;
          const int col = q * 64 + nt * 8 + tig * 2;
          const float bb0 = s_b2[col], bb1 = s_b2[col + 1];
          h2[2 * t + 0] = gelu(acc[nt][0] + bb0, acc[nt][1] + bb1);
          h2[2 * t + 1] = gelu(acc[nt][2] + bb0, acc[nt][3] + bb1);
        }
        uint32_t b0, b1;
        // W3 rows k = q*64 + kk*16 + lr + (lj&1)*8 (lanes 16..31 repeat lanes 0..15)
        ldsm_x2_t(b0, b1, w3_base + 2u * ((q * 64 + kk * 16 + lr + (lj & 1) * 8) * kOutPad));
        mma16816(o, h2, b0, b1);
      }
    }
    // o[0..1]: row g, columns 2*tig, 2*tig+1; o[2..3]: row g+8. Columns 0..3
    // live in lanes with tig 0 and 1; lane tig=0 collects its row's four.
    const float c2 = __shfl_down_sync(0xffffffffu, o[0], 1);
    const float c3 = __shfl_down_sync(0xffffffffu, o[1], 1);
    const float d2 = __shfl_down_sync(0xffffffffu, o[2], 1);
    const float d3 = __shfl_down_sync(0xffffffffu, o[3], 1);
    if (tig == 0) {
      float4 y0 = make_float4((o[0] + s_b3[0]) * ysig[0] + ymu[0], (o[1] + s_b3[1]) * ysig[1] + ymu[1],
                              (c2 + s_b3[2]) * ysig[2] + ymu[2], (c3 + s_b3[3]) * ysig[3] + ymu[3]);
      float4 y1 = make_float4((o[2] + s_b3[0]) * ysig[0] + ymu[0], (o[3] + s_b3[1]) * ysig[1] + ymu[1],
                              (d2 + s_b3[2]) * ysig[2] + ymu[2], (d3 + s_b3[3]) * ysig[3] + ymu[3]);
      if (r0 < rows) store(r0, y0);
      if (r1 < rows) store(r1, y1);
    }
  }
}

// ---------------------------------------------------------------------------
// Tiled GEMM for training: C[M][N] = sum_k A[m][k] * B[k][n].
// A_K: A stored [M][K] (lda = row stride), else stored [K][M].
// B_K: B stored [N][K], else stored [K][N].
// Epilogue functors of the training GEMM (k_gemm_tc in clsph_mlp_tc.cuh),
// called on every (row, even column) pair of the product.

// z = acc + bias; Z (fp32) and H = GELU(z) (bf16), both [M][ld]
struct EpiHidden {
  const float* bias;
  float* z;
  bf16* h;
  int ld;
  __device__ void operator()(int row, int col, float v0, float v1) const {
    const float z0 = v0 + bias[col], z1 = v1 + bias[col + 1];
    const size_t o = (size_t)row * ld + col;
    *reinterpret_cast<float2*>(z + o) = make_float2(z0, z1);
    *reinterpret_cast<uint32_t*>(h + o) = GeluConsts()(z0, z1);
  }
};

// dZ = acc * GELU'(Z), stored bf16 [M][ld]
struct EpiGeluGrad {
  const float* z;
  bf16* dz;
  int ld;
  __device__ void operator()(int row, int col, float v0, float v1) const {
    const size_t o = (size_t)row * ld + col;
    const float2 zz = *reinterpret_cast<const float2*>(z + o);
    *reinterpret_cast<uint32_t*>(dz + o) = pack_bf16(v0 * gelu_grad(zz.x), v1 * gelu_grad(zz.y));
  }
};

// split-K partial sums, ws[blockIdx.z][M][ld]
struct EpiPartial {
  float* ws;
  int ld;
  size_t split_stride;
  __device__ void operator()(int row, int col, float v0, float v1) const {
    *reinterpret_cast<float2*>(ws + blockIdx.z * split_stride + (size_t)row * ld + col) =
        make_float2(v0, v1);
  }
};

// split-K partial sums of a transposed product: the GEMM computes C^T, so
// element (row, col) of it is C's (col, row), ws[blockIdx.z][col][ld]
struct EpiPartialT {
  float* ws;
  int ld;
  size_t split_stride;
  __device__ void operator()(int row, int col, float v0, float v1) const {
    float* w = ws + blockIdx.z * split_stride + row;
    w[(size_t)col * ld] = v0;
    w[(size_t)(col + 1) * ld] = v1;
  }
};

// ---------------------------------------------------------------------------
// Training: elementwise and reduction kernels

// Batch rows from the sample set: x standardised to bf16, y standardised fp32.
__global__ void k_gather_batch(const float* __restrict__ x_raw, const float* __restrict__ y_raw,
                               const uint32_t* __restrict__ idx, uint32_t rows,
                               const float* __restrict__ norm /* blob + kOffXMu */,
                               bf16* __restrict__ xb, float* __restrict__ yb) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t r = t / (kIn + kOut), c = t % (kIn + kOut);
  if (r >= rows) return;
  const size_t s = idx[r];
  if (c < kIn) {
    const float v = standardise(x_raw[s * kIn + c], norm[c], norm[kIn + c]);
    xb[(size_t)r * kIn + c] = __float2bfloat16_rn(v);
  } else {
    const int k = c - kIn;
    yb[(size_t)r * kOut + k] = (y_raw[s * kOut + k] - norm[2 * kIn + k]) / norm[2 * kIn + kOut + k];
  }
}

// raw feature rows -> standardised BF16 rows
__global__ void k_standardize(const float* __restrict__ x_raw, uint32_t rows, const float* __restrict__ norm,
                              bf16* __restrict__ xb) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)rows * kIn) return;
  const int c = (int)(i % kIn);
  xb[i] = __float2bfloat16_rn(standardise(x_raw[i], norm[c], norm[kIn + c]));
}

// Layer 3 forward + loss + backward to dZ2, one block of 256 threads (one per
// hidden unit) walking `rows_per_block` rows:
//   y = H2 W3 + b3, loss = mean over rows of sum_k (y_k - t_k)^2,
//   dY = 2 (y - t) / rows, dZ2 = (dY W3^T) * GELU'(Z2),
//   dW3 += H2^T dY, db3 += sum dY, loss_sum += sum of squared errors.
__global__ void __launch_bounds__(kHid)
    k_head(const bf16* __restrict__ h2, const float* __restrict__ z2, const float* __restrict__ w3,
           const float* __restrict__ b3, const float* __restrict__ yt, uint32_t rows,
           uint32_t rows_per_block, float inv_rows, bf16* __restrict__ dz2, float* __restrict__ dw3,
           float* __restrict__ db3, float* __restrict__ loss_sum, float* __restrict__ y_out) {
  __shared__ float red[kHid / 32][kOut];
  __shared__ float dy_s[kOut];
  const int k = threadIdx.x, lane = k & 31, warp = k >> 5;
  float w[kOut];  // BF16 values, as the inference kernels use them
#pragma unroll
  for (int j = 0; j < kOut; ++j) w[j] = __bfloat162float(__float2bfloat16_rn(w3[k * kOut + j]));
  float gw[kOut] = {}, gb[kOut] = {}, lsum = 0.f;
  const uint32_t r_begin = blockIdx.x * rows_per_block;
  const uint32_t r_end = min(rows, r_begin + rows_per_block);
  for (uint32_t r = r_begin; r < r_end; ++r) {
    const size_t o = (size_t)r * kHid + k;
    const float hv = __bfloat162float(h2[o]);
    float p[kOut];
#pragma unroll
    for (int j = 0; j < kOut; ++j) {
      p[j] = hv * w[j];
#pragma unroll
      for (int s = 16; s > 0; s >>= 1) p[j] += __shfl_xor_sync(0xffffffffu, p[j], s);
    }
    if (lane == 0)
#pragma unroll
      for (int j = 0; j < kOut; ++j) red[warp][j] = p[j];
    __syncthreads();
    if (k < kOut) {
      float y = b3[k];
      for (int q = 0; q < kHid / 32; ++q) y += red[q][k];
      const float e = y - yt[(size_t)r * kOut + k];
      dy_s[k] = 2.f * e * inv_rows;
      if (y_out) y_out[(size_t)r * kOut + k] = y;
      lsum += e * e;
    }
    __syncthreads();
    float dh = 0.f;
#pragma unroll
    for (int j = 0; j < kOut; ++j) {
      const float d = dy_s[j];
      dh += d * w[j];
      gw[j] += hv * d;
      gb[j] += d;
    }
    dz2[o] = __float2bfloat16_rn(dh * gelu_grad(z2[o]));
    __syncthreads();
  }
#pragma unroll
  for (int j = 0; j < kOut; ++j) atomicAdd(&dw3[k * kOut + j], gw[j]);
  if (k < kOut) {
    atomicAdd(&db3[k], gb[k]);
    atomicAdd(loss_sum, lsum);
  }
}

// db[c] += sum over rows of dz[r][c] (bf16 [rows][cols])
__global__ void k_colsum(const bf16* __restrict__ dz, uint32_t rows, int cols, uint32_t rows_per_block,
                         float* __restrict__ db) {
  const int c = threadIdx.x;
  if (c >= cols) return;
  const uint32_t r_begin = blockIdx.x * rows_per_block;
  const uint32_t r_end = min(rows, r_begin + rows_per_block);
  float s = 0.f;
  for (uint32_t r = r_begin; r < r_end; ++r) s += __bfloat162float(dz[(size_t)r * cols + c]);
  atomicAdd(&db[c], s);
}

// out[i] = sum over splits of ws[s][i]
__global__ void k_reduce_splits(const float* __restrict__ ws, int splits, size_t count,
                                float* __restrict__ out) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  float s = 0.f;
  for (int z = 0; z < splits; ++z) s += ws[(size_t)z * count + i];
  out[i] = s;
}

// BF16 copies of the weights used by the kernels: W1, W2 as stored
// ([in][out], training GEMMs and the mma.sync path), W1t, W2t transposed
// ([out][in], tcgen05 operands), W3 padded to 8 columns.
// BF16 copies of the weights: w1..w3 for the mma.sync kernels and training,
// w1t..w3t transposed for the tcgen05 kernel, whose w2t and w3t hold half the
// weights (its activations are twice GELU, gelu2x2_bf16).
struct Bf16Weights {
  bf16* w1;
  bf16* w2;
  bf16* w3;
  bf16* w1t;
  bf16* w2t;
  bf16* w3t;  // [16][256], rows 4..15 zero
  __device__ void put(int i, float v) const {
    const bf16 b = __float2bfloat16_rn(v);
    const bf16 half = __float2bfloat16_rn(0.5f * v);  // = b / 2 exactly for |v| >= 2^-125
    if (i < kOffB1) {
      w1[i] = b;
      w1t[(i % kHid) * kIn + i / kHid] = b;
    } else if (i >= kOffW2 && i < kOffB2) {
      const int j = i - kOffW2;
      w2[j] = b;
      w2t[(j % kHid) * kHid + j / kHid] = half;
    } else if (i >= kOffW3 && i < kOffB3) {
      const int j = i - kOffW3;
      w3[(j / kOut) * kOutPad + j % kOut] = b;
      w3t[(j % kOut) * kHid + j / kOut] = half;
    }
  }
};

// Adam on the fp32 parameters; refreshes the bf16 copies.
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ grad, float* __restrict__ m,
                       float* __restrict__ v, int count, float lr, float beta1, float beta2, float eps,
                       float bc1, float bc2, Bf16Weights wb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float gr = grad[i];
  const float mi = beta1 * m[i] + (1.f - beta1) * gr;
  const float vi = beta2 * v[i] + (1.f - beta2) * gr * gr;
  m[i] = mi;
  v[i] = vi;
  const float pi = p[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  p[i] = pi;
  wb.put(i, pi);
}

// bf16 copies of the weights from the fp32 blob (padding columns of W3 zero)
__global__ void k_refresh_bf16(const float* __restrict__ p, Bf16Weights wb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < kParams) wb.put(i, p[i]);
  if (i < kHid * kOutPad && i % kOutPad >= kOut) wb.w3[i] = __float2bfloat16_rn(0.f);
  if (i >= kOut * kHid && i < 16 * kHid) wb.w3t[i] = __float2bfloat16_rn(0.f);
}

// Standardisation statistics of the sample set: sums of x, x^2 (cols
// 0..35 = 32 inputs then 4 targets) in double.
__global__ void k_moments(const float* __restrict__ x_raw, const float* __restrict__ y_raw,
                          uint64_t samples, uint64_t per_block, double* __restrict__ sums) {
  const int c = threadIdx.x;
  if (c >= kIn + kOut) return;
  const uint64_t b = blockIdx.x * per_block;
  const uint64_t e = b + per_block < samples ? b + per_block : samples;
  double s = 0.0, s2 = 0.0;
  for (uint64_t r = b; r < e; ++r) {
    const float v = c < kIn ? x_raw[r * kIn + c] : y_raw[r * kOut + (c - kIn)];
    s += v;
    s2 += (double)v * v;
  }
  atomicAdd(&sums[c], s);
  atomicAdd(&sums[kIn + kOut + c], s2);
}

}  // namespace clsph_nn
