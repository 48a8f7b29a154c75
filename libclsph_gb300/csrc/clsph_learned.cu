// Learned 4x-dt stepper, sample collector and MLP training
// (include/clsph_learned.h). No counterpart in the reference.
//
// The learned step reuses the plain substep's neighbour build, density and
// force kernels on the handle's buffers, then runs
//   k_forces<.., FeatureHook>  the plain forces kernel that also gathers 32
//                   neighbour features per particle (sorted slot order),
//                   standardised to BF16 rows
//   k_mlp_tc        fused BF16 MLP on the tcgen05 tensor cores -> the
//                   network's de-standardised outputs
//   k_advect<true>  outputs -> acceleration correction and predicted density,
//                   then one leapfrog + collision pass over dt_mult time steps
// and, at the next step, k_gate compares the density reached with the
// prediction to accept the step or roll it back.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <string>
#include <vector>

#include "clsph_handle.cuh"
#include "clsph_learned.h"
#include "clsph_mlp.cuh"
#include "clsph_mlp_tc.cuh"

using namespace clsph_host;
using clsph_nn::bf16;
using clsph_nn::kBlob;
using clsph_nn::kHid;
using clsph_nn::kIn;
using clsph_nn::kOut;
using clsph_nn::kOutPad;
using clsph_nn::kParams;

namespace {

constexpr int kFeat = 32;
static_assert(kFeat == kIn, "feature count");
constexpr int kRing = 36;           // floats per tracked particle and level: features + naive v
constexpr uint32_t kRowBlock = 2048;  // training rows come in multiples of this
constexpr uint32_t kSplitK = 1024;    // batch rows per split of the weight-gradient GEMMs

// ---------------------------------------------------------------------------
// Features, gathered by k_forces in its neighbour walk (FeatureHook)

enum FeatureMode { kFeatStd = 0, kFeatRaw = 1, kFeatRing = 2 };

struct FeatureHook {
  State st;  // sorted state of the current substep
  const float4* aux;
  const Consts* consts;
  const uint16_t* scene_of;
  int mode;
  const float* norm;  // x_mu[32], x_sigma[32] (kFeatStd)
  bf16* xstd;         // [n][32] (kFeatStd)
  float* raw;         // [n][32] (kFeatRaw) or a ring level [m][kRing] (kFeatRing)
  const uint32_t* ids;
  uint32_t stride, m;

  struct Acc {
    float inv_h, vs;
    float s[22];  // sum w d (3), w d d^T (6), w u (3), w u u^T (6), w d.u, w d x u (3)
    uint32_t cnt;
  };

  __device__ __forceinline__ Acc begin(uint32_t i) const {
    Acc a;
    const Consts& c = consts[scene_of[i]];
    a.inv_h = 1.f / c.h;
    a.vs = c.time_delta * c.scale * a.inv_h;
#pragma unroll
    for (int k = 0; k < 22; ++k) a.s[k] = 0.f;
    a.cnt = 0;
    return a;
  }

  // d = p_i - p_j and dv = v_j - v_i: the force evaluation's own exact
  // differences (p_j - p_i is exactly -d)
  __device__ __forceinline__ void pair(Acc& a, uint32_t i, uint32_t j, const V3& d, const V3& dv) const {
    ++a.cnt;
    if (j == i) return;
    const float dx = -d.x * a.inv_h, dy = -d.y * a.inv_h, dz = -d.z * a.inv_h;
    const float ux = dv.x * a.vs, uy = dv.y * a.vs, uz = dv.z * a.vs;
    const float w = fmaxf(0.f, 1.f - (dx * dx + dy * dy + dz * dz));
    a.s[0] += w * dx;
    a.s[1] += w * dy;
    a.s[2] += w * dz;
    a.s[3] += w * dx * dx;
    a.s[4] += w * dy * dy;
    a.s[5] += w * dz * dz;
    a.s[6] += w * dx * dy;
    a.s[7] += w * dx * dz;
    a.s[8] += w * dy * dz;
    a.s[9] += w * ux;
    a.s[10] += w * uy;
    a.s[11] += w * uz;
    a.s[12] += w * ux * ux;
    a.s[13] += w * uy * uy;
    a.s[14] += w * uz * uz;
    a.s[15] += w * ux * uy;
    a.s[16] += w * ux * uz;
    a.s[17] += w * uy * uz;
    a.s[18] += w * (dx * ux + dy * uy + dz * uz);
    a.s[19] += w * (dy * uz - dz * uy);
    a.s[20] += w * (dz * ux - dx * uz);
    a.s[21] += w * (dx * uy - dy * ux);
  }

  __device__ __forceinline__ void end(Acc& a, uint32_t i, const float4& acc) const {
    uint32_t q = 0;
    if (mode == kFeatRing) {
      const uint32_t id = ids[i];
      if (id % stride) return;
      q = id / stride;
      if (q >= m) return;
    }
    const Consts& c = consts[scene_of[i]];
    const float4 ax = aux[i];
    const float dt = c.time_delta * c.scale;
    const float as = dt * dt * a.inv_h;
    float f[kFeat];
    f[0] = ax.x / c.rho0 - 1.f;
    f[1] = c.K != 0.f ? ax.y / c.K : ax.y;
    f[2] = (float)a.cnt * (1.f / 32.f);
    f[3] = acc.x * as;
    f[4] = acc.y * as;
    f[5] = acc.z * as;
    const float4 vh = st.ivel[i];  // the intermediate velocity the step integrates
    f[6] = vh.x * a.vs;
    f[7] = vh.y * a.vs;
    f[8] = vh.z * a.vs;
    f[9] = c.vmax > 0.f ? sqrtf(vh.x * vh.x + vh.y * vh.y + vh.z * vh.z) / c.vmax : 0.f;
#pragma unroll
    for (int k = 0; k < 22; ++k) f[10 + k] = a.s[k];
    if (mode == kFeatStd) {
      uint4* row = reinterpret_cast<uint4*>(xstd + (size_t)i * kFeat);
#pragma unroll
      for (int qq = 0; qq < kFeat / 8; ++qq) {
        uint32_t w[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int k = qq * 8 + 2 * e;
          w[e] = clsph_nn::pack_bf16(clsph_nn::standardise(f[k], norm[k], norm[kFeat + k]),
                                      clsph_nn::standardise(f[k + 1], norm[k + 1], norm[kFeat + k + 1]));
        }
        row[qq] = make_uint4(w[0], w[1], w[2], w[3]);
      }
    } else {
      float* out = mode == kFeatRaw ? raw + (size_t)i * kFeat : raw + (size_t)q * kRing;
#pragma unroll
      for (int k = 0; k < kFeat; ++k) out[k] = f[k];
    }
  }
};

// the naive dt_mult step's velocity (units h/dt) of the tracked particles
__global__ void __launch_bounds__(kBlock)
    k_ring_naive(uint32_t n, const uint32_t* __restrict__ ids, uint32_t stride, uint32_t m,
                 const float4* __restrict__ naive_ivel, const Consts* __restrict__ consts,
                 const uint16_t* __restrict__ scene_of, float* __restrict__ level) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t id = ids[i];
  if (id % stride) return;
  const uint32_t q = id / stride;
  if (q >= m) return;
  const Consts& c = consts[scene_of[i]];
  const float vs = c.time_delta * c.scale / c.h;
  const float4 v = naive_ivel[i];
  float* out = level + (size_t)q * kRing;
  out[32] = v.x * vs;
  out[33] = v.y * vs;
  out[34] = v.z * vs;
  out[35] = 0.f;
}

// samples from two ring levels dt_mult substeps apart
__global__ void k_sample(const float* __restrict__ old_level, const float* __restrict__ now_level,
                         uint32_t m, float inv_mult, float* __restrict__ xs, float* __restrict__ ys,
                         uint64_t base, uint64_t capacity) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= m) return;
  const uint64_t s = base + q;
  if (s >= capacity) return;
  const float* o = old_level + (size_t)q * kRing;
  const float* w = now_level + (size_t)q * kRing;
  for (int k = 0; k < kFeat; ++k) xs[s * kFeat + k] = o[k];
  ys[s * kOut + 0] = (w[6] - o[32]) * inv_mult;
  ys[s * kOut + 1] = (w[7] - o[33]) * inv_mult;
  ys[s * kOut + 2] = (w[8] - o[34]) * inv_mult;
  ys[s * kOut + 3] = (w[0] + 1.f) / (o[0] + 1.f) - 1.f;
}

// Density statistics of the state just evaluated against the densities the
// network predicted for it (vel.w): sums over particles of
//   [0] |rho/rho0 - 1|   [1] |rho_pred/rho0 - 1|   [2] rho/rho0   [3] rho_pred/rho0
//   [4] |rho - rho_pred| / rho0
constexpr int kGateSums = 5;
__global__ void __launch_bounds__(kBlock)
    k_gate(uint32_t n, const float4* __restrict__ aux, const float4* __restrict__ vel,
           const Consts* __restrict__ consts, const uint16_t* __restrict__ scene_of,
           float* __restrict__ sums) {
  __shared__ float red[kGateSums][kBlock / 32];
  float s[kGateSums] = {0.f, 0.f, 0.f, 0.f, 0.f};
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float inv = 1.f / consts[scene_of[i]].rho0;
    const float r = aux[i].x * inv, rp = vel[i].w * inv;
    s[0] += fabsf(r - 1.f);
    s[1] += fabsf(rp - 1.f);
    s[2] += r;
    s[3] += rp;
    s[4] += fabsf(r - rp);
  }
#pragma unroll
  for (int k = 0; k < kGateSums; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s[k] += __shfl_xor_sync(0xffffffffu, s[k], o);
    if ((threadIdx.x & 31) == 0) red[k][threadIdx.x >> 5] = s[k];
  }
  __syncthreads();
  if (threadIdx.x < kGateSums) {
    float t = 0.f;
    for (int w = 0; w < kBlock / 32; ++w) t += red[threadIdx.x][w];
    atomicAdd(&sums[threadIdx.x], t);
  }
}

// The learned step's MLP stores its de-standardised outputs as they are
// (clsph_nn::StoreRaw); k_advect<true> turns them into the acceleration
// correction and the predicted density (learned_correction), where the loads
// it needs for that are hidden by many resident warps.

template <class Store>
int launch_infer(cudaStream_t stream, uint32_t sms, const bf16* x, uint32_t rows,
                 const clsph_nn::InferWeights& w, Store store, clsph_gpu* h, int cls) {
  // set on every launch: the attribute belongs to the current device
  cudaError_t e = cudaFuncSetAttribute(clsph_nn::k_mlp_infer<Store>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)clsph_nn::kInferSmem);
  if (e != cudaSuccess)
    return fail(CLSPH_ERR_CUDA, std::string("mlp: shared memory attribute: ") + cudaGetErrorString(e));
  const uint32_t tiles = (rows + 15) / 16;
  uint32_t blocks = (tiles + clsph_nn::kInferWarps - 1) / clsph_nn::kInferWarps;
  blocks = std::max(1u, std::min(blocks, sms));
  if (h)
    h->launch_smem(cls, clsph_nn::k_mlp_infer<Store>, dim3(blocks), dim3(clsph_nn::kInferWarps * 32),
                   clsph_nn::kInferSmem, x, rows, w, store);
  else
    clsph_nn::k_mlp_infer<Store><<<blocks, clsph_nn::kInferWarps * 32, clsph_nn::kInferSmem, stream>>>(
        x, rows, w, store);
  return 0;
}

static_assert(clsph_nn::kTcWaitLimit == CLSPH_DEFAULT_MLP_WAIT_POLLS, "default MLP wait bound");

// tcgen05 inference; *err collects wait timeouts (see k_mlp_tc)
template <class Store>
int launch_tc(cudaStream_t stream, uint32_t sms, const bf16* x, uint32_t rows, const clsph_nn::TcWeights& w,
              Store store, uint32_t* err, clsph_gpu* h, int cls) {
  const uint32_t wait_limit = h ? h->mlp_wait_limit : clsph_nn::kTcWaitLimit;
  cudaError_t e = cudaFuncSetAttribute(clsph_nn::k_mlp_tc<Store>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)clsph_nn::kTcSmem);
  if (e != cudaSuccess)
    return fail(CLSPH_ERR_CUDA, std::string("mlp: shared memory attribute: ") + cudaGetErrorString(e));
  const uint32_t tiles = (rows + clsph_nn::kTcRows - 1) / clsph_nn::kTcRows;
  const uint32_t blocks = std::max(1u, std::min(tiles, sms));
  if (h)
    h->launch_smem(cls, clsph_nn::k_mlp_tc<Store>, dim3(blocks), dim3(clsph_nn::kTcThreads), clsph_nn::kTcSmem,
                   x, rows, w, store, err, wait_limit);
  else
    clsph_nn::k_mlp_tc<Store><<<blocks, clsph_nn::kTcThreads, clsph_nn::kTcSmem, stream>>>(x, rows, w, store, err,
                                                                                          wait_limit);
  return 0;
}

// weight of the end-of-step velocity in the position update of one step over
// m time steps: sum_{k=1..m} v_k dt = m dt ((1 - w) v_0 + w v_m), w = (m + 1) / 2m,
// for constant acceleration
float position_weight(uint32_t m) { return (float)(m + 1) / (float)(2 * m); }

FeatureHook feature_hook(clsph_gpu* h, int mode) {
  FeatureHook f{};
  f.st = h->st[1];
  f.aux = h->aux;
  f.consts = h->consts;
  f.scene_of = h->scene_of;
  f.mode = mode;
  f.stride = 1;
  return f;
}

// the forces kernel of the current substep again (same accelerations), with
// the feature gathering
int launch_forces_hooked(clsph_gpu* h, const FeatureHook& hook) {
  const int b = h->forces_block;
  const dim3 grid((h->n + b - 1) / b);
  auto go = [&](auto kernel) {
    h->launch(K_FEATURES, kernel, grid, dim3(b), h->n, (const DevGrid*)h->grids,
              (const uint16_t*)h->scene_of, (const uint32_t*)h->ctl, (const uint32_t*)h->keys, h->st[1],
              (const float4*)h->aux, h->ci, (const Consts*)h->consts, (const uint16_t*)h->nlist,
              (const uint32_t*)h->ncount, h->nlist_cap, h->acc, hook, (const float4*)h->frec,
              (const uint32_t*)h->nb_start);
  };
  if (b == 64) go(k_forces<64, FeatureHook>);
  else if (b == 256) go(k_forces<256, FeatureHook>);
  else go(k_forces<128, FeatureHook>);
  return 0;
}

}  // namespace

// ---------------------------------------------------------------------------
// MLP handle

struct clsph_mlp {
  int device = 0;
  uint32_t sms = 152;
  cudaStream_t stream = nullptr;
  float* blob = nullptr;  // kBlob floats
  bf16* w1b = nullptr;    // [32][256]
  bf16* w2b = nullptr;    // [256][256]
  bf16* w3b = nullptr;    // [256][8]
  uint64_t serial = 0;    // unique per network made in this process (keys cached graphs)
  bf16* w1t = nullptr;    // [256][32]
  bf16* w2t = nullptr;    // [256][256]
  bf16* w3t = nullptr;    // [16][256]
  uint32_t* err = nullptr;  // tensor-core wait timeouts of clsph_mlp_forward
  // training state, made on first use
  uint32_t rows_cap = 0;
  float* grad = nullptr;
  float* adam_m = nullptr;
  float* adam_v = nullptr;
  uint64_t adam_t = 0;
  bf16 *xb = nullptr, *h1 = nullptr, *h2 = nullptr, *dz1 = nullptr, *dz2 = nullptr;
  float *yb = nullptr, *z1 = nullptr, *z2 = nullptr, *ws = nullptr, *loss = nullptr;
  uint32_t loss_cap = 0;
  uint32_t* idx = nullptr;
  uint64_t idx_cap = 0;
  double* moments = nullptr;

};

namespace {

clsph_nn::Bf16Weights bf16_weights(const clsph_mlp* m) {
  return clsph_nn::Bf16Weights{m->w1b, m->w2b, m->w3b, m->w1t, m->w2t, m->w3t};
}

clsph_nn::TcWeights tc_weights(const clsph_mlp* m) {
  return clsph_nn::TcWeights{m->w1t,
                             m->w2t,
                             m->w3t,
                             m->blob + clsph_nn::kOffB1,
                             m->blob + clsph_nn::kOffB2,
                             m->blob + clsph_nn::kOffB3,
                             m->blob + clsph_nn::kOffYMu,
                             m->blob + clsph_nn::kOffYSigma};
}

clsph_nn::InferWeights infer_weights(const clsph_mlp* m) {
  return clsph_nn::InferWeights{m->w1b,
                                 m->w2b,
                                 m->w3b,
                                 m->blob + clsph_nn::kOffB1,
                                 m->blob + clsph_nn::kOffB2,
                                 m->blob + clsph_nn::kOffB3,
                                 m->blob + clsph_nn::kOffYMu,
                                 m->blob + clsph_nn::kOffYSigma};
}

}  // namespace

namespace {

using clsph_nn::EpiGeluGrad;
using clsph_nn::EpiHidden;
using clsph_nn::EpiPartial;

// Training GEMMs on the tensor cores (clsph_nn::k_gemm_tc); timeouts of its
// bounded waits set bit kTrainWaitBit of the network's error word.
constexpr uint32_t kTrainWaitBit = 4u;

template <int BN, bool A_K, bool B_K, class Epi>
int gemm_tc(cudaStream_t s, uint32_t* err, const bf16* A, int lda, const bf16* B, int ldb, int M, int N, int K,
            int k_split, Epi epi) {
  using L = clsph_nn::GemmTcLayout<BN>;
  (void)sizeof(L);
  if (N != BN || M % clsph_nn::kGtRows || k_split <= 0 || K % k_split || k_split % clsph_nn::kGtBK ||
      lda % 8 || ldb % 8)
    return fail(CLSPH_ERR_ARGUMENT, "mlp: GEMM shape not tileable");
  auto kernel = clsph_nn::k_gemm_tc<BN, A_K, B_K, Epi>;
  // set on every launch: the attribute belongs to the current device
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)clsph_nn::kGtSmem);
  if (e != cudaSuccess) return fail(CLSPH_ERR_CUDA, std::string("mlp: GEMM shared memory: ") + cudaGetErrorString(e));
  dim3 grid(1, M / clsph_nn::kGtRows, K / k_split);
  kernel<<<grid, clsph_nn::kGtThreads, clsph_nn::kGtSmem, s>>>(A, lda, B, ldb, K, k_split, epi, err);
  return 0;
}

// the training GEMMs' wait timeouts since the last check
int check_train_waits(clsph_mlp* m) {
  uint32_t e = 0;
  CUDA_TRY(cudaStreamSynchronize(m->stream));
  CUDA_TRY(cudaMemcpy(&e, m->err, sizeof(e), cudaMemcpyDeviceToHost));
  if (e & kTrainWaitBit) {
    const uint32_t keep = e & ~kTrainWaitBit;
    CUDA_TRY(cudaMemcpy(m->err, &keep, sizeof(keep), cudaMemcpyHostToDevice));
    return fail(CLSPH_ERR_CUDA, "mlp: a tensor-core wait of a training GEMM timed out");
  }
  return 0;
}

template <class T>
int alloc(T** p, size_t count) {
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * (count ? count : 1));
  if (e != cudaSuccess) return fail(CLSPH_ERR_CUDA, std::string("mlp: cudaMalloc: ") + cudaGetErrorString(e));
  return 0;
}

int ensure_training(clsph_mlp* m, uint32_t rows) {
  if (!m->grad) {
    int rc;
    if ((rc = alloc(&m->grad, kParams)) || (rc = alloc(&m->adam_m, kParams)) ||
        (rc = alloc(&m->adam_v, kParams)) || (rc = alloc(&m->moments, 2 * (kIn + kOut))))
      return rc;
    CUDA_TRY(cudaMemset(m->adam_m, 0, sizeof(float) * kParams));
    CUDA_TRY(cudaMemset(m->adam_v, 0, sizeof(float) * kParams));
    m->adam_t = 0;
  }
  if (rows > m->rows_cap) {
    void* bufs[] = {m->xb, m->h1, m->h2, m->dz1, m->dz2, m->yb, m->z1, m->z2, m->ws};
    for (void* b : bufs) cudaFree(b);
    const size_t r = rows;
    int rc;
    if ((rc = alloc(&m->xb, r * kIn)) || (rc = alloc(&m->h1, r * kHid)) || (rc = alloc(&m->h2, r * kHid)) ||
        (rc = alloc(&m->dz1, r * kHid)) || (rc = alloc(&m->dz2, r * kHid)) || (rc = alloc(&m->yb, r * kOut)) ||
        (rc = alloc(&m->z1, r * kHid)) || (rc = alloc(&m->z2, r * kHid)) ||
        (rc = alloc(&m->ws, (r / kSplitK) * (size_t)kHid * kHid)))
      return rc;
    m->rows_cap = rows;
  }
  return 0;
}

int ensure_idx(clsph_mlp* m, uint64_t count) {
  if (count > m->idx_cap) {
    cudaFree(m->idx);
    m->idx = nullptr;
    int rc = alloc(&m->idx, count);
    if (rc) return rc;
    m->idx_cap = count;
  }
  return 0;
}

int ensure_loss(clsph_mlp* m, uint32_t count) {
  if (count > m->loss_cap) {
    cudaFree(m->loss);
    m->loss = nullptr;
    int rc = alloc(&m->loss, count);
    if (rc) return rc;
    m->loss_cap = count;
  }
  return 0;
}

// Forward + loss (into *loss_slot) and, when `backward`, gradients into
// m->grad for the `rows` rows already in m->xb / m->yb.
int pass(clsph_mlp* m, uint32_t rows, float* loss_slot, bool backward) {
  cudaStream_t s = m->stream;
  const float* p = m->blob;
  int rc;
  if (backward) CUDA_TRY(cudaMemsetAsync(m->grad, 0, sizeof(float) * kParams, s));
  uint32_t* err = m->err;
  // Z1 = X W1 + b1, H1 = GELU(Z1)
  if ((rc = gemm_tc<kHid, true, false>(s, err, m->xb, kIn, m->w1b, kHid, rows, kHid, kIn, kIn,
                                       EpiHidden{p + clsph_nn::kOffB1, m->z1, m->h1, kHid})))
    return rc;
  // Z2 = H1 W2 + b2, H2 = GELU(Z2)
  if ((rc = gemm_tc<kHid, true, false>(s, err, m->h1, kHid, m->w2b, kHid, rows, kHid, kHid, kHid,
                                       EpiHidden{p + clsph_nn::kOffB2, m->z2, m->h2, kHid})))
    return rc;
  // Y = H2 W3 + b3, loss, dZ2, dW3, db3
  clsph_nn::k_head<<<rows / 256, kHid, 0, s>>>(m->h2, m->z2, p + clsph_nn::kOffW3, p + clsph_nn::kOffB3, m->yb,
                                               rows, 256, 1.f / rows, m->dz2, m->grad + clsph_nn::kOffW3,
                                               m->grad + clsph_nn::kOffB3, loss_slot, nullptr);
  if (!backward) return 0;
  const int splits = rows / kSplitK;
  const size_t split_stride = (size_t)kHid * kHid;
  // dW2 = H1^T dZ2 (split over rows), db2 = column sums of dZ2
  if ((rc = gemm_tc<kHid, false, false>(s, err, m->h1, kHid, m->dz2, kHid, kHid, kHid, rows, kSplitK,
                                        EpiPartial{m->ws, kHid, split_stride})))
    return rc;
  clsph_nn::k_reduce_splits<<<(kHid * kHid + 255) / 256, 256, 0, s>>>(m->ws, splits, (size_t)kHid * kHid,
                                                                      m->grad + clsph_nn::kOffW2);
  clsph_nn::k_colsum<<<rows / 256, kHid, 0, s>>>(m->dz2, rows, kHid, 256, m->grad + clsph_nn::kOffB2);
  // dZ1 = (dZ2 W2^T) * GELU'(Z1)
  if ((rc = gemm_tc<kHid, true, true>(s, err, m->dz2, kHid, m->w2b, kHid, rows, kHid, kHid, kHid,
                                      EpiGeluGrad{m->z1, m->dz1, kHid})))
    return rc;
  // dW1 = X^T dZ1 as its transpose dZ1^T X (M = 256 hidden rows, N = 32
  // inputs, stored transposed), db1
  if ((rc = gemm_tc<kIn, false, false>(s, err, m->dz1, kHid, m->xb, kIn, kHid, kIn, rows, kSplitK,
                                       clsph_nn::EpiPartialT{m->ws, kHid, (size_t)kIn * kHid})))
    return rc;
  clsph_nn::k_reduce_splits<<<(kIn * kHid + 255) / 256, 256, 0, s>>>(m->ws, splits, (size_t)kIn * kHid,
                                                                    m->grad + clsph_nn::kOffW1);
  clsph_nn::k_colsum<<<rows / 256, kHid, 0, s>>>(m->dz1, rows, kHid, 256, m->grad + clsph_nn::kOffB1);
  return 0;
}

int refresh_bf16(clsph_mlp* m) {
  clsph_nn::k_refresh_bf16<<<(kParams + 255) / 256, 256, 0, m->stream>>>(m->blob, bf16_weights(m));
  static_assert(kParams > 16 * kHid, "refresh grid covers the W3 padding");
  CUDA_TRY(cudaGetLastError());
  return 0;
}

// Learned-step buffers of one engine handle.
struct Snapshot {
  float4 *pos = nullptr, *vel = nullptr, *ivel = nullptr;
  uint32_t* ids = nullptr;
  uint32_t* bbox = nullptr;
  int ids_sel = 0;
};

struct LearnedCache {
  bf16* x = nullptr;       // [n][32]
  float4* corr = nullptr;  // [n]
  Snapshot snap[2];
  float* dev_sum = nullptr;   // [0..4] gate sums, [5] tensor-core error word
  float* dev_host = nullptr;  // pinned copy
  cudaEvent_t ev = nullptr;
  // online calibration of the predicted density statistics against the plain
  // substeps run as fallback (exponential average of plain - predicted)
  const clsph_mlp* calibrated_for = nullptr;
  double bias_d = 0.0, bias_m = 0.0;
  bool calib_pending = false;        // a fallback interval awaits its plain statistics
  double rejected_d = 0.0, rejected_m = 0.0;  // predictions for that interval
  // unchecked learned steps replayed from a CUDA graph, one per buffer the
  // particle ids start in; rebuilt when the network, dt_mult, the collision
  // cap or the handle's launch shapes (graph_epoch) change
  cudaGraphExec_t nc_graph[2] = {};
  uint64_t nc_mlp[2] = {};
  uint32_t nc_mult[2] = {}, nc_max_iters[2] = {}, nc_epoch[2] = {};
  uint64_t nc_launches[2] = {};  // kernels in one replay
};

void free_cache(clsph_gpu* h) {
  auto* L = static_cast<LearnedCache*>(h->learned);
  if (!L) return;
  cudaFree(L->x);
  cudaFree(L->corr);
  for (auto& s : L->snap) {
    cudaFree(s.pos);
    cudaFree(s.vel);
    cudaFree(s.ivel);
    cudaFree(s.ids);
    cudaFree(s.bbox);
  }
  cudaFree(L->dev_sum);
  if (L->dev_host) cudaFreeHost(L->dev_host);
  if (L->ev) cudaEventDestroy(L->ev);
  for (auto& g : L->nc_graph)
    if (g) cudaGraphExecDestroy(g);
  delete L;
  h->learned = nullptr;
}

int ensure_cache(clsph_gpu* h, LearnedCache** out) {
  if (h->learned) {
    *out = static_cast<LearnedCache*>(h->learned);
    return 0;
  }
  auto* L = new LearnedCache();
  h->learned = L;
  h->free_learned = free_cache;
  // a failed allocation leaves no half-made cache behind
  auto bail = [&](int code) {
    free_cache(h);
    return code;
  };
  const size_t n = h->n;
  int rc;
  if ((rc = dev_alloc(&L->x, n * kFeat)) || (rc = dev_alloc(&L->corr, n)) ||
      (rc = dev_alloc(&L->dev_sum, kGateSums + 1)))
    return bail(rc);
  for (auto& s : L->snap)
    if ((rc = dev_alloc(&s.pos, n)) || (rc = dev_alloc(&s.vel, n)) || (rc = dev_alloc(&s.ivel, n)) ||
        (rc = dev_alloc(&s.ids, n)) || (rc = dev_alloc(&s.bbox, 6 * (size_t)h->nscenes)))
      return bail(rc);
  // the correction and feature rows start defined: a learned step whose MLP
  // stopped early (a wait ran out, reported as an error) reads them as they are
  if (cudaMemset(L->dev_sum, 0, (kGateSums + 1) * sizeof(float)) != cudaSuccess ||
      cudaMemset(L->corr, 0, sizeof(float4) * n) != cudaSuccess ||
      cudaMemset(L->x, 0, sizeof(bf16) * n * kFeat) != cudaSuccess ||
      cudaMallocHost(reinterpret_cast<void**>(&L->dev_host), (kGateSums + 1) * sizeof(float)) != cudaSuccess ||
      cudaEventCreateWithFlags(&L->ev, cudaEventDisableTiming) != cudaSuccess)
    return bail(fail(CLSPH_ERR_CUDA, "step_learned: buffer set-up"));
  *out = L;
  return 0;
}

int save(clsph_gpu* h, Snapshot& s) {
  const size_t b = sizeof(float4) * h->n;
  CUDA_TRY(cudaMemcpyAsync(s.pos, h->st[0].pos, b, cudaMemcpyDeviceToDevice, h->stream));
  CUDA_TRY(cudaMemcpyAsync(s.vel, h->st[0].vel, b, cudaMemcpyDeviceToDevice, h->stream));
  CUDA_TRY(cudaMemcpyAsync(s.ivel, h->st[0].ivel, b, cudaMemcpyDeviceToDevice, h->stream));
  CUDA_TRY(cudaMemcpyAsync(s.ids, h->ids[h->ids_sel], sizeof(uint32_t) * h->n, cudaMemcpyDeviceToDevice,
                           h->stream));
  CUDA_TRY(cudaMemcpyAsync(s.bbox, h->bbox, sizeof(uint32_t) * 6 * h->nscenes, cudaMemcpyDeviceToDevice,
                           h->stream));
  s.ids_sel = h->ids_sel;
  return 0;
}

int restore(clsph_gpu* h, const Snapshot& s) {
  const size_t b = sizeof(float4) * h->n;
  CUDA_TRY(cudaMemcpyAsync(h->st[0].pos, s.pos, b, cudaMemcpyDeviceToDevice, h->stream));
  CUDA_TRY(cudaMemcpyAsync(h->st[0].vel, s.vel, b, cudaMemcpyDeviceToDevice, h->stream));
  CUDA_TRY(cudaMemcpyAsync(h->st[0].ivel, s.ivel, b, cudaMemcpyDeviceToDevice, h->stream));
  CUDA_TRY(cudaMemcpyAsync(h->ids[s.ids_sel], s.ids, sizeof(uint32_t) * h->n, cudaMemcpyDeviceToDevice,
                           h->stream));
  CUDA_TRY(cudaMemcpyAsync(h->bbox, s.bbox, sizeof(uint32_t) * 6 * h->nscenes, cudaMemcpyDeviceToDevice,
                           h->stream));
  h->ids_sel = s.ids_sel;
  return 0;
}

// density check of the state just sorted and evaluated
int enqueue_gate(clsph_gpu* h, LearnedCache* L) {
  CUDA_TRY(cudaMemsetAsync(L->dev_sum, 0, kGateSums * sizeof(float), h->stream));
  h->launch(K_GATE, k_gate, dim3(grid_blocks(h->n, h->sm_count * 4)), dim3(kBlock), h->n,
            (const float4*)h->aux, (const float4*)h->st[1].vel, (const Consts*)h->consts,
            (const uint16_t*)h->scene_of, L->dev_sum);
  CUDA_TRY(cudaMemcpyAsync(L->dev_host, L->dev_sum, (kGateSums + 1) * sizeof(float), cudaMemcpyDeviceToHost,
                           h->stream));
  CUDA_TRY(cudaEventRecord(L->ev, h->stream));
  return 0;
}

// Density statistics read back by enqueue_gate: D = mean |rho/rho0 - 1| and
// M = mean rho/rho0 of the state just evaluated, D_pred and M_pred of the
// densities predicted for it, P = mean |rho - rho_pred| / rho0.
struct GateStats {
  double d, d_pred, m, m_pred, particle;
};

int wait_gate(clsph_gpu* h, LearnedCache* L, GateStats* g) {
  CUDA_TRY(cudaEventSynchronize(L->ev));
  uint32_t errw;
  std::memcpy(&errw, L->dev_host + kGateSums, sizeof(errw));
  if (errw) return fail(CLSPH_ERR_CUDA, "step_learned: a tensor-core wait of the MLP kernel timed out");
  const double inv = 1.0 / (double)h->n;
  g->d = L->dev_host[0] * inv;
  g->d_pred = L->dev_host[1] * inv;
  g->m = L->dev_host[2] * inv;
  g->m_pred = L->dev_host[3] * inv;
  g->particle = L->dev_host[4] * inv;
  return 0;
}

// The predicted density deviation of a learned step: how far the density
// statistics it reached lie from those predicted for the plain solver (after
// the calibration), max(|D - D_pred - b_D|, |M - M_pred - b_M|).
double predicted_deviation(const GateStats& g, const LearnedCache* L) {
  return std::max(std::fabs(g.d - g.d_pred - L->bias_d), std::fabs(g.m - g.m_pred - L->bias_m));
}

constexpr double kCalibrationWeight = 0.3;

// forces + features -> MLP -> one advection over dt_mult time steps
int enqueue_learned_tail(clsph_gpu* h, clsph_mlp* m, LearnedCache* L, uint32_t dt_mult) {
  const uint32_t n = h->n;
  FeatureHook fh = feature_hook(h, kFeatStd);
  fh.norm = m->blob + clsph_nn::kOffXMu;
  fh.xstd = L->x;
  int rc = launch_forces_hooked(h, fh);
  if (rc) return rc;
  rc = launch_tc(h->stream, h->sm_count, L->x, n, tc_weights(m), clsph_nn::StoreRaw{L->corr},
                 reinterpret_cast<uint32_t*>(L->dev_sum + kGateSums), h, K_MLP);
  if (rc) return rc;
  h->launch(K_LEARNED_ADVECT, k_advect<true>, dim3(grid_blocks(n, h->sm_count * h->advect_blocks_per_sm)),
            dim3(kBlock), n, h->st[1], (const float4*)h->acc, h->st[0], (const DevMesh*)h->meshes,
            (const Consts*)h->consts, (const uint16_t*)h->scene_of, h->max_iters, h->bbox, h->status,
            h->capped, (const float4*)L->corr, (float)dt_mult, position_weight(dt_mult),
            (const float4*)h->aux, (const float*)(m->blob + clsph_nn::kOffYMu));
  return 0;
}

int plain_substeps(clsph_gpu* h, uint32_t count) {
  for (uint32_t k = 0; k < count; ++k) {
    int rc = enqueue_substep(h, CLSPH_STAGE_ADVECT);
    if (rc) return rc;
    ++h->substeps;
  }
  return 0;
}

// An even number of unchecked learned steps (density pass + learned tail),
// captured once and replayed like the plain substeps' graphs. The particle
// ids alternate between their two buffers once per step, so an even count
// returns them to the buffer it started from; one graph per starting buffer.
constexpr uint32_t kLearnedGraphLen = 4;

int ensure_nocheck_graph(clsph_gpu* h, clsph_mlp* m, LearnedCache* L, uint32_t mult) {
  const int par = h->ids_sel;
  cudaGraphExec_t& ge = L->nc_graph[par];
  if (ge && L->nc_mlp[par] == m->serial && L->nc_mult[par] == mult && L->nc_max_iters[par] == h->max_iters &&
      L->nc_epoch[par] == h->graph_epoch)
    return 0;
  if (ge) cudaGraphExecDestroy(ge);
  ge = nullptr;
  cudaGraph_t graph = nullptr;
  CUDA_TRY(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  const uint64_t launches = h->launches;
  int rc = 0;
  for (uint32_t k = 0; k < kLearnedGraphLen && !rc; ++k) {
    rc = enqueue_substep(h, CLSPH_STAGE_DENSITY);
    if (!rc) rc = enqueue_learned_tail(h, m, L, mult);
  }
  L->nc_launches[par] = h->launches - launches;
  h->launches = launches;
  cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
  if (rc) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (e != cudaSuccess) return fail(CLSPH_ERR_CUDA, std::string("learned graph capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(&ge, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    ge = nullptr;
    return fail(CLSPH_ERR_CUDA, std::string("learned graph instantiate: ") + cudaGetErrorString(e));
  }
  if (h->ids_sel != par) return fail(CLSPH_ERR_STATE, "learned graph: particle ids did not return to their buffer");
  L->nc_mlp[par] = m->serial;
  L->nc_mult[par] = mult;
  L->nc_max_iters[par] = h->max_iters;
  L->nc_epoch[par] = h->graph_epoch;
  return 0;
}

}  // namespace

// ---------------------------------------------------------------------------
// Collector

struct clsph_collector {
  clsph_gpu* h = nullptr;
  uint32_t stride = 1, m = 0, dt_mult = 4;
  uint64_t capacity = 0, count = 0, t = 0;
  float* ring = nullptr;  // (dt_mult + 1) levels x m x kRing
  float* xs = nullptr;
  float* ys = nullptr;
  State scratch{};
  float4* zero = nullptr;
  uint32_t* sbbox = nullptr;
  uint32_t* sstatus = nullptr;
  unsigned long long* scapped = nullptr;
};

extern "C" {

uint64_t clsph_mlp_blob_size(void) { return kBlob; }

int clsph_mlp_destroy(clsph_mlp* m) {
  if (!m) return CLSPH_OK;
  if (m->stream) cudaStreamSynchronize(m->stream);
  void* bufs[] = {m->blob, m->w1b, m->w2b, m->w3b, m->w1t,  m->w2t,    m->w3t,    m->err,    m->grad,
                  m->adam_m, m->adam_v, m->xb, m->h1, m->h2, m->dz1, m->dz2, m->yb, m->z1, m->z2,
                  m->ws,   m->loss, m->idx, m->moments};
  for (void* b : bufs) cudaFree(b);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
  return CLSPH_OK;
}

int clsph_mlp_create(uint64_t seed, clsph_mlp** out) {
  if (!out) return fail(CLSPH_ERR_ARGUMENT, "mlp_create: null output");
  int devices = 0;
  if (cudaGetDeviceCount(&devices) != cudaSuccess || devices == 0)
    return fail(CLSPH_ERR_NO_DEVICE, "mlp_create: no CUDA device");
  auto* m = new clsph_mlp();
  static std::atomic<uint64_t> next_serial{1};
  m->serial = next_serial++;
  cudaGetDevice(&m->device);
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, m->device) == cudaSuccess && sms > 0)
    m->sms = (uint32_t)sms;
  auto bail = [&](int rc) {
    clsph_mlp_destroy(m);
    return rc;
  };
  if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(CLSPH_ERR_CUDA, "mlp_create: stream"));
  int rc;
  if ((rc = alloc(&m->blob, kBlob)) || (rc = alloc(&m->w1b, kIn * kHid)) || (rc = alloc(&m->w2b, kHid * kHid)) ||
      (rc = alloc(&m->w3b, kHid * kOutPad)) || (rc = alloc(&m->w1t, kIn * kHid)) ||
      (rc = alloc(&m->w2t, kHid * kHid)) || (rc = alloc(&m->w3t, 16 * kHid)) || (rc = alloc(&m->err, 1)))
    return bail(rc);
  if (cudaMemset(m->err, 0, sizeof(uint32_t)) != cudaSuccess) return bail(fail(CLSPH_ERR_CUDA, "mlp_create: memset"));
  std::vector<float> blob(kBlob, 0.f);
  std::mt19937_64 rng(seed);
  std::normal_distribution<float> nd(0.f, 1.f);
  const float s1 = std::sqrt(2.f / kIn), s2 = std::sqrt(2.f / kHid), s3 = 0.01f * std::sqrt(1.f / kHid);
  for (int i = 0; i < kIn * kHid; ++i) blob[clsph_nn::kOffW1 + i] = nd(rng) * s1;
  for (int i = 0; i < kHid * kHid; ++i) blob[clsph_nn::kOffW2 + i] = nd(rng) * s2;
  for (int i = 0; i < kHid * kOut; ++i) blob[clsph_nn::kOffW3 + i] = nd(rng) * s3;
  for (int i = 0; i < kIn; ++i) blob[clsph_nn::kOffXSigma + i] = 1.f;
  for (int i = 0; i < kOut; ++i) blob[clsph_nn::kOffYSigma + i] = 1.f;
  if (cudaMemcpy(m->blob, blob.data(), sizeof(float) * kBlob, cudaMemcpyHostToDevice) != cudaSuccess)
    return bail(fail(CLSPH_ERR_CUDA, "mlp_create: upload"));
  if ((rc = refresh_bf16(m)) || cudaStreamSynchronize(m->stream) != cudaSuccess)
    return bail(rc ? rc : fail(CLSPH_ERR_CUDA, "mlp_create: weight conversion"));
  *out = m;
  return CLSPH_OK;
}

int clsph_mlp_set_blob(clsph_mlp* m, const float* blob, uint64_t count) {
  if (!m || !blob || count != kBlob) return fail(CLSPH_ERR_ARGUMENT, "mlp_set_blob: bad argument");
  for (int i = 0; i < kIn; ++i)
    if (!(blob[clsph_nn::kOffXSigma + i] > 0.f)) return fail(CLSPH_ERR_ARGUMENT, "mlp_set_blob: x_sigma <= 0");
  CUDA_TRY(cudaStreamSynchronize(m->stream));
  CUDA_TRY(cudaMemcpy(m->blob, blob, sizeof(float) * kBlob, cudaMemcpyHostToDevice));
  int rc = refresh_bf16(m);
  if (rc) return rc;
  CUDA_TRY(cudaStreamSynchronize(m->stream));
  m->adam_t = 0;
  if (m->adam_m) {
    CUDA_TRY(cudaMemset(m->adam_m, 0, sizeof(float) * kParams));
    CUDA_TRY(cudaMemset(m->adam_v, 0, sizeof(float) * kParams));
  }
  return CLSPH_OK;
}

int clsph_mlp_get_blob(clsph_mlp* m, float* blob, uint64_t count) {
  if (!m || !blob || count != kBlob) return fail(CLSPH_ERR_ARGUMENT, "mlp_get_blob: bad argument");
  CUDA_TRY(cudaStreamSynchronize(m->stream));
  CUDA_TRY(cudaMemcpy(blob, m->blob, sizeof(float) * kBlob, cudaMemcpyDeviceToHost));
  return CLSPH_OK;
}

int clsph_mlp_forward(clsph_mlp* m, const uint16_t* x_bf16, uint32_t rows, float* y, void* cuda_stream) {
  if (!m || (rows && (!x_bf16 || !y))) return fail(CLSPH_ERR_ARGUMENT, "mlp_forward: bad argument");
  if (!rows) return CLSPH_OK;
  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  CUDA_TRY(cudaStreamSynchronize(m->stream));
  int rc = launch_tc(s, m->sms, reinterpret_cast<const bf16*>(x_bf16), rows, tc_weights(m),
                     clsph_nn::StoreRaw{reinterpret_cast<float4*>(y)}, m->err, nullptr, 0);
  if (rc) return rc;
  CUDA_TRY(cudaGetLastError());
  return CLSPH_OK;
}

int clsph_mlp_forward_mma_sync(clsph_mlp* m, const uint16_t* x_bf16, uint32_t rows, float* y, void* cuda_stream) {
  if (!m || (rows && (!x_bf16 || !y))) return fail(CLSPH_ERR_ARGUMENT, "mlp_forward_mma_sync: bad argument");
  if (!rows) return CLSPH_OK;
  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  CUDA_TRY(cudaStreamSynchronize(m->stream));
  int rc = launch_infer(s, m->sms, reinterpret_cast<const bf16*>(x_bf16), rows, infer_weights(m),
                        clsph_nn::StoreRaw{reinterpret_cast<float4*>(y)}, nullptr, 0);
  if (rc) return rc;
  CUDA_TRY(cudaGetLastError());
  return CLSPH_OK;
}

int clsph_mlp_predict(clsph_mlp* m, const float* x_raw, uint64_t rows, float* y_host) {
  if (!m || (rows && (!x_raw || !y_host))) return fail(CLSPH_ERR_ARGUMENT, "mlp_predict: bad argument");
  const uint32_t chunk = 65536;
  int rc;
  if ((rc = ensure_training(m, chunk))) return rc;
  for (uint64_t off = 0; off < rows; off += chunk) {
    const uint32_t r = (uint32_t)std::min<uint64_t>(chunk, rows - off);
    clsph_nn::k_standardize<<<(r * kIn + 255) / 256, 256, 0, m->stream>>>(x_raw + off * kIn, r,
                                                                        m->blob + clsph_nn::kOffXMu, m->xb);
    if ((rc = launch_tc(m->stream, m->sms, m->xb, r, tc_weights(m), clsph_nn::StoreRaw{reinterpret_cast<float4*>(m->yb)},
                        m->err, nullptr, 0)))
      return rc;
    CUDA_TRY(cudaMemcpyAsync(y_host + off * kOut, m->yb, sizeof(float) * kOut * r, cudaMemcpyDeviceToHost,
                             m->stream));
    CUDA_TRY(cudaStreamSynchronize(m->stream));
  }
  uint32_t e = 0;
  CUDA_TRY(cudaMemcpy(&e, m->err, sizeof(e), cudaMemcpyDeviceToHost));
  if (e) return fail(CLSPH_ERR_CUDA, "mlp_predict: a tensor-core wait timed out");
  return CLSPH_OK;
}

int clsph_mlp_status(clsph_mlp* m, uint32_t* flags) {
  if (!m || !flags) return fail(CLSPH_ERR_ARGUMENT, "mlp_status: bad argument");
  CUDA_TRY(cudaDeviceSynchronize());
  CUDA_TRY(cudaMemcpy(flags, m->err, sizeof(uint32_t), cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemset(m->err, 0, sizeof(uint32_t)));
  return CLSPH_OK;
}

int clsph_mlp_gradients(clsph_mlp* m, const float* x_raw, const float* y_raw, uint32_t rows,
                        float* grads_host, float* loss) {
  if (!m || !x_raw || !y_raw || rows == 0 || rows % kRowBlock)
    return fail(CLSPH_ERR_ARGUMENT, "mlp_gradients: rows must be a positive multiple of 2048");
  int rc;
  if ((rc = ensure_training(m, rows)) || (rc = ensure_idx(m, rows)) || (rc = ensure_loss(m, 1))) return rc;
  std::vector<uint32_t> iota(rows);
  std::iota(iota.begin(), iota.end(), 0u);
  CUDA_TRY(cudaMemcpyAsync(m->idx, iota.data(), sizeof(uint32_t) * rows, cudaMemcpyHostToDevice, m->stream));
  CUDA_TRY(cudaMemsetAsync(m->loss, 0, sizeof(float), m->stream));
  clsph_nn::k_gather_batch<<<(rows * (kIn + kOut) + 255) / 256, 256, 0, m->stream>>>(
      x_raw, y_raw, m->idx, rows, m->blob + clsph_nn::kOffXMu, m->xb, m->yb);
  if ((rc = pass(m, rows, m->loss, true))) return rc;
  float l = 0.f;
  CUDA_TRY(cudaMemcpyAsync(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream));
  if (grads_host)
    CUDA_TRY(cudaMemcpyAsync(grads_host, m->grad, sizeof(float) * kParams, cudaMemcpyDeviceToHost, m->stream));
  CUDA_TRY(cudaStreamSynchronize(m->stream));
  if ((rc = check_train_waits(m))) return rc;
  if (loss) *loss = l / rows;
  return CLSPH_OK;
}

int clsph_mlp_loss(clsph_mlp* m, const float* x_raw, const float* y_raw, uint64_t samples, float* loss) {
  if (!m || !x_raw || !y_raw || !loss) return fail(CLSPH_ERR_ARGUMENT, "mlp_loss: bad argument");
  const uint32_t rows = (uint32_t)std::min<uint64_t>(samples - samples % kRowBlock, 65536);
  if (rows == 0) return fail(CLSPH_ERR_ARGUMENT, "mlp_loss: fewer than 2048 samples");
  const uint64_t blocks = samples / rows;
  int rc;
  if ((rc = ensure_training(m, rows)) || (rc = ensure_idx(m, rows)) || (rc = ensure_loss(m, 1))) return rc;
  CUDA_TRY(cudaMemsetAsync(m->loss, 0, sizeof(float), m->stream));
  std::vector<uint32_t> iota(rows);
  for (uint64_t b = 0; b < blocks; ++b) {
    for (uint32_t r = 0; r < rows; ++r) iota[r] = (uint32_t)(b * rows + r);
    CUDA_TRY(cudaMemcpyAsync(m->idx, iota.data(), sizeof(uint32_t) * rows, cudaMemcpyHostToDevice, m->stream));
    clsph_nn::k_gather_batch<<<(rows * (kIn + kOut) + 255) / 256, 256, 0, m->stream>>>(
        x_raw, y_raw, m->idx, rows, m->blob + clsph_nn::kOffXMu, m->xb, m->yb);
    if ((rc = pass(m, rows, m->loss, false))) return rc;
    CUDA_TRY(cudaStreamSynchronize(m->stream));  // iota is reused
  }
  float l = 0.f;
  CUDA_TRY(cudaMemcpy(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost));
  if ((rc = check_train_waits(m))) return rc;
  *loss = l / (float)(blocks * rows);
  return CLSPH_OK;
}

int clsph_mlp_train(clsph_mlp* m, const float* x_raw, const float* y_raw, uint64_t samples,
                    const clsph_train_config* cfg, float* loss_log, uint32_t log_len, uint32_t* logged) {
  if (!m || !x_raw || !y_raw || !cfg || cfg->batch == 0 || cfg->batch % kRowBlock || cfg->epochs == 0)
    return fail(CLSPH_ERR_ARGUMENT, "mlp_train: bad argument (batch must be a multiple of 2048)");
  if (samples < cfg->batch || samples >= (1ull << 32))
    return fail(CLSPH_ERR_ARGUMENT, "mlp_train: sample count out of range");
  const uint32_t rows = cfg->batch;
  int rc;
  if ((rc = ensure_training(m, rows)) || (rc = ensure_idx(m, samples))) return rc;
  cudaStream_t s = m->stream;
  if (cfg->fit_normalisation) {
    CUDA_TRY(cudaMemsetAsync(m->moments, 0, sizeof(double) * 2 * (kIn + kOut), s));
    const uint64_t per = 4096;
    clsph_nn::k_moments<<<(unsigned)((samples + per - 1) / per), 64, 0, s>>>(x_raw, y_raw, samples, per,
                                                                             m->moments);
    double mom[2 * (kIn + kOut)];
    CUDA_TRY(cudaMemcpyAsync(mom, m->moments, sizeof(mom), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    float norm[2 * kIn + 2 * kOut];
    for (int c = 0; c < kIn + kOut; ++c) {
      const double mu = mom[c] / samples;
      const double var = std::max(0.0, mom[kIn + kOut + c] / samples - mu * mu);
      const float sd = (float)std::max(std::sqrt(var), 1e-6);
      if (c < kIn) {
        norm[c] = (float)mu;
        norm[kIn + c] = sd;
      } else {
        norm[2 * kIn + (c - kIn)] = (float)mu;
        norm[2 * kIn + kOut + (c - kIn)] = sd;
      }
    }
    CUDA_TRY(cudaMemcpyAsync(m->blob + clsph_nn::kOffXMu, norm, sizeof(norm), cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaStreamSynchronize(s));
  }
  const uint64_t per_epoch = samples / rows;
  const uint64_t total = per_epoch * cfg->epochs;
  if (total >= (1ull << 31)) return fail(CLSPH_ERR_ARGUMENT, "mlp_train: too many steps");
  if ((rc = ensure_loss(m, (uint32_t)total))) return rc;
  CUDA_TRY(cudaMemsetAsync(m->loss, 0, sizeof(float) * total, s));
  std::vector<uint32_t> perm(samples);
  std::mt19937_64 rng(cfg->seed);
  const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
  uint64_t step = 0;
  for (uint32_t e = 0; e < cfg->epochs; ++e) {
    std::iota(perm.begin(), perm.end(), 0u);
    std::shuffle(perm.begin(), perm.end(), rng);
    CUDA_TRY(cudaStreamSynchronize(s));  // the previous epoch's gathers read m->idx
    CUDA_TRY(cudaMemcpyAsync(m->idx, perm.data(), sizeof(uint32_t) * samples, cudaMemcpyHostToDevice, s));
    for (uint64_t b = 0; b < per_epoch; ++b, ++step) {
      clsph_nn::k_gather_batch<<<(rows * (kIn + kOut) + 255) / 256, 256, 0, s>>>(
          x_raw, y_raw, m->idx + b * rows, rows, m->blob + clsph_nn::kOffXMu, m->xb, m->yb);
      if ((rc = pass(m, rows, m->loss + step, true))) return rc;
      const float frac = total > 1 ? (float)step / (float)(total - 1) : 0.f;
      const float lr = cfg->lr + (cfg->lr_final - cfg->lr) * frac;
      ++m->adam_t;
      const float bc1 = 1.f - std::pow(beta1, (float)m->adam_t);
      const float bc2 = 1.f - std::pow(beta2, (float)m->adam_t);
      clsph_nn::k_adam<<<(kParams + 255) / 256, 256, 0, s>>>(m->blob, m->grad, m->adam_m, m->adam_v, kParams,
                                                            lr, beta1, beta2, eps, bc1, bc2, bf16_weights(m));
    }
  }
  CUDA_TRY(cudaGetLastError());
  std::vector<float> losses(total);
  CUDA_TRY(cudaMemcpyAsync(losses.data(), m->loss, sizeof(float) * total, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  uint32_t nlog = 0;
  if (loss_log && log_len) {
    const uint32_t every = std::max<uint32_t>(1, cfg->log_every);
    for (uint64_t b0 = 0; b0 < total && nlog < log_len; b0 += every) {
      const uint64_t b1 = std::min<uint64_t>(total, b0 + every);
      double acc = 0.0;
      for (uint64_t b = b0; b < b1; ++b) acc += losses[b];
      loss_log[nlog++] = (float)(acc / (double)(b1 - b0) / rows);
    }
  }
  if (logged) *logged = nlog;
  return check_train_waits(m);
}

// ---- collector

int clsph_collector_destroy(clsph_collector* c) {
  if (!c) return CLSPH_OK;
  if (c->h && c->h->stream) cudaStreamSynchronize(c->h->stream);
  void* bufs[] = {c->ring, c->xs, c->ys, c->scratch.pos, c->scratch.vel, c->scratch.ivel,
                  c->zero, c->sbbox, c->sstatus, c->scapped};
  for (void* b : bufs) cudaFree(b);
  delete c;
  return CLSPH_OK;
}

int clsph_collector_create(clsph_gpu* h, uint32_t id_stride, uint32_t dt_mult, uint64_t capacity,
                           clsph_collector** out) {
  if (!h || !out || id_stride == 0 || dt_mult == 0 || dt_mult > 64 || capacity == 0)
    return fail(CLSPH_ERR_ARGUMENT, "collector_create: bad argument");
  auto* c = new clsph_collector();
  c->h = h;
  c->stride = id_stride;
  c->dt_mult = dt_mult;
  c->m = (h->n + id_stride - 1) / id_stride;
  c->capacity = capacity;
  const size_t n = h->n;
  int rc;
  if ((rc = dev_alloc(&c->ring, (size_t)(dt_mult + 1) * c->m * kRing)) ||
      (rc = dev_alloc(&c->xs, capacity * kFeat)) || (rc = dev_alloc(&c->ys, capacity * kOut)) ||
      (rc = dev_alloc(&c->scratch.pos, n)) || (rc = dev_alloc(&c->scratch.vel, n)) ||
      (rc = dev_alloc(&c->scratch.ivel, n)) || (rc = dev_alloc(&c->zero, n)) ||
      (rc = dev_alloc(&c->sbbox, 6 * (size_t)h->nscenes)) || (rc = dev_alloc(&c->sstatus, 1)) ||
      (rc = dev_alloc(&c->scapped, 1))) {
    clsph_collector_destroy(c);
    return rc;
  }
  if (cudaMemset(c->zero, 0, sizeof(float4) * n) != cudaSuccess ||
      cudaMemset(c->sbbox, 0, sizeof(uint32_t) * 6 * h->nscenes) != cudaSuccess) {
    clsph_collector_destroy(c);
    return fail(CLSPH_ERR_CUDA, "collector_create: memset");
  }
  *out = c;
  return CLSPH_OK;
}

namespace {

// Density, forces and the tracked particles' ring entry (features and the
// naive dt_mult step's velocity) of the handle's current state; leaves the
// substep ready for its advection.
int collect_level(clsph_collector* c, float* level) {
  clsph_gpu* h = c->h;
  const uint32_t n = h->n;
  int rc = enqueue_substep(h, CLSPH_STAGE_DENSITY);
  if (rc) return rc;
  FeatureHook fh = feature_hook(h, kFeatRing);
  fh.raw = level;
  fh.ids = h->ids[h->ids_sel];
  fh.stride = c->stride;
  fh.m = c->m;
  if ((rc = launch_forces_hooked(h, fh))) return rc;
  h->launch(K_MISC, k_advect<true>, dim3(grid_blocks(n, h->sm_count * h->advect_blocks_per_sm)), dim3(kBlock),
            n, h->st[1], (const float4*)h->acc, c->scratch, (const DevMesh*)h->meshes, (const Consts*)h->consts,
            (const uint16_t*)h->scene_of, h->max_iters, c->sbbox, c->sstatus, c->scapped,
            (const float4*)c->zero, (float)c->dt_mult, position_weight(c->dt_mult), (const float4*)nullptr,
            (const float*)nullptr);
  h->launch(K_MISC, k_ring_naive, dim3(grid_blocks(n)), dim3(kBlock), n, (const uint32_t*)h->ids[h->ids_sel],
            c->stride, c->m, (const float4*)c->scratch.ivel, (const Consts*)h->consts,
            (const uint16_t*)h->scene_of, level);
  return 0;
}

void emit_samples(clsph_collector* c, const float* old_level, const float* level) {
  if (c->count >= c->capacity) return;
  c->h->launch(K_MISC, k_sample, dim3((c->m + 255) / 256), dim3(256), old_level, level, c->m,
               1.f / (float)c->dt_mult, c->xs, c->ys, c->count, c->capacity);
  c->count = std::min<uint64_t>(c->capacity, c->count + c->m);
}

}  // namespace

int clsph_collector_step(clsph_collector* c, uint32_t substeps) {
  if (!c) return fail(CLSPH_ERR_ARGUMENT, "collector_step: null collector");
  clsph_gpu* h = c->h;
  if (!h->uploaded || h->partial) return fail(CLSPH_ERR_STATE, "collector_step: upload particles first");
  const uint32_t levels = c->dt_mult + 1;
  for (uint32_t k = 0; k < substeps; ++k) {
    float* level = c->ring + (size_t)(c->t % levels) * c->m * kRing;
    int rc = collect_level(c, level);
    if (rc) return rc;
    if (c->t >= c->dt_mult)
      emit_samples(c, c->ring + (size_t)((c->t - c->dt_mult) % levels) * c->m * kRing, level);
    if ((rc = enqueue_advect(h))) return rc;
    ++h->substeps;
    ++c->t;
  }
  if (substeps) h->have_fields = true;
  return check_launch(h);
}

int clsph_collector_step_learned(clsph_collector* c, clsph_mlp* m, uint32_t steps) {
  if (!c || !m) return fail(CLSPH_ERR_ARGUMENT, "collector_step_learned: bad argument");
  clsph_gpu* h = c->h;
  if (!h->uploaded || h->partial) return fail(CLSPH_ERR_STATE, "collector_step_learned: upload particles first");
  if (m->device != h->device) return fail(CLSPH_ERR_ARGUMENT, "collector_step_learned: MLP on another device");
  LearnedCache* L = nullptr;
  int rc = ensure_cache(h, &L);
  if (rc) return rc;
  CUDA_TRY(cudaStreamSynchronize(m->stream));
  float* lv0 = c->ring;
  float* lv1 = c->ring + (size_t)c->m * kRing;
  for (uint32_t k = 0; k < steps; ++k) {
    // the plain outcome of the visited state: dt_mult substeps, features at both ends
    if ((rc = save(h, L->snap[0]))) return rc;
    if ((rc = collect_level(c, lv0)) || (rc = enqueue_advect(h))) return rc;
    for (uint32_t q = 1; q < c->dt_mult; ++q)
      if ((rc = enqueue_substep(h, CLSPH_STAGE_ADVECT))) return rc;
    if ((rc = collect_level(c, lv1))) return rc;
    emit_samples(c, lv0, lv1);
    // back to the visited state, then one learned step onward
    if ((rc = restore(h, L->snap[0]))) return rc;
    if ((rc = enqueue_substep(h, CLSPH_STAGE_DENSITY))) return rc;
    if ((rc = enqueue_learned_tail(h, m, L, c->dt_mult))) return rc;
    h->substeps += 1;
  }
  c->t = 0;  // the plain-trajectory ring restarts after this
  h->have_fields = false;
  return check_launch(h);
}

int clsph_collector_samples(clsph_collector* c, const float** x_raw, const float** y_raw, uint64_t* count) {
  if (!c) return fail(CLSPH_ERR_ARGUMENT, "collector_samples: null collector");
  CUDA_TRY(cudaStreamSynchronize(c->h->stream));
  if (x_raw) *x_raw = c->xs;
  if (y_raw) *y_raw = c->ys;
  if (count) *count = c->count;
  return CLSPH_OK;
}

int clsph_collector_copy(clsph_collector* c, float* x_host, float* y_host, uint64_t first, uint64_t count) {
  if (!c || (count && (!x_host || !y_host))) return fail(CLSPH_ERR_ARGUMENT, "collector_copy: bad argument");
  CUDA_TRY(cudaStreamSynchronize(c->h->stream));
  if (first > c->count || count > c->count - first)
    return fail(CLSPH_ERR_ARGUMENT, "collector_copy: range beyond the samples collected");
  if (!count) return CLSPH_OK;
  CUDA_TRY(cudaMemcpy(x_host, c->xs + first * kFeat, sizeof(float) * kFeat * count, cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemcpy(y_host, c->ys + first * kOut, sizeof(float) * kOut * count, cudaMemcpyDeviceToHost));
  return CLSPH_OK;
}

int clsph_gpu_read_features(clsph_gpu* h, float* features_host) {
  if (!h || !features_host) return fail(CLSPH_ERR_ARGUMENT, "read_features: bad argument");
  if (!h->have_fields) return fail(CLSPH_ERR_STATE, "read_features: run a substep to CLSPH_STAGE_FORCES first");
  float* d = nullptr;
  int rc = dev_alloc(&d, (size_t)h->n * kFeat);
  if (rc) return rc;
  FeatureHook fh = feature_hook(h, kFeatRaw);
  fh.raw = d;
  rc = launch_forces_hooked(h, fh);
  if (rc) {
    cudaFree(d);
    return rc;
  }
  cudaError_t e = cudaMemcpyAsync(features_host, d, sizeof(float) * h->n * kFeat, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(d);
  if (e != cudaSuccess) return fail(CLSPH_ERR_CUDA, std::string("read_features: ") + cudaGetErrorString(e));
  return check_launch(h);
}

// ---- learned step

int clsph_gpu_step_learned(clsph_gpu* h, clsph_mlp* m, uint32_t steps, const clsph_learned_config* cfg,
                           clsph_learned_stats* stats) {
  if (!h || !m || !cfg || cfg->dt_mult == 0 || cfg->dt_mult > 64 || !(cfg->threshold >= 0.f))
    return fail(CLSPH_ERR_ARGUMENT, "step_learned: bad argument");
  if (!h->uploaded || h->partial) return fail(CLSPH_ERR_STATE, "step_learned: upload particles first");
  if (m->device != h->device) return fail(CLSPH_ERR_ARGUMENT, "step_learned: MLP on another device");
  LearnedCache* L = nullptr;
  int rc = ensure_cache(h, &L);
  if (rc) return rc;
  if (L->calibrated_for != m || !(cfg->flags & CLSPH_LEARNED_CALIBRATE)) {
    L->calibrated_for = m;
    L->bias_d = L->bias_m = 0.0;
    L->calib_pending = false;
  }
  CUDA_TRY(cudaStreamSynchronize(m->stream));  // weights in place
  // the MLP kernel's error word collects this call's wait timeouts only
  CUDA_TRY(cudaMemsetAsync(L->dev_sum + kGateSums, 0, sizeof(float), h->stream));
  const uint32_t mult = cfg->dt_mult;
  clsph_learned_stats st{};
  auto record = [&](const GateStats& g, double dev) {
    ++st.checks;
    st.deviation_sum += dev;
    st.particle_deviation_sum += g.particle;
    st.deviation_max = std::max(st.deviation_max, dev);
  };
  // roll the learned step whose input is `snap` back, redo its interval with
  // plain substeps and calibrate on their result at the next density pass
  auto fall_back = [&](const Snapshot& snap, const GateStats& g) -> int {
    int r;
    if ((r = restore(h, snap))) return r;
    if ((r = plain_substeps(h, mult))) return r;
    ++st.rejected;
    st.plain_substeps += mult;
    L->calib_pending = true;
    L->rejected_d = g.d_pred;
    L->rejected_m = g.m_pred;
    return 0;
  };
  if (cfg->flags & CLSPH_LEARNED_NO_CHECK) {
    // back to back on the stream: no snapshot, no gate, no host wait per step;
    // groups of kLearnedGraphLen steps replay one CUDA graph when the handle
    // uses graphs
    uint32_t k = 0;
    if (h->use_graph && !h->profiling && steps >= kLearnedGraphLen) {
      if ((rc = ensure_nocheck_graph(h, m, L, mult))) return rc;
      for (; k + kLearnedGraphLen <= steps; k += kLearnedGraphLen) {
        CUDA_TRY(cudaGraphLaunch(L->nc_graph[h->ids_sel], h->stream));
        h->launches += L->nc_launches[h->ids_sel];
        h->substeps += kLearnedGraphLen;
      }
    }
    for (; k < steps; ++k) {
      if ((rc = enqueue_substep(h, CLSPH_STAGE_DENSITY))) return rc;
      if ((rc = enqueue_learned_tail(h, m, L, mult))) return rc;
      ++h->substeps;
    }
    // the MLP kernel's error word, read once for the whole run
    CUDA_TRY(cudaMemcpyAsync(L->dev_host + kGateSums, L->dev_sum + kGateSums, sizeof(float),
                             cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    uint32_t errw;
    std::memcpy(&errw, L->dev_host + kGateSums, sizeof(errw));
    if (errw) return fail(CLSPH_ERR_CUDA, "step_learned: a tensor-core wait of the MLP kernel timed out");
    h->have_fields = false;
    if (stats) {
      stats->learned_steps += steps;
      stats->calibration_d = L->bias_d;
      stats->calibration_m = L->bias_m;
    }
    return check_launch(h);
  }
  int cur = 0;
  bool pending = false;  // the last learned step awaits its density check; its input is snap[cur ^ 1]
  uint32_t done = 0;
  while (done < steps) {
    if ((rc = save(h, L->snap[cur]))) return rc;
    if ((rc = enqueue_substep(h, CLSPH_STAGE_DENSITY))) return rc;
    const bool calib = !pending && L->calib_pending && (cfg->flags & CLSPH_LEARNED_CALIBRATE);
    if ((pending || calib) && (rc = enqueue_gate(h, L))) return rc;
    if ((rc = enqueue_learned_tail(h, m, L, mult))) return rc;
    ++h->substeps;
    if (calib) {
      GateStats g;
      if ((rc = wait_gate(h, L, &g))) return rc;
      L->bias_d += kCalibrationWeight * ((g.d - L->rejected_d) - L->bias_d);
      L->bias_m += kCalibrationWeight * ((g.m - L->rejected_m) - L->bias_m);
      L->calib_pending = false;
    }
    if (pending) {
      GateStats g;
      if ((rc = wait_gate(h, L, &g))) return rc;
      const double dev = predicted_deviation(g, L);
      record(g, dev);
      if (!(dev <= cfg->threshold)) {
        if ((rc = fall_back(L->snap[cur ^ 1], g))) return rc;
        pending = false;
        continue;
      }
      ++st.learned_steps;
    }
    pending = true;
    ++done;
    cur ^= 1;
  }
  if (pending) {
    // check the last learned step with one neighbour build and density pass
    if ((rc = save(h, L->snap[cur]))) return rc;
    if ((rc = enqueue_substep(h, CLSPH_STAGE_DENSITY))) return rc;
    if ((rc = enqueue_gate(h, L))) return rc;
    GateStats g;
    if ((rc = wait_gate(h, L, &g))) return rc;
    if ((rc = restore(h, L->snap[cur]))) return rc;
    const double dev = predicted_deviation(g, L);
    record(g, dev);
    if (!(dev <= cfg->threshold)) {
      if ((rc = fall_back(L->snap[cur ^ 1], g))) return rc;
    } else {
      ++st.learned_steps;
    }
  }
  h->have_fields = false;
  if (stats) {
    stats->learned_steps += st.learned_steps;
    stats->rejected += st.rejected;
    stats->plain_substeps += st.plain_substeps;
    stats->checks += st.checks;
    stats->deviation_sum += st.deviation_sum;
    stats->particle_deviation_sum += st.particle_deviation_sum;
    stats->deviation_max = std::max(stats->deviation_max, st.deviation_max);
    stats->calibration_d = L->bias_d;
    stats->calibration_m = L->bias_m;
  }
  return check_launch(h);
}

}  // extern "C"
