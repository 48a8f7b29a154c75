// Allocation-free stable key sort: clsph_gpu_sort_keys_noalloc.
//
// Some callers cannot allocate device memory themselves: a host application
// or framework that owns every device allocation through its own allocator
// and forbids raw cudaMalloc/cudaFree (whose implicit device-wide
// synchronisation would stall its other work), or a fixed-budget real-time
// loop that must not allocate after start-up. This entry point runs the
// substep's stable sort (the 4 x 8-bit LSD radix sort of
// libclsph/sph_simulation.cpp:107-156 + kernels/sort.cl, with 32-bit offsets)
// on caller-provided device buffers and takes its scratch space from one
// file-scope __device__ array instead of cudaMalloc.
//
// Limits and rules:
//  * at most kNoAllocMaxKeys (1,048,576) keys per call; larger n is rejected
//    with CLSPH_ERR_TOO_LARGE before any GPU work;
//  * the scratch array (8.3 MB) is part of the library's device image: every
//    GPU that loads the library holds it until the process exits;
//  * all calls share that one array and it keeps the last call's contents;
//    each call clears what must start at zero itself. Calls whose GPU work
//    overlaps (other streams, other host threads on the same device) race on
//    it, so the caller must serialise them;
//  * the first call on each device looks up the array's device address with
//    cudaGetSymbolAddress (with that device current); make that first call
//    before any stream capture.
// It makes no cudaMalloc, cudaFree or other allocating call.

#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "clsph_common.cuh"
#include "clsph_gpu.h"

void clsph_set_last_error(const std::string& msg);

namespace {

constexpr uint32_t kNoAllocMaxKeys = 1u << 20;
constexpr int kThreads = 256;
constexpr int kItems = 16;
constexpr uint32_t kTile = kThreads * kItems;  // 4096 keys per tile
constexpr uint32_t kMaxTiles = kNoAllocMaxKeys / kTile;
constexpr int kWarps = kThreads / 32;
constexpr uint32_t kWarpSpan = kTile / kWarps;

// scratch layout, in 32-bit words
constexpr size_t kOffKeys = 0;                                    // ping-pong keys
constexpr size_t kOffVals = kOffKeys + kNoAllocMaxKeys;           // ping-pong slots
constexpr size_t kOffHist = kOffVals + kNoAllocMaxKeys;           // [256][tiles]
constexpr size_t kOffTotals = kOffHist + 256 * (size_t)kMaxTiles; // [4][256]
constexpr size_t kOffCtl = kOffTotals + 4 * 256;                  // [0] = largest key
constexpr size_t kScratchWords = kOffCtl + 64;

static __device__ __align__(256) uint32_t g_sort_scratch[kScratchWords];

struct Buffers {
  const uint32_t* in_keys;  // caller's input (never written)
  uint32_t* out_keys;       // caller's sorted keys
  uint32_t* out_vals;       // caller's permutation
  uint32_t* tmp_keys;       // scratch
  uint32_t* tmp_vals;       // scratch
  uint32_t* hist;
  uint32_t* totals;
  uint32_t* ctl;
};

__device__ __forceinline__ uint32_t passes_for(uint32_t maxkey) {
  uint32_t k = maxkey | 1u, bits = 0;
  while (k) {
    ++bits;
    k >>= 1;
  }
  return (bits + 7u) / 8u;
}

// Pass p writes to the caller's buffers when an even number of passes
// follows it, so the last pass always lands in the caller's output.
__device__ __forceinline__ void pass_buffers(const Buffers& b, int pass, uint32_t passes,
                                             const uint32_t** ks, const uint32_t** vs,
                                             uint32_t** kd, uint32_t** vd) {
  auto dst_is_out = [&](int p) { return ((passes - 1u - (uint32_t)p) & 1u) == 0u; };
  if (pass == 0) {
    *ks = b.in_keys;
    *vs = nullptr;
  } else {
    bool prev_out = dst_is_out(pass - 1);
    *ks = prev_out ? b.out_keys : b.tmp_keys;
    *vs = prev_out ? b.out_vals : b.tmp_vals;
  }
  bool out = dst_is_out(pass);
  *kd = out ? b.out_keys : b.tmp_keys;
  *vd = out ? b.out_vals : b.tmp_vals;
}

__global__ void k_na_clear(Buffers b) {
  for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x) b.totals[i] = 0u;
  if (threadIdx.x == 0) b.ctl[0] = 0u;
}

__global__ void k_na_maxkey(Buffers b, uint32_t n) {
  __shared__ uint32_t block_max;
  if (threadIdx.x == 0) block_max = 0u;
  __syncthreads();
  uint32_t m = 0u;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    m = max(m, b.in_keys[i]);
  m = __reduce_max_sync(0xFFFFFFFFu, m);
  if ((threadIdx.x & 31) == 0) atomicMax(&block_max, m);
  __syncthreads();
  if (threadIdx.x == 0) atomicMax(&b.ctl[0], block_max);
}

__global__ void k_na_count(Buffers b, uint32_t n, int pass, uint32_t ntiles) {
  const uint32_t passes = passes_for(b.ctl[0]);
  if ((uint32_t)pass >= passes) return;
  const uint32_t *ks, *vs;
  uint32_t *kd, *vd;
  pass_buffers(b, pass, passes, &ks, &vs, &kd, &vd);
  __shared__ uint32_t hist[256];
  hist[threadIdx.x] = 0u;
  __syncthreads();
  const uint32_t base = blockIdx.x * kTile;
  const int shift = 8 * pass;
  for (int k = 0; k < kItems; ++k) {
    uint32_t idx = base + k * kThreads + threadIdx.x;
    if (idx < n) atomicAdd(&hist[(ks[idx] >> shift) & 0xFFu], 1u);
  }
  __syncthreads();
  uint32_t c = hist[threadIdx.x];
  b.hist[(size_t)threadIdx.x * ntiles + blockIdx.x] = c;
  if (c) atomicAdd(&b.totals[pass * 256 + threadIdx.x], c);
}

__global__ void k_na_scan(Buffers b, uint32_t ntiles, int pass) {
  if ((uint32_t)pass >= passes_for(b.ctl[0])) return;
  __shared__ uint32_t warp_sums[kThreads / 32];
  __shared__ uint32_t base_s;
  const uint32_t d = blockIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t part = threadIdx.x < d ? b.totals[pass * 256 + threadIdx.x] : 0u;
  for (int off = 16; off > 0; off >>= 1) part += __shfl_xor_sync(0xFFFFFFFFu, part, off);
  if (lane == 0) warp_sums[warp] = part;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t s = 0;
    for (int w = 0; w < kThreads / 32; ++w) s += warp_sums[w];
    base_s = s;
  }
  __syncthreads();
  uint32_t carry = base_s;
  uint32_t* row = b.hist + (size_t)d * ntiles;
  for (uint32_t chunk = 0; chunk < ntiles; chunk += kThreads) {
    uint32_t idx = chunk + threadIdx.x;
    uint32_t v = idx < ntiles ? row[idx] : 0u;
    uint32_t x = v;
    for (int off = 1; off < 32; off <<= 1) {
      uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, off);
      if (lane >= off) x += y;
    }
    __syncthreads();
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    uint32_t wbase = 0, total = 0;
    for (int w = 0; w < kThreads / 32; ++w) {
      uint32_t s = warp_sums[w];
      if (w < warp) wbase += s;
      total += s;
    }
    if (idx < ntiles) row[idx] = carry + wbase + x - v;
    carry += total;
  }
}

__global__ void __launch_bounds__(kThreads) k_na_scatter(Buffers b, uint32_t n, int pass, uint32_t ntiles) {
  const uint32_t passes = passes_for(b.ctl[0]);
  if ((uint32_t)pass >= passes) return;
  const uint32_t *ks, *vs;
  uint32_t *kd, *vd;
  pass_buffers(b, pass, passes, &ks, &vs, &kd, &vd);
  __shared__ uint32_t cnt[kWarps][256];
  __shared__ uint32_t tile_off[256];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int w = 0; w < kWarps; ++w) cnt[w][threadIdx.x] = 0u;
  tile_off[threadIdx.x] = b.hist[(size_t)threadIdx.x * ntiles + blockIdx.x];
  __syncthreads();
  const int shift = 8 * pass;
  const uint32_t lt_mask = (1u << lane) - 1u;
  const uint32_t base = blockIdx.x * kTile + warp * kWarpSpan;
  uint32_t key[kItems], val[kItems], rank[kItems];
#pragma unroll
  for (int r = 0; r < kItems; ++r) {
    const uint32_t idx = base + r * 32 + lane;
    const bool valid = idx < n;
    key[r] = valid ? ks[idx] : 0u;
    val[r] = valid ? (vs ? vs[idx] : idx) : 0u;
    const uint32_t d = valid ? ((key[r] >> shift) & 0xFFu) : 256u;
    const uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
    uint32_t rk = 0;
    if (valid) rk = cnt[warp][d] + __popc(peers & lt_mask);
    __syncwarp();
    if (valid && (peers & lt_mask) == 0u) cnt[warp][d] += __popc(peers);
    __syncwarp();
    rank[r] = valid ? ((rk << 8) | d) : 0xFFFFFFFFu;
  }
  __syncthreads();
  {
    uint32_t run = 0;
    for (int w = 0; w < kWarps; ++w) {
      uint32_t t = cnt[w][threadIdx.x];
      cnt[w][threadIdx.x] = run;
      run += t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < kItems; ++r) {
    if (rank[r] == 0xFFFFFFFFu) continue;
    const uint32_t d = rank[r] & 0xFFu;
    const uint32_t dst = tile_off[d] + cnt[warp][d] + (rank[r] >> 8);
    kd[dst] = key[r];
    vd[dst] = val[r];
  }
}

// Device address of g_sort_scratch, looked up once per device and kept for
// the life of the process (a cudaDeviceReset reloads the device code and
// makes it stale; the header tells callers not to use the entry point on a
// device after resetting it).
constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
uint32_t* g_scratch_addr[kMaxDevices] = {};

int scratch_for_current_device(uint32_t** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    clsph_set_last_error(std::string("sort_keys_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
    return CLSPH_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    clsph_set_last_error("sort_keys_noalloc: device ordinal out of range");
    return CLSPH_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_sort_scratch);
    if (e != cudaSuccess || p == nullptr) {
      clsph_set_last_error(std::string("sort_keys_noalloc: cudaGetSymbolAddress: ") +
                           cudaGetErrorString(e));
      return CLSPH_ERR_CUDA;
    }
    g_scratch_addr[dev] = static_cast<uint32_t*>(p);
  }
  *out = g_scratch_addr[dev];
  return CLSPH_OK;
}

}  // namespace

extern "C" int clsph_gpu_sort_keys_noalloc(const uint32_t* keys_in, uint32_t* keys_out,
                                           uint32_t* perm_out, uint32_t n, void* stream) {
  if (n > kNoAllocMaxKeys) {
    clsph_set_last_error("sort_keys_noalloc: n = " + std::to_string(n) +
                         " exceeds the maximum of 1048576 keys");
    return CLSPH_ERR_TOO_LARGE;
  }
  if (n == 0) return CLSPH_OK;
  if (!keys_in || !keys_out || !perm_out) {
    clsph_set_last_error("sort_keys_noalloc: null buffer");
    return CLSPH_ERR_ARGUMENT;
  }
  uint32_t* scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Buffers b;
  b.in_keys = keys_in;
  b.out_keys = keys_out;
  b.out_vals = perm_out;
  b.tmp_keys = scratch + kOffKeys;
  b.tmp_vals = scratch + kOffVals;
  b.hist = scratch + kOffHist;
  b.totals = scratch + kOffTotals;
  b.ctl = scratch + kOffCtl;
  const uint32_t ntiles = (n + kTile - 1) / kTile;
  k_na_clear<<<1, 256, 0, s>>>(b);
  uint32_t blocks = (n + 255) / 256;
  if (blocks > 1024) blocks = 1024;
  k_na_maxkey<<<blocks, 256, 0, s>>>(b, n);
  for (int pass = 0; pass < 4; ++pass) {
    k_na_count<<<ntiles, kThreads, 0, s>>>(b, n, pass, ntiles);
    k_na_scan<<<256, kThreads, 0, s>>>(b, ntiles, pass);
    k_na_scatter<<<ntiles, kThreads, 0, s>>>(b, n, pass, ntiles);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    clsph_set_last_error(std::string("sort_keys_noalloc: launch: ") + cudaGetErrorString(e));
    return CLSPH_ERR_CUDA;
  }
  return CLSPH_OK;
}
