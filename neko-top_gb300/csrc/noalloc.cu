// Masked dot product that allocates nothing: the variant of
// cuda_glsc2_mask for callers that cannot allocate device memory.
//
// Who needs it: code that runs while device memory belongs to someone else
// or is exhausted -- a host application whose caching allocator has
// reserved the whole GPU, an out-of-memory recovery path that must still
// measure a residual, or a Fortran solver that hands the library all its
// memory up front and forbids allocation afterwards.  cudaMalloc can fail
// there, and cudaMalloc/cudaFree may also synchronise the device, which such
// callers cannot afford in the middle of a solve.
//
// How: the block partial sums, the result slot and the last-block ticket
// live in one file-scope __device__ array (kNoAllocScratch doubles,
// 128 KiB plus 16 bytes), which every GPU that loads the library keeps until
// the process exits.  Each block reduces kNoAllocPerBlock mask entries, so
// the largest accepted mask has kNoAllocMaxBlocks * kNoAllocPerBlock =
// 16,777,216 entries; longer masks are rejected with NTG_ERR_INVALID.
//
// Host code never uses the array's name as an address (on the host it is a
// stand-in, not device memory): the first call on each device, made with
// that device current, asks cudaGetSymbolAddress for the device address
// and caches it.  Make that first call before any stream capture.
//
// Every call shares the one array.  The ticket is cleared at the start of
// each call (an async memset on the caller's stream); the result of the last
// call stays in the array.  Two calls whose kernels overlap on the GPU (on
// different streams, or on different host threads without ordering) race
// on the array and give wrong results: order them on one stream.
#include <mutex>

#include "common.cuh"

namespace ntg {

constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocPerThread = 4;
constexpr int kNoAllocPerBlock = kNoAllocThreads * kNoAllocPerThread;  // 1024 mask entries
constexpr int kNoAllocMaxBlocks = 16384;
constexpr int64_t kNoAllocMaxEntries = (int64_t)kNoAllocMaxBlocks * kNoAllocPerBlock;
// [0, kNoAllocMaxBlocks): block partials; [kNoAllocMaxBlocks]: result;
// [kNoAllocMaxBlocks + 1]: ticket (as unsigned long long)
constexpr int kNoAllocScratch = kNoAllocMaxBlocks + 2;

static __device__ __align__(256) double g_glsc2_noalloc_scratch[kNoAllocScratch];

__device__ __forceinline__ double na_warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double na_block_sum(double v, double* sred) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = na_warp_sum(v);
  if (lane == 0) sred[warp] = v;
  __syncthreads();
  double t = (threadIdx.x < kNoAllocThreads / 32) ? sred[lane] : 0.0;
  if (warp == 0) t = na_warp_sum(t);
  __syncthreads();
  return t;  // valid in thread 0
}

// 1-based mask (as the reference's masked kernels); deterministic: fixed
// per-block ranges, fixed trees, partials summed by the last block in order.
__global__ void __launch_bounds__(kNoAllocThreads)
    k_glsc2_mask_noalloc(const double* __restrict__ a, const double* __restrict__ b, const int* __restrict__ mask,
                         int m, double* __restrict__ scratch, double* __restrict__ out) {
  __shared__ double sred[kNoAllocThreads / 32];
  __shared__ int s_last;
  const int64_t base = (int64_t)blockIdx.x * kNoAllocPerBlock;
  double s = 0.0;
#pragma unroll
  for (int q = 0; q < kNoAllocPerThread; ++q) {
    const int64_t i = base + q * kNoAllocThreads + threadIdx.x;
    if (i < m) {
      const int l = mask[i] - 1;
      s += a[l] * b[l];
    }
  }
  s = na_block_sum(s, sred);
  unsigned long long* ticket = reinterpret_cast<unsigned long long*>(scratch + kNoAllocMaxBlocks + 1);
  if (threadIdx.x == 0) {
    scratch[blockIdx.x] = s;
    __threadfence();
    s_last = (atomicAdd(ticket, 1ull) == (unsigned long long)(gridDim.x - 1));
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  double t = 0.0;
  for (int blk = threadIdx.x; blk < (int)gridDim.x; blk += kNoAllocThreads) t += __ldcg(scratch + blk);
  t = na_block_sum(t, sred);
  if (threadIdx.x == 0) {
    scratch[kNoAllocMaxBlocks] = t;
    *out = t;
    *ticket = 0ull;
  }
}

// Device address of the scratch array, looked up once per device.
static std::mutex g_na_mu;
static double* g_na_addr[64] = {};

static int noalloc_scratch(double** ptr) {
  int dev = 0;
  NTG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    set_error("ntg_glsc2_mask_noalloc: device ordinal %d out of range", dev);
    return NTG_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(g_na_mu);
  if (!g_na_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_glsc2_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      set_error("ntg_glsc2_mask_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
      return NTG_ERR_CUDA;
    }
    g_na_addr[dev] = static_cast<double*>(p);
  }
  *ptr = g_na_addr[dev];
  return NTG_OK;
}

}  // namespace ntg

using namespace ntg;

extern "C" int ntg_glsc2_mask_noalloc(const double* a_d, const double* b_d, const int* mask_d, int mask_size,
                                      double* out_d, void* stream) {
  clear_error();
  NTG_CHECK_ARG(out_d, "ntg_glsc2_mask_noalloc: null output pointer");
  if (mask_size < 0) {
    set_error("ntg_glsc2_mask_noalloc: negative mask size %d", mask_size);
    return NTG_ERR_INVALID;
  }
  if ((int64_t)mask_size > kNoAllocMaxEntries) {
    set_error("ntg_glsc2_mask_noalloc: mask of %d entries exceeds the maximum of %lld (static scratch of %d blocks)",
              mask_size, (long long)kNoAllocMaxEntries, kNoAllocMaxBlocks);
    return NTG_ERR_INVALID;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (mask_size == 0) {
    NTG_CUDA_TRY(cudaMemsetAsync(out_d, 0, sizeof(double), s));
    return NTG_OK;
  }
  NTG_CHECK_ARG(a_d && b_d && mask_d, "ntg_glsc2_mask_noalloc: null input pointer");
  double* scratch = nullptr;
  NTG_TRY(noalloc_scratch(&scratch));
  // the ticket must start at zero
  NTG_CUDA_TRY(cudaMemsetAsync(scratch + kNoAllocMaxBlocks + 1, 0, sizeof(double), s));
  const int grid = (int)(((int64_t)mask_size + kNoAllocPerBlock - 1) / kNoAllocPerBlock);
  { k_glsc2_mask_noalloc<<<grid, kNoAllocThreads, 0, s>>>(a_d, b_d, mask_d, mask_size, scratch, out_d); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}
