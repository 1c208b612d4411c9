// FP64 FMA throughput probe: the denominator the FP64-bound kernels (FP64
// ax_helm, the derivative and dealiasing kernels, the MMA) are reported
// against.  Eight independent FMA chains per thread, grid = 8 blocks of 256
// threads per SM, timed with CUDA events on the given stream.
//
// A measurement tool, not part of the drop-in: it is built into its own
// library (lib/libntgb300_probe.so) that only bench.py --fp64-peak loads.
#include <cuda_runtime.h>

namespace {

__global__ void __launch_bounds__(256) k_fp64_fma(double* __restrict__ out, int iters, double c, double d) {
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = 1.0 + 1e-3 * (threadIdx.x + k);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fma(a[k], c, d);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the chains live
}

}  // namespace

// Returns 0 and the FMA rate in TFLOP/s (an FMA counts 2), or a CUDA error
// code.
extern "C" __attribute__((visibility("default"))) int ntgprobe_fp64(int iters, double* tflops, void* stream) {
  if (iters <= 0 || iters > (1 << 24) || !tflops) return -1;
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) return -2;
  const int blocks = sms * 8, threads = 256;
  double* out = nullptr;
  cudaError_t err = cudaMalloc(&out, sizeof(double) * blocks * threads);
  if (err != cudaSuccess) return (int)err;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fp64_fma<<<blocks, threads, 0, s>>>(out, iters / 8 + 1, 0.999999, 1e-7);  // warm-up
  cudaEventRecord(e0, s);
  k_fp64_fma<<<blocks, threads, 0, s>>>(out, iters, 0.999999, 1e-7);
  cudaEventRecord(e1, s);
  err = cudaEventSynchronize(e1);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return (int)err;
  *tflops = 2.0 * 8.0 * (double)iters * blocks * threads / (ms * 1e-3) / 1e12;
  return 0;
}
