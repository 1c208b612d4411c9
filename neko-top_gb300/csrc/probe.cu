// FP64 FMA throughput probe: the denominator the FP64-bound kernels (FP64
// ax_helm, the derivative and dealiasing kernels, the MMA) are reported
// against.  Eight independent FMA chains per thread, grid = 8 blocks of 256
// threads per SM, timed with CUDA events on the given stream.
#include "common.cuh"

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

extern "C" int ntg_probe_fp64(int iters, double* tflops, void* stream) {
  ntg::clear_error();
  NTG_CHECK_ARG(iters > 0 && iters <= (1 << 24) && tflops, "ntg_probe_fp64: bad argument");
  cudaStream_t s = (cudaStream_t)stream;
  const int blocks = ntg::num_sms() * 8, threads = 256;
  double* out = nullptr;
  NTG_TRY(ntg::dev_alloc(&out, (size_t)blocks * threads));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fp64_fma<<<blocks, threads, 0, s>>>(out, iters / 8 + 1, 0.999999, 1e-7);  // warm-up
  cudaEventRecord(e0, s);
  k_fp64_fma<<<blocks, threads, 0, s>>>(out, iters, 0.999999, 1e-7);
  cudaEventRecord(e1, s);
  NTG_COUNT_LAUNCH();
  NTG_COUNT_LAUNCH();
  const cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ntg::dev_free(out);
  if (err != cudaSuccess) {
    ntg::set_error("ntg_probe_fp64: %s", cudaGetErrorString(err));
    return NTG_ERR_CUDA;
  }
  *tflops = 2.0 * 8.0 * (double)iters * blocks * threads / (ms * 1e-3) / 1e12;
  return NTG_OK;
}
