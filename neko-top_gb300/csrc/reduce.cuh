// Deterministic block + grid reductions in FP64.
//
// Every reducing kernel accumulates NL partial sums per thread, reduces them
// inside the block with warp shuffles in a fixed tree, writes one partial per
// block to part[lane * kRedSlots + blockIdx.x], and the last block to finish
// (atomic ticket in Scalars) sums the partials in index order and hands the
// totals to a finaliser run by thread 0.  The result depends only on the
// grid size, never on block scheduling, so two runs are bit-identical.
#pragma once
#include "common.cuh"

namespace ntg {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum of NL values; result valid in thread 0.  NT = blockDim.
template <int NL>
__device__ __forceinline__ void block_sum(double (&v)[NL], double (*sred)[32]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int q = 0; q < NL; ++q) v[q] = warp_sum(v[q]);
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < NL; ++q) sred[q][warp] = v[q];
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int q = 0; q < NL; ++q) {
      double t = lane < nwarps ? sred[q][lane] : 0.0;
      v[q] = warp_sum(t);
    }
  }
  __syncthreads();
}

// Grid reduction with a last-block finaliser.  Must be called by every
// thread of every block (blockDim.x threads, 1-D thread index).
template <int NL, typename Fin>
__device__ __forceinline__ void grid_reduce(double (&v)[NL], double* __restrict__ part, Scalars* sc, Fin fin) {
  __shared__ double sred[NL][32];
  __shared__ int s_last;
  block_sum<NL>(v, sred);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < NL; ++q) part[q * kRedSlots + blockIdx.x] = v[q];
    __threadfence();
    unsigned t = atomicAdd(&sc->ticket, 1u);
    s_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  double acc[NL];
#pragma unroll
  for (int q = 0; q < NL; ++q) {
    acc[q] = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) acc[q] += __ldcg(part + q * kRedSlots + b);
  }
  block_sum<NL>(acc, sred);
  if (threadIdx.x == 0) {
    fin(acc, sc);
    sc->ticket = 0;
    __threadfence();
  }
}

// Fused dot finaliser: pap = sum p.(A p)_local; alpha = rz / pap.
struct FinPap {
  __device__ void operator()(const double* acc, Scalars* sc) const {
    double pap = acc[0];
    sc->pap = pap;
    if (!(pap > 0.0) || !isfinite(pap)) {
      sc->status = isfinite(pap) ? NTG_BREAKDOWN : NTG_NONFINITE;
      sc->done = 1;
      sc->alpha = 0.0;
    } else {
      sc->alpha = sc->rz / pap;
    }
  }
};

// (r, z) finaliser of a preconditioned CG step.
struct FinRz {
  int mode;  // 0 iteration / confirmation: beta = new / rz; 1 replacement: rz only; 3 start: rz, beta = 0
  __device__ void operator()(const double* acc, Scalars* sc) const {
    const double rz = acc[0];
    if (!isfinite(rz) || !(rz > 0.0)) {
      sc->status = isfinite(rz) ? NTG_BREAKDOWN : NTG_NONFINITE;
      sc->done = 1;
      return;
    }
    if (mode == 0) sc->beta = rz / sc->rz;
    if (mode == 3) sc->beta = 0.0;
    sc->rz = rz;
  }
};

}  // namespace ntg
