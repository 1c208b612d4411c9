// FP32 ax_helm for lx = 8, HBM-bound, fed by bulk-copy (TMA) pipelines.
//
// The FP32 operator streams (2 + 6 + c) * 4 bytes per local DOF and does
// ~57 FMA per DOF, well under the FP32 roof, so its speed is the HBM stream.
// Each block is persistent (one per SM) and walks groups of 4 consecutive
// elements.  For every group one thread issues cp.async.bulk copies of the
// group's u, G11..G33 (and h1 / h2*B) -- 8 KB contiguous per array -- into a
// shared-memory stage and arms an mbarrier with the byte count; NSTAGE
// stages are in flight, so the copies of the next groups overlap the
// contractions of the current one.  Compute is the same column mapping as
// the generic kernel (thread (i,j) owns the column over k; r/s contractions
// read the staged tile, t on registers).  w is stored straight to global
// memory (coalesced 128-byte rows).  Every mbarrier wait is bounded: on
// timeout the kernel raises a flag, drains its own copies (bounded) and
// returns, so it can never hang the GPU.
#include "common.cuh"
#include "reduce.cuh"

namespace ntg {

namespace tma {

constexpr int LX = 8, LX2 = 64, LX3 = 512;
constexpr int EPB = 4;                       // elements per group
constexpr int NT = LX2 * EPB;                // 256 threads
constexpr int ARR_BYTES = EPB * LX3 * 4;     // 8 KB per array per group
constexpr unsigned kSpinLimit = 1u << 26;    // bounded waits (seconds)

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

template <int NARR>
struct Stages {
  static constexpr int STAGE_BYTES = NARR * ARR_BYTES;
  static constexpr int NSTAGE = (3 * STAGE_BYTES + 2 * EPB * LX3 * 4 + 1024 <= 220 * 1024) ? 3 : 2;
  static constexpr int SMEM = NSTAGE * STAGE_BYTES + 2 * EPB * LX3 * 4 + 64;
};

struct F32Params {
  float d[LX * LX];
};

// Arrays in stage order: 0 u, 1..6 G11 G12 G13 G22 G23 G33, then h1, then hB.
template <bool H1ARR, bool H2, bool DOT>
__global__ void __launch_bounds__(NT, 1)
    k_ax_helm_f32_tma(float* __restrict__ w, const float* __restrict__ u, const float* __restrict__ g11,
                      const float* __restrict__ g12, const float* __restrict__ g13, const float* __restrict__ g22,
                      const float* __restrict__ g23, const float* __restrict__ g33, const float* __restrict__ h1,
                      float h1c, const float* __restrict__ hB, int64_t nelv, const __grid_constant__ F32Params Dp,
                      double* __restrict__ part, Scalars* sc, int* __restrict__ err) {
  constexpr int NARR = 7 + (H1ARR ? 1 : 0) + (H2 ? 1 : 0);
  using St = Stages<NARR>;
  constexpr int NSTAGE = St::NSTAGE;
  if (DOT && sc->done) return;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  float* stage_base = reinterpret_cast<float*>(smem_raw);
  float* s_r = reinterpret_cast<float*>(smem_raw + NSTAGE * St::STAGE_BYTES);
  float* s_s = s_r + EPB * LX3;
  uint64_t* bars = reinterpret_cast<uint64_t*>(s_s + EPB * LX3);

  const int tid = threadIdx.x;
  const int le = tid >> 6;
  const int ij = tid & 63;
  const int i = ij & 7, j = ij >> 3;
  const int64_t ngroups = (nelv + EPB - 1) / EPB;
  const float* srcs[9] = {u, g11, g12, g13, g22, g23, g33, H1ARR ? h1 : nullptr, H2 ? hB : nullptr};

  if (tid == 0) {
    for (int s = 0; s < NSTAGE; ++s) mbar_init(&bars[s], 1);
    fence_mbar_init();
  }
  __syncthreads();

  auto issue = [&](int64_t grp, int s) {
    const int64_t e0 = grp * EPB;
    const int nvalid = (int)((nelv - e0) < EPB ? (nelv - e0) : EPB);
    const unsigned bytes = (unsigned)nvalid * LX3 * 4;
    fence_proxy_async();
    mbar_expect_tx(&bars[s], bytes * NARR);
    float* dst = stage_base + (size_t)s * (St::STAGE_BYTES / 4);
    int a = 0;
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      if (q == 7 && !H1ARR) continue;
      if (q == 8 && !H2) continue;
      bulk_g2s(dst + (size_t)a * (ARR_BYTES / 4), srcs[q] + e0 * LX3, bytes, &bars[s]);
      ++a;
    }
  };

  // my groups: blockIdx.x, blockIdx.x + gridDim.x, ...
  const int64_t my_first = blockIdx.x;
  const int64_t stride = gridDim.x;
  int64_t nmine = my_first < ngroups ? (ngroups - 1 - my_first) / stride + 1 : 0;
  if (tid == 0) {
    for (int s = 0; s < NSTAGE && s < nmine; ++s) issue(my_first + s * stride, s);
  }
  float Dri[LX], Dsj[LX], DTi[LX], DTj[LX];
#pragma unroll
  for (int l = 0; l < LX; ++l) {
    Dri[l] = Dp.d[i * LX + l];
    Dsj[l] = Dp.d[j * LX + l];
    DTi[l] = Dp.d[l * LX + i];
    DTj[l] = Dp.d[l * LX + j];
  }
  float dot = 0.f;
  bool failed = false;
  int64_t t_fail = 0;
  for (int64_t t = 0; t < nmine; ++t) {
    t_fail = t;
    const int s = (int)(t % NSTAGE);
    const unsigned parity = (unsigned)((t / NSTAGE) & 1);
    unsigned spins = 0;
    while (!mbar_try_wait(&bars[s], parity)) {
      if (++spins > kSpinLimit) {
        failed = true;
        break;
      }
    }
    if (__syncthreads_or(failed)) {
      failed = true;
      break;
    }
    const int64_t grp = my_first + t * stride;
    const int64_t e = grp * EPB + le;
    const bool active = e < nelv;
    const float* st = stage_base + (size_t)s * (St::STAGE_BYTES / 4);
    const float* su = st + le * LX3;
    const float* sg11 = st + 1 * (ARR_BYTES / 4) + le * LX3;
    const float* sg12 = st + 2 * (ARR_BYTES / 4) + le * LX3;
    const float* sg13 = st + 3 * (ARR_BYTES / 4) + le * LX3;
    const float* sg22 = st + 4 * (ARR_BYTES / 4) + le * LX3;
    const float* sg23 = st + 5 * (ARR_BYTES / 4) + le * LX3;
    const float* sg33 = st + 6 * (ARR_BYTES / 4) + le * LX3;
    const float* sh1 = st + 7 * (ARR_BYTES / 4) + le * LX3;
    const float* shB = st + (H1ARR ? 8 : 7) * (ARR_BYTES / 4) + le * LX3;
    float* mr = s_r + le * LX3;
    float* ms = s_s + le * LX3;
    float ureg[LX], wt[LX];
    if (active) {
#pragma unroll
      for (int k = 0; k < LX; ++k) ureg[k] = su[ij + k * LX2];
#pragma unroll
      for (int k = 0; k < LX; ++k) {
        float ur = 0.f, us = 0.f, ut = 0.f;
        const float4* row = reinterpret_cast<const float4*>(su + k * LX2 + j * LX);
        const float4 r0 = row[0], r1 = row[1];
        ur = fmaf(Dri[0], r0.x, ur); ur = fmaf(Dri[1], r0.y, ur); ur = fmaf(Dri[2], r0.z, ur);
        ur = fmaf(Dri[3], r0.w, ur); ur = fmaf(Dri[4], r1.x, ur); ur = fmaf(Dri[5], r1.y, ur);
        ur = fmaf(Dri[6], r1.z, ur); ur = fmaf(Dri[7], r1.w, ur);
#pragma unroll
        for (int l = 0; l < LX; ++l) {
          us = fmaf(Dsj[l], su[k * LX2 + l * LX + i], us);
          ut = fmaf(Dp.d[k * LX + l], ureg[l], ut);
        }
        const int q = ij + k * LX2;
        const float a11 = sg11[q], a12 = sg12[q], a13 = sg13[q], a22 = sg22[q], a23 = sg23[q], a33 = sg33[q];
        const float hh = H1ARR ? sh1[q] : h1c;
        mr[q] = hh * (a11 * ur + a12 * us + a13 * ut);
        ms[q] = hh * (a12 * ur + a22 * us + a23 * ut);
        wt[k] = hh * (a13 * ur + a23 * us + a33 * ut);
      }
    }
    __syncthreads();
    if (active) {
      float* wout = w + e * LX3;
#pragma unroll
      for (int k = 0; k < LX; ++k) {
        float acc = 0.f;
        const float4* rrow = reinterpret_cast<const float4*>(mr + k * LX2 + j * LX);
        const float4 r0 = rrow[0], r1 = rrow[1];
        acc = fmaf(DTi[0], r0.x, acc); acc = fmaf(DTi[1], r0.y, acc); acc = fmaf(DTi[2], r0.z, acc);
        acc = fmaf(DTi[3], r0.w, acc); acc = fmaf(DTi[4], r1.x, acc); acc = fmaf(DTi[5], r1.y, acc);
        acc = fmaf(DTi[6], r1.z, acc); acc = fmaf(DTi[7], r1.w, acc);
#pragma unroll
        for (int l = 0; l < LX; ++l) {
          acc = fmaf(DTj[l], ms[k * LX2 + l * LX + i], acc);
          acc = fmaf(Dp.d[l * LX + k], wt[l], acc);
        }
        const int q = ij + k * LX2;
        if (H2) acc = fmaf(shB[q], ureg[k], acc);
        wout[q] = acc;
        if (DOT) dot = fmaf(ureg[k], acc, dot);
      }
    }
    __syncthreads();  // stage s and s_r/s_s are free again
    if (tid == 0 && t + NSTAGE < nmine) issue(my_first + (t + NSTAGE) * stride, s);
  }
  if (failed) {
    if (tid == 0) {
      atomicExch(err, 1);
      // drain: the groups t_fail .. t_fail+NSTAGE-1 were issued and not yet
      // consumed; wait (bounded) for each one's phase before leaving
      for (int64_t g = t_fail; g < t_fail + NSTAGE && g < nmine; ++g) {
        const int s = (int)(g % NSTAGE);
        const unsigned par = (unsigned)((g / NSTAGE) & 1);
        unsigned spins = 0;
        while (spins < kSpinLimit && !mbar_try_wait(&bars[s], par)) ++spins;
      }
    }
    __syncthreads();
    if (DOT && tid == 0) {
      sc->status = NTG_ERR_CUDA;
      sc->done = 1;
    }
    return;
  }
  if (DOT) {
    double v[1] = {(double)dot};
    grid_reduce<1>(v, part, sc, FinPap());
  }
}

template <bool H1ARR, bool H2, bool DOT>
static int launch_variant(ntg_plan* p, float* w, const float* u, const float* const* g, const float* h1, float h1c,
                          const float* hB, Scalars* sc, cudaStream_t s) {
  constexpr int NARR = 7 + (H1ARR ? 1 : 0) + (H2 ? 1 : 0);
  constexpr int SMEM = Stages<NARR>::SMEM;
  static bool attr_done[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  auto kern = k_ax_helm_f32_tma<H1ARR, H2, DOT>;
  if (dev >= 0 && dev < 64 && !attr_done[dev]) {
    NTG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM));
    attr_done[dev] = true;
  }
  F32Params Dp;
  for (int q = 0; q < LX * LX; ++q) Dp.d[q] = p->Df[q];
  const int64_t ngroups = (p->nelv + EPB - 1) / EPB;
  int grid = num_sms();
  if (ngroups < grid) grid = (int)ngroups;
  { kern<<<grid, NT, SMEM, s>>>(w, u, g[0], g[1], g[2], g[3], g[4], g[5], h1, h1c, hB, p->nelv, Dp, p->red_part, sc, p->dev_err); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

}  // namespace tma

static bool aligned16(const void* q) { return q == nullptr || (reinterpret_cast<uintptr_t>(q) & 15u) == 0; }

int ax_f32_tma_launch(ntg_plan* p, float* w, const float* u, const float* const* g, const float* h1, float h1c,
                      const float* hB, Scalars* sc, cudaStream_t s) {
  if (p->lx != 8 || !p->dev_err) return NTG_ERR_UNSUPPORTED;
  // a bulk copy must start on a 16-byte boundary: every element group starts
  // at a multiple of 2 KB from the array base, so the bases decide
  const void* ptrs[10] = {w, u, g[0], g[1], g[2], g[3], g[4], g[5], h1, hB};
  for (const void* q : ptrs)
    if (!aligned16(q)) return NTG_ERR_UNSUPPORTED;
  const bool h1a = h1 != nullptr, h2 = hB != nullptr, dot = sc != nullptr;
#define NTG_TMA_CASE(A, B, C)                                                     \
  if (h1a == A && h2 == B && dot == C) return tma::launch_variant<A, B, C>(p, w, u, g, h1, h1c, hB, sc, s);
  NTG_TMA_CASE(false, false, false)
  NTG_TMA_CASE(false, true, false)
  NTG_TMA_CASE(true, false, false)
  NTG_TMA_CASE(true, true, false)
  NTG_TMA_CASE(false, false, true)
  NTG_TMA_CASE(false, true, true)
  NTG_TMA_CASE(true, false, true)
  NTG_TMA_CASE(true, true, true)
#undef NTG_TMA_CASE
  return NTG_ERR_UNSUPPORTED;
}

}  // namespace ntg

using namespace ntg;

// Select the FP32 Ax path of a plan: 1 = bulk-copy pipeline (lx = 8), 0 =
// the generic kernel.
extern "C" int ntg_plan_set_ax_path(ntg_plan* plan, int use_tma) {
  clear_error();
  NTG_CHECK_ARG(plan, "ntg_plan_set_ax_path: null plan");
  plan->use_tma = use_tma ? 1 : 0;
  return NTG_OK;
}

// Select the gather-scatter kernel: 1 = by multiplicity class (default),
// 0 = one thread per shared group.  Both give bit-identical results.
extern "C" int ntg_plan_set_gs_path(ntg_plan* plan, int by_class) {
  clear_error();
  NTG_CHECK_ARG(plan, "ntg_plan_set_gs_path: null plan");
  plan->gs_classes = by_class ? 1 : 0;
  return NTG_OK;
}

// 1 if a bounded wait of a kernel of this plan ran out (the flag is cleared).
extern "C" int ntg_plan_check_error(ntg_plan* plan, int* flag) {
  clear_error();
  NTG_CHECK_ARG(plan && flag, "ntg_plan_check_error: null argument");
  int h = 0;
  NTG_CUDA_TRY(cudaMemcpyAsync(&h, plan->dev_err, sizeof(int), cudaMemcpyDeviceToHost, plan->stream));
  NTG_CUDA_TRY(cudaStreamSynchronize(plan->stream));
  if (h) NTG_CUDA_TRY(cudaMemsetAsync(plan->dev_err, 0, sizeof(int), plan->stream));
  *flag = h;
  return NTG_OK;
}
