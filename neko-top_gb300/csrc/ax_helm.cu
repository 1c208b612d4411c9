// Matrix-free spectral-element Helmholtz operator (ax_helm) on sm_103a:
//   w = h1 * (D^T G D) u + h2 * B * u   (element-local, unassembled)
//
// Replaces Neko's ax_helm (created by ax_helm_factory(Ax, full_formulation =
// .false.) at sources/mapping_functions/PDE_filter_mapping.f90:177 and
// sources/adjoint/adjoint_pnpn.f90:207,217; applied inside ksp%solve).
//
// Mapping: one element per 64-thread group (thread (i,j) owns the column
// u(i,j,0..LX-1)); EPB elements per block.  The t-direction contraction runs
// on the column held in registers with D taken from the kernel-parameter
// (constant) bank at compile-time indices; the r- and s-direction
// contractions read the element tile from shared memory, where a warp's
// reads are broadcasts or 8 consecutive words (conflict-free).  Each thread
// keeps its D rows/columns in registers.  The transposed contractions reuse
// the same pattern on the metric-mixed fluxes.
//
// Bounds: FP64 is FP64-pipe bound on GB300 (about 1.2 TFLOP/s against ~116
// flop per DOF); FP32 is HBM bound (32 B/DOF for Poisson).
#include "common.cuh"
#include "reduce.cuh"

namespace ntg {

template <typename T, int LX>
struct DParam {
  T d[LX * LX];
};

template <typename T, int LX>
struct AxShape {
  static constexpr int LX2 = LX * LX, LX3 = LX * LX * LX;
  static constexpr int EPB_T = (256 / LX2) < 1 ? 1 : ((256 / LX2) > 8 ? 8 : 256 / LX2);
  static constexpr int EPB_S = 49152 / (3 * LX3 * (int)sizeof(T));
  static constexpr int EPB = EPB_T < EPB_S ? EPB_T : (EPB_S < 1 ? 1 : EPB_S);
  static constexpr int NW = LX2 * EPB;             // working threads
  static constexpr int NT = (NW + 31) / 32 * 32;   // launched threads
};

template <typename T, int LX, bool H1ARR, bool H2, bool DOT>
__global__ void __launch_bounds__(AxShape<T, LX>::NT)
    k_ax_helm(T* __restrict__ w, const T* __restrict__ u, const T* __restrict__ g11, const T* __restrict__ g12,
              const T* __restrict__ g13, const T* __restrict__ g22, const T* __restrict__ g23,
              const T* __restrict__ g33, const T* __restrict__ h1, T h1c, const T* __restrict__ hB, int64_t nelv,
              const __grid_constant__ DParam<T, LX> Dp, double* __restrict__ part, Scalars* sc) {
  using S = AxShape<T, LX>;
  constexpr int LX2 = S::LX2, LX3 = S::LX3, EPB = S::EPB;
  if (DOT && sc->done) return;
  __shared__ T s_u[EPB][LX3];
  __shared__ T s_r[EPB][LX3];
  __shared__ T s_s[EPB][LX3];
  const int tid = threadIdx.x;
  const bool worker = tid < S::NW;
  const int le = worker ? tid / LX2 : 0;  // element slot in the block
  const int ij = worker ? tid - le * LX2 : 0;
  const int i = ij % LX, j = ij / LX;
  T Dri[LX], Dsj[LX], DTi[LX], DTj[LX];
#pragma unroll
  for (int l = 0; l < LX; ++l) {
    Dri[l] = Dp.d[i * LX + l];
    Dsj[l] = Dp.d[j * LX + l];
    DTi[l] = Dp.d[l * LX + i];
    DTj[l] = Dp.d[l * LX + j];
  }
  T dot = 0;  // per-thread partial in the kernel's precision (FP64 math is scarce on GB300)
  const int64_t ngroups = (nelv + EPB - 1) / EPB;
  for (int64_t grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
    const int64_t e = grp * EPB + le;
    const bool active = worker && e < nelv;
    const int64_t base = e * LX3 + ij;
    T ureg[LX];
#pragma unroll
    for (int k = 0; k < LX; ++k) {
      ureg[k] = active ? u[base + k * LX2] : T(0);
      if (worker) s_u[le][ij + k * LX2] = ureg[k];
    }
    __syncthreads();
    T wt[LX];
#pragma unroll
    for (int k = 0; k < LX; ++k) {
      T ur = 0, us = 0, ut = 0;
#pragma unroll
      for (int l = 0; l < LX; ++l) {
        ur = fma(Dri[l], s_u[le][k * LX2 + j * LX + l], ur);
        us = fma(Dsj[l], s_u[le][k * LX2 + l * LX + i], us);
        ut = fma(Dp.d[k * LX + l], ureg[l], ut);
      }
      T a11 = 0, a12 = 0, a13 = 0, a22 = 0, a23 = 0, a33 = 0, hh = h1c;
      if (active) {
        const int64_t q = base + k * LX2;
        a11 = g11[q]; a12 = g12[q]; a13 = g13[q]; a22 = g22[q]; a23 = g23[q]; a33 = g33[q];
        if (H1ARR) hh = h1[q];
      }
      T wr = a11 * ur + a12 * us + a13 * ut;
      T ws = a12 * ur + a22 * us + a23 * ut;
      T wtt = a13 * ur + a23 * us + a33 * ut;
      if (worker) {
        s_r[le][ij + k * LX2] = hh * wr;
        s_s[le][ij + k * LX2] = hh * ws;
      }
      wt[k] = hh * wtt;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < LX; ++k) {
      T acc = 0;
#pragma unroll
      for (int l = 0; l < LX; ++l) {
        acc = fma(DTi[l], s_r[le][k * LX2 + j * LX + l], acc);
        acc = fma(DTj[l], s_s[le][k * LX2 + l * LX + i], acc);
        acc = fma(Dp.d[l * LX + k], wt[l], acc);
      }
      if (active) {
        const int64_t q = base + k * LX2;
        if (H2) acc = fma(hB[q], ureg[k], acc);
        w[q] = acc;
        if (DOT) dot = fma(ureg[k], acc, dot);
      }
    }
    __syncthreads();
  }
  if (DOT) {
    double v[1] = {(double)dot};
    grid_reduce<1>(v, part, sc, FinPap());
  }
}

// TMA-pipelined FP32 kernel for lx = 8 (ax_helm_f32_tma.cu); returns
// NTG_ERR_UNSUPPORTED when a pointer is not 16-byte aligned.
int ax_f32_tma_launch(ntg_plan* p, float* w, const float* u, const float* const* g, const float* h1, float h1c,
                      const float* hB, Scalars* sc, cudaStream_t s);

template <typename T, int LX>
static int launch_lx(ntg_plan* p, T* w, const T* u, const T* const* g, const T* h1, T h1c, const T* hB,
                     Scalars* sc, cudaStream_t s) {
  constexpr int EPB = AxShape<T, LX>::EPB;
  constexpr int NT = AxShape<T, LX>::NT;
  DParam<T, LX> Dp;
  for (int q = 0; q < LX * LX; ++q) Dp.d[q] = (T)p->D[q];
  int64_t ngroups = (p->nelv + EPB - 1) / EPB;
  int64_t cap = sc ? kRedSlots : (int64_t)num_sms() * 32;
  int grid = (int)(ngroups < cap ? ngroups : cap);
  const bool h1arr = h1 != nullptr, h2 = hB != nullptr;
#define NTG_AX_CASE(H1A, HH2, DT)                                                                              \
  if (h1arr == H1A && h2 == HH2 && (sc != nullptr) == DT) {                                                 \
    { k_ax_helm<T, LX, H1A, HH2, DT><<<grid, NT, 0, s>>>(w, u, g[0], g[1], g[2], g[3], g[4], g[5], h1, h1c, \
                                                            hB, p->nelv, Dp, p->red_part, sc); NTG_COUNT_LAUNCH(); }              \
  }
  NTG_AX_CASE(false, false, false)
  NTG_AX_CASE(false, true, false)
  NTG_AX_CASE(true, false, false)
  NTG_AX_CASE(true, true, false)
  NTG_AX_CASE(false, false, true)
  NTG_AX_CASE(false, true, true)
  NTG_AX_CASE(true, false, true)
  NTG_AX_CASE(true, true, true)
#undef NTG_AX_CASE
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

template <typename T>
static int ax_dispatch(ntg_plan* p, T* w, const T* u, const T* const* g, const T* h1, T h1c, const T* hB,
                       Scalars* sc, cudaStream_t s) {
  switch (p->lx) {
    case 2: return launch_lx<T, 2>(p, w, u, g, h1, h1c, hB, sc, s);
    case 3: return launch_lx<T, 3>(p, w, u, g, h1, h1c, hB, sc, s);
    case 4: return launch_lx<T, 4>(p, w, u, g, h1, h1c, hB, sc, s);
    case 5: return launch_lx<T, 5>(p, w, u, g, h1, h1c, hB, sc, s);
    case 6: return launch_lx<T, 6>(p, w, u, g, h1, h1c, hB, sc, s);
    case 7: return launch_lx<T, 7>(p, w, u, g, h1, h1c, hB, sc, s);
    case 8: return launch_lx<T, 8>(p, w, u, g, h1, h1c, hB, sc, s);
    case 9: return launch_lx<T, 9>(p, w, u, g, h1, h1c, hB, sc, s);
    case 10: return launch_lx<T, 10>(p, w, u, g, h1, h1c, hB, sc, s);
    default: set_error("ax_helm: lx=%d not compiled", p->lx); return NTG_ERR_UNSUPPORTED;
  }
}

int ax_launch(ntg_plan* p, double* w, const double* u, Scalars* dot_scal, int, cudaStream_t s) {
  const double* g[6] = {p->g[0], p->g[1], p->g[2], p->g[3], p->g[4], p->g[5]};
  timer_start(TM_AX64, s);
  int st = ax_dispatch<double>(p, w, u, g, p->h1_const ? nullptr : p->h1, p->h1c, p->ifh2 ? p->hB : nullptr,
                               dot_scal, s);
  timer_stop(TM_AX64, s);
  return st;
}

int ax_launch_f32(ntg_plan* p, float* w, const float* u, Scalars* dot_scal, int, cudaStream_t s) {
  NTG_TRY(ensure_fp32(p));
  const float* g[6] = {p->gf[0], p->gf[1], p->gf[2], p->gf[3], p->gf[4], p->gf[5]};
  timer_start(TM_AX32, s);
  const float* h1 = p->h1_const ? nullptr : p->h1f;
  const float* hB = p->ifh2 ? p->hBf : nullptr;
  int st = NTG_ERR_UNSUPPORTED;
  if (p->lx == 8 && p->use_tma) st = ax_f32_tma_launch(p, w, u, g, h1, (float)p->h1c, hB, dot_scal, s);
  if (st == NTG_ERR_UNSUPPORTED) st = ax_dispatch<float>(p, w, u, g, h1, (float)p->h1c, hB, dot_scal, s);
  timer_stop(TM_AX32, s);
  return st;
}

}  // namespace ntg

using namespace ntg;

extern "C" int ntg_ax_helm(ntg_plan* plan, double* w_d, const double* u_d) {
  clear_error();
  NTG_CHECK_ARG(plan && w_d && u_d, "ntg_ax_helm: null argument");
  return ax_launch(plan, w_d, u_d, nullptr, 0, plan->stream);
}

extern "C" int ntg_ax_helm_f32(ntg_plan* plan, float* w_d, const float* u_d) {
  clear_error();
  NTG_CHECK_ARG(plan && w_d && u_d, "ntg_ax_helm_f32: null argument");
  return ax_launch_f32(plan, w_d, u_d, nullptr, 0, plan->stream);
}
