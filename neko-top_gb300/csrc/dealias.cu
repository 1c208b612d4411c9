// Dealiased (over-integrated) adjoint and linearised advection, FP64
// (sources/adjoint/adv_adjoint_dealias.f90: init_dealias :137-224,
// compute_adjoint_advection_dealias :235-462, compute_linear_advection_dealias
// :470-600).  The fields are interpolated from the LX GLL points to LXD
// Gauss-Legendre points per direction (J), the products are formed there with
// the GL weights and the metric cofactors interpolated to GL, and the result
// comes back with J^T:
//
//   adjoint  f_i -= J^T [ sum_j u_j opgrad_i(Ub_j) + sum_d cdtp_d(u_i Ub_d) ]
//   linear   f_i -= J^T [ u . opgrad(Ub_i) + Ub . opgrad(u_i) ]
//
// One element per block, everything between the GLL loads and the GLL
// update in shared memory (12 GL tiles + interpolation buffers: 185 KB at
// LX = 8, LXD = 12), so the six interpolated fields, the 27 GL derivatives
// and the fluxes never touch HBM; only the GL cofactors (9 doubles per GL
// point, interpolated once at create) stream from memory.  The reference
// round-trips each of those through device arrays (20 GL-sized scratch
// fields).  The sums are rewritten with contravariant fluxes V_r =
// sum_d drdx_d Ub_d (etc.), so the three cdtp of a component become one D^T
// contraction of u_i V and the linear term needs no contraction at all.
#include <cmath>

#include "deriv.cuh"

struct ntg_dealias {
  ntg_plan* p = nullptr;
  int lx = 0, lxd = 0;
  int64_t ngl = 0;  // nelv * lxd^3
  double J[16 * NTG_LXMAX];
  double Dg[16 * 16];
  double wg[16];
  double* met_gl = nullptr;  // 9 x ngl cofactors at the GL points
  int grid = 0;
  size_t smem = 0;
};

namespace ntg {
namespace dl {

constexpr int NT = 256;

template <int LX, int LXD>
struct GLMat {
  double J[LXD * LX];  // J[A * LX + a] = l_a(xg_A)
  double D[LXD * LXD]; // D[A * LXD + l] = l_l'(xg_A) on the GL points
  double w[LXD];
};

template <int LX, int LXD>
struct Smem {
  static constexpr int N3 = LXD * LXD * LXD, TA = LXD * LX * LX, TB = LXD * LXD * LX, G3 = LX * LX * LX;
  static constexpr int DOUBLES = 12 * N3 + TA + TB + G3 + LXD * LX + LXD * LXD + LXD;
  static constexpr size_t BYTES = sizeof(double) * DOUBLES;
};

// dst[C][B][A] = sum J[C][c] J[B][b] J[A][a] src[c][b][a] (block-cooperative)
template <int LX, int LXD>
__device__ __forceinline__ void to_gl(double* dst, const double* src, double* tA, double* tB, const double* J) {
  for (int t = threadIdx.x; t < LX * LX * LXD; t += NT) {
    const int A = t % LXD, cb = t / LXD;
    double acc = 0.0;
#pragma unroll
    for (int a = 0; a < LX; ++a) acc = fma(J[A * LX + a], src[cb * LX + a], acc);
    tA[t] = acc;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < LX * LXD * LXD; t += NT) {
    const int A = t % LXD, B = (t / LXD) % LXD, c = t / (LXD * LXD);
    double acc = 0.0;
#pragma unroll
    for (int b = 0; b < LX; ++b) acc = fma(J[B * LX + b], tA[(c * LX + b) * LXD + A], acc);
    tB[t] = acc;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < LXD * LXD * LXD; t += NT) {
    const int BA = t % (LXD * LXD), C = t / (LXD * LXD);
    double acc = 0.0;
#pragma unroll
    for (int c = 0; c < LX; ++c) acc = fma(J[C * LX + c], tB[c * LXD * LXD + BA], acc);
    dst[t] = acc;
  }
  __syncthreads();
}

// out[c][b][a] (+)= sign * sum J[C][c] J[B][b] J[A][a] src[C][B][A]; out in global memory
template <int LX, int LXD>
__device__ __forceinline__ void to_gll(double* __restrict__ out, const double* src, double* tA, double* tB,
                                       const double* J, bool sub) {
  for (int t = threadIdx.x; t < LX * LXD * LXD; t += NT) {
    const int BA = t % (LXD * LXD), c = t / (LXD * LXD);
    double acc = 0.0;
#pragma unroll
    for (int C = 0; C < LXD; ++C) acc = fma(J[C * LX + c], src[C * LXD * LXD + BA], acc);
    tB[t] = acc;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < LX * LX * LXD; t += NT) {
    const int A = t % LXD, b = (t / LXD) % LX, c = t / (LXD * LX);
    double acc = 0.0;
#pragma unroll
    for (int B = 0; B < LXD; ++B) acc = fma(J[B * LX + b], tB[(c * LXD + B) * LXD + A], acc);
    tA[t] = acc;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < LX * LX * LX; t += NT) {
    const int a = t % LX, cb = t / LX;
    double acc = 0.0;
#pragma unroll
    for (int A = 0; A < LXD; ++A) acc = fma(J[A * LX + a], tA[cb * LXD + A], acc);
    if (sub) out[t] -= acc;
    else out[t] = acc;
  }
  __syncthreads();
}

template <int LXD>
__device__ __forceinline__ void glgrad(const double* s, const double* D, int A, int B, int C, double& r, double& q,
                                       double& t) {
  constexpr int L2 = LXD * LXD;
  r = q = t = 0.0;
#pragma unroll
  for (int l = 0; l < LXD; ++l) {
    r = fma(D[A * LXD + l], s[C * L2 + B * LXD + l], r);
    q = fma(D[B * LXD + l], s[C * L2 + l * LXD + A], q);
    t = fma(D[C * LXD + l], s[l * L2 + B * LXD + A], t);
  }
}

template <int LX, int LXD>
__device__ __forceinline__ double* stage_mats(double* sm, const GLMat<LX, LXD>& M, double*& J, double*& D,
                                              double*& w) {
  using S = Smem<LX, LXD>;
  J = sm + 12 * S::N3 + S::TA + S::TB + S::G3;
  D = J + LXD * LX;
  w = D + LXD * LXD;
  for (int t = threadIdx.x; t < LXD * LX; t += NT) J[t] = M.J[t];
  for (int t = threadIdx.x; t < LXD * LXD; t += NT) D[t] = M.D[t];
  for (int t = threadIdx.x; t < LXD; t += NT) w[t] = M.w[t];
  return sm;
}

// out = to_gl(in) (DIR 0) or to_gll(in) (DIR 1) for `nf` fields (stride = field size)
template <int LX, int LXD, int DIR>
__global__ void __launch_bounds__(NT) k_map(double* __restrict__ out, const double* __restrict__ in, int nf,
                                            int64_t nelv, int64_t n_in, int64_t n_out,
                                            const __grid_constant__ GLMat<LX, LXD> M) {
  using S = Smem<LX, LXD>;
  extern __shared__ double sm[];
  double *J, *D, *w;
  stage_mats<LX, LXD>(sm, M, J, D, w);
  double* tile = sm;
  double* tA = sm + 12 * S::N3;
  double* tB = tA + S::TA;
  constexpr int NIN = DIR == 0 ? S::G3 : S::N3;
  constexpr int NOUT = DIR == 0 ? S::N3 : S::G3;
  __syncthreads();
  for (int64_t e = blockIdx.x; e < nelv; e += gridDim.x) {
    for (int f = 0; f < nf; ++f) {
      const double* src = in + f * n_in + e * NIN;
      double* dst = out + f * n_out + e * NOUT;
      for (int t = threadIdx.x; t < NIN; t += NT) tile[t] = src[t];
      __syncthreads();
      if (DIR == 0) {
        to_gl<LX, LXD>(tile + S::N3, tile, tA, tB, J);
        for (int t = threadIdx.x; t < S::N3; t += NT) dst[t] = tile[S::N3 + t];
      } else {
        to_gll<LX, LXD>(dst, tile, tA, tB, J, false);
      }
      __syncthreads();
    }
  }
}

// MODE 0: adjoint, MODE 1: linear
template <int LX, int LXD, int MODE>
__global__ void __launch_bounds__(NT)
    k_adv(double* __restrict__ f0, double* __restrict__ f1, double* __restrict__ f2, const double* __restrict__ u0,
          const double* __restrict__ u1, const double* __restrict__ u2, const double* __restrict__ b0,
          const double* __restrict__ b1, const double* __restrict__ b2, const double* __restrict__ met, int64_t ngl,
          int64_t nelv, const __grid_constant__ GLMat<LX, LXD> M) {
  using S = Smem<LX, LXD>;
  constexpr int N3 = S::N3, G3 = S::G3;
  extern __shared__ double sm[];
  double *J, *D, *w;
  stage_mats<LX, LXD>(sm, M, J, D, w);
  double* sU = sm;            // 3 x N3: u on GL
  double* sB = sm + 3 * N3;   // 3 x N3: Ub on GL
  double* sW = sm + 6 * N3;   // 3 x N3: w3 V_r, w3 V_s, w3 V_t (adjoint)
  double* sT = sm + 9 * N3;   // 3 x N3: the GL result per component
  double* tA = sm + 12 * N3;
  double* tB = tA + S::TA;
  double* sIn = tB + S::TB;
  double* fo[3] = {f0, f1, f2};
  const double* ui[6] = {u0, u1, u2, b0, b1, b2};
  __syncthreads();
  for (int64_t e = blockIdx.x; e < nelv; e += gridDim.x) {
    for (int fld = 0; fld < 6; ++fld) {
      const double* src = ui[fld] + e * G3;
      for (int t = threadIdx.x; t < G3; t += NT) sIn[t] = src[t];
      __syncthreads();
      to_gl<LX, LXD>(fld < 3 ? sU + fld * N3 : sB + (fld - 3) * N3, sIn, tA, tB, J);
    }
    for (int t = threadIdx.x; t < N3; t += NT) {
      const int A = t % LXD, B = (t / LXD) % LXD, C = t / (LXD * LXD);
      const int64_t q = e * N3 + t;
      double c[9];
#pragma unroll
      for (int m = 0; m < 9; ++m) c[m] = met[m * ngl + q];
      const double w3 = w[A] * w[B] * w[C];
      const double U[3] = {sU[t], sU[N3 + t], sU[2 * N3 + t]};
      const double V[3] = {sB[t], sB[N3 + t], sB[2 * N3 + t]};
      const double vr = c[0] * V[0] + c[1] * V[1] + c[2] * V[2];
      const double vs = c[3] * V[0] + c[4] * V[1] + c[5] * V[2];
      const double vt = c[6] * V[0] + c[7] * V[1] + c[8] * V[2];
      if (MODE == 0) {
        double acc[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          double r, s, tt;
          glgrad<LXD>(sB + j * N3, D, A, B, C, r, s, tt);
#pragma unroll
          for (int i = 0; i < 3; ++i) acc[i] = fma(U[j], c[i] * r + c[3 + i] * s + c[6 + i] * tt, acc[i]);
        }
#pragma unroll
        for (int i = 0; i < 3; ++i) sT[i * N3 + t] = w3 * acc[i];
        sW[t] = w3 * vr;
        sW[N3 + t] = w3 * vs;
        sW[2 * N3 + t] = w3 * vt;
      } else {
        const double ur_ = c[0] * U[0] + c[1] * U[1] + c[2] * U[2];
        const double us_ = c[3] * U[0] + c[4] * U[1] + c[5] * U[2];
        const double ut_ = c[6] * U[0] + c[7] * U[1] + c[8] * U[2];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          double br, bs, bt, ar, as, at;
          glgrad<LXD>(sB + i * N3, D, A, B, C, br, bs, bt);
          glgrad<LXD>(sU + i * N3, D, A, B, C, ar, as, at);
          sT[i * N3 + t] = w3 * (br * ur_ + bs * us_ + bt * ut_ + ar * vr + as * vs + at * vt);
        }
      }
    }
    __syncthreads();
    if (MODE == 0) {
      constexpr int L2 = LXD * LXD;
      for (int t = threadIdx.x; t < N3; t += NT) {
        const int A = t % LXD, B = (t / LXD) % LXD, C = t / L2;
#pragma unroll 1
        for (int i = 0; i < 3; ++i) {
          const double* su = sU + i * N3;
          double acc = 0.0;
#pragma unroll
          for (int l = 0; l < LXD; ++l) {
            const int pr = C * L2 + B * LXD + l, ps = C * L2 + l * LXD + A, pt = l * L2 + B * LXD + A;
            acc = fma(D[l * LXD + A], su[pr] * sW[pr], acc);
            acc = fma(D[l * LXD + B], su[ps] * sW[N3 + ps], acc);
            acc = fma(D[l * LXD + C], su[pt] * sW[2 * N3 + pt], acc);
          }
          sT[i * N3 + t] += acc;
        }
      }
      __syncthreads();
    }
    for (int i = 0; i < 3; ++i) to_gll<LX, LXD>(fo[i] + e * G3, sT + i * N3, tA, tB, J, true);
  }
}

template <int LX, int LXD>
GLMat<LX, LXD> glmat(const ntg_dealias* d) {
  GLMat<LX, LXD> M;
  for (int q = 0; q < LXD * LX; ++q) M.J[q] = d->J[q];
  for (int q = 0; q < LXD * LXD; ++q) M.D[q] = d->Dg[q];
  for (int q = 0; q < LXD; ++q) M.w[q] = d->wg[q];
  return M;
}

template <typename F>
int dispatch(int lx, int lxd, F&& f) {
  if (lx == 4 && lxd == 6) return f(std::integral_constant<int, 4>{}, std::integral_constant<int, 6>{});
  if (lx == 5 && lxd == 7) return f(std::integral_constant<int, 5>{}, std::integral_constant<int, 7>{});
  if (lx == 6 && lxd == 9) return f(std::integral_constant<int, 6>{}, std::integral_constant<int, 9>{});
  if (lx == 7 && lxd == 10) return f(std::integral_constant<int, 7>{}, std::integral_constant<int, 10>{});
  if (lx == 8 && lxd == 12) return f(std::integral_constant<int, 8>{}, std::integral_constant<int, 12>{});
  set_error("dealiasing: (lx, lxd) = (%d, %d) not compiled; pairs: (4,6) (5,7) (6,9) (7,10) (8,12)", lx, lxd);
  return NTG_ERR_UNSUPPORTED;
}

// Gauss-Legendre points and weights (Newton on the three-term recurrence of
// P_n from the Chebyshev-like start cos(pi (i + 3/4) / (n + 1/2)))
void gauss_legendre(int n, double* x, double* w) {
  for (int i = 0; i < n; ++i) {
    double z = cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; ++k) {
        const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      const double dz = p1 / dp;
      z -= dz;
      if (fabs(dz) < 1e-16) break;
    }
    double p0 = 1.0, p1 = z;
    for (int k = 2; k <= n; ++k) {
      const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    dp = n * (z * p1 - p0) / (z * z - 1.0);
    x[n - 1 - i] = z;  // ascending
    w[n - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

}  // namespace dl
}  // namespace ntg

using namespace ntg;

extern "C" {

int ntg_dealias_create(ntg_dealias** out, ntg_plan* p, int lxd) {
  clear_error();
  NTG_CHECK_ARG(out && p, "ntg_dealias_create: null argument");
  NTG_TRY(need_metrics(p));
  if (lxd <= 0) lxd = 3 * p->lx / 2;
  NTG_TRY(dl::dispatch(p->lx, lxd, [](auto, auto) { return NTG_OK; }));
  ntg_dealias* d = new ntg_dealias();
  d->p = p;
  d->lx = p->lx;
  d->lxd = lxd;
  d->ngl = p->nelv * (int64_t)lxd * lxd * lxd;
  const int lx = p->lx;
  double xi[NTG_LXMAX], wq[NTG_LXMAX], Dm[NTG_LXMAX * NTG_LXMAX];
  gll_basis(lx, xi, wq, Dm);
  double xg[16];
  dl::gauss_legendre(lxd, xg, d->wg);
  for (int A = 0; A < lxd; ++A)
    for (int a = 0; a < lx; ++a) {
      double v = 1.0;
      for (int k = 0; k < lx; ++k)
        if (k != a) v *= (xg[A] - xi[k]) / (xi[a] - xi[k]);
      d->J[A * lx + a] = v;
    }
  // GL differentiation matrix from barycentric weights
  double lam[16];
  for (int j = 0; j < lxd; ++j) {
    double pr = 1.0;
    for (int k = 0; k < lxd; ++k)
      if (k != j) pr *= xg[j] - xg[k];
    lam[j] = 1.0 / pr;
  }
  for (int i = 0; i < lxd; ++i) {
    double diag = 0.0;
    for (int j = 0; j < lxd; ++j) {
      if (j == i) continue;
      const double v = lam[j] / lam[i] / (xg[i] - xg[j]);
      d->Dg[i * lxd + j] = v;
      diag -= v;
    }
    d->Dg[i * lxd + i] = diag;
  }
  int st = dev_alloc(&d->met_gl, (size_t)(9 * d->ngl));
  if (!st) {
    st = dl::dispatch(lx, lxd, [&](auto L, auto LD) -> int {
      constexpr int LX = decltype(L)::value, LXD = decltype(LD)::value;
      using S = dl::Smem<LX, LXD>;
      d->smem = S::BYTES;
      NTG_CUDA_TRY(cudaFuncSetAttribute(dl::k_map<LX, LXD, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)S::BYTES));
      NTG_CUDA_TRY(cudaFuncSetAttribute(dl::k_map<LX, LXD, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)S::BYTES));
      NTG_CUDA_TRY(cudaFuncSetAttribute(dl::k_adv<LX, LXD, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)S::BYTES));
      NTG_CUDA_TRY(cudaFuncSetAttribute(dl::k_adv<LX, LXD, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)S::BYTES));
      int occ = 0;
      NTG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, dl::k_adv<LX, LXD, 0>, dl::NT, S::BYTES));
      if (occ < 1) occ = 1;
      const int64_t g = (int64_t)num_sms() * occ;
      d->grid = (int)(p->nelv < g ? p->nelv : g);
      dl::k_map<LX, LXD, 0><<<d->grid, dl::NT, S::BYTES, p->stream>>>(d->met_gl, p->met, 9, p->nelv, p->n, d->ngl,
                                                                       dl::glmat<LX, LXD>(d));
      NTG_COUNT_LAUNCH();
      NTG_CUDA_TRY(cudaGetLastError());
      return NTG_OK;
    });
  }
  if (st) {
    dev_free(d->met_gl);
    delete d;
    return st;
  }
  *out = d;
  return NTG_OK;
}

int ntg_dealias_destroy(ntg_dealias* d) {
  if (!d) return NTG_OK;
  if (d->p) cudaStreamSynchronize(d->p->stream);
  dev_free(d->met_gl);
  delete d;
  return NTG_OK;
}

int ntg_dealias_info(const ntg_dealias* d, int* lxd, int64_t* ngl) {
  clear_error();
  NTG_CHECK_ARG(d, "ntg_dealias_info: null handle");
  if (lxd) *lxd = d->lxd;
  if (ngl) *ngl = d->ngl;
  return NTG_OK;
}

int ntg_dealias_map(ntg_dealias* d, double* out_d, const double* in_d, int to_gl) {
  clear_error();
  NTG_CHECK_ARG(d && out_d && in_d, "ntg_dealias_map: null argument");
  ntg_plan* p = d->p;
  return dl::dispatch(d->lx, d->lxd, [&](auto L, auto LD) -> int {
    constexpr int LX = decltype(L)::value, LXD = decltype(LD)::value;
    if (to_gl)
      dl::k_map<LX, LXD, 0><<<d->grid, dl::NT, d->smem, p->stream>>>(out_d, in_d, 1, p->nelv, p->n, d->ngl,
                                                                      dl::glmat<LX, LXD>(d));
    else
      dl::k_map<LX, LXD, 1><<<d->grid, dl::NT, d->smem, p->stream>>>(out_d, in_d, 1, p->nelv, d->ngl, p->n,
                                                                      dl::glmat<LX, LXD>(d));
    NTG_COUNT_LAUNCH();
    NTG_CUDA_TRY(cudaGetLastError());
    return NTG_OK;
  });
}

static int adv_dealias(ntg_dealias* d, int mode, double* fx, double* fy, double* fz, const double* vx,
                       const double* vy, const double* vz, const double* vxb, const double* vyb, const double* vzb) {
  clear_error();
  NTG_CHECK_ARG(d && fx && fy && fz && vx && vy && vz && vxb && vyb && vzb, "dealiased advection: null argument");
  ntg_plan* p = d->p;
  return dl::dispatch(d->lx, d->lxd, [&](auto L, auto LD) -> int {
    constexpr int LX = decltype(L)::value, LXD = decltype(LD)::value;
    if (mode == 0)
      dl::k_adv<LX, LXD, 0><<<d->grid, dl::NT, d->smem, p->stream>>>(fx, fy, fz, vx, vy, vz, vxb, vyb, vzb,
                                                                      d->met_gl, d->ngl, p->nelv,
                                                                      dl::glmat<LX, LXD>(d));
    else
      dl::k_adv<LX, LXD, 1><<<d->grid, dl::NT, d->smem, p->stream>>>(fx, fy, fz, vx, vy, vz, vxb, vyb, vzb,
                                                                      d->met_gl, d->ngl, p->nelv,
                                                                      dl::glmat<LX, LXD>(d));
    NTG_COUNT_LAUNCH();
    NTG_CUDA_TRY(cudaGetLastError());
    return NTG_OK;
  });
}

int ntg_adjoint_advection_dealias(ntg_dealias* d, double* fx_d, double* fy_d, double* fz_d, const double* vx_d,
                                  const double* vy_d, const double* vz_d, const double* vxb_d, const double* vyb_d,
                                  const double* vzb_d) {
  return adv_dealias(d, 0, fx_d, fy_d, fz_d, vx_d, vy_d, vz_d, vxb_d, vyb_d, vzb_d);
}

int ntg_linear_advection_dealias(ntg_dealias* d, double* fx_d, double* fy_d, double* fz_d, const double* vx_d,
                                 const double* vy_d, const double* vz_d, const double* vxb_d, const double* vyb_d,
                                 const double* vzb_d) {
  return adv_dealias(d, 1, fx_d, fy_d, fz_d, vx_d, vy_d, vz_d, vxb_d, vyb_d, vzb_d);
}

}  // extern "C"
