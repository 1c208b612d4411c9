// Spectral-element derivative operators (FP64) and the adjoint-equation
// terms built on them:
//
//   metrics      drdx .. dtdz (cofactors of dx/dr) and 1/jac from the coordinates
//   dudxyz       strong derivative (dr u_r + ds u_s + dt u_t) / jac   (Neko dudxyz)
//   opgrad       weak gradient w3 (drdx u_r + dsdx u_s + dtdx u_t), ... (= B grad u)
//   cdtp         D_r^T (w3 dr x) + D_s^T (w3 ds x) + D_t^T (w3 dt x) (transpose of opgrad)
//   conv1        vx du/dx + vy du/dy + vz du/dz (strong, pointwise)
//   curl         strong curl averaged across element copies: Binv gs(B curl u)
//
//   adjoint advection (no dealiasing), sources/adjoint/adv_adjoint_no_dealias.f90:118-302:
//       f_i -= sum_j u_j opgrad_i(Ub_j) + sum_d cdtp_d(u_i Ub_d)
//     (the device branch there; its CPU branch adds two of the three cdtp terms)
//   linearised advection (no dealiasing), same file :331-400:
//       f_i -= B conv1(u_i; Ub) + B conv1(Ub_i; u)
//   minimum-dissipation adjoint forcing,
//   sources/source_terms/adjoint_minimum_dissipation_source_term.f90:175-249:
//       f += scale curl(curl(u)), kept inside a zone (mask_exterior_const,
//       sources/neko_ext/mask_ops.f90:55-82) when one is given
//
// Layout and mapping as ax_helm: one element per LX x LX thread group
// (thread (i, j) owns the column k = 0..LX-1), element tiles in shared
// memory, D from the kernel-parameter bank.  FP64 throughout (these feed the
// adjoint right-hand sides and sensitivities).
#include "deriv.cuh"

namespace ntg {
namespace dv {

// 9 cofactors (drdx, drdy, drdz, dsdx, ..., dtdz) and 1/jac, stored m * n + l
template <int LX>
__global__ void __launch_bounds__(Shape<LX, 3>::THREADS)
    k_metrics(const double* __restrict__ x, const double* __restrict__ y, const double* __restrict__ z, int64_t nelv,
              const __grid_constant__ DMat<LX> M, double* __restrict__ met, int64_t n) {
  using S = Shape<LX, 3>;
  constexpr int LX2 = S::LX2, LX3 = S::LX3, EPB = S::EPB;
  __shared__ double sx[EPB][LX3], sy[EPB][LX3], sz[EPB][LX3];
  const int tid = threadIdx.x, le = tid / LX2, ij = tid - le * LX2, i = ij % LX, j = ij / LX;
  const bool worker = tid < S::NW;
  for (int64_t g = blockIdx.x; g * EPB < nelv; g += gridDim.x) {
    const int64_t e = g * EPB + le;
    const bool act = worker && e < nelv;
    for (int k = 0; k < LX && worker; ++k) {
      const int64_t q = e * LX3 + k * LX2 + ij;
      sx[le][k * LX2 + ij] = act ? x[q] : 0.0;
      sy[le][k * LX2 + ij] = act ? y[q] : 0.0;
      sz[le][k * LX2 + ij] = act ? z[q] : 0.0;
    }
    __syncthreads();
    if (act) {
      for (int k = 0; k < LX; ++k) {
        double xr, xs, xt, yr, ys, yt, zr, zs, zt;
        rgrad<LX>(sx[le], M, i, j, k, xr, xs, xt);
        rgrad<LX>(sy[le], M, i, j, k, yr, ys, yt);
        rgrad<LX>(sz[le], M, i, j, k, zr, zs, zt);
        const double c[9] = {ys * zt - yt * zs, xt * zs - xs * zt, xs * yt - xt * ys,
                             yt * zr - yr * zt, xr * zt - xt * zr, xt * yr - xr * yt,
                             yr * zs - ys * zr, xs * zr - xr * zs, xr * ys - xs * yr};
        const double jac = xr * c[0] + yr * c[1] + zr * c[2];
        const int64_t q = e * LX3 + k * LX2 + ij;
#pragma unroll
        for (int m = 0; m < 9; ++m) met[m * n + q] = c[m];
        met[9 * n + q] = 1.0 / jac;
      }
    }
    __syncthreads();
  }
}

// Gradient of u with the cofactors.  MODE 0: out_d = (strong) or w3 * (weak)
// derivative, d in {0, 1, 2} selected by mask bits; MODE 1: f_d -= mul *
// opgrad_d(u) for all d (the first term of the adjoint advection).
template <int LX, int MODE, bool WEAK>
__global__ void __launch_bounds__(Shape<LX, 1>::THREADS)
    k_grad(double* __restrict__ o0, double* __restrict__ o1, double* __restrict__ o2, const double* __restrict__ u,
           const double* __restrict__ mul, int64_t nelv, const __grid_constant__ DMat<LX> M,
           const double* __restrict__ met, int64_t n) {
  using S = Shape<LX, 1>;
  constexpr int LX2 = S::LX2, LX3 = S::LX3, EPB = S::EPB;
  __shared__ double su[EPB][LX3];
  const int tid = threadIdx.x, le = tid / LX2, ij = tid - le * LX2, i = ij % LX, j = ij / LX;
  const bool worker = tid < S::NW;
  for (int64_t g = blockIdx.x; g * EPB < nelv; g += gridDim.x) {
    const int64_t e = g * EPB + le;
    const bool act = worker && e < nelv;
    for (int k = 0; k < LX && worker; ++k) su[le][k * LX2 + ij] = act ? u[e * LX3 + k * LX2 + ij] : 0.0;
    __syncthreads();
    if (act) {
      for (int k = 0; k < LX; ++k) {
        double ur, us, ut;
        rgrad<LX>(su[le], M, i, j, k, ur, us, ut);
        const int64_t q = e * LX3 + k * LX2 + ij;
        const double sc = WEAK ? M.w[i] * M.w[j] * M.w[k] : met[9 * n + q];
        double* outs[3] = {o0, o1, o2};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          if (MODE == 0 && !outs[d]) continue;
          const double v = sc * (met[d * n + q] * ur + met[(3 + d) * n + q] * us + met[(6 + d) * n + q] * ut);
          if (MODE == 0) outs[d][q] = v;
          else outs[d][q] -= mul[q] * v;
        }
      }
    }
    __syncthreads();
  }
}

// out (= or -=) sum_d cdtp_d(a_d), a_d = mul * in_d (mul null: 1; in_d null: 0)
template <int LX, bool SUB>
__global__ void __launch_bounds__(Shape<LX, 3>::THREADS)
    k_cdtp(double* __restrict__ out, const double* __restrict__ in0, const double* __restrict__ in1,
           const double* __restrict__ in2, const double* __restrict__ mul, int64_t nelv,
           const __grid_constant__ DMat<LX> M, const double* __restrict__ met, int64_t n) {
  using S = Shape<LX, 3>;
  constexpr int LX2 = S::LX2, LX3 = S::LX3, EPB = S::EPB;
  __shared__ double fr[EPB][LX3], fs[EPB][LX3], ft[EPB][LX3];
  const int tid = threadIdx.x, le = tid / LX2, ij = tid - le * LX2, i = ij % LX, j = ij / LX;
  const bool worker = tid < S::NW;
  for (int64_t g = blockIdx.x; g * EPB < nelv; g += gridDim.x) {
    const int64_t e = g * EPB + le;
    const bool act = worker && e < nelv;
    for (int k = 0; k < LX && worker; ++k) {
      const int64_t q = e * LX3 + k * LX2 + ij;
      double a[3] = {0.0, 0.0, 0.0};
      if (act) {
        const double mq = mul ? mul[q] : 1.0;
        if (in0) a[0] = mq * in0[q];
        if (in1) a[1] = mq * in1[q];
        if (in2) a[2] = mq * in2[q];
      }
      const double w3 = M.w[i] * M.w[j] * M.w[k];
      double r = 0.0, s = 0.0, t = 0.0;
      if (act) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          r = fma(met[d * n + q], a[d], r);
          s = fma(met[(3 + d) * n + q], a[d], s);
          t = fma(met[(6 + d) * n + q], a[d], t);
        }
      }
      fr[le][k * LX2 + ij] = w3 * r;
      fs[le][k * LX2 + ij] = w3 * s;
      ft[le][k * LX2 + ij] = w3 * t;
    }
    __syncthreads();
    if (act) {
      for (int k = 0; k < LX; ++k) {
        double acc = 0.0;
#pragma unroll
        for (int l = 0; l < LX; ++l) {
          acc = fma(M.d[l * LX + i], fr[le][k * LX2 + j * LX + l], acc);
          acc = fma(M.d[l * LX + j], fs[le][k * LX2 + l * LX + i], acc);
          acc = fma(M.d[l * LX + k], ft[le][l * LX2 + j * LX + i], acc);
        }
        const int64_t q = e * LX3 + k * LX2 + ij;
        if (SUB) out[q] -= acc;
        else out[q] = acc;
      }
    }
    __syncthreads();
  }
}

// MODE 0: out = va . grad(a) (conv1, strong);  MODE 1: out -= B (va . grad a + vb . grad b)
template <int LX, int MODE>
__global__ void __launch_bounds__(Shape<LX, 2>::THREADS)
    k_conv(double* __restrict__ out, const double* __restrict__ a, const double* __restrict__ va0,
           const double* __restrict__ va1, const double* __restrict__ va2, const double* __restrict__ b,
           const double* __restrict__ vb0, const double* __restrict__ vb1, const double* __restrict__ vb2,
           int64_t nelv, const __grid_constant__ DMat<LX> M, const double* __restrict__ met, int64_t n) {
  using S = Shape<LX, 2>;
  constexpr int LX2 = S::LX2, LX3 = S::LX3, EPB = S::EPB;
  __shared__ double sa[EPB][LX3], sb[EPB][LX3];
  const int tid = threadIdx.x, le = tid / LX2, ij = tid - le * LX2, i = ij % LX, j = ij / LX;
  const bool worker = tid < S::NW;
  for (int64_t g = blockIdx.x; g * EPB < nelv; g += gridDim.x) {
    const int64_t e = g * EPB + le;
    const bool act = worker && e < nelv;
    for (int k = 0; k < LX && worker; ++k) {
      const int64_t q = e * LX3 + k * LX2 + ij;
      sa[le][k * LX2 + ij] = act ? a[q] : 0.0;
      if (MODE == 1) sb[le][k * LX2 + ij] = act ? b[q] : 0.0;
    }
    __syncthreads();
    if (act) {
      for (int k = 0; k < LX; ++k) {
        const int64_t q = e * LX3 + k * LX2 + ij;
        double ur, us, ut;
        rgrad<LX>(sa[le], M, i, j, k, ur, us, ut);
        const double* vv[3] = {va0, va1, va2};
        double acc = 0.0;
#pragma unroll
        for (int d = 0; d < 3; ++d)
          acc = fma(vv[d][q], met[d * n + q] * ur + met[(3 + d) * n + q] * us + met[(6 + d) * n + q] * ut, acc);
        if (MODE == 0) {
          out[q] = acc * met[9 * n + q];
        } else {
          rgrad<LX>(sb[le], M, i, j, k, ur, us, ut);
          const double* vw[3] = {vb0, vb1, vb2};
#pragma unroll
          for (int d = 0; d < 3; ++d)
            acc = fma(vw[d][q], met[d * n + q] * ur + met[(3 + d) * n + q] * us + met[(6 + d) * n + q] * ut, acc);
          out[q] -= M.w[i] * M.w[j] * M.w[k] * acc;  // B / jac = w3
        }
      }
    }
    __syncthreads();
  }
}

// B curl(u) (strong curl times B = w3 * cofactor combinations)
template <int LX>
__global__ void __launch_bounds__(Shape<LX, 3>::THREADS)
    k_curl(double* __restrict__ w0, double* __restrict__ w1, double* __restrict__ w2, const double* __restrict__ ux,
           const double* __restrict__ uy, const double* __restrict__ uz, int64_t nelv,
           const __grid_constant__ DMat<LX> M, const double* __restrict__ met, int64_t n) {
  using S = Shape<LX, 3>;
  constexpr int LX2 = S::LX2, LX3 = S::LX3, EPB = S::EPB;
  __shared__ double sx[EPB][LX3], sy[EPB][LX3], sz[EPB][LX3];
  const int tid = threadIdx.x, le = tid / LX2, ij = tid - le * LX2, i = ij % LX, j = ij / LX;
  const bool worker = tid < S::NW;
  for (int64_t g = blockIdx.x; g * EPB < nelv; g += gridDim.x) {
    const int64_t e = g * EPB + le;
    const bool act = worker && e < nelv;
    for (int k = 0; k < LX && worker; ++k) {
      const int64_t q = e * LX3 + k * LX2 + ij;
      sx[le][k * LX2 + ij] = act ? ux[q] : 0.0;
      sy[le][k * LX2 + ij] = act ? uy[q] : 0.0;
      sz[le][k * LX2 + ij] = act ? uz[q] : 0.0;
    }
    __syncthreads();
    if (act) {
      for (int k = 0; k < LX; ++k) {
        const int64_t q = e * LX3 + k * LX2 + ij;
        double g[3][3];  // g[f][r|s|t]: reference derivatives of field f
        rgrad<LX>(sx[le], M, i, j, k, g[0][0], g[0][1], g[0][2]);
        rgrad<LX>(sy[le], M, i, j, k, g[1][0], g[1][1], g[1][2]);
        rgrad<LX>(sz[le], M, i, j, k, g[2][0], g[2][1], g[2][2]);
        auto d = [&](int f, int dir) {
          return met[dir * n + q] * g[f][0] + met[(3 + dir) * n + q] * g[f][1] + met[(6 + dir) * n + q] * g[f][2];
        };
        const double w3 = M.w[i] * M.w[j] * M.w[k];
        w0[q] = w3 * (d(2, 1) - d(1, 2));
        w1[q] = w3 * (d(0, 2) - d(2, 0));
        w2[q] = w3 * (d(1, 0) - d(0, 1));
      }
    }
    __syncthreads();
  }
}

// The adjoint advection without dealiasing in one element pass:
//   f_i -= sum_j u_j opgrad_i(Ub_j) + sum_d cdtp_d(u_i Ub_d).
// The cdtp fluxes of all three components share the contravariant fluxes
// V_r = w3 (drdx . Ub), V_s = w3 (dsdx . Ub), V_t = w3 (dtdx . Ub):
// component i's fluxes are u_i V_r, u_i V_s, u_i V_t.  Phase 1 takes the
// reference gradients of Ub from its tiles, subtracts the opgrad part and
// stores V; then per component the Ub tiles hold u_i V and D^T is applied.
// Inputs and the cofactors are read once per node instead of by six
// separate kernels; the FP64 operation count is the separate kernels' less
// the repeated flux sums (198 instead of 216 per node).
template <int LX>
__global__ void __launch_bounds__(Shape<LX, 6>::THREADS)
    k_adv_adj_nd(double* __restrict__ f0, double* __restrict__ f1, double* __restrict__ f2,
                 const double* __restrict__ u0, const double* __restrict__ u1, const double* __restrict__ u2,
                 const double* __restrict__ b0, const double* __restrict__ b1, const double* __restrict__ b2,
                 int64_t nelv, const __grid_constant__ DMat<LX> M, const double* __restrict__ met, int64_t n) {
  using S = Shape<LX, 6>;
  constexpr int LX2 = S::LX2, LX3 = S::LX3, EPB = S::EPB;
  __shared__ double sA[EPB][3][LX3];  // Ub, then u_i V_r, u_i V_s, u_i V_t
  __shared__ double sV[EPB][3][LX3];  // V_r, V_s, V_t
  const int tid = threadIdx.x, le = tid / LX2, ij = tid - le * LX2, i = ij % LX, j = ij / LX;
  const bool worker = tid < S::NW;
  const double* ub[3] = {b0, b1, b2};
  const double* uu[3] = {u0, u1, u2};
  double* ff[3] = {f0, f1, f2};
  for (int64_t g = blockIdx.x; g * EPB < nelv; g += gridDim.x) {
    const int64_t e = g * EPB + le;
    const bool act = worker && e < nelv;
    for (int k = 0; k < LX && worker; ++k)
#pragma unroll
      for (int c = 0; c < 3; ++c) sA[le][c][k * LX2 + ij] = act ? ub[c][e * LX3 + k * LX2 + ij] : 0.0;
    __syncthreads();
    if (act) {
#pragma unroll 1
      for (int k = 0; k < LX; ++k) {
        const int64_t q = e * LX3 + k * LX2 + ij;
        const int p = k * LX2 + ij;
        double gr[3][3];
#pragma unroll
        for (int c = 0; c < 3; ++c) rgrad<LX>(sA[le][c], M, i, j, k, gr[c][0], gr[c][1], gr[c][2]);
        double m[9];
#pragma unroll
        for (int t = 0; t < 9; ++t) m[t] = met[t * n + q];
        const double w3 = M.w[i] * M.w[j] * M.w[k];
        const double uq[3] = {u0[q], u1[q], u2[q]};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          double acc = 0.0;
#pragma unroll
          for (int jj = 0; jj < 3; ++jj)
            acc = fma(uq[jj], m[c] * gr[jj][0] + m[3 + c] * gr[jj][1] + m[6 + c] * gr[jj][2], acc);
          ff[c][q] -= w3 * acc;
        }
        const double bq[3] = {sA[le][0][p], sA[le][1][p], sA[le][2][p]};
#pragma unroll
        for (int d = 0; d < 3; ++d)
          sV[le][d][p] = w3 * (m[3 * d] * bq[0] + m[3 * d + 1] * bq[1] + m[3 * d + 2] * bq[2]);
      }
    }
#pragma unroll 1
    for (int c = 0; c < 3; ++c) {
      __syncthreads();
      if (act) {
        for (int k = 0; k < LX; ++k) {
          const int p = k * LX2 + ij;
          const double uc = uu[c][e * LX3 + p];
#pragma unroll
          for (int d = 0; d < 3; ++d) sA[le][d][p] = uc * sV[le][d][p];
        }
      }
      __syncthreads();
      if (act) {
        const double* fr = sA[le][0];
        const double* fs = sA[le][1];
        const double* ft = sA[le][2];
#pragma unroll 1
        for (int k = 0; k < LX; ++k) {
          double acc = 0.0;
#pragma unroll
          for (int l = 0; l < LX; ++l) {
            acc = fma(M.d[l * LX + i], fr[k * LX2 + j * LX + l], acc);
            acc = fma(M.d[l * LX + j], fs[k * LX2 + l * LX + i], acc);
            acc = fma(M.d[l * LX + k], ft[l * LX2 + j * LX + i], acc);
          }
          ff[c][e * LX3 + k * LX2 + ij] -= acc;
        }
      }
    }
    __syncthreads();
  }
}

// The linearised advection without dealiasing in one element pass:
//   f_i -= B conv1(u_i; Ub) + B conv1(Ub_i; u)
//        = w3 sum_d (Ub_d (drdx_d . grad u_i) + u_d (drdx_d . grad Ub_i)),
// with u and Ub in six tiles, the cofactors read once per node.
template <int LX>
__global__ void __launch_bounds__(Shape<LX, 6>::THREADS)
    k_adv_lin_nd(double* __restrict__ f0, double* __restrict__ f1, double* __restrict__ f2,
                 const double* __restrict__ u0, const double* __restrict__ u1, const double* __restrict__ u2,
                 const double* __restrict__ b0, const double* __restrict__ b1, const double* __restrict__ b2,
                 int64_t nelv, const __grid_constant__ DMat<LX> M, const double* __restrict__ met, int64_t n) {
  using S = Shape<LX, 6>;
  constexpr int LX2 = S::LX2, LX3 = S::LX3, EPB = S::EPB;
  __shared__ double sU[EPB][3][LX3], sB[EPB][3][LX3];
  const int tid = threadIdx.x, le = tid / LX2, ij = tid - le * LX2, i = ij % LX, j = ij / LX;
  const bool worker = tid < S::NW;
  const double* ub[3] = {b0, b1, b2};
  const double* uu[3] = {u0, u1, u2};
  double* ff[3] = {f0, f1, f2};
  for (int64_t g = blockIdx.x; g * EPB < nelv; g += gridDim.x) {
    const int64_t e = g * EPB + le;
    const bool act = worker && e < nelv;
    for (int k = 0; k < LX && worker; ++k)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        sU[le][c][k * LX2 + ij] = act ? uu[c][e * LX3 + k * LX2 + ij] : 0.0;
        sB[le][c][k * LX2 + ij] = act ? ub[c][e * LX3 + k * LX2 + ij] : 0.0;
      }
    __syncthreads();
    if (act) {
#pragma unroll 1
      for (int k = 0; k < LX; ++k) {
        const int64_t q = e * LX3 + k * LX2 + ij;
        const int p = k * LX2 + ij;
        double m[9];
#pragma unroll
        for (int t = 0; t < 9; ++t) m[t] = met[t * n + q];
        const double w3 = M.w[i] * M.w[j] * M.w[k];
        const double uq[3] = {sU[le][0][p], sU[le][1][p], sU[le][2][p]};
        const double bq[3] = {sB[le][0][p], sB[le][1][p], sB[le][2][p]};
#pragma unroll 1
        for (int c = 0; c < 3; ++c) {
          double gu[3], gb[3];
          rgrad<LX>(sU[le][c], M, i, j, k, gu[0], gu[1], gu[2]);
          rgrad<LX>(sB[le][c], M, i, j, k, gb[0], gb[1], gb[2]);
          double acc = 0.0;
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            acc = fma(bq[d], m[d] * gu[0] + m[3 + d] * gu[1] + m[6 + d] * gu[2], acc);
            acc = fma(uq[d], m[d] * gb[0] + m[3 + d] * gb[1] + m[6 + d] * gb[2], acc);
          }
          ff[c][q] -= w3 * acc;
        }
      }
    }
    __syncthreads();
  }
}

__global__ void k_mul3(double* __restrict__ a, double* __restrict__ b, double* __restrict__ c,
                       const double* __restrict__ s, int64_t n) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    a[q] *= s[q];
    b[q] *= s[q];
    c[q] *= s[q];
  }
}

__global__ void k_inv(double* __restrict__ a, int64_t n) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
    a[q] = 1.0 / a[q];
}

// f_c += scale w_c on all nodes (zone null) or on the zone's nodes only
__global__ void k_add_zone(double* __restrict__ f0, double* __restrict__ f1, double* __restrict__ f2,
                           const double* __restrict__ w0, const double* __restrict__ w1,
                           const double* __restrict__ w2, double scale, const int32_t* __restrict__ zone,
                           int64_t nzone, int base, int64_t n) {
  const int64_t cnt = zone ? nzone : n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < cnt; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = zone ? (int64_t)zone[t] - base : t;
    if (q < 0 || q >= n) continue;
    f0[q] += scale * w0[q];
    f1[q] += scale * w1[q];
    f2[q] += scale * w2[q];
  }
}

}  // namespace dv

double* plan_scratch(ntg_plan* p, int64_t count) {
  if (p->dscr_n < count) {
    // the stream may still use the old buffer
    if (p->dscr && cudaStreamSynchronize(p->stream) != cudaSuccess) return nullptr;
    dev_free(p->dscr);
    p->dscr_n = 0;
    if (dev_alloc(&p->dscr, (size_t)count)) return nullptr;
    p->dscr_n = count;
  }
  return p->dscr;
}

// w = B curl u (unassembled)
int bcurl(ntg_plan* p, double* w0, double* w1, double* w2, const double* ux, const double* uy, const double* uz) {
  cudaStream_t s = p->stream;
  return dv::dispatch<3>(p->lx, [&](auto L) -> int {
    constexpr int LX = decltype(L)::value;
    dv::k_curl<LX><<<dv::grid_of<LX, 3>(p), dv::Shape<LX, 3>::THREADS, 0, s>>>(w0, w1, w2, ux, uy, uz, p->nelv,
                                                                                 dv::dmat<LX>(p), p->met, p->n);
    NTG_COUNT_LAUNCH();
    return NTG_OK;
  });
}

// w = Binv gs(B curl u)
int curl_avg(ntg_plan* p, double* w0, double* w1, double* w2, const double* ux, const double* uy,
             const double* uz) {
  cudaStream_t s = p->stream;
  NTG_TRY(bcurl(p, w0, w1, w2, ux, uy, uz));
  NTG_TRY(gs_launch(p, w0, NTG_GS_ADD, s));
  NTG_TRY(gs_launch(p, w1, NTG_GS_ADD, s));
  NTG_TRY(gs_launch(p, w2, NTG_GS_ADD, s));
  { dv::k_mul3<<<grid_for(p->n, 256), 256, 0, s>>>(w0, w1, w2, p->binv, p->n); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

}  // namespace ntg

using namespace ntg;

extern "C" {

int ntg_metrics_set(ntg_plan* p, const double* x_d, const double* y_d, const double* z_d) {
  clear_error();
  NTG_CHECK_ARG(p && x_d && y_d && z_d, "ntg_metrics_set: null argument");
  if (!p->met) NTG_TRY(dev_alloc(&p->met, (size_t)p->n * 10));
  if (!p->binv) NTG_TRY(dev_alloc(&p->binv, (size_t)p->n));
  cudaStream_t s = p->stream;
  NTG_TRY(dv::dispatch<3>(p->lx, [&](auto L) -> int {
    constexpr int LX = decltype(L)::value;
    dv::k_metrics<LX><<<dv::grid_of<LX, 3>(p), dv::Shape<LX, 3>::THREADS, 0, s>>>(x_d, y_d, z_d, p->nelv,
                                                                                    dv::dmat<LX>(p), p->met, p->n);
    NTG_COUNT_LAUNCH();
    return NTG_OK;
  }));
  NTG_CUDA_TRY(cudaMemcpyAsync(p->binv, p->B, sizeof(double) * p->n, cudaMemcpyDeviceToDevice, s));
  NTG_TRY(gs_launch(p, p->binv, NTG_GS_ADD, s));
  { dv::k_inv<<<grid_for(p->n, 256), 256, 0, s>>>(p->binv, p->n); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

int ntg_dudxyz(ntg_plan* p, double* du_d, const double* u_d, int dir) {
  clear_error();
  NTG_CHECK_ARG(p && du_d && u_d && dir >= 0 && dir <= 2, "ntg_dudxyz: bad argument");
  NTG_TRY(need_metrics(p));
  double* o[3] = {nullptr, nullptr, nullptr};
  o[dir] = du_d;
  return dv::dispatch<1>(p->lx, [&](auto L) -> int {
    constexpr int LX = decltype(L)::value;
    dv::k_grad<LX, 0, false><<<dv::grid_of<LX, 1>(p), dv::Shape<LX, 1>::THREADS, 0, p->stream>>>(
        o[0], o[1], o[2], u_d, nullptr, p->nelv, dv::dmat<LX>(p), p->met, p->n);
    NTG_COUNT_LAUNCH();
    NTG_CUDA_TRY(cudaGetLastError());
    return NTG_OK;
  });
}

int ntg_opgrad(ntg_plan* p, double* ux_d, double* uy_d, double* uz_d, const double* u_d) {
  clear_error();
  NTG_CHECK_ARG(p && ux_d && uy_d && uz_d && u_d, "ntg_opgrad: null argument");
  NTG_TRY(need_metrics(p));
  return dv::dispatch<1>(p->lx, [&](auto L) -> int {
    constexpr int LX = decltype(L)::value;
    dv::k_grad<LX, 0, true><<<dv::grid_of<LX, 1>(p), dv::Shape<LX, 1>::THREADS, 0, p->stream>>>(
        ux_d, uy_d, uz_d, u_d, nullptr, p->nelv, dv::dmat<LX>(p), p->met, p->n);
    NTG_COUNT_LAUNCH();
    NTG_CUDA_TRY(cudaGetLastError());
    return NTG_OK;
  });
}

int ntg_cdtp(ntg_plan* p, double* dtx_d, const double* x_d, int dir) {
  clear_error();
  NTG_CHECK_ARG(p && dtx_d && x_d && dir >= 0 && dir <= 2, "ntg_cdtp: bad argument");
  NTG_TRY(need_metrics(p));
  const double* in[3] = {nullptr, nullptr, nullptr};
  in[dir] = x_d;
  return dv::dispatch<3>(p->lx, [&](auto L) -> int {
    constexpr int LX = decltype(L)::value;
    dv::k_cdtp<LX, false><<<dv::grid_of<LX, 3>(p), dv::Shape<LX, 3>::THREADS, 0, p->stream>>>(
        dtx_d, in[0], in[1], in[2], nullptr, p->nelv, dv::dmat<LX>(p), p->met, p->n);
    NTG_COUNT_LAUNCH();
    NTG_CUDA_TRY(cudaGetLastError());
    return NTG_OK;
  });
}

int ntg_conv1(ntg_plan* p, double* du_d, const double* u_d, const double* vx_d, const double* vy_d,
              const double* vz_d) {
  clear_error();
  NTG_CHECK_ARG(p && du_d && u_d && vx_d && vy_d && vz_d, "ntg_conv1: null argument");
  NTG_TRY(need_metrics(p));
  return dv::dispatch<2>(p->lx, [&](auto L) -> int {
    constexpr int LX = decltype(L)::value;
    dv::k_conv<LX, 0><<<dv::grid_of<LX, 2>(p), dv::Shape<LX, 2>::THREADS, 0, p->stream>>>(
        du_d, u_d, vx_d, vy_d, vz_d, nullptr, nullptr, nullptr, nullptr, p->nelv, dv::dmat<LX>(p), p->met, p->n);
    NTG_COUNT_LAUNCH();
    NTG_CUDA_TRY(cudaGetLastError());
    return NTG_OK;
  });
}

int ntg_curl(ntg_plan* p, double* w1_d, double* w2_d, double* w3_d, const double* u1_d, const double* u2_d,
             const double* u3_d) {
  clear_error();
  NTG_CHECK_ARG(p && w1_d && w2_d && w3_d && u1_d && u2_d && u3_d, "ntg_curl: null argument");
  NTG_TRY(need_metrics(p));
  return curl_avg(p, w1_d, w2_d, w3_d, u1_d, u2_d, u3_d);
}

int ntg_adjoint_advection_no_dealias(ntg_plan* p, double* fx, double* fy, double* fz, const double* vx,
                                     const double* vy, const double* vz, const double* vxb, const double* vyb,
                                     const double* vzb) {
  clear_error();
  NTG_CHECK_ARG(p && fx && fy && fz && vx && vy && vz && vxb && vyb && vzb,
                "ntg_adjoint_advection_no_dealias: null argument");
  NTG_TRY(need_metrics(p));
  const double* u[3] = {vx, vy, vz};
  const double* ub[3] = {vxb, vyb, vzb};
  double* f[3] = {fx, fy, fz};
  cudaStream_t s = p->stream;
  // f_i -= sum_j u_j opgrad_i(Ub_j) + sum_d cdtp_d(u_i Ub_d), one element pass
  NTG_TRY(dv::dispatch<6>(p->lx, [&](auto L) -> int {
    constexpr int LX = decltype(L)::value;
    dv::k_adv_adj_nd<LX><<<dv::grid_of<LX, 6>(p), dv::Shape<LX, 6>::THREADS, 0, s>>>(
        f[0], f[1], f[2], u[0], u[1], u[2], ub[0], ub[1], ub[2], p->nelv, dv::dmat<LX>(p), p->met, p->n);
    NTG_COUNT_LAUNCH();
    return NTG_OK;
  }));
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

int ntg_linear_advection_no_dealias(ntg_plan* p, double* fx, double* fy, double* fz, const double* vx,
                                    const double* vy, const double* vz, const double* vxb, const double* vyb,
                                    const double* vzb) {
  clear_error();
  NTG_CHECK_ARG(p && fx && fy && fz && vx && vy && vz && vxb && vyb && vzb,
                "ntg_linear_advection_no_dealias: null argument");
  NTG_TRY(need_metrics(p));
  const double* u[3] = {vx, vy, vz};
  const double* ub[3] = {vxb, vyb, vzb};
  double* f[3] = {fx, fy, fz};
  // f_i -= B conv1(u_i; Ub) + B conv1(Ub_i; u), one element pass
  NTG_TRY(dv::dispatch<6>(p->lx, [&](auto L) -> int {
    constexpr int LX = decltype(L)::value;
    dv::k_adv_lin_nd<LX><<<dv::grid_of<LX, 6>(p), dv::Shape<LX, 6>::THREADS, 0, p->stream>>>(
        f[0], f[1], f[2], u[0], u[1], u[2], ub[0], ub[1], ub[2], p->nelv, dv::dmat<LX>(p), p->met, p->n);
    NTG_COUNT_LAUNCH();
    return NTG_OK;
  }));
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

int ntg_adjoint_min_dissipation(ntg_plan* p, double* fx, double* fy, double* fz, const double* u, const double* v,
                                const double* w, double scale, const int32_t* zone_d, int64_t nzone, int base) {
  clear_error();
  NTG_CHECK_ARG(p && fx && fy && fz && u && v && w && (nzone == 0 || zone_d) && nzone >= 0,
                "ntg_adjoint_min_dissipation: bad argument");
  NTG_TRY(need_metrics(p));
  const int64_t n = p->n;
  double* t = plan_scratch(p, 6 * n);
  if (!t) return NTG_ERR_ALLOC;
  NTG_TRY(curl_avg(p, t, t + n, t + 2 * n, u, v, w));
  NTG_TRY(curl_avg(p, t + 3 * n, t + 4 * n, t + 5 * n, t, t + n, t + 2 * n));
  dv::k_add_zone<<<grid_for(nzone ? nzone : n, 256), 256, 0, p->stream>>>(
      fx, fy, fz, t + 3 * n, t + 4 * n, t + 5 * n, scale, nzone ? zone_d : nullptr, nzone, base, n);
  NTG_COUNT_LAUNCH();
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

}  // extern "C"
