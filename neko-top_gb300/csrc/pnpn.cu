// Pn/Pn splitting residuals on either side of the pressure and velocity
// solves (FP64), as the adjoint/forward step calls them
// (sources/adjoint/adjoint_pnpn.f90:716-723 prs_res%compute and :747-753
// vel_res%compute):
//
//   pressure  wa = curl(curl(u_e)),  ta_d = Binv gs(f_d / rho - (mu / rho) B wa_d)
//             p_res = -A(h1 = 1/rho) p + sum_d cdtp_d(ta_d)
//                     - (bd/dt) sum_c u_c s_c   on velocity-surface nodes
//                     - sum_c ta_c s'_c         on symmetry-surface nodes
//   velocity  u_res_c = f_c - (mu K + rho (bd/dt) B) u_c - opgrad_c(p)
//
// (s, s': outward normal times facet area, per surface node, from the
// caller.)  Neither residual is gs-assembled or masked: the caller does that
// next, as the reference does.
//
// Fusion: the pressure residual's Laplacian of p and its three cdtp terms
// are one element-tile pass (both end in the transposed reference
// derivatives, so their r/s/t fluxes are summed before one D^T contraction);
// the velocity residual computes all three components and the pressure
// gradient in one pass, so G, B and the cofactors are read once instead of
// three times.  mu and rho are fields or constants (null pointer -> the
// constant).
#include "deriv.cuh"

namespace ntg {
namespace pn {

using dv::DMat;
using dv::rgrad;
using dv::Shape;

struct GPtr {
  const double* g[6];
};

struct Coefs {
  const double* mu;
  const double* rho;
  double muc, rhoc;
  __device__ __forceinline__ double m(int64_t q) const { return mu ? mu[q] : muc; }
  __device__ __forceinline__ double r(int64_t q) const { return rho ? rho[q] : rhoc; }
};

// X_c holds gs(B curl t)_c; becomes f_c / rho - (mu / rho) B (Binv X_c)
__global__ void k_ta(double* __restrict__ x0, double* __restrict__ x1, double* __restrict__ x2,
                     const double* __restrict__ f0, const double* __restrict__ f1, const double* __restrict__ f2,
                     const double* __restrict__ B, const double* __restrict__ binv, Coefs c, int64_t n) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const double rho = c.r(q), mr = c.m(q) / rho, bb = B[q], bi = binv[q];
    x0[q] = f0[q] / rho - mr * bb * (bi * x0[q]);
    x1[q] = f1[q] / rho - mr * bb * (bi * x1[q]);
    x2[q] = f2[q] / rho - mr * bb * (bi * x2[q]);
  }
}

// p_res = -D^T (h1 G D p) + sum_d cdtp_d(binv ta_d), h1 = 1 / rho
template <int LX>
__global__ void __launch_bounds__(Shape<LX, 4>::THREADS)
    k_prs_core(double* __restrict__ pres, const double* __restrict__ p, const double* __restrict__ ta0,
               const double* __restrict__ ta1, const double* __restrict__ ta2, const double* __restrict__ binv,
               Coefs c, int64_t nelv, const __grid_constant__ DMat<LX> M, GPtr G, const double* __restrict__ met,
               int64_t n) {
  using S = Shape<LX, 4>;
  constexpr int LX2 = S::LX2, LX3 = S::LX3, EPB = S::EPB;
  __shared__ double sp[EPB][LX3], fr[EPB][LX3], fs[EPB][LX3], ft[EPB][LX3];
  const int tid = threadIdx.x, le = tid / LX2, ij = tid - le * LX2, i = ij % LX, j = ij / LX;
  const bool worker = tid < S::NW;
  for (int64_t g = blockIdx.x; g * EPB < nelv; g += gridDim.x) {
    const int64_t e = g * EPB + le;
    const bool act = worker && e < nelv;
    for (int k = 0; k < LX && worker; ++k) sp[le][k * LX2 + ij] = act ? p[e * LX3 + k * LX2 + ij] : 0.0;
    __syncthreads();
    if (act) {
      for (int k = 0; k < LX; ++k) {
        const int64_t q = e * LX3 + k * LX2 + ij;
        double ur, us, ut;
        rgrad<LX>(sp[le], M, i, j, k, ur, us, ut);
        const double h1 = 1.0 / c.r(q), w3 = M.w[i] * M.w[j] * M.w[k], bi = binv[q];
        const double a0 = bi * ta0[q], a1 = bi * ta1[q], a2 = bi * ta2[q];
        const double g11 = G.g[0][q], g12 = G.g[1][q], g13 = G.g[2][q], g22 = G.g[3][q], g23 = G.g[4][q],
                     g33 = G.g[5][q];
        const double cr = met[0 * n + q] * a0 + met[1 * n + q] * a1 + met[2 * n + q] * a2;
        const double cs = met[3 * n + q] * a0 + met[4 * n + q] * a1 + met[5 * n + q] * a2;
        const double ct = met[6 * n + q] * a0 + met[7 * n + q] * a1 + met[8 * n + q] * a2;
        fr[le][k * LX2 + ij] = w3 * cr - h1 * (g11 * ur + g12 * us + g13 * ut);
        fs[le][k * LX2 + ij] = w3 * cs - h1 * (g12 * ur + g22 * us + g23 * ut);
        ft[le][k * LX2 + ij] = w3 * ct - h1 * (g13 * ur + g23 * us + g33 * ut);
      }
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
        pres[e * LX3 + k * LX2 + ij] = acc;
      }
    }
    __syncthreads();
  }
}

// res_c = f_c - D^T (mu G D u_c) - rho (bd/dt) B u_c - opgrad_c(p), c = 0..2
template <int LX>
__global__ void __launch_bounds__(Shape<LX, 5>::THREADS)
    k_vel_res(double* __restrict__ r0, double* __restrict__ r1, double* __restrict__ r2,
              const double* __restrict__ u0, const double* __restrict__ u1, const double* __restrict__ u2,
              const double* __restrict__ p, const double* __restrict__ f0, const double* __restrict__ f1,
              const double* __restrict__ f2, Coefs c, double bddt, int64_t nelv,
              const __grid_constant__ DMat<LX> M, GPtr G, const double* __restrict__ B,
              const double* __restrict__ met, int64_t n) {
  using S = Shape<LX, 5>;
  constexpr int LX2 = S::LX2, LX3 = S::LX3, EPB = S::EPB;
  __shared__ double su[EPB][LX3], sp[EPB][LX3], fr[EPB][LX3], fs[EPB][LX3], ft[EPB][LX3];
  const int tid = threadIdx.x, le = tid / LX2, ij = tid - le * LX2, i = ij % LX, j = ij / LX;
  const bool worker = tid < S::NW;
  for (int64_t g = blockIdx.x; g * EPB < nelv; g += gridDim.x) {
    const int64_t e = g * EPB + le;
    const bool act = worker && e < nelv;
    for (int k = 0; k < LX && worker; ++k) sp[le][k * LX2 + ij] = act ? p[e * LX3 + k * LX2 + ij] : 0.0;
    __syncthreads();
    // res_c = f_c - opgrad_c(p) first (the pressure gradient once for all
    // three components); the thread that writes a node updates it below
    if (act) {
      for (int k = 0; k < LX; ++k) {
        const int64_t q = e * LX3 + k * LX2 + ij;
        double pr, ps, pt;
        rgrad<LX>(sp[le], M, i, j, k, pr, ps, pt);
        const double w3 = M.w[i] * M.w[j] * M.w[k];
        r0[q] = f0[q] - w3 * (met[0 * n + q] * pr + met[3 * n + q] * ps + met[6 * n + q] * pt);
        r1[q] = f1[q] - w3 * (met[1 * n + q] * pr + met[4 * n + q] * ps + met[7 * n + q] * pt);
        r2[q] = f2[q] - w3 * (met[2 * n + q] * pr + met[5 * n + q] * ps + met[8 * n + q] * pt);
      }
    }
#pragma unroll 1
    for (int cc = 0; cc < 3; ++cc) {
      const double* u = cc == 0 ? u0 : (cc == 1 ? u1 : u2);
      double* r = cc == 0 ? r0 : (cc == 1 ? r1 : r2);
      for (int k = 0; k < LX && worker; ++k) su[le][k * LX2 + ij] = act ? u[e * LX3 + k * LX2 + ij] : 0.0;
      __syncthreads();
      if (act) {
        for (int k = 0; k < LX; ++k) {
          const int64_t q = e * LX3 + k * LX2 + ij;
          double ur, us, ut;
          rgrad<LX>(su[le], M, i, j, k, ur, us, ut);
          const double h1 = c.m(q);
          const double g11 = G.g[0][q], g12 = G.g[1][q], g13 = G.g[2][q], g22 = G.g[3][q], g23 = G.g[4][q],
                       g33 = G.g[5][q];
          fr[le][k * LX2 + ij] = h1 * (g11 * ur + g12 * us + g13 * ut);
          fs[le][k * LX2 + ij] = h1 * (g12 * ur + g22 * us + g23 * ut);
          ft[le][k * LX2 + ij] = h1 * (g13 * ur + g23 * us + g33 * ut);
        }
      }
      __syncthreads();
      if (act) {
        for (int k = 0; k < LX; ++k) {
          const int64_t q = e * LX3 + k * LX2 + ij;
          double acc = 0.0;
#pragma unroll
          for (int l = 0; l < LX; ++l) {
            acc = fma(M.d[l * LX + i], fr[le][k * LX2 + j * LX + l], acc);
            acc = fma(M.d[l * LX + j], fs[le][k * LX2 + l * LX + i], acc);
            acc = fma(M.d[l * LX + k], ft[le][l * LX2 + j * LX + i], acc);
          }
          const double h2 = c.r(q) * bddt;
          r[q] -= acc + h2 * B[q] * su[le][k * LX2 + ij];
        }
      }
      __syncthreads();
    }
  }
}

// res[q] -= scale sum_c (mul[q]) v_c[q] s_c[t] over the surface entries t
__global__ void k_surface(double* __restrict__ res, const int32_t* __restrict__ idx, const double* __restrict__ s,
                          int64_t ns, int base, const double* __restrict__ v0, const double* __restrict__ v1,
                          const double* __restrict__ v2, const double* __restrict__ mul, double scale, int64_t n) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ns; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = (int64_t)idx[t] - base;
    if (q < 0 || q >= n) continue;
    const double m = mul ? mul[q] : 1.0;
    res[q] -= scale * (m * v0[q] * s[t] + m * v1[q] * s[ns + t] + m * v2[q] * s[2 * ns + t]);
  }
}

GPtr gptr(const ntg_plan* p) {
  GPtr G;
  for (int a = 0; a < 6; ++a) G.g[a] = p->g[a];
  return G;
}

}  // namespace pn
}  // namespace ntg

using namespace ntg;

extern "C" {

int ntg_pnpn_prs_res(ntg_plan* p, double* p_res, const double* pr, const double* u, const double* v, const double* w,
                     const double* ue, const double* ve, const double* we, const double* fx, const double* fy,
                     const double* fz, const double* mu_d, double mu_c, const double* rho_d, double rho_c, double bd,
                     double dt, const int32_t* prs_idx, const double* prs_s, int64_t nprs, const int32_t* sym_idx,
                     const double* sym_s, int64_t nsym, int base) {
  clear_error();
  NTG_CHECK_ARG(p && p_res && pr && u && v && w && ue && ve && we && fx && fy && fz,
                "ntg_pnpn_prs_res: null field argument");
  NTG_CHECK_ARG(nprs >= 0 && nsym >= 0 && (nprs == 0 || (prs_idx && prs_s)) && (nsym == 0 || (sym_idx && sym_s)),
                "ntg_pnpn_prs_res: bad surface list");
  NTG_CHECK_ARG(dt > 0.0 && (rho_d || rho_c != 0.0), "ntg_pnpn_prs_res: need dt > 0 and rho != 0");
  NTG_TRY(need_metrics(p));
  const int64_t n = p->n;
  double* t = plan_scratch(p, 6 * n);
  if (!t) return NTG_ERR_ALLOC;
  double *t0 = t, *t1 = t + n, *t2 = t + 2 * n, *x0 = t + 3 * n, *x1 = t + 4 * n, *x2 = t + 5 * n;
  cudaStream_t s = p->stream;
  const pn::Coefs c{mu_d, rho_d, mu_c, rho_c};
  // t = curl(u_e); X = gs(B curl t)
  NTG_TRY(curl_avg(p, t0, t1, t2, ue, ve, we));
  NTG_TRY(bcurl(p, x0, x1, x2, t0, t1, t2));
  NTG_TRY(gs_launch(p, x0, NTG_GS_ADD, s));
  NTG_TRY(gs_launch(p, x1, NTG_GS_ADD, s));
  NTG_TRY(gs_launch(p, x2, NTG_GS_ADD, s));
  // ta = gs(f / rho - (mu / rho) B wa); its Binv is applied where ta is read
  { pn::k_ta<<<grid_for(n, 256), 256, 0, s>>>(x0, x1, x2, fx, fy, fz, p->B, p->binv, c, n); NTG_COUNT_LAUNCH(); }
  NTG_TRY(gs_launch(p, x0, NTG_GS_ADD, s));
  NTG_TRY(gs_launch(p, x1, NTG_GS_ADD, s));
  NTG_TRY(gs_launch(p, x2, NTG_GS_ADD, s));
  NTG_TRY(dv::dispatch<4>(p->lx, [&](auto L) -> int {
    constexpr int LX = decltype(L)::value;
    pn::k_prs_core<LX><<<dv::grid_of<LX, 4>(p), dv::Shape<LX, 4>::THREADS, 0, s>>>(
        p_res, pr, x0, x1, x2, p->binv, c, p->nelv, dv::dmat<LX>(p), pn::gptr(p), p->met, n);
    NTG_COUNT_LAUNCH();
    return NTG_OK;
  }));
  if (nprs) {
    pn::k_surface<<<grid_for(nprs, 256), 256, 0, s>>>(p_res, prs_idx, prs_s, nprs, base, u, v, w, nullptr, bd / dt,
                                                      n);
    NTG_COUNT_LAUNCH();
  }
  if (nsym) {
    pn::k_surface<<<grid_for(nsym, 256), 256, 0, s>>>(p_res, sym_idx, sym_s, nsym, base, x0, x1, x2, p->binv, 1.0,
                                                      n);
    NTG_COUNT_LAUNCH();
  }
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

int ntg_pnpn_vel_res(ntg_plan* p, double* u_res, double* v_res, double* w_res, const double* u, const double* v,
                     const double* w, const double* pr, const double* fx, const double* fy, const double* fz,
                     const double* mu_d, double mu_c, const double* rho_d, double rho_c, double bd, double dt) {
  clear_error();
  NTG_CHECK_ARG(p && u_res && v_res && w_res && u && v && w && pr && fx && fy && fz,
                "ntg_pnpn_vel_res: null field argument");
  NTG_CHECK_ARG(dt > 0.0, "ntg_pnpn_vel_res: need dt > 0");
  NTG_TRY(need_metrics(p));
  const pn::Coefs c{mu_d, rho_d, mu_c, rho_c};
  return dv::dispatch<5>(p->lx, [&](auto L) -> int {
    constexpr int LX = decltype(L)::value;
    pn::k_vel_res<LX><<<dv::grid_of<LX, 5>(p), dv::Shape<LX, 5>::THREADS, 0, p->stream>>>(
        u_res, v_res, w_res, u, v, w, pr, fx, fy, fz, c, bd / dt, p->nelv, dv::dmat<LX>(p), pn::gptr(p), p->B,
        p->met, p->n);
    NTG_COUNT_LAUNCH();
    NTG_CUDA_TRY(cudaGetLastError());
    return NTG_OK;
  });
}

}  // extern "C"
