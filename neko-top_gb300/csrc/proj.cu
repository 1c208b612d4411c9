// Fischer residual projection (projection_t) and the PDE density filter.
//
// Projection replaces Neko's projection_t%pre_solving / post_solving
// (sources/adjoint/adjoint_pnpn.f90:365-374,729-741): the basis holds L
// A-orthonormal earlier solutions x_k together with A x_k (assembled), so
//   pre:  alpha_k = (x_k, b);  xbar = sum alpha_k x_k;  b <- b - sum alpha_k A x_k
//   post: dx (the solve's answer) is A-orthogonalised against the basis by
//         classical Gram-Schmidt applied twice, normalised and appended;
//         x = xbar + dx.  A full basis restarts from the normalised full
//         solution (its A-image is A xbar + A dx, no extra application).
// All inner products are mult-weighted (unique-node) FP64 sums from one
// multi-dot kernel that streams the basis once per call.
//
// The filter replaces PDE_filter_t%apply_forward/backward
// (sources/mapping_functions/PDE_filter_mapping.f90:212-363).
#include <cmath>
#include <cstring>

#include "common.cuh"
#include "reduce.cuh"

namespace ntg {

int jacobi_update(ntg_plan* p);

constexpr int kProjMax = 32;

// out[k] = sum_l mult_l a_l B_k,l for k < m (B_k = base + k*n)
template <int MAXL>
__global__ void k_multidot(const double* __restrict__ a, const double* __restrict__ base, int m, int64_t n,
                           const double* __restrict__ mult, double* __restrict__ part, Scalars* sc,
                           double* __restrict__ out) {
  double acc[MAXL];
#pragma unroll
  for (int k = 0; k < MAXL; ++k) acc[k] = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double ai = a[i] * mult[i];
#pragma unroll
    for (int k = 0; k < MAXL; ++k)
      if (k < m) acc[k] += ai * base[(int64_t)k * n + i];
  }
  struct Fin {
    double* out;
    int m;
    __device__ void operator()(const double* t, Scalars*) const {
      for (int k = 0; k < m; ++k) out[k] = t[k];
    }
  };
  grid_reduce<MAXL>(acc, part, sc, Fin{out, m});
}

// y1 -= sum c_k B1_k ; y2 -= sum c_k B2_k  (y2/B2 optional)
__global__ void k_multiaxpy(double* __restrict__ y1, const double* __restrict__ B1, double* __restrict__ y2,
                            const double* __restrict__ B2, const double* __restrict__ c, int m, int64_t n) {
  __shared__ double sc_[kProjMax];
  if (threadIdx.x < m) sc_[threadIdx.x] = c[threadIdx.x];
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double v1 = y1[i];
    double v2 = y2 ? y2[i] : 0.0;
    for (int k = 0; k < m; ++k) {
      v1 -= sc_[k] * B1[(int64_t)k * n + i];
      if (y2) v2 -= sc_[k] * B2[(int64_t)k * n + i];
    }
    y1[i] = v1;
    if (y2) y2[i] = v2;
  }
}

// xbar = sum alpha_k x_k; axbar = sum alpha_k A x_k; b -= axbar
__global__ void k_proj_pre(double* __restrict__ xbar, double* __restrict__ axbar, double* __restrict__ b,
                           const double* __restrict__ xs, const double* __restrict__ axs,
                           const double* __restrict__ c, int m, int64_t n) {
  __shared__ double sc_[kProjMax];
  if (threadIdx.x < m) sc_[threadIdx.x] = c[threadIdx.x];
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double xb = 0.0, ab = 0.0;
    for (int k = 0; k < m; ++k) {
      xb += sc_[k] * xs[(int64_t)k * n + i];
      ab += sc_[k] * axs[(int64_t)k * n + i];
    }
    xbar[i] = xb;
    axbar[i] = ab;
    b[i] -= ab;
  }
}

// xbar += beta v; axbar += beta A v; b -= beta A v  (beta = c[0])
__global__ void k_proj_add(double* __restrict__ xbar, double* __restrict__ axbar, double* __restrict__ b,
                           const double* __restrict__ v, const double* __restrict__ av, const double* __restrict__ c,
                           int64_t n) {
  const double beta = c[0];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    xbar[i] += beta * v[i];
    axbar[i] += beta * av[i];
    b[i] -= beta * av[i];
  }
}

// v += beta g; av += beta A g  (beta = c[0])
__global__ void k_proj_add_back(double* __restrict__ v, double* __restrict__ av, const double* __restrict__ g,
                                const double* __restrict__ ag, const double* __restrict__ c, int64_t n) {
  const double beta = c[0];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    v[i] += beta * g[i];
    av[i] += beta * ag[i];
  }
}

// a *= 1/sqrt(nrm2), b likewise
__global__ void k_scale2(double* __restrict__ a, double* __restrict__ b, const double* __restrict__ nrm2, int64_t n) {
  const double s = 1.0 / sqrt(*nrm2);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    a[i] *= s;
    b[i] *= s;
  }
}
// o = a + b
__global__ void k_sum3(double* __restrict__ o, const double* __restrict__ a, const double* __restrict__ b,
                       int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    o[i] = a[i] + b[i];
}
// o = a - b
__global__ void k_sub3(double* __restrict__ o, const double* __restrict__ a, const double* __restrict__ b,
                       int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    o[i] = a[i] - b[i];
}
// o = a * B
__global__ void k_mulB(double* __restrict__ o, const double* __restrict__ a, const double* __restrict__ B, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    o[i] = a[i] * B[i];
}

int multidot(ntg_plan* p, const double* a, const double* base, int m, double* out_d, Scalars* sc, cudaStream_t s) {
  if (m <= 0) return NTG_OK;
  const int T = 256;
  int G = grid_for(p->n, T);
  if (m <= 8) { k_multidot<8><<<G, T, 0, s>>>(a, base, m, p->n, p->mult, p->red_part, sc, out_d); NTG_COUNT_LAUNCH(); }
  else if (m <= 16) { k_multidot<16><<<G, T, 0, s>>>(a, base, m, p->n, p->mult, p->red_part, sc, out_d); NTG_COUNT_LAUNCH(); }
  else { k_multidot<32><<<G, T, 0, s>>>(a, base, m, p->n, p->mult, p->red_part, sc, out_d); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

}  // namespace ntg

struct ntg_proj {
  ntg_plan* plan = nullptr;
  int L = 0, m = 0;
  double* xs = nullptr;   // L*n
  double* axs = nullptr;  // L*n
  double* xbar = nullptr;
  double* axbar = nullptr;  // A xbar = b_original - b_reduced
  double* adx = nullptr;
  double* gv = nullptr;     // extra direction and its A-image (pre_solving_with)
  double* gav = nullptr;
  double* coef = nullptr;   // kProjMax + 1 device coefficients
  ntg::Scalars* sc = nullptr;
  double* hcoef = nullptr;  // pinned
  int have_pre = 0;
  int have_extra = 0;       // this solve's xbar includes beta * gv (coef[kProjMax + 2])
};

using namespace ntg;

static void proj_free(ntg_proj* q) {
  dev_free(q->xs); dev_free(q->axs); dev_free(q->xbar); dev_free(q->axbar); dev_free(q->adx);
  dev_free(q->gv); dev_free(q->gav);
  dev_free(q->coef); dev_free(q->sc);
  if (q->hcoef) cudaFreeHost(q->hcoef);
  q->hcoef = nullptr;
}

extern "C" {

int ntg_proj_create(ntg_plan* plan, int L, ntg_proj** proj) {
  clear_error();
  NTG_CHECK_ARG(plan && proj, "ntg_proj_create: null argument");
  NTG_CHECK_ARG(L >= 1 && L <= kProjMax, "ntg_proj_create: L must be in [1, 32]");
  *proj = nullptr;
  ntg_proj* q = new ntg_proj();
  q->plan = plan;
  q->L = L;
  const int64_t n = plan->n;
  int st = NTG_OK;
  do {
    if ((st = dev_alloc(&q->xs, (size_t)L * n))) break;
    if ((st = dev_alloc(&q->axs, (size_t)L * n))) break;
    if ((st = dev_alloc(&q->xbar, n))) break;
    if ((st = dev_alloc(&q->axbar, n))) break;
    if ((st = dev_alloc(&q->adx, n))) break;
    if ((st = dev_alloc(&q->gv, n))) break;
    if ((st = dev_alloc(&q->gav, n))) break;
    if ((st = dev_alloc(&q->coef, kProjMax + 4))) break;
    if ((st = dev_alloc(&q->sc, 1))) break;
    if (cudaMemset(q->sc, 0, sizeof(Scalars)) != cudaSuccess) { st = NTG_ERR_CUDA; break; }
    if (cudaMallocHost(&q->hcoef, sizeof(double) * (kProjMax + 1)) != cudaSuccess) { st = NTG_ERR_ALLOC; break; }
  } while (0);
  if (st) {
    proj_free(q);
    delete q;
    return st;
  }
  *proj = q;
  return NTG_OK;
}

int ntg_proj_destroy(ntg_proj* proj) {
  clear_error();
  if (!proj) return NTG_OK;
  cudaStreamSynchronize(proj->plan->stream);
  proj_free(proj);
  delete proj;
  return NTG_OK;
}

int ntg_proj_size(const ntg_proj* proj) { return proj ? proj->m : 0; }

int ntg_proj_pre_solving(ntg_proj* q, double* b_d) {
  clear_error();
  NTG_CHECK_ARG(q && b_d, "ntg_proj_pre_solving: null argument");
  ntg_plan* p = q->plan;
  cudaStream_t s = p->stream;
  const int64_t n = p->n;
  const int G = grid_for(n, 256);
  if (q->m > 0) {
    NTG_TRY(multidot(p, b_d, q->xs, q->m, q->coef, q->sc, s));
    { k_proj_pre<<<G, 256, 0, s>>>(q->xbar, q->axbar, b_d, q->xs, q->axs, q->coef, q->m, n); NTG_COUNT_LAUNCH(); }
    NTG_CUDA_TRY(cudaGetLastError());
  } else {
    NTG_CUDA_TRY(cudaMemsetAsync(q->xbar, 0, sizeof(double) * n, s));
    NTG_CUDA_TRY(cudaMemsetAsync(q->axbar, 0, sizeof(double) * n, s));
  }
  q->have_pre = 1;
  q->have_extra = 0;
  return NTG_OK;
}

// pre_solving with one extra direction g (e.g. a learned guess): after the
// usual projection, g is A-orthogonalised against the basis (classical
// Gram-Schmidt, twice), A-normalised, and the Galerkin component of b along
// it is moved into xbar as well.  The direction is used for this solve only.
// Costs one FP64 operator application.  *used = 0 when g adds nothing.
int ntg_proj_pre_solving_with(ntg_proj* q, double* b_d, const double* g_d, int* used) {
  clear_error();
  NTG_CHECK_ARG(q && b_d && g_d && used, "ntg_proj_pre_solving_with: null argument");
  *used = 0;
  NTG_TRY(ntg_proj_pre_solving(q, b_d));
  ntg_plan* p = q->plan;
  cudaStream_t s = p->stream;
  const int64_t n = p->n;
  const int G = grid_for(n, 256);
  double* v = q->gv;
  double* av = q->gav;
  NTG_CUDA_TRY(cudaMemcpyAsync(v, g_d, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  NTG_TRY(op_apply(p, av, v, s));
  // (g, A g) for the rank test
  NTG_TRY(multidot(p, v, av, 1, q->coef + kProjMax, q->sc, s));
  NTG_CUDA_TRY(cudaMemcpyAsync(q->hcoef + 1, q->coef + kProjMax, sizeof(double), cudaMemcpyDeviceToHost, s));
  for (int pass = 0; pass < 2 && q->m > 0; ++pass) {
    NTG_TRY(multidot(p, av, q->xs, q->m, q->coef, q->sc, s));
    { k_multiaxpy<<<G, 256, 0, s>>>(v, q->xs, av, q->axs, q->coef, q->m, n); NTG_COUNT_LAUNCH(); }
  }
  NTG_TRY(multidot(p, v, av, 1, q->coef + kProjMax, q->sc, s));
  NTG_CUDA_TRY(cudaMemcpyAsync(q->hcoef, q->coef + kProjMax, sizeof(double), cudaMemcpyDeviceToHost, s));
  NTG_CUDA_TRY(cudaStreamSynchronize(s));
  const double nrm2 = q->hcoef[0], gag = q->hcoef[1];
  if (!(nrm2 > 1e-14 * gag) || !std::isfinite(nrm2)) return NTG_OK;
  { k_scale2<<<G, 256, 0, s>>>(v, av, q->coef + kProjMax, n); NTG_COUNT_LAUNCH(); }
  // beta = (v, b); keep the direction only if it lowers the residual norm:
  // ||b - beta A v||^2 - ||b||^2 = beta^2 (Av, Av) - 2 beta (Av, b)
  NTG_TRY(multidot(p, b_d, v, 1, q->coef + kProjMax + 2, q->sc, s));
  NTG_TRY(multidot(p, av, b_d, 1, q->coef + kProjMax + 1, q->sc, s));
  NTG_TRY(multidot(p, av, av, 1, q->coef + kProjMax + 3, q->sc, s));
  NTG_CUDA_TRY(cudaMemcpyAsync(q->hcoef, q->coef + kProjMax + 1, 3 * sizeof(double), cudaMemcpyDeviceToHost, s));
  NTG_CUDA_TRY(cudaStreamSynchronize(s));
  const double bav = q->hcoef[0], beta = q->hcoef[1], avav = q->hcoef[2];
  if (!(beta * beta * avav - 2.0 * beta * bav < 0.0)) return NTG_OK;
  // xbar += beta v; b -= beta A v
  { k_proj_add<<<G, 256, 0, s>>>(q->xbar, q->axbar, b_d, v, av, q->coef + kProjMax + 2, n); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  q->have_extra = 1;
  *used = 1;
  return NTG_OK;
}

int ntg_proj_post_solving(ntg_proj* q, double* x_d) {
  clear_error();
  NTG_CHECK_ARG(q && x_d, "ntg_proj_post_solving: null argument");
  NTG_CHECK_ARG(q->have_pre, "ntg_proj_post_solving: pre_solving was not called");
  ntg_plan* p = q->plan;
  cudaStream_t s = p->stream;
  const int64_t n = p->n;
  const int G = grid_for(n, 256);
  q->have_pre = 0;
  NTG_TRY(op_apply(p, q->adx, x_d, s));
  if (q->m >= q->L) {
    // restart from the full solution x = xbar + dx, A x = A xbar + A dx
    { k_sum3<<<G, 256, 0, s>>>(q->xs, q->xbar, x_d, n); NTG_COUNT_LAUNCH(); }
    { k_sum3<<<G, 256, 0, s>>>(q->axs, q->axbar, q->adx, n); NTG_COUNT_LAUNCH(); }
    NTG_TRY(multidot(p, q->xs, q->axs, 1, q->coef + kProjMax, q->sc, s));
    NTG_CUDA_TRY(cudaMemcpyAsync(q->hcoef, q->coef + kProjMax, sizeof(double), cudaMemcpyDeviceToHost, s));
    NTG_CUDA_TRY(cudaStreamSynchronize(s));
    if (q->hcoef[0] > 0.0 && std::isfinite(q->hcoef[0])) {
      { k_scale2<<<G, 256, 0, s>>>(q->xs, q->axs, q->coef + kProjMax, n); NTG_COUNT_LAUNCH(); }
      q->m = 1;
    } else {
      q->m = 0;
    }
  } else {
    double* v = q->xs + (int64_t)q->m * n;
    double* av = q->axs + (int64_t)q->m * n;
    NTG_CUDA_TRY(cudaMemcpyAsync(v, x_d, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    NTG_CUDA_TRY(cudaMemcpyAsync(av, q->adx, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    if (q->have_extra) {
      // the basis takes x minus its projection on the old basis: add back the
      // extra direction's share so no part of it enters the basis as noise
      { k_proj_add_back<<<G, 256, 0, s>>>(v, av, q->gv, q->gav, q->coef + kProjMax + 2, n); NTG_COUNT_LAUNCH(); }
    }
    for (int pass = 0; pass < 2 && q->m > 0; ++pass) {
      NTG_TRY(multidot(p, v, q->axs, q->m, q->coef, q->sc, s));
      { k_multiaxpy<<<G, 256, 0, s>>>(v, q->xs, av, q->axs, q->coef, q->m, n); NTG_COUNT_LAUNCH(); }
    }
    NTG_TRY(multidot(p, v, av, 1, q->coef + kProjMax, q->sc, s));
    NTG_CUDA_TRY(cudaMemcpyAsync(q->hcoef, q->coef + kProjMax, sizeof(double), cudaMemcpyDeviceToHost, s));
    NTG_CUDA_TRY(cudaStreamSynchronize(s));
    if (q->hcoef[0] > 1e-300 && std::isfinite(q->hcoef[0])) {
      { k_scale2<<<G, 256, 0, s>>>(v, av, q->coef + kProjMax, n); NTG_COUNT_LAUNCH(); }
      q->m += 1;
    }
  }
  // x = xbar + dx
  { k_sum3<<<G, 256, 0, s>>>(x_d, q->xbar, x_d, n); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

// post_solving for a solution found elsewhere: x_d is the full solution of
// the right-hand side given to the preceding pre_solving (not the reduced
// one), e.g. the same solve made by another solver or read from a restart.
// The basis takes dx = x - xbar exactly as post_solving(dx) would; x_d is
// left unchanged.  Not after pre_solving_with (its extra direction is
// for one solve only).
int ntg_proj_post_solving_full(ntg_proj* q, const double* x_d) {
  clear_error();
  NTG_CHECK_ARG(q && x_d, "ntg_proj_post_solving_full: null argument");
  NTG_CHECK_ARG(q->have_pre, "ntg_proj_post_solving_full: pre_solving was not called");
  NTG_CHECK_ARG(!q->have_extra, "ntg_proj_post_solving_full: not after pre_solving_with");
  ntg_plan* p = q->plan;
  cudaStream_t s = p->stream;
  const int64_t n = p->n;
  const int G = grid_for(n, 256);
  // dx = x - xbar into the (unused) extra-direction buffer
  { k_sub3<<<G, 256, 0, s>>>(q->gv, x_d, q->xbar, n); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  return ntg_proj_post_solving(q, q->gv);
}

// The basis for checkpoints: m (vectors held), and with dir = 0 copies the
// m basis vectors and their A-images out to xs_d / axs_d (m*n doubles
// each), with dir = 1 loads m of them (m <= L) back in.
int ntg_proj_state(ntg_proj* q, int* m, double* xs_d, double* axs_d, int dir) {
  clear_error();
  NTG_CHECK_ARG(q && m && (dir == 0 || dir == 1), "ntg_proj_state: bad argument");
  ntg_plan* p = q->plan;
  cudaStream_t s = p->stream;
  const size_t bytes = sizeof(double) * (size_t)p->n;
  if (dir == 0) {
    *m = q->m;
    if (xs_d && q->m) NTG_CUDA_TRY(cudaMemcpyAsync(xs_d, q->xs, bytes * q->m, cudaMemcpyDeviceToDevice, s));
    if (axs_d && q->m) NTG_CUDA_TRY(cudaMemcpyAsync(axs_d, q->axs, bytes * q->m, cudaMemcpyDeviceToDevice, s));
  } else {
    NTG_CHECK_ARG(*m >= 0 && *m <= q->L, "ntg_proj_state: m must be in [0, L]");
    NTG_CHECK_ARG(*m == 0 || (xs_d && axs_d), "ntg_proj_state: null basis");
    if (*m) {
      NTG_CUDA_TRY(cudaMemcpyAsync(q->xs, xs_d, bytes * *m, cudaMemcpyDeviceToDevice, s));
      NTG_CUDA_TRY(cudaMemcpyAsync(q->axs, axs_d, bytes * *m, cudaMemcpyDeviceToDevice, s));
    }
    q->m = *m;
    q->have_pre = 0;
    q->have_extra = 0;
  }
  NTG_CUDA_TRY(cudaStreamSynchronize(s));
  return NTG_OK;
}

// PDE filter: (r^2 K + B) X_out = B X_in with all-Neumann boundaries and
// X_in as initial guess (PDE_filter_mapping.f90:212-278; the backward map at
// :298-363 is the same solve applied to dF/dX_out).  The solve uses the
// ksp's Jacobi-PCG; the plan's Dirichlet mask is suspended during the call.
int ntg_filter_apply(ntg_plan* p, ntg_ksp* ksp, double* X_out_d, const double* X_in_d, double r,
                     ntg_monitor* mon) {
  clear_error();
  NTG_CHECK_ARG(p && ksp && X_out_d && X_in_d, "ntg_filter_apply: null argument");
  cudaStream_t s = p->stream;
  const int64_t n = p->n;
  const int G = grid_for(n, 256);
  // h1 = r^2, h2 = 1 (the filter overwrites the shared coefficients)
  NTG_TRY(ntg_coef_set(p, nullptr, r * r, nullptr, 1.0, 1));
  double* rhs = nullptr;
  NTG_TRY(dev_alloc(&rhs, n));
  int32_t* saved_mask = p->mask;
  int64_t saved_nmask = p->nmask;
  p->mask = nullptr;
  p->nmask = 0;
  int st = NTG_OK;
  do {
    { k_mulB<<<G, 256, 0, s>>>(rhs, X_in_d, p->B, n); NTG_COUNT_LAUNCH(); }
    if (cudaGetLastError() != cudaSuccess) { st = NTG_ERR_CUDA; set_error("filter rhs"); break; }
    if ((st = gs_launch(p, rhs, NTG_GS_ADD, s))) break;
    if (cudaMemcpyAsync(X_out_d, X_in_d, sizeof(double) * n, cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
      st = NTG_ERR_CUDA; set_error("filter guess copy"); break;
    }
    if ((st = jacobi_update(p))) break;
    st = ntg_ksp_solve(ksp, X_out_d, rhs, mon);
  } while (0);
  p->mask = saved_mask;
  p->nmask = saved_nmask;
  p->jacobi_ready = 0;  // the next solve rebuilds the diagonal with its mask
  cudaStreamSynchronize(s);
  dev_free(rhs);
  return st;
}

}  // extern "C"
