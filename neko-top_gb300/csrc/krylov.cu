// Jacobi preconditioner, Jacobi-PCG (FP64 drop-in), the mixed-precision
// flexible CG (FP32 inner PCG, FP64 outer residuals and dots), Fischer
// residual projection, the PDE filter driver and generic dot products.
//
// Replaces Neko's pc_t (jacobi), ksp_t (cg) and projection_t, used by the
// reference at sources/adjoint/adjoint_pnpn.f90:729-741,781-794 and
// sources/mapping_functions/PDE_filter_mapping.f90:180-184,246-262.
//
// Solver state lives on the device (Scalars); every iteration is a fixed
// sequence of kernels (Ax with the fused (p, Ap) dot, gather-scatter, mask,
// update with fused (r, z) and (r, r) dots, direction update), each of which
// returns at once after the device-side convergence flag is set.  The host
// reads the flag every `check_every` iterations, so the iteration count is
// exact and no per-iteration host round trip is needed.
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "reduce.cuh"

namespace ntg {

// ---------------------------------------------------------------------------
// Jacobi diagonal of the element operator (see the derivation in the oracle):
//   sum_l D_li^2 G11(l,j,k) h1 + D_lj^2 G22(i,l,k) h1 + D_lk^2 G33(i,j,l) h1
//   + 2 h1 (D_ii D_jj G12 + D_ii D_kk G13 + D_jj D_kk G23) + h2 B
// ---------------------------------------------------------------------------
struct DBig {
  double d[NTG_LXMAX * NTG_LXMAX];
};

__global__ void k_helm_diag(int64_t nelv, int lx, const __grid_constant__ DBig D, const double* __restrict__ g11,
                            const double* __restrict__ g12, const double* __restrict__ g13,
                            const double* __restrict__ g22, const double* __restrict__ g23,
                            const double* __restrict__ g33, const double* __restrict__ h1, double h1c,
                            const double* __restrict__ hB, double* __restrict__ d) {
  const int64_t lx3 = (int64_t)lx * lx * lx;
  const int64_t n = nelv * lx3;
  for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < n; m += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = m / lx3;
    const int r = (int)(m - e * lx3);
    const int i = r % lx, j = (r / lx) % lx, k = r / (lx * lx);
    const int64_t base = e * lx3;
    double acc = 0.0;
    for (int l = 0; l < lx; ++l) {
      int64_t qr = base + l + lx * (j + lx * k);
      int64_t qs = base + i + lx * (l + lx * k);
      int64_t qt = base + i + lx * (j + lx * l);
      double hr = h1 ? h1[qr] : h1c, hs = h1 ? h1[qs] : h1c, ht = h1 ? h1[qt] : h1c;
      double a = D.d[l * lx + i], b = D.d[l * lx + j], c = D.d[l * lx + k];
      acc += a * a * g11[qr] * hr;
      acc += b * b * g22[qs] * hs;
      acc += c * c * g33[qt] * ht;
    }
    double hm = h1 ? h1[m] : h1c;
    double di = D.d[i * lx + i], dj = D.d[j * lx + j], dk = D.d[k * lx + k];
    acc += 2.0 * hm * (di * dj * g12[m] + di * dk * g13[m] + dj * dk * g23[m]);
    if (hB) acc += hB[m];
    d[m] = acc;
  }
}

__global__ void k_set_masked(double* __restrict__ u, const int32_t* __restrict__ mask, int64_t m, double v) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < m; q += (int64_t)gridDim.x * blockDim.x)
    u[mask[q]] = v;
}
__global__ void k_invert(double* __restrict__ d, float* __restrict__ df, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double v = 1.0 / d[i];
    d[i] = v;
    df[i] = (float)v;
  }
}
__global__ void k_col3(double* __restrict__ z, const double* __restrict__ a, const double* __restrict__ b, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    z[i] = a[i] * b[i];
}

int jacobi_update(ntg_plan* p) {
  cudaStream_t s = p->stream;
  if (!p->dinv) NTG_TRY(dev_alloc(&p->dinv, p->n));
  if (!p->dinvf) NTG_TRY(dev_alloc(&p->dinvf, p->n));
  DBig D;
  memcpy(D.d, p->D, sizeof(double) * p->lx * p->lx);
  { k_helm_diag<<<grid_for(p->n, 256), 256, 0, s>>>(p->nelv, p->lx, D, p->g[0], p->g[1], p->g[2], p->g[3], p->g[4],
                                                    p->g[5], p->h1_const ? nullptr : p->h1, p->h1c,
                                                    p->ifh2 ? p->hB : nullptr, p->dinv); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  NTG_TRY(gs_launch(p, p->dinv, NTG_GS_ADD, s));
  if (p->nmask) { k_set_masked<<<grid_for(p->nmask, 256), 256, 0, s>>>(p->dinv, p->mask, p->nmask, 1.0); NTG_COUNT_LAUNCH(); }
  { k_invert<<<grid_for(p->n, 256), 256, 0, s>>>(p->dinv, p->dinvf, p->n); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  p->jacobi_ready = 1;
  return NTG_OK;
}

// ---------------------------------------------------------------------------
// Generic reductions
// ---------------------------------------------------------------------------
struct FinStore {
  int slot;
  __device__ void operator()(const double* acc, Scalars* sc) const { sc->red[slot] = acc[0]; }
};

__global__ void k_wdot(const double* __restrict__ a, const double* __restrict__ b, const double* __restrict__ c,
                       int64_t n, double* __restrict__ part, Scalars* sc) {
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s += c ? a[i] * b[i] * c[i] : a[i] * b[i];
  double v[1] = {s};
  grid_reduce<1>(v, part, sc, FinStore{0});
}

int wdot(ntg_plan* p, const double* a, const double* b, const double* c, int64_t n, double* host_out,
         cudaStream_t s) {
  { k_wdot<<<grid_for(n, 256), 256, 0, s>>>(a, b, c, n, p->red_part, p->scal); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  NTG_CUDA_TRY(cudaMemcpyAsync(p->host_red, &p->scal->red[0], sizeof(double), cudaMemcpyDeviceToHost, s));
  NTG_CUDA_TRY(cudaStreamSynchronize(s));
  *host_out = p->host_red[0];
  return NTG_OK;
}

// ---------------------------------------------------------------------------
// PCG kernels (T = double for the FP64 solver, float for the inner solve;
// reductions always accumulate in FP64).
// ---------------------------------------------------------------------------
struct FinInit {
  __device__ void operator()(const double* acc, Scalars* sc) const {
    // acc: ff, rr, rz
    sc->ff = acc[0];
    sc->rr = acc[1];
    sc->rr0 = acc[1];
    sc->rz = acc[2];
    double t = sc->rtol * sqrt(acc[0]);
    if (sc->abstol > t) t = sc->abstol;
    sc->tol2 = t * t;
    sc->iter = 0;
    sc->status = NTG_OK;
    sc->done = 0;
    if (!isfinite(acc[0]) || !isfinite(acc[1]) || !isfinite(acc[2])) {
      sc->status = NTG_NONFINITE;
      sc->done = 1;
    } else if (acc[1] <= sc->tol2) {
      sc->done = 1;
    } else if (sc->max_iter <= 0) {
      sc->status = NTG_MAXITER;
      sc->done = 1;
    }
  }
};

// r = f - w (w == null: r = f); z = dinv r; p = z; sums ff, rr, rz
template <typename T>
__global__ void k_cg_init(const T* __restrict__ f, const T* __restrict__ w, const T* __restrict__ dinv,
                          const T* __restrict__ mult, T* __restrict__ r, T* __restrict__ p, int64_t n,
                          double* __restrict__ part, Scalars* sc) {
  double ff = 0, rr = 0, rz = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    T fi = f[i];
    T ri = w ? fi - w[i] : fi;
    T zi = dinv[i] * ri;
    r[i] = ri;
    p[i] = zi;
    double m = (double)mult[i];
    ff += m * (double)fi * (double)fi;
    rr += m * (double)ri * (double)ri;
    rz += m * (double)ri * (double)zi;
  }
  double v[3] = {ff, rr, rz};
  grid_reduce<3>(v, part, sc, FinInit());
}

struct FinUpd {
  __device__ void operator()(const double* acc, Scalars* sc) const {
    // acc: rz_new, rr
    sc->iter += 1;
    sc->rr = acc[1];
    if (!isfinite(acc[0]) || !isfinite(acc[1])) {
      sc->status = NTG_NONFINITE;
      sc->done = 1;
      return;
    }
    if (sc->ru_mode) {
      // FP32 residual: a converged one is only a candidate (the host
      // confirms it with an FP64 residual); a drop by delta since the last
      // FP64 residual asks for a replacement.  Both stop the FP32 iteration
      // here, before the direction update, so the replacement comes at once
      // (iterating on to the host's next poll can carry the FP32 recurrence
      // decades past what FP32 resolves); the host completes the iteration.
      const double rn = sqrt(acc[1]);
      if (rn > sc->rmax) sc->rmax = rn;
      if (acc[1] <= sc->tol2 || rn < sc->delta * sc->rmax) {
        sc->need_ru = 2;
        sc->done = 1;
        return;
      }
    } else if (acc[1] <= sc->tol2) {
      sc->done = 1;
      return;
    }
    if (sc->iter >= sc->max_iter) {
      sc->status = NTG_MAXITER;
      sc->done = 1;
      return;
    }
    if (sc->ext_pc) return;  // beta and (r, z) come with the preconditioner application
    sc->beta = acc[0] / sc->rz;
    sc->rz = acc[0];
  }
};

// x += alpha p; r -= alpha w; sums (r, dinv r), (r, r)
template <typename T>
__global__ void k_cg_update(T* __restrict__ x, const T* __restrict__ p, T* __restrict__ r, const T* __restrict__ w,
                            const T* __restrict__ dinv, const T* __restrict__ mult, int64_t n,
                            double* __restrict__ part, Scalars* sc) {
  if (sc->done) return;
  const T alpha = (T)sc->alpha;
  // per-thread partials in T: FP64 arithmetic is 1/58 of FP32 on GB300, so
  // the FP32 iteration accumulates its short per-thread sums in FP32 and
  // only the block/grid levels in FP64
  T rz = 0, rr = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    T xi = x[i] + alpha * p[i];
    T ri = r[i] - alpha * w[i];
    x[i] = xi;
    r[i] = ri;
    T mr = mult[i] * ri;
    rz += mr * (dinv[i] * ri);
    rr += mr * ri;
  }
  double v[2] = {(double)rz, (double)rr};
  grid_reduce<2>(v, part, sc, FinUpd());
}

// p = dinv r + beta p
template <typename T>
__global__ void k_cg_dir(T* __restrict__ p, const T* __restrict__ r, const T* __restrict__ dinv, int64_t n,
                         const Scalars* sc) {
  if (sc->done) return;
  const T beta = (T)sc->beta;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = dinv[i] * r[i] + beta * p[i];
}

template <typename T>
struct PcgVecs {
  T *r = nullptr, *p = nullptr, *w = nullptr;
};

// Runs Jacobi-PCG on x (guess in, solution out) for rhs f.  `zero_guess`
// skips the initial operator application.  Returns the final host copy of
// the scalars in *hs.
template <typename T>
static int run_pcg(ntg_plan* pl, Scalars* sc, Scalars* hs_pinned, PcgVecs<T>& v, T* x, const T* f,
                   const T* dinv, const T* mult, double rtol, double abstol, int max_iter, bool zero_guess,
                   int check_every, cudaStream_t s, int* fp_ax) {
  const int64_t n = pl->n;
  const int TPB = 256;
  const int G = grid_for(n, TPB);
  // reset the scalar block
  memset(hs_pinned, 0, sizeof(Scalars));
  hs_pinned->rtol = rtol;
  hs_pinned->abstol = abstol;
  hs_pinned->max_iter = max_iter;
  NTG_CUDA_TRY(cudaMemcpyAsync(sc, hs_pinned, sizeof(Scalars), cudaMemcpyHostToDevice, s));
  if (!zero_guess) {
    if (sizeof(T) == 8) NTG_TRY(op_apply(pl, (double*)v.w, (const double*)x, s));
    else NTG_TRY(op_apply_f32(pl, (float*)v.w, (const float*)x, s));
    if (fp_ax && sizeof(T) == 8) (*fp_ax)++;
  }
  { k_cg_init<T><<<G, TPB, 0, s>>>(f, zero_guess ? nullptr : v.w, dinv, mult, v.r, v.p, n, pl->red_part, sc); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  int launched = 0;
  for (;;) {
    NTG_CUDA_TRY(cudaMemcpyAsync(hs_pinned, sc, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
    NTG_CUDA_TRY(cudaStreamSynchronize(s));
    if (hs_pinned->done) break;
    if (launched >= max_iter + check_every) break;  // defensive: device cap reached
    for (int c = 0; c < check_every; ++c) {
      if (sizeof(T) == 8) {
        NTG_TRY(ax_launch(pl, (double*)v.w, (const double*)v.p, sc, 0, s));
        NTG_TRY(gs_add_guarded(pl, (double*)v.w, s, sc));
        NTG_TRY(mask_guarded(pl, (double*)v.w, s, sc));
      } else {
        NTG_TRY(ax_launch_f32(pl, (float*)v.w, (const float*)v.p, sc, 0, s));
        NTG_TRY(gs_add_guarded_f32(pl, (float*)v.w, s, sc));
        NTG_TRY(mask_guarded_f32(pl, (float*)v.w, s, sc));
      }
      timer_start(sizeof(T) == 8 ? TM_UPD64 : TM_UPD32, s);
      { k_cg_update<T><<<G, TPB, 0, s>>>(x, v.p, v.r, v.w, dinv, mult, n, pl->red_part, sc); NTG_COUNT_LAUNCH(); }
      timer_stop(sizeof(T) == 8 ? TM_UPD64 : TM_UPD32, s);
      timer_start(sizeof(T) == 8 ? TM_DIR64 : TM_DIR32, s);
      { k_cg_dir<T><<<G, TPB, 0, s>>>(v.p, v.r, dinv, n, sc); NTG_COUNT_LAUNCH(); }
      timer_stop(sizeof(T) == 8 ? TM_DIR64 : TM_DIR32, s);
      NTG_CUDA_TRY(cudaGetLastError());
      ++launched;
    }
  }
  // each iteration that ran did exactly one FP64 Ax when T == double
  if (fp_ax && sizeof(T) == 8) *fp_ax += hs_pinned->iter;
  return NTG_OK;
}

// ---------------------------------------------------------------------------
// Mixed-precision flexible CG kernels
// ---------------------------------------------------------------------------
struct FinResid {
  __device__ void operator()(const double* acc, Scalars* sc) const {
    // acc: ff, rr
    sc->ff = acc[0];
    sc->rr = acc[1];
    sc->rr0 = acc[1];
    double t = sc->rtol * sqrt(acc[0]);
    if (sc->abstol > t) t = sc->abstol;
    sc->tol2 = t * t;
    sc->iter = 0;
    sc->status = NTG_OK;
    sc->done = 0;
    sc->pap_prev = 0.0;
    if (!isfinite(acc[0]) || !isfinite(acc[1])) {
      sc->status = NTG_NONFINITE;
      sc->done = 1;
    } else if (acc[1] <= sc->tol2) {
      sc->done = 1;
    }
  }
};

// r = f - w; sums ff, rr
__global__ void k_resid(const double* __restrict__ f, const double* __restrict__ w, const double* __restrict__ mult,
                        double* __restrict__ r, int64_t n, double* __restrict__ part, Scalars* sc) {
  double ff = 0, rr = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double fi = f[i];
    double ri = w ? fi - w[i] : fi;
    r[i] = ri;
    ff += mult[i] * fi * fi;
    rr += mult[i] * ri * ri;
  }
  double v[2] = {ff, rr};
  grid_reduce<2>(v, part, sc, FinResid());
}

// x32 = (float)x
__global__ void k_to_f32(const double* __restrict__ x, float* __restrict__ x32, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x32[i] = (float)x[i];
}

// the guard's residual from an FP32 operator image: w = (double)w32, r = f - w
__global__ void k_resid_w32(const double* __restrict__ f, const float* __restrict__ w32, double* __restrict__ w,
                            const double* __restrict__ mult, double* __restrict__ r, int64_t n,
                            double* __restrict__ part, Scalars* sc) {
  double ff = 0, rr = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double fi = f[i], wi = (double)w32[i];
    w[i] = wi;
    const double ri = fi - wi;
    r[i] = ri;
    ff += mult[i] * fi * fi;
    rr += mult[i] * ri * ri;
  }
  double v[2] = {ff, rr};
  grid_reduce<2>(v, part, sc, FinResid());
}

// inner right-hand side: rin = (float)(r / ||r||)
__global__ void k_to_f32_scaled(const double* __restrict__ r, float* __restrict__ rin, int64_t n, const Scalars* sc) {
  const double s = 1.0 / sqrt(sc->rr);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    rin[i] = (float)(r[i] * s);
}

struct FinGamma {
  __device__ void operator()(const double* acc, Scalars* sc) const {
    sc->gamma = sc->pap_prev > 0.0 ? acc[0] / sc->pap_prev : 0.0;
  }
};
// z = ||r|| * (double)din; sums (z, qprev)_mult.  z is continuous and q
// assembled, so the mult-weighted local sum is the unique-node product.
__global__ void k_from_f32(const float* __restrict__ din, double* __restrict__ z, const double* __restrict__ qprev,
                           const double* __restrict__ mult, int64_t n, double* __restrict__ part, Scalars* sc) {
  const double s = sqrt(sc->rr);
  double zq = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double zi = s * (double)din[i];
    z[i] = zi;
    if (qprev) zq += mult[i] * zi * qprev[i];
  }
  double v[1] = {zq};
  grid_reduce<1>(v, part, sc, FinGamma());
}
struct FinPr {
  __device__ void operator()(const double* acc, Scalars* sc) const { sc->rz = acc[0]; }
};
// p = z - gamma pprev; sums (p, r)_mult
__global__ void k_fcg_orth(double* __restrict__ p, const double* __restrict__ pprev, const double* __restrict__ r,
                           const double* __restrict__ mult, int64_t n, double* __restrict__ part, Scalars* sc) {
  const double g = sc->gamma;
  double pr = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double pi = p[i];
    if (pprev) pi -= g * pprev[i];
    p[i] = pi;
    pr += mult[i] * pi * r[i];
  }
  double v[1] = {pr};
  grid_reduce<1>(v, part, sc, FinPr());
}
struct FinOuter {
  __device__ void operator()(const double* acc, Scalars* sc) const {
    sc->iter += 1;
    sc->rr = acc[0];
    sc->pap_prev = sc->pap;
    if (!isfinite(acc[0])) {
      sc->status = NTG_NONFINITE;
      sc->done = 1;
    } else if (acc[0] <= sc->tol2) {
      sc->done = 1;
    } else if (sc->iter >= sc->max_iter) {
      sc->status = NTG_MAXITER;
      sc->done = 1;
    }
  }
};
// x += alpha p; r -= alpha q; sums (r, r)_mult
__global__ void k_fcg_update(double* __restrict__ x, const double* __restrict__ p, double* __restrict__ r,
                             const double* __restrict__ q, const double* __restrict__ mult, int64_t n,
                             double* __restrict__ part, Scalars* sc) {
  const double a = sc->alpha;
  double rr = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] += a * p[i];
    double ri = r[i] - a * q[i];
    r[i] = ri;
    rr += mult[i] * ri * ri;
  }
  double v[1] = {rr};
  grid_reduce<1>(v, part, sc, FinOuter());
}

__global__ void k_zero_f(float* __restrict__ a, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) a[i] = 0.f;
}

// ---------------------------------------------------------------------------
// Mixed-precision CG with reliable updates (Sleijpen & van der Vorst 1996;
// the residual-replacement scheme lattice-QCD solvers use for mixed
// precision).  One Jacobi-PCG runs in FP32 (operator, preconditioner,
// vectors); the FP32 iterate y accumulates a correction that is folded into
// the FP64 solution x whenever the FP32 residual has dropped by `delta`
// since the last replacement, at which point the residual is recomputed in
// FP64 (r = f - A x) and rounded back into the FP32 iteration.  The search
// direction is kept across replacements, so the Krylov space is never
// restarted.  Convergence is only declared on an FP64 residual.
// ---------------------------------------------------------------------------
struct FinRUInit {
  __device__ void operator()(const double* acc, Scalars* sc) const {
    // acc: ff, rr (FP64), rz (FP32 iteration)
    sc->ff = acc[0];
    sc->rr = acc[1];
    sc->rr0 = acc[1];
    sc->rz = acc[2];
    sc->rmax = sqrt(acc[1]);
    double t = sc->rtol * sqrt(acc[0]);
    if (sc->abstol > t) t = sc->abstol;
    sc->tol2 = t * t;
    sc->iter = 0;
    sc->status = NTG_OK;
    sc->done = 0;
    sc->need_ru = 0;
    if (!isfinite(acc[0]) || !isfinite(acc[1]) || !isfinite(acc[2])) {
      sc->status = NTG_NONFINITE;
      sc->done = 1;
    } else if (acc[1] <= sc->tol2) {
      sc->done = 1;
    } else if (sc->max_iter <= 0) {
      sc->status = NTG_MAXITER;
      sc->done = 1;
    }
  }
};

// r = f - w (w null: r = f); r32 = (float) r; p32 = dinv32 r32; y32 = 0
__global__ void k_ru_init(const double* __restrict__ f, const double* __restrict__ w, const float* __restrict__ dinv,
                          const double* __restrict__ mult, double* __restrict__ r, float* __restrict__ r32,
                          float* __restrict__ p32, float* __restrict__ y32, int64_t n, double* __restrict__ part,
                          Scalars* sc) {
  double ff = 0, rr = 0;
  float rz = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double fi = f[i];
    const double ri = w ? fi - w[i] : fi;
    const float rf = (float)ri;
    const float zf = dinv[i] * rf;
    r[i] = ri;
    r32[i] = rf;
    p32[i] = zf;
    y32[i] = 0.f;
    const double m = mult[i];
    ff += m * fi * fi;
    rr += m * ri * ri;
    rz += (float)m * rf * zf;
  }
  double v[3] = {ff, rr, (double)rz};
  grid_reduce<3>(v, part, sc, FinRUInit());
}

// x += (double) y; y = 0
__global__ void k_ru_accum(double* __restrict__ x, float* __restrict__ y, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] += (double)y[i];
    y[i] = 0.f;
  }
}

struct FinRU {
  int mode;  // 1: replacement during the iteration; 2: confirm a converged FP32 residual
  __device__ void operator()(const double* acc, Scalars* sc) const {
    // acc: rr (FP64), rz of the new FP32 residual
    sc->rr = acc[0];
    sc->rmax = sqrt(acc[0]);
    sc->need_ru = 0;
    if (!isfinite(acc[0]) || !isfinite(acc[1])) {
      sc->status = NTG_NONFINITE;
      sc->done = 1;
      return;
    }
    if (acc[0] <= sc->tol2) {
      sc->status = NTG_OK;
      sc->done = 1;
      return;
    }
    if (sc->iter >= sc->max_iter) {
      sc->status = NTG_MAXITER;
      sc->done = 1;
      return;
    }
    // a confirmation that failed resumes the iteration: the direction update
    // skipped at the candidate uses the replaced residual
    sc->done = 0;
    if (sc->ext_pc) return;  // (r, z) of the new residual comes with the preconditioner application
    if (mode == 2) sc->beta = acc[1] / sc->rz;
    sc->rz = acc[1];
  }
};

// ---------------------------------------------------------------------------
// Explicit-preconditioner variant of the FP32 iteration (Schwarz): the
// update forms only (r, r); z = M r is applied by its own kernels, the last
// of which also forms (r, z) and beta; k_dir_z sets p = z + beta p.
// Both stream float4s (a scalar tail covers n % 4).
// ---------------------------------------------------------------------------
__global__ void k_update_rr(float* __restrict__ y, const float* __restrict__ p, float* __restrict__ r,
                            const float* __restrict__ w, const float* __restrict__ mult, int64_t n,
                            double* __restrict__ part, Scalars* sc) {
  if (sc->done) return;
  const float alpha = (float)sc->alpha;
  float rr = 0.f;
  const int64_t n4 = n >> 2, g0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, gs = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = g0; i < n4; i += gs) {
    float4 y4 = reinterpret_cast<float4*>(y)[i];
    const float4 p4 = reinterpret_cast<const float4*>(p)[i], w4 = reinterpret_cast<const float4*>(w)[i];
    const float4 m4 = reinterpret_cast<const float4*>(mult)[i];
    float4 r4 = reinterpret_cast<float4*>(r)[i];
    y4.x += alpha * p4.x; y4.y += alpha * p4.y; y4.z += alpha * p4.z; y4.w += alpha * p4.w;
    r4.x -= alpha * w4.x; r4.y -= alpha * w4.y; r4.z -= alpha * w4.z; r4.w -= alpha * w4.w;
    reinterpret_cast<float4*>(y)[i] = y4;
    reinterpret_cast<float4*>(r)[i] = r4;
    rr += m4.x * r4.x * r4.x + m4.y * r4.y * r4.y + m4.z * r4.z * r4.z + m4.w * r4.w * r4.w;
  }
  for (int64_t i = 4 * n4 + g0; i < n; i += gs) {
    y[i] += alpha * p[i];
    const float ri = r[i] - alpha * w[i];
    r[i] = ri;
    rr += mult[i] * ri * ri;
  }
  double v[2] = {0.0, (double)rr};
  grid_reduce<2>(v, part, sc, FinUpd());
}

// The update of k_update_rr with the gather-scatter and the mask of w done
// in the same pass, on a structured box (elements x fastest): a thread owns
// one row (j, k) of an element and sums, per node, the local w of every
// element holding it -- the rows of the 1, 2 or 4 elements covering the row
// in y and z, and the x neighbours' end values -- in ascending element
// order (z-major, y, x), the order of the gather-scatter's groups, so every
// copy of a node receives the same sum.  Then w is masked (one mask byte per
// row) and y += alpha p, r -= alpha w; (r, r)_mult is summed over each
// node's owning copy (no lower neighbour in any direction), which the
// mult-weighted sum over copies equals, with no multiplicity stream.
template <int LX>
__global__ void __launch_bounds__(256)
    k_update_box(float* __restrict__ y, const float* __restrict__ p, float* __restrict__ r,
                 const float* __restrict__ w, const uint8_t* __restrict__ maskrow, int Ex,
                 int Ey, int Ez, double* __restrict__ part, Scalars* sc) {
  constexpr int N = LX - 1, LX2 = LX * LX, LX3 = LX2 * LX;
  if (sc->done) return;
  const float alpha = (float)sc->alpha;
  const int64_t nrow = (int64_t)Ex * Ey * Ez * LX2;
  const int64_t sy = (int64_t)Ex * LX3, sz = (int64_t)Ex * Ey * LX3;
  float rr = 0.f;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nrow; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = t / LX2;
    const int m = (int)(t - e * LX2), j = m % LX, k = m / LX;
    const int64_t o = e * LX3 + (int64_t)m * LX;
    const int64_t exy = e / Ex;
    const int cx = (int)(e - exy * Ex), cz = (int)(exy / Ey), cy = (int)(exy - (int64_t)cz * Ey);
    // covering rows, lower element first: offsets from the own row
    int64_t zo[2] = {0, 0}, yo[2] = {0, 0};
    int nz = 1, ny = 1;
    if (k == 0 && cz > 0) { zo[0] = -sz + (int64_t)N * LX2; nz = 2; }
    else if (k == N && cz < Ez - 1) { zo[1] = sz - (int64_t)N * LX2; nz = 2; }
    if (j == 0 && cy > 0) { yo[0] = -sy + (int64_t)N * LX; ny = 2; }
    else if (j == N && cy < Ey - 1) { yo[1] = sy - (int64_t)N * LX; ny = 2; }
    const bool xl = cx > 0, xh = cx < Ex - 1;
    float acc[LX];
#pragma unroll
    for (int i = 0; i < LX; ++i) acc[i] = 0.f;
#pragma unroll
    for (int vz = 0; vz < 2; ++vz) {
      if (vz >= nz) break;
#pragma unroll
      for (int vy = 0; vy < 2; ++vy) {
        if (vy >= ny) break;
        const float* row = w + o + (nz == 2 ? zo[vz] : 0) + (ny == 2 ? yo[vy] : 0);
        if (xl) acc[0] += row[N - LX3];
#pragma unroll
        for (int i = 0; i < LX; i += 2) {
          const float2 v = *reinterpret_cast<const float2*>(row + i);
          acc[i] += v.x;
          acc[i + 1] += v.y;
        }
        if (xh) acc[N] += row[LX3];
      }
    }
    const unsigned mb = maskrow[t];
    const bool own_jk = (j > 0 || cy == 0) && (k > 0 || cz == 0);
#pragma unroll
    for (int i = 0; i < LX; i += 2) {
      const float2 pp = *reinterpret_cast<const float2*>(p + o + i);
      float2 yy = *reinterpret_cast<const float2*>(y + o + i);
      float2 rv = *reinterpret_cast<const float2*>(r + o + i);
      yy.x += alpha * pp.x;
      yy.y += alpha * pp.y;
      rv.x -= alpha * (((mb >> i) & 1u) ? 0.f : acc[i]);
      rv.y -= alpha * (((mb >> (i + 1)) & 1u) ? 0.f : acc[i + 1]);
      *reinterpret_cast<float2*>(y + o + i) = yy;
      *reinterpret_cast<float2*>(r + o + i) = rv;
      if (own_jk) {
        if (i > 0 || cx == 0) rr += rv.x * rv.x;
        rr += rv.y * rv.y;  // node i + 1 > 0
      }
    }
  }
  double v[2] = {0.0, (double)rr};
  grid_reduce<2>(v, part, sc, FinUpd());
}

__global__ void k_dir_z(float* __restrict__ p, const float* __restrict__ z, int64_t n, int init, const Scalars* sc) {
  if (sc->done) return;
  const float beta = init ? 0.f : (float)sc->beta;
  const int64_t n4 = n >> 2, g0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, gs = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = g0; i < n4; i += gs) {
    const float4 z4 = reinterpret_cast<const float4*>(z)[i];
    float4 p4 = init ? make_float4(0.f, 0.f, 0.f, 0.f) : reinterpret_cast<const float4*>(p)[i];
    p4.x = z4.x + beta * p4.x; p4.y = z4.y + beta * p4.y; p4.z = z4.z + beta * p4.z; p4.w = z4.w + beta * p4.w;
    reinterpret_cast<float4*>(p)[i] = p4;
  }
  for (int64_t i = 4 * n4 + g0; i < n; i += gs) p[i] = init ? z[i] : z[i] + beta * p[i];
}
// start: r = f - w (w null: f); r32 = (float) r; y = 0; sums ff, rr
__global__ void k_ru_init_pc(const double* __restrict__ f, const double* __restrict__ w, const double* __restrict__ mult,
                             double* __restrict__ r, float* __restrict__ r32, float* __restrict__ y32, int64_t n,
                             double* __restrict__ part, Scalars* sc) {
  double ff = 0, rr = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double fi = f[i];
    const double ri = w ? fi - w[i] : fi;
    r[i] = ri;
    r32[i] = (float)ri;
    y32[i] = 0.f;
    ff += mult[i] * fi * fi;
    rr += mult[i] * ri * ri;
  }
  double v[3] = {ff, rr, 1.0};
  grid_reduce<3>(v, part, sc, FinRUInit());
}

// r = f - w (FP64); r32 = (float) r; sums (r, r)_mult, (r32, dinv32 r32)_mult
__global__ void k_ru_resid(const double* __restrict__ f, const double* __restrict__ w, const float* __restrict__ dinv,
                           const double* __restrict__ mult, double* __restrict__ r, float* __restrict__ r32, int64_t n,
                           int mode, double* __restrict__ part, Scalars* sc) {
  double rr = 0;
  float rz = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double ri = f[i] - w[i];
    const float rf = (float)ri;
    r[i] = ri;
    r32[i] = rf;
    const double m = mult[i];
    rr += m * ri * ri;
    rz += (float)m * rf * (dinv[i] * rf);
  }
  double v[2] = {rr, (double)rz};
  grid_reduce<2>(v, part, sc, FinRU{mode});
}

}  // namespace ntg

// ---------------------------------------------------------------------------
// ksp object
// ---------------------------------------------------------------------------
struct ntg_ksp {
  ntg_plan* plan = nullptr;
  int type = NTG_KSP_CG;
  int max_iter = 800;
  double rtol = 1e-10, abstol = 0.0;
  double inner_rtol = 1e-4;
  int inner_max_iter = 400;
  int check_every = 16;
  int guess_guard = 0;
  int ax_ready = 0;  // the guard left A x0 (assembled, masked) in v64.w for this solve: 1 FP64, 2 FP32 operator
  int box_update = 1;  // structured-box Schwarz: gather-scatter + mask + update in one kernel
  ntg_schwarz* sw = nullptr;  // explicit FP32 preconditioner of the cg_mixed / gmres iterations
  int restart = 30;            // gmres restart length
  ntg::GmresWork* gm = nullptr;
  float* z32 = nullptr;
  // FP64 workspace
  ntg::PcgVecs<double> v64;
  double *pd = nullptr, *qd = nullptr, *pprev = nullptr, *qprev = nullptr;
  // FP32 workspace
  ntg::PcgVecs<float> v32;
  float *rin = nullptr, *din = nullptr;
  ntg::Scalars* sc = nullptr;      // outer / plain solve
  ntg::Scalars* sc_in = nullptr;   // inner solve
  ntg::Scalars* hs = nullptr;      // pinned host mirror (outer)
  ntg::Scalars* hs_in = nullptr;   // pinned host mirror (inner)
};

using namespace ntg;

static void ksp_free(ntg_ksp* k) {
  dev_free(k->v64.r); dev_free(k->v64.p); dev_free(k->v64.w);
  dev_free(k->pd); dev_free(k->qd); dev_free(k->pprev); dev_free(k->qprev);
  dev_free(k->v32.r); dev_free(k->v32.p); dev_free(k->v32.w);
  dev_free(k->rin); dev_free(k->din); dev_free(k->z32);
  dev_free(k->sc); dev_free(k->sc_in);
  gmres_free(k->gm);
  k->gm = nullptr;
  if (k->hs) cudaFreeHost(k->hs);
  if (k->hs_in) cudaFreeHost(k->hs_in);
  k->hs = nullptr;
  k->hs_in = nullptr;
}

static int ksp_solve_cg(ntg_ksp* k, double* x, const double* f, ntg_monitor* mon) {
  ntg_plan* p = k->plan;
  cudaStream_t s = p->stream;
  if (!p->jacobi_ready) NTG_TRY(jacobi_update(p));
  // a zero initial guess skips one operator application
  double xx = 0.0;
  NTG_TRY(wdot(p, x, x, nullptr, p->n, &xx, s));
  int fpax = 0;
  NTG_TRY(run_pcg<double>(p, k->sc, k->hs, k->v64, x, f, p->dinv, p->mult, k->rtol, k->abstol, k->max_iter,
                          xx == 0.0, k->check_every, s, &fpax));
  if (mon) {
    mon->iter = k->hs->iter;
    mon->inner_iter = 0;
    mon->res_start = sqrt(k->hs->rr0);
    mon->res_final = sqrt(k->hs->rr);
    mon->rhs_norm = sqrt(k->hs->ff);
    mon->status = k->hs->status;
    mon->fp64_ax = fpax;
  }
  return NTG_OK;
}

static int ksp_solve_mixed(ntg_ksp* k, double* x, const double* f, ntg_monitor* mon) {
  ntg_plan* p = k->plan;
  cudaStream_t s = p->stream;
  const int64_t n = p->n;
  const int TPB = 256;
  const int G = grid_for(n, TPB);
  NTG_TRY(ensure_fp32(p));
  if (!p->jacobi_ready) NTG_TRY(jacobi_update(p));
  double xx = 0.0;
  NTG_TRY(wdot(p, x, x, nullptr, n, &xx, s));
  int fpax = 0, inner_total = 0;
  // outer residual r = f - A x (FP64)
  Scalars* hs = k->hs;
  memset(hs, 0, sizeof(Scalars));
  hs->rtol = k->rtol;
  hs->abstol = k->abstol;
  hs->max_iter = k->max_iter;
  NTG_CUDA_TRY(cudaMemcpyAsync(k->sc, hs, sizeof(Scalars), cudaMemcpyHostToDevice, s));
  if (xx != 0.0) {
    NTG_TRY(op_apply(p, k->qd, x, s));
    fpax++;
  }
  { k_resid<<<G, TPB, 0, s>>>(f, xx != 0.0 ? k->qd : nullptr, p->mult, k->v64.r, n, p->red_part, k->sc); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  NTG_CUDA_TRY(cudaMemcpyAsync(hs, k->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
  NTG_CUDA_TRY(cudaStreamSynchronize(s));
  const double rr0 = hs->rr0, ff = hs->ff;
  double* pd = k->pd;
  double* qd = k->qd;
  double* pprev = k->pprev;
  double* qprev = k->qprev;
  bool have_prev = false;
  Scalars& hin = *k->hs_in;
  double last_rr = hs->rr;
  int stagnant = 0;
  int outer_status = hs->status;
  bool fallback = false;
  while (!hs->done) {
    // inner FP32 Jacobi-PCG on the normalised residual, zero guess
    { k_to_f32_scaled<<<G, TPB, 0, s>>>(k->v64.r, k->rin, n, k->sc); NTG_COUNT_LAUNCH(); }
    { k_zero_f<<<G, TPB, 0, s>>>(k->din, n); NTG_COUNT_LAUNCH(); }
    NTG_CUDA_TRY(cudaGetLastError());
    NTG_TRY(run_pcg<float>(p, k->sc_in, &hin, k->v32, k->din, k->rin, p->dinvf, p->multf, k->inner_rtol, 0.0,
                           k->inner_max_iter, true, k->check_every, s, nullptr));
    inner_total += hin.iter;
    // direction: z = ||r|| din, FCG(1) orthogonalisation against pprev
    { k_from_f32<<<G, TPB, 0, s>>>(k->din, pd, have_prev ? qprev : nullptr, p->mult, n, p->red_part, k->sc); NTG_COUNT_LAUNCH(); }
    { k_fcg_orth<<<G, TPB, 0, s>>>(pd, have_prev ? pprev : nullptr, k->v64.r, p->mult, n, p->red_part, k->sc); NTG_COUNT_LAUNCH(); }
    // q = A p (FP64) with fused (p, Ap) -> alpha = (p, r) / (p, Ap)
    NTG_TRY(ax_launch(p, qd, pd, k->sc, 0, s));
    NTG_TRY(gs_launch(p, qd, NTG_GS_ADD, s));
    NTG_TRY(mask_launch(p, qd, s));
    fpax++;
    { k_fcg_update<<<G, TPB, 0, s>>>(x, pd, k->v64.r, qd, p->mult, n, p->red_part, k->sc); NTG_COUNT_LAUNCH(); }
    NTG_CUDA_TRY(cudaGetLastError());
    NTG_CUDA_TRY(cudaMemcpyAsync(hs, k->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
    NTG_CUDA_TRY(cudaStreamSynchronize(s));
    // swap direction buffers
    double* t = pprev; pprev = pd; pd = t;
    t = qprev; qprev = qd; qd = t;
    have_prev = true;
    // stagnation guard: two outer steps that each fail to halve the
    // residual hand the rest of the solve to the FP64 PCG
    if (!hs->done) {
      if (hs->rr > 0.25 * last_rr) ++stagnant;
      else stagnant = 0;
      last_rr = hs->rr;
      if (stagnant >= 2) {
        fallback = true;
        break;
      }
    }
  }
  outer_status = hs->status;
  int outer_iter = hs->iter;
  double rr_final = hs->rr;
  if (fallback) {
    int fp2 = 0;
    NTG_TRY(run_pcg<double>(p, k->sc, k->hs, k->v64, x, f, p->dinv, p->mult, k->rtol, k->abstol,
                            k->max_iter, false, k->check_every, s, &fp2));
    fpax += fp2;
    outer_iter += k->hs->iter;
    rr_final = k->hs->rr;
    outer_status = k->hs->status;
  }
  k->pd = pd; k->qd = qd; k->pprev = pprev; k->qprev = qprev;
  if (mon) {
    mon->iter = outer_iter;
    mon->inner_iter = inner_total;
    mon->res_start = sqrt(rr0);
    mon->res_final = sqrt(rr_final);
    mon->rhs_norm = sqrt(ff);
    mon->status = outer_status;
    mon->fp64_ax = fpax;
  }
  return NTG_OK;
}

// Reliable-update mixed CG (NTG_KSP_CG_MIXED); see the kernels above.
static int ksp_solve_mixed_ru(ntg_ksp* k, double* x, const double* f, ntg_monitor* mon) {
  ntg_plan* p = k->plan;
  cudaStream_t s = p->stream;
  const int64_t n = p->n;
  const int TPB = 256;
  const int G = grid_for(n, TPB);
  NTG_TRY(ensure_fp32(p));
  if (!p->jacobi_ready) NTG_TRY(jacobi_update(p));
  double xx = 0.0;
  NTG_TRY(wdot(p, x, x, nullptr, n, &xx, s));
  int fpax = 0, nru = 0;
  Scalars* hs = k->hs;
  memset(hs, 0, sizeof(Scalars));
  hs->rtol = k->rtol;
  hs->abstol = k->abstol;
  hs->max_iter = k->max_iter;
  hs->ru_mode = 1;
  hs->delta = k->inner_rtol;
  NTG_CUDA_TRY(cudaMemcpyAsync(k->sc, hs, sizeof(Scalars), cudaMemcpyHostToDevice, s));
  if (xx != 0.0) {
    if (!k->ax_ready) NTG_TRY(op_apply(p, k->v64.w, x, s));  // else the guess guard's A x0 is in v64.w
    if (k->ax_ready != 2) fpax++;  // 2: the FP32 operator's image
  }
  float* y32 = k->din;
  { k_ru_init<<<G, TPB, 0, s>>>(f, xx != 0.0 ? k->v64.w : nullptr, p->dinvf, p->mult, k->v64.r, k->v32.r, k->v32.p, y32, n, p->red_part, k->sc); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  auto poll = [&]() -> int {
    NTG_CUDA_TRY(cudaMemcpyAsync(hs, k->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
    NTG_CUDA_TRY(cudaStreamSynchronize(s));
    return NTG_OK;
  };
  auto replace = [&](int mode) -> int {
    { k_ru_accum<<<G, TPB, 0, s>>>(x, y32, n); NTG_COUNT_LAUNCH(); }
    NTG_TRY(op_apply(p, k->v64.w, x, s));
    fpax++;
    nru++;
    { k_ru_resid<<<G, TPB, 0, s>>>(f, k->v64.w, p->dinvf, p->mult, k->v64.r, k->v32.r, n, mode, p->red_part, k->sc); NTG_COUNT_LAUNCH(); }
    NTG_CUDA_TRY(cudaGetLastError());
    return poll();
  };
  double rr0 = 0, ff = 0;
  NTG_TRY(poll());
  rr0 = hs->rr0;
  ff = hs->ff;
  bool y_dirty = false;  // y32 holds a correction not yet folded into x
  int guard = 0;
  for (;;) {
    if (hs->done) {
      if (hs->need_ru == 2) {
        NTG_TRY(replace(2));
        y_dirty = false;
        if (hs->done) break;
        { k_cg_dir<float><<<G, TPB, 0, s>>>(k->v32.p, k->v32.r, p->dinvf, n, k->sc); NTG_COUNT_LAUNCH(); }
        continue;
      }
      break;
    }
    if (hs->need_ru == 1) {
      NTG_TRY(replace(1));
      y_dirty = false;
      if (hs->done) break;
    }
    if (++guard > k->max_iter / k->check_every + 64) break;  // defensive: the device cap ends the loop first
    for (int c = 0; c < k->check_every; ++c) {
      NTG_TRY(ax_launch_f32(p, k->v32.w, k->v32.p, k->sc, 0, s));
      NTG_TRY(gs_add_guarded_f32(p, k->v32.w, s, k->sc));
      NTG_TRY(mask_guarded_f32(p, k->v32.w, s, k->sc));
      timer_start(TM_UPD32, s);
      { k_cg_update<float><<<G, TPB, 0, s>>>(y32, k->v32.p, k->v32.r, k->v32.w, p->dinvf, p->multf, n, p->red_part, k->sc); NTG_COUNT_LAUNCH(); }
      timer_stop(TM_UPD32, s);
      timer_start(TM_DIR32, s);
      { k_cg_dir<float><<<G, TPB, 0, s>>>(k->v32.p, k->v32.r, p->dinvf, n, k->sc); NTG_COUNT_LAUNCH(); }
      timer_stop(TM_DIR32, s);
    }
    y_dirty = true;
    NTG_TRY(poll());
  }
  int status = hs->status;
  double rr_final = hs->rr;
  if (y_dirty) {
    // stopped inside the FP32 iteration (cap, breakdown, non-finite): fold
    // the correction in and report the FP64 residual
    const int iters = hs->iter;
    NTG_TRY(replace(1));
    rr_final = hs->rr;
    hs->iter = iters;
  }
  if (mon) {
    mon->iter = hs->iter;
    mon->inner_iter = nru;
    mon->res_start = sqrt(rr0);
    mon->res_final = sqrt(rr_final);
    mon->rhs_norm = sqrt(ff);
    mon->status = status;
    mon->fp64_ax = fpax;
  }
  return NTG_OK;
}

// Reliable-update mixed CG with an explicit FP32 preconditioner (Schwarz).
static int ksp_solve_mixed_ru_pc(ntg_ksp* k, double* x, const double* f, ntg_monitor* mon) {
  ntg_plan* p = k->plan;
  cudaStream_t s = p->stream;
  const int64_t n = p->n;
  const int TPB = 256;
  const int G = grid_for(n, TPB);
  NTG_TRY(ensure_fp32(p));
  double xx = 0.0;
  NTG_TRY(wdot(p, x, x, nullptr, n, &xx, s));
  int fpax = 0, nru = 0;
  Scalars* hs = k->hs;
  memset(hs, 0, sizeof(Scalars));
  hs->rtol = k->rtol;
  hs->abstol = k->abstol;
  hs->max_iter = k->max_iter;
  hs->ru_mode = 1;
  hs->ext_pc = 1;
  hs->delta = k->inner_rtol;
  NTG_CUDA_TRY(cudaMemcpyAsync(k->sc, hs, sizeof(Scalars), cudaMemcpyHostToDevice, s));
  if (xx != 0.0) {
    if (!k->ax_ready) NTG_TRY(op_apply(p, k->v64.w, x, s));  // else the guess guard's A x0 is in v64.w
    if (k->ax_ready != 2) fpax++;  // 2: the FP32 operator's image
  }
  float* y32 = k->din;
  float* r32 = k->v32.r;
  float* p32 = k->v32.p;
  float* w32 = k->v32.w;
  float* z32 = k->z32;
  { k_ru_init_pc<<<G, TPB, 0, s>>>(f, xx != 0.0 ? k->v64.w : nullptr, p->mult, k->v64.r, r32, y32, n, p->red_part, k->sc); NTG_COUNT_LAUNCH(); }
  auto poll = [&]() -> int {
    NTG_CUDA_TRY(cudaMemcpyAsync(hs, k->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
    NTG_CUDA_TRY(cudaStreamSynchronize(s));
    return NTG_OK;
  };
  // z = M r, then (r, z) in the given mode
  auto precondition = [&](int mode) -> int {
    return schwarz_apply(k->sw, z32, r32, s, k->sc, p->multf, p->red_part, mode);
  };
  auto replace = [&](int mode) -> int {
    { k_ru_accum<<<G, TPB, 0, s>>>(x, y32, n); NTG_COUNT_LAUNCH(); }
    NTG_TRY(op_apply(p, k->v64.w, x, s));
    fpax++;
    nru++;
    { k_ru_resid<<<G, TPB, 0, s>>>(f, k->v64.w, p->dinvf ? p->dinvf : r32, p->mult, k->v64.r, r32, n, mode, p->red_part, k->sc); NTG_COUNT_LAUNCH(); }
    NTG_CUDA_TRY(cudaGetLastError());
    NTG_TRY(poll());
    if (hs->done) return NTG_OK;
    NTG_TRY(precondition(mode == 2 ? 0 : 1));
    if (mode == 2) { k_dir_z<<<G, TPB, 0, s>>>(p32, z32, n, 0, k->sc); NTG_COUNT_LAUNCH(); }
    return poll();
  };
  // structured box (the Schwarz preconditioner's form): the gather-scatter of
  // w folds into the update
  int bx = 0, by = 0, bz = 0, box_lx = 0;
  if (k->box_update && schwarz_box(k->sw, &bx, &by, &bz) && (p->lx == 4 || p->lx == 6 || p->lx == 8) &&
      (int64_t)bx * by * bz == p->nelv) {
    NTG_TRY(ensure_maskrow(p));
    box_lx = p->lx;
  }
  NTG_TRY(poll());
  const double rr0 = hs->rr0, ff = hs->ff;
  if (!hs->done) {
    NTG_TRY(precondition(3));
    { k_dir_z<<<G, TPB, 0, s>>>(p32, z32, n, 1, k->sc); NTG_COUNT_LAUNCH(); }
    NTG_TRY(poll());
  }
  bool y_dirty = false;
  int guard = 0;
  for (;;) {
    if (hs->done) {
      if (hs->need_ru == 2) {
        NTG_TRY(replace(2));
        y_dirty = false;
        if (hs->done) break;
        continue;
      }
      break;
    }
    if (hs->need_ru == 1) {
      NTG_TRY(replace(1));
      y_dirty = false;
      if (hs->done) break;
    }
    if (++guard > k->max_iter / k->check_every + 64) break;  // defensive: the device cap ends the loop first
    for (int c = 0; c < k->check_every; ++c) {
      NTG_TRY(ax_launch_f32(p, w32, p32, k->sc, 0, s));
      timer_start(TM_UPD32, s);
      if (box_lx) {
        // gather-scatter, mask and update in one pass over the box
        const int GB = grid_for(n / p->lx, TPB);
        if (box_lx == 8) k_update_box<8><<<GB, TPB, 0, s>>>(y32, p32, r32, w32, p->maskrow, bx, by, bz, p->red_part, k->sc);
        else if (box_lx == 6) k_update_box<6><<<GB, TPB, 0, s>>>(y32, p32, r32, w32, p->maskrow, bx, by, bz, p->red_part, k->sc);
        else k_update_box<4><<<GB, TPB, 0, s>>>(y32, p32, r32, w32, p->maskrow, bx, by, bz, p->red_part, k->sc);
        NTG_COUNT_LAUNCH();
      } else {
        timer_stop(TM_UPD32, s);
        NTG_TRY(gs_add_guarded_f32(p, w32, s, k->sc));
        NTG_TRY(mask_guarded_f32(p, w32, s, k->sc));
        timer_start(TM_UPD32, s);
        { k_update_rr<<<G, TPB, 0, s>>>(y32, p32, r32, w32, p->multf, n, p->red_part, k->sc); NTG_COUNT_LAUNCH(); }
      }
      timer_stop(TM_UPD32, s);
      timer_start(TM_PC32, s);
      NTG_TRY(precondition(0));
      timer_stop(TM_PC32, s);
      timer_start(TM_DIR32, s);
      { k_dir_z<<<G, TPB, 0, s>>>(p32, z32, n, 0, k->sc); NTG_COUNT_LAUNCH(); }
      timer_stop(TM_DIR32, s);
    }
    y_dirty = true;
    NTG_TRY(poll());
  }
  int status = hs->status;
  double rr_final = hs->rr;
  if (y_dirty) {
    const int iters = hs->iter;
    { k_ru_accum<<<G, TPB, 0, s>>>(x, y32, n); NTG_COUNT_LAUNCH(); }
    NTG_TRY(op_apply(p, k->v64.w, x, s));
    fpax++;
    { k_resid<<<G, TPB, 0, s>>>(f, k->v64.w, p->mult, k->v64.r, n, p->red_part, k->sc); NTG_COUNT_LAUNCH(); }
    NTG_TRY(poll());
    rr_final = hs->rr;
    hs->iter = iters;
  }
  if (mon) {
    mon->iter = hs->iter;
    mon->inner_iter = nru;
    mon->res_start = sqrt(rr0);
    mon->res_final = sqrt(rr_final);
    mon->rhs_norm = sqrt(ff);
    mon->status = status;
    mon->fp64_ax = fpax;
  }
  return NTG_OK;
}

extern "C" {

int ntg_ksp_set_schwarz(ntg_ksp* ksp, ntg_schwarz* sw_) {
  clear_error();
  NTG_CHECK_ARG(ksp, "ntg_ksp_set_schwarz: null argument");
  NTG_CHECK_ARG(ksp->type == NTG_KSP_CG_MIXED || ksp->type == NTG_KSP_GMRES || ksp->type == NTG_KSP_GMRES_MIXED,
                "ntg_ksp_set_schwarz: the cg_mixed and gmres solvers take Schwarz");
  if (sw_ && ksp->type == NTG_KSP_CG_MIXED && !ksp->z32) NTG_TRY(dev_alloc(&ksp->z32, ksp->plan->n));
  ksp->sw = sw_;
  return NTG_OK;
}

int ntg_pc_jacobi_update(ntg_plan* plan) {
  clear_error();
  NTG_CHECK_ARG(plan, "ntg_pc_jacobi_update: null plan");
  return jacobi_update(plan);
}

int ntg_pc_jacobi_solve(ntg_plan* plan, double* z_d, const double* r_d) {
  clear_error();
  NTG_CHECK_ARG(plan && z_d && r_d, "ntg_pc_jacobi_solve: null argument");
  if (!plan->jacobi_ready) NTG_TRY(jacobi_update(plan));
  { k_col3<<<grid_for(plan->n, 256), 256, 0, plan->stream>>>(z_d, plan->dinv, r_d, plan->n); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

int ntg_pc_jacobi_get(const ntg_plan* plan, double* dinv_d) {
  clear_error();
  NTG_CHECK_ARG(plan && dinv_d, "ntg_pc_jacobi_get: null argument");
  NTG_CHECK_ARG(plan->jacobi_ready, "ntg_pc_jacobi_get: call ntg_pc_jacobi_update first");
  NTG_CUDA_TRY(cudaMemcpyAsync(dinv_d, plan->dinv, sizeof(double) * plan->n, cudaMemcpyDeviceToDevice, plan->stream));
  return NTG_OK;
}

int ntg_glsc3(ntg_plan* plan, const double* a_d, const double* b_d, const double* c_d, int64_t n, double* out) {
  clear_error();
  NTG_CHECK_ARG(plan && a_d && b_d && out && n >= 0, "ntg_glsc3: bad argument");
  return wdot(plan, a_d, b_d, c_d, n, out, plan->stream);
}

int ntg_ksp_create(ntg_plan* plan, int type, int max_iter, double rtol, double abstol, ntg_ksp** ksp) {
  clear_error();
  NTG_CHECK_ARG(plan && ksp, "ntg_ksp_create: null argument");
  NTG_CHECK_ARG(type == NTG_KSP_CG || type == NTG_KSP_FCG_MIXED || type == NTG_KSP_CG_MIXED ||
                    type == NTG_KSP_GMRES || type == NTG_KSP_GMRES_MIXED,
                "ntg_ksp_create: unknown solver type");
  NTG_CHECK_ARG(max_iter >= 0 && rtol >= 0 && abstol >= 0, "ntg_ksp_create: bad tolerance or iteration cap");
  *ksp = nullptr;
  ntg_ksp* k = new ntg_ksp();
  k->plan = plan;
  k->type = type;
  k->max_iter = max_iter;
  k->rtol = rtol;
  k->abstol = abstol;
  const int64_t n = plan->n;
  int st = NTG_OK;
  do {
    if ((st = dev_alloc(&k->v64.r, n))) break;
    if ((st = dev_alloc(&k->v64.p, n))) break;
    if ((st = dev_alloc(&k->v64.w, n))) break;
    if ((st = dev_alloc(&k->sc, 1))) break;
    if ((st = dev_alloc(&k->sc_in, 1))) break;
    if (cudaMallocHost(&k->hs, sizeof(Scalars)) != cudaSuccess) { st = NTG_ERR_ALLOC; break; }
    if (cudaMallocHost(&k->hs_in, sizeof(Scalars)) != cudaSuccess) { st = NTG_ERR_ALLOC; break; }
    if (cudaMemset(k->sc, 0, sizeof(Scalars)) != cudaSuccess) { st = NTG_ERR_CUDA; break; }
    if (cudaMemset(k->sc_in, 0, sizeof(Scalars)) != cudaSuccess) { st = NTG_ERR_CUDA; break; }
    if (type == NTG_KSP_GMRES_MIXED) k->inner_rtol = 1e-4;  // residual reduction per FP32 cycle
    if (type == NTG_KSP_CG_MIXED) {
      k->inner_rtol = 0.1;  // reliable-update threshold delta
      if ((st = dev_alloc(&k->v32.r, n))) break;
      if ((st = dev_alloc(&k->v32.p, n))) break;
      if ((st = dev_alloc(&k->v32.w, n))) break;
      if ((st = dev_alloc(&k->din, n))) break;
    }
    if (type == NTG_KSP_FCG_MIXED) {
      if ((st = dev_alloc(&k->pd, n))) break;
      if ((st = dev_alloc(&k->qd, n))) break;
      if ((st = dev_alloc(&k->pprev, n))) break;
      if ((st = dev_alloc(&k->qprev, n))) break;
      if ((st = dev_alloc(&k->v32.r, n))) break;
      if ((st = dev_alloc(&k->v32.p, n))) break;
      if ((st = dev_alloc(&k->v32.w, n))) break;
      if ((st = dev_alloc(&k->rin, n))) break;
      if ((st = dev_alloc(&k->din, n))) break;
    }
  } while (0);
  if (st) {
    ksp_free(k);
    delete k;
    return st;
  }
  *ksp = k;
  return NTG_OK;
}

int ntg_ksp_destroy(ntg_ksp* ksp) {
  clear_error();
  if (!ksp) return NTG_OK;
  cudaStreamSynchronize(ksp->plan->stream);
  ksp_free(ksp);
  delete ksp;
  return NTG_OK;
}

int ntg_ksp_set_inner(ntg_ksp* ksp, double inner_rtol, int inner_max_iter) {
  clear_error();
  NTG_CHECK_ARG(ksp && inner_rtol > 0 && inner_rtol < 1 && inner_max_iter > 0, "ntg_ksp_set_inner: bad argument");
  ksp->inner_rtol = inner_rtol;
  ksp->inner_max_iter = inner_max_iter;
  return NTG_OK;
}

int ntg_ksp_set_restart(ntg_ksp* ksp, int m) {
  clear_error();
  NTG_CHECK_ARG(ksp && m >= 1 && m <= 31, "ntg_ksp_set_restart: restart length must be in [1, 31]");
  ksp->restart = m;
  return NTG_OK;
}

int ntg_ksp_set_check_every(ntg_ksp* ksp, int every) {
  clear_error();
  NTG_CHECK_ARG(ksp && every > 0 && every <= 1024, "ntg_ksp_set_check_every: bad argument");
  ksp->check_every = every;
  return NTG_OK;
}

int ntg_ksp_set_tol(ntg_ksp* ksp, double rtol, double abstol) {
  clear_error();
  NTG_CHECK_ARG(ksp && rtol >= 0 && abstol >= 0, "ntg_ksp_set_tol: bad argument");
  ksp->rtol = rtol;
  ksp->abstol = abstol;
  return NTG_OK;
}

// the cg_mixed iteration with a structured-box Schwarz preconditioner folds
// the gather-scatter and mask of A p into its update kernel (default on)
int ntg_ksp_set_fused_update(ntg_ksp* ksp, int on) {
  clear_error();
  NTG_CHECK_ARG(ksp, "ntg_ksp_set_fused_update: null argument");
  ksp->box_update = on ? 1 : 0;
  return NTG_OK;
}

int ntg_ksp_set_guess_guard(ntg_ksp* ksp, int on) {
  clear_error();
  NTG_CHECK_ARG(ksp, "ntg_ksp_set_guess_guard: null argument");
  ksp->guess_guard = on ? 1 : 0;
  return NTG_OK;
}

int ntg_ksp_solve(ntg_ksp* ksp, double* x_d, const double* f_d, ntg_monitor* mon) {
  clear_error();
  NTG_CHECK_ARG(ksp && x_d && f_d, "ntg_ksp_solve: null argument");
  if (mon) memset(mon, 0, sizeof(*mon));
  int rejected = 0;
  if (ksp->guess_guard) {
    // a guess is kept only if its residual is below ||f||: one operator
    // application and two dots decide.  For the reliable-update mixed CG
    // the operator is the FP32 one: its image of the guess becomes the
    // initial residual, which the first FP64 residual replacement of that
    // solver recomputes exactly (the FP64 operator costs 20x the FP32 one
    // on GB300's FP64 pipe); every other solver takes the FP64 operator.
    ntg_plan* p = ksp->plan;
    cudaStream_t s = p->stream;
    double xx = 0.0;
    NTG_TRY(wdot(p, x_d, x_d, nullptr, p->n, &xx, s));
    const bool fp32 = ksp->type == NTG_KSP_CG_MIXED;
    if (xx != 0.0 && fp32) {
      NTG_TRY(ensure_fp32(p));
      { k_to_f32<<<grid_for(p->n, 256), 256, 0, s>>>(x_d, ksp->v32.p, p->n); NTG_COUNT_LAUNCH(); }
      NTG_TRY(ax_launch_f32(p, ksp->v32.w, ksp->v32.p, nullptr, 0, s));
      NTG_TRY(gs_add_guarded_f32(p, ksp->v32.w, s, nullptr));
      NTG_TRY(mask_guarded_f32(p, ksp->v32.w, s, nullptr));
      { k_resid_w32<<<grid_for(p->n, 256), 256, 0, s>>>(f_d, ksp->v32.w, ksp->v64.w, p->mult, ksp->v64.r, p->n, p->red_part, ksp->sc); NTG_COUNT_LAUNCH(); }
    } else if (xx != 0.0) {
      NTG_TRY(op_apply(p, ksp->v64.w, x_d, s));
      { k_resid<<<grid_for(p->n, 256), 256, 0, s>>>(f_d, ksp->v64.w, p->mult, ksp->v64.r, p->n, p->red_part, ksp->sc); NTG_COUNT_LAUNCH(); }
    }
    if (xx != 0.0) {
      NTG_CUDA_TRY(cudaMemcpyAsync(ksp->hs, ksp->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
      NTG_CUDA_TRY(cudaStreamSynchronize(s));
      if (!(ksp->hs->rr <= ksp->hs->ff)) {
        NTG_CUDA_TRY(cudaMemsetAsync(x_d, 0, sizeof(double) * p->n, s));
        rejected = 1;
      } else {
        ksp->ax_ready = fp32 ? 2 : 1;  // the mixed CG reuses this A x0 for its initial residual
      }
    }
  }
  int st = NTG_OK;
  if (ksp->type == NTG_KSP_GMRES || ksp->type == NTG_KSP_GMRES_MIXED) {
    GmresOpts o;
    o.restart = ksp->restart;
    o.fp32 = ksp->type == NTG_KSP_GMRES_MIXED;
    o.max_iter = ksp->max_iter;
    o.rtol = ksp->rtol;
    o.abstol = ksp->abstol;
    o.delta = ksp->inner_rtol;
    st = gmres_solve(ksp->plan, ksp->gm, ksp->sc, ksp->sw, o, x_d, f_d, mon);
  } else if (ksp->type == NTG_KSP_FCG_MIXED) st = ksp_solve_mixed(ksp, x_d, f_d, mon);
  else if (ksp->type == NTG_KSP_CG_MIXED)
    st = ksp->sw ? ksp_solve_mixed_ru_pc(ksp, x_d, f_d, mon) : ksp_solve_mixed_ru(ksp, x_d, f_d, mon);
  else st = ksp_solve_cg(ksp, x_d, f_d, mon);
  if (mon) {
    mon->guess_rejected = rejected;
    if (rejected && ksp->type != NTG_KSP_CG_MIXED) mon->fp64_ax += 1;
  }
  ksp->ax_ready = 0;
  return st;
}

int ntg_ksp_solve_coupled(ntg_ksp* ksp, double* x_d, double* y_d, double* z_d, const double* fx_d,
                          const double* fy_d, const double* fz_d, ntg_monitor* mon3) {
  clear_error();
  NTG_CHECK_ARG(ksp && x_d && y_d && z_d && fx_d && fy_d && fz_d, "ntg_ksp_solve_coupled: null argument");
  double* xs[3] = {x_d, y_d, z_d};
  const double* fs[3] = {fx_d, fy_d, fz_d};
  for (int c = 0; c < 3; ++c) NTG_TRY(ntg_ksp_solve(ksp, xs[c], fs[c], mon3 ? mon3 + c : nullptr));
  return NTG_OK;
}

}  // extern "C"
