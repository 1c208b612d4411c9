// Restarted flexible GMRES, device resident: Neko's pressure solver type
// ('gmres', selected with the hsmg preconditioner by the reference's cases,
// examples/rugby_ball/rugby_ball.case:46-52, and the filter's default,
// sources/mapping_functions/PDE_filter_mapping.f90:136).
//
// Right-preconditioned FGMRES(m) (Saad 1993): the preconditioned vectors
// Z_j = M V_j are kept, so the preconditioner may vary between steps (the
// FP32 Schwarz applied to FP64 data, or any inexact one).  Arnoldi by
// classical Gram-Schmidt applied twice, every dot a deterministic
// mult-weighted grid reduction; the Hessenberg matrix, its Givens rotations
// and the residual estimate |g_{j+1}| live on the device and are updated by
// the finaliser of the norm reduction, so a step needs no host round trip.
//
//   NTG_KSP_GMRES        FP64 vectors, FP64 operator (the plain drop-in)
//   NTG_KSP_GMRES_MIXED  FP32 vectors, operator and preconditioner in each
//                        cycle; every restart starts from the FP64 residual
//                        r = f - A x, and x accumulates in FP64 (GMRES-based
//                        iterative refinement, Carson & Higham 2018)
//
// Convergence is always judged on the FP64 residual of the FP64 solution.
#include <cmath>
#include <cstring>

#include "common.cuh"
#include "reduce.cuh"

namespace ntg {

constexpr int kGmMax = 31;  // restart cap: the dots of one Arnoldi pass share one reduction
static_assert(kGmMax + 1 <= kRedLanes, "one reduction lane per basis vector");

struct GmState {
  double H[(kGmMax + 1) * kGmMax];  // column-major, leading dimension kGmMax + 1
  double cs[kGmMax], sn[kGmMax], g[kGmMax + 1], y[kGmMax], h2[kGmMax + 1];
  double beta, tol, hnext, rr, ff;
  int j;     // completed Arnoldi columns of the current cycle
  int conv;  // the cycle reached its tolerance (or broke down)
  int pad[2];
};

struct GmresWork {
  int64_t n = 0;
  int m = 0, fp32 = 0;
  void* V = nullptr;  // (m + 1) basis vectors, T
  void* Z = nullptr;  // m preconditioned vectors, T
  void* w = nullptr;  // T
  void* rT = nullptr; // T residual (FP32 variant)
  double* r64 = nullptr;
  double* w64 = nullptr;
  float* a32 = nullptr;  // FP32 staging for the Schwarz preconditioner
  float* b32 = nullptr;
  GmState* gs = nullptr;
  GmState* hgs = nullptr;  // pinned host mirror
};

namespace gm {

constexpr int TPB = 256;

// r = f - w (w null: f); rT = (T) r (rT may alias r for T = double);
// (r, r)_mult and (f, f)_mult into gs
struct FinResid {
  GmState* gs;
  __device__ void operator()(const double* acc, Scalars*) const {
    gs->rr = acc[0];
    gs->ff = acc[1];
  }
};
template <typename T>
__global__ void k_resid(const double* __restrict__ f, const double* __restrict__ w, const double* __restrict__ mult,
                        double* __restrict__ r, T* __restrict__ rT, int64_t n, double* __restrict__ part, Scalars* sc,
                        GmState* gs) {
  double rr = 0, ff = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double fi = f[i];
    const double ri = w ? fi - w[i] : fi;
    r[i] = ri;
    if ((const void*)rT != (const void*)r) rT[i] = (T)ri;
    rr += mult[i] * ri * ri;
    ff += mult[i] * fi * fi;
  }
  double v[2] = {rr, ff};
  grid_reduce<2>(v, part, sc, FinResid{gs});
}

// beta = ||r||_mult starts a cycle: g = beta e1
struct FinBeta {
  GmState* gs;
  __device__ void operator()(const double* acc, Scalars* sc) const {
    const double beta = sqrt(acc[0]);
    gs->beta = beta;
    gs->g[0] = beta;
    gs->j = 0;
    gs->conv = !(beta > gs->tol);
    sc->done = gs->conv;
    if (!isfinite(beta)) {
      sc->status = NTG_NONFINITE;
      gs->conv = 1;
      sc->done = 1;
    }
  }
};
template <typename T>
__global__ void k_beta(const T* __restrict__ r, const T* __restrict__ mult, int64_t n, double* __restrict__ part,
                       Scalars* sc, GmState* gs) {
  T s = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s += mult[i] * r[i] * r[i];
  double v[1] = {(double)s};
  grid_reduce<1>(v, part, sc, FinBeta{gs});
}

// v = w / s, s = beta (which = 0) or the last norm (which = 1)
template <typename T>
__global__ void k_scale(T* __restrict__ v, const T* __restrict__ w, int64_t n, const GmState* gs, int which,
                        const Scalars* sc) {
  if (sc->done) return;
  const T inv = (T)(1.0 / (which ? gs->hnext : gs->beta));
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    v[i] = w[i] * inv;
}

// z = dinv r
template <typename T>
__global__ void k_jacobi(T* __restrict__ z, const T* __restrict__ r, const T* __restrict__ dinv, int64_t n,
                         const Scalars* sc) {
  if (sc->done) return;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    z[i] = dinv[i] * r[i];
}

template <typename A, typename B>
__global__ void k_convert(A* __restrict__ a, const B* __restrict__ b, int64_t n, const Scalars* sc) {
  if (sc->done) return;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    a[i] = (A)b[i];
}

// h_k = (V_k, w)_mult, k <= j; pass 0 stores column j of H, pass 1 adds to it
// (and keeps the correction for the second orthogonalisation)
struct FinDots {
  GmState* gs;
  int j, pass;
  __device__ void operator()(const double* acc, Scalars*) const {
    constexpr int LD = kGmMax + 1;
    for (int k = 0; k <= j; ++k) {
      if (pass == 0) {
        gs->H[k + LD * j] = acc[k];
      } else {
        gs->h2[k] = acc[k];
        gs->H[k + LD * j] += acc[k];
      }
    }
  }
};
template <typename T, int MAXL>
__global__ void k_dots(const T* __restrict__ w, const T* __restrict__ V, int j, int64_t n, const T* __restrict__ mult,
                       double* __restrict__ part, Scalars* sc, GmState* gs, int pass) {
  if (sc->done) return;
  T acc[MAXL];
#pragma unroll
  for (int k = 0; k < MAXL; ++k) acc[k] = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T wi = w[i] * mult[i];
#pragma unroll
    for (int k = 0; k < MAXL; ++k)
      if (k <= j) acc[k] += wi * V[(int64_t)k * n + i];
  }
  double v[MAXL];
#pragma unroll
  for (int k = 0; k < MAXL; ++k) v[k] = (double)acc[k];
  grid_reduce<MAXL>(v, part, sc, FinDots{gs, j, pass});
}

// w -= sum_k c_k V_k, c = column j of H (pass 0) or the correction (pass 1)
template <typename T>
__global__ void k_orth(T* __restrict__ w, const T* __restrict__ V, int j, int64_t n, const GmState* gs, int pass,
                       const Scalars* sc) {
  if (sc->done) return;
  __shared__ T c[kGmMax + 1];
  constexpr int LD = kGmMax + 1;
  if (threadIdx.x <= j) c[threadIdx.x] = (T)(pass == 0 ? gs->H[threadIdx.x + LD * j] : gs->h2[threadIdx.x]);
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    T v = w[i];
    for (int k = 0; k <= j; ++k) v -= c[k] * V[(int64_t)k * n + i];
    w[i] = v;
  }
}

// ||w||: H[j+1, j], the Givens rotations of column j, the residual estimate
struct FinNorm {
  GmState* gs;
  int j;
  __device__ void operator()(const double* acc, Scalars* sc) const {
    constexpr int LD = kGmMax + 1;
    const double hn = sqrt(acc[0]);
    gs->hnext = hn;
    double* Hj = gs->H + LD * j;
    Hj[j + 1] = hn;
    for (int i = 0; i < j; ++i) {
      const double a = Hj[i], b = Hj[i + 1];
      Hj[i] = gs->cs[i] * a + gs->sn[i] * b;
      Hj[i + 1] = -gs->sn[i] * a + gs->cs[i] * b;
    }
    const double a = Hj[j], b = Hj[j + 1];
    const double rho = hypot(a, b);
    const double c = rho > 0 ? a / rho : 1.0, s = rho > 0 ? b / rho : 0.0;
    gs->cs[j] = c;
    gs->sn[j] = s;
    Hj[j] = rho;
    Hj[j + 1] = 0.0;
    gs->g[j + 1] = -s * gs->g[j];
    gs->g[j] = c * gs->g[j];
    gs->j = j + 1;
    if (!isfinite(hn) || !isfinite(rho)) {
      sc->status = NTG_NONFINITE;
      gs->conv = 1;
      sc->done = 1;
      return;
    }
    // converged, or breakdown (the Krylov space holds the solution)
    if (fabs(gs->g[j + 1]) <= gs->tol || !(hn > 0.0)) {
      gs->conv = 1;
      sc->done = 1;
    }
  }
};
template <typename T>
__global__ void k_norm(const T* __restrict__ w, const T* __restrict__ mult, int64_t n, double* __restrict__ part,
                       Scalars* sc, GmState* gs, int j) {
  if (sc->done) return;
  T s = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s += mult[i] * w[i] * w[i];
  double v[1] = {(double)s};
  grid_reduce<1>(v, part, sc, FinNorm{gs, j});
}

// y = R^-1 g over the completed columns (one thread; at most kGmMax)
__global__ void k_solve_y(GmState* gs) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  constexpr int LD = kGmMax + 1;
  const int jc = gs->j;
  for (int i = jc - 1; i >= 0; --i) {
    double v = gs->g[i];
    for (int k = i + 1; k < jc; ++k) v -= gs->H[i + LD * k] * gs->y[k];
    const double d = gs->H[i + LD * i];
    gs->y[i] = d != 0.0 ? v / d : 0.0;
  }
}

// x += sum_k y_k Z_k (the correction in T, accumulated into the FP64 x)
template <typename T>
__global__ void k_update(double* __restrict__ x, const T* __restrict__ Z, int64_t n, const GmState* gs) {
  __shared__ T y[kGmMax];
  const int jc = gs->j;
  if (threadIdx.x < jc) y[threadIdx.x] = (T)gs->y[threadIdx.x];
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    T e = 0;
    for (int k = 0; k < jc; ++k) e += y[k] * Z[(int64_t)k * n + i];
    x[i] += (double)e;
  }
}

template <typename T, int MAXL>
int dots_launch(ntg_plan* p, const T* w, const T* V, int j, const T* mult, Scalars* sc, GmState* gs, int pass,
                cudaStream_t s) {
  k_dots<T, MAXL><<<grid_for(p->n, TPB), TPB, 0, s>>>(w, V, j, p->n, mult, p->red_part, sc, gs, pass);
  NTG_COUNT_LAUNCH();
  return NTG_OK;
}

template <typename T>
int dots(ntg_plan* p, const T* w, const T* V, int j, const T* mult, Scalars* sc, GmState* gs, int pass,
         cudaStream_t s) {
  if (j < 8) return dots_launch<T, 8>(p, w, V, j, mult, sc, gs, pass, s);
  if (j < 16) return dots_launch<T, 16>(p, w, V, j, mult, sc, gs, pass, s);
  return dots_launch<T, 32>(p, w, V, j, mult, sc, gs, pass, s);
}

}  // namespace gm

void gmres_free(GmresWork* g) {
  if (!g) return;
  dev_free(g->V); dev_free(g->Z); dev_free(g->w); dev_free(g->rT);
  dev_free(g->r64); dev_free(g->w64); dev_free(g->a32); dev_free(g->b32); dev_free(g->gs);
  if (g->hgs) cudaFreeHost(g->hgs);
  delete g;
}

static int gmres_alloc(GmresWork*& g, ntg_plan* p, int m, int fp32) {
  if (g && g->n == p->n && g->m == m && g->fp32 == fp32) return NTG_OK;
  gmres_free(g);
  g = new GmresWork();
  g->n = p->n;
  g->m = m;
  g->fp32 = fp32;
  const size_t n = (size_t)p->n, es = fp32 ? sizeof(float) : sizeof(double);
  auto bytes = [&](void** ptr, size_t count) -> int {
    if (cudaMalloc(ptr, count) != cudaSuccess) {
      cudaGetLastError();
      set_error("gmres: cannot allocate %zu bytes", count);
      return NTG_ERR_ALLOC;
    }
    return NTG_OK;
  };
  NTG_TRY(bytes(&g->V, es * n * (m + 1)));
  NTG_TRY(bytes(&g->Z, es * n * m));
  NTG_TRY(bytes(&g->w, es * n));
  if (fp32) NTG_TRY(bytes(&g->rT, es * n));
  NTG_TRY(dev_alloc(&g->r64, n));
  NTG_TRY(dev_alloc(&g->w64, n));
  NTG_TRY(dev_alloc(&g->gs, 1));
  if (cudaMallocHost(&g->hgs, sizeof(GmState)) != cudaSuccess) {
    set_error("gmres: cannot allocate pinned host memory");
    return NTG_ERR_ALLOC;
  }
  return NTG_OK;
}

// One GMRES solve.  sw: FP32 Schwarz preconditioner (null: Jacobi).  delta:
// the FP32 variant's relative reduction per cycle.
template <typename T>
static int gmres_run(ntg_plan* p, GmresWork* g, Scalars* sc, ntg_schwarz* sw, const GmresOpts& o, double* x,
                     const double* f, ntg_monitor* mon) {
  cudaStream_t s = p->stream;
  const int64_t n = p->n;
  const int G = grid_for(n, gm::TPB), m = g->m;
  T* V = (T*)g->V;
  T* Z = (T*)g->Z;
  T* w = (T*)g->w;
  T* rT = g->fp32 ? (T*)g->rT : (T*)g->r64;
  const T* mult = g->fp32 ? (const T*)p->multf : (const T*)p->mult;
  const T* dinv = g->fp32 ? (const T*)p->dinvf : (const T*)p->dinv;
  GmState* hg = g->hgs;
  int fpax = 0, iters = 0, cycles = 0;
  auto poll = [&]() -> int {
    NTG_CUDA_TRY(cudaMemcpyAsync(hg, g->gs, sizeof(GmState), cudaMemcpyDeviceToHost, s));
    NTG_CUDA_TRY(cudaStreamSynchronize(s));
    return NTG_OK;
  };
  auto residual = [&](bool nonzero_x) -> int {
    if (nonzero_x) {
      NTG_TRY(op_apply(p, g->w64, x, s));
      fpax++;
    }
    { gm::k_resid<T><<<G, gm::TPB, 0, s>>>(f, nonzero_x ? g->w64 : nullptr, p->mult, g->r64, rT, n, p->red_part, sc, g->gs); NTG_COUNT_LAUNCH(); }
    NTG_CUDA_TRY(cudaGetLastError());
    return poll();
  };
  auto precondition = [&](T* z, const T* v) -> int {
    if (sw) {
      if constexpr (sizeof(T) == sizeof(float)) {
        return schwarz_apply(sw, (float*)z, (const float*)v, s, sc);
      } else {
        { gm::k_convert<float, double><<<G, gm::TPB, 0, s>>>(g->a32, (const double*)v, n, sc); NTG_COUNT_LAUNCH(); }
        NTG_TRY(schwarz_apply(sw, g->b32, g->a32, s, sc));
        { gm::k_convert<double, float><<<G, gm::TPB, 0, s>>>((double*)z, g->b32, n, sc); NTG_COUNT_LAUNCH(); }
        return NTG_OK;
      }
    }
    { gm::k_jacobi<T><<<G, gm::TPB, 0, s>>>(z, v, dinv, n, sc); NTG_COUNT_LAUNCH(); }
    return NTG_OK;
  };
  auto op = [&](T* out, const T* in) -> int {
    if constexpr (sizeof(T) == sizeof(float)) {
      NTG_TRY(ax_launch_f32(p, (float*)out, (const float*)in, nullptr, 0, s));
      NTG_TRY(gs_add_guarded_f32(p, (float*)out, s, sc));
      return mask_guarded_f32(p, (float*)out, s, sc);
    } else {
      NTG_TRY(ax_launch(p, (double*)out, (const double*)in, nullptr, 0, s));
      NTG_TRY(gs_add_guarded(p, (double*)out, s, sc));
      return mask_guarded(p, (double*)out, s, sc);
    }
  };
  // start: r = f - A x
  double xx = 0.0;
  NTG_TRY(wdot(p, x, x, nullptr, n, &xx, s));
  NTG_TRY(residual(xx != 0.0));
  const double ff = hg->ff, rr0 = hg->rr;
  const double tol = fmax(o.abstol, o.rtol * sqrt(ff));
  double rr = rr0;
  int status = NTG_OK;
  for (;;) {
    if (!(sqrt(rr) > tol)) break;
    if (!std::isfinite(rr)) { status = NTG_NONFINITE; break; }
    if (iters >= o.max_iter) { status = NTG_MAXITER; break; }
    // a cycle on the current residual
    Scalars zero{};
    NTG_CUDA_TRY(cudaMemcpyAsync(sc, &zero, sizeof(Scalars), cudaMemcpyHostToDevice, s));
    const double tin = g->fp32 ? fmax(tol, o.delta * sqrt(rr)) : tol;
    NTG_CUDA_TRY(cudaMemcpyAsync(&g->gs->tol, &tin, sizeof(double), cudaMemcpyHostToDevice, s));
    { gm::k_beta<T><<<G, gm::TPB, 0, s>>>(rT, mult, n, p->red_part, sc, g->gs); NTG_COUNT_LAUNCH(); }
    { gm::k_scale<T><<<G, gm::TPB, 0, s>>>(V, rT, n, g->gs, 0, sc); NTG_COUNT_LAUNCH(); }
    const int mm = m < o.max_iter - iters ? m : o.max_iter - iters;
    for (int j = 0; j < mm; ++j) {
      T* Vj = V + (int64_t)j * n;
      T* Zj = Z + (int64_t)j * n;
      NTG_TRY(precondition(Zj, Vj));
      NTG_TRY(op(w, Zj));
      NTG_TRY(gm::dots<T>(p, w, V, j, mult, sc, g->gs, 0, s));
      { gm::k_orth<T><<<G, gm::TPB, 0, s>>>(w, V, j, n, g->gs, 0, sc); NTG_COUNT_LAUNCH(); }
      NTG_TRY(gm::dots<T>(p, w, V, j, mult, sc, g->gs, 1, s));
      { gm::k_orth<T><<<G, gm::TPB, 0, s>>>(w, V, j, n, g->gs, 1, sc); NTG_COUNT_LAUNCH(); }
      { gm::k_norm<T><<<G, gm::TPB, 0, s>>>(w, mult, n, p->red_part, sc, g->gs, j); NTG_COUNT_LAUNCH(); }
      { gm::k_scale<T><<<G, gm::TPB, 0, s>>>(V + (int64_t)(j + 1) * n, w, n, g->gs, 1, sc); NTG_COUNT_LAUNCH(); }
      NTG_CUDA_TRY(cudaGetLastError());
      if ((j + 1) % o.check_every == 0 || j + 1 == mm) {
        NTG_TRY(poll());
        if (hg->conv) break;
      }
    }
    NTG_TRY(poll());
    const int jc = hg->j;
    if (jc > 0) {
      { gm::k_solve_y<<<1, 32, 0, s>>>(g->gs); NTG_COUNT_LAUNCH(); }
      { gm::k_update<T><<<G, gm::TPB, 0, s>>>(x, Z, n, g->gs); NTG_COUNT_LAUNCH(); }
    }
    iters += jc;
    cycles++;
    NTG_TRY(residual(true));
    rr = hg->rr;
    if (jc == 0) {  // a cycle that cannot move (zero or non-finite start)
      if (!(sqrt(rr) > tol)) break;
      status = std::isfinite(rr) ? NTG_BREAKDOWN : NTG_NONFINITE;
      break;
    }
  }
  if (mon) {
    mon->iter = iters;
    mon->inner_iter = cycles;
    mon->res_start = sqrt(rr0);
    mon->res_final = sqrt(rr);
    mon->rhs_norm = sqrt(ff);
    mon->status = status;
    mon->fp64_ax = fpax;
  }
  return NTG_OK;
}

int gmres_solve(ntg_plan* p, GmresWork*& g, Scalars* sc, ntg_schwarz* sw, const GmresOpts& o, double* x,
                const double* f, ntg_monitor* mon) {
  NTG_CHECK_ARG(o.restart >= 1 && o.restart <= kGmMax, "gmres: restart length must be in [1, 31]");
  if (!p->jacobi_ready) NTG_TRY(jacobi_update(p));
  if (o.fp32 || sw) NTG_TRY(ensure_fp32(p));
  NTG_TRY(gmres_alloc(g, p, o.restart, o.fp32));
  if (sw && !o.fp32 && !g->a32) {
    NTG_TRY(dev_alloc(&g->a32, (size_t)p->n));
    NTG_TRY(dev_alloc(&g->b32, (size_t)p->n));
  }
  if (o.fp32) return gmres_run<float>(p, g, sc, sw, o, x, f, mon);
  return gmres_run<double>(p, g, sc, sw, o, x, f, mon);
}

}  // namespace ntg
