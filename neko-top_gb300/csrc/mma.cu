// The method of moving asymptotes on the GPU (FP64): the reference's MMA
// optimiser (sources/mma/mma.f90, sources/mma/bcknd/cpu/mma_cpu.f90), i.e.
// Svanberg's MMA with the primal-dual interior-point subproblem solver.
//
// Layout: every n-sized quantity (design, asymptotes, move limits, p0/q0,
// the m rows of P/Q stored row by row so each row is contiguous, the
// interior-point x/xsi/eta, their Newton directions and line-search
// origins) lives on the device; the m-sized dual quantities (y, z, lambda,
// s, mu, zeta) and the (m+1) x (m+1) Newton system live on the host, as in
// the reference, where they are scalars per rank.  Each Newton step is
// three kernels with fused reductions (residual, assembly, direction) and
// one per line-search trial; each reduction is deterministic (per-block
// partials summed in block order by the last block) and its m + 2 .. m(m+5)/2
// totals come back in one small copy, the GPU stand-in for the reference's
// MPI_Allreduce calls.  m <= 4 constraints.
#include <cmath>
#include <vector>

#include "reduce.cuh"

namespace ntg {
namespace mm {

constexpr int NT = 256;
constexpr int MMAX = 4;
constexpr int LANES = 2 * MMAX + MMAX * (MMAX + 1) / 2 + 2;  // sums + 1 max

// the reference's default-kind (single precision) literals
constexpr double C001 = (double)0.01f, C01 = (double)0.1f, C09 = (double)0.9f, C101 = (double)1.01f;

// 1/a and 1/b from one division (1/(ab) times the other factor): the FP64
// pipe, not memory, bounds these kernels, and a division costs it about ten
// FMAs.  Each result is within a few ulp of the quotient.
__device__ __forceinline__ void rcp2(double a, double b, double& ra, double& rb) {
  const double r = 1.0 / (a * b);
  ra = b * r;
  rb = a * r;
}

// 1/a, 1/b, 1/c, 1/d from one division
__device__ __forceinline__ void rcp4(double a, double b, double c, double d, double& ra, double& rb, double& rc,
                                     double& rd) {
  const double ab = a * b, cd = c * d, r = 1.0 / (ab * cd), rab = cd * r, rcd = ab * r;
  ra = b * rab;
  rb = a * rab;
  rc = d * rcd;
  rd = c * rcd;
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Reduce NS sums and one max over the grid; the last block writes them to
// out[0..NS) and out[NS].
template <int NS>
__device__ __forceinline__ void reduce_out(double (&v)[NS], double mx, double* __restrict__ part, unsigned* ticket,
                                           double* __restrict__ out) {
  __shared__ double sred[NS + 1][32];
  __shared__ int s_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int q = 0; q < NS; ++q) v[q] = warp_sum(v[q]);
  mx = warp_max(mx);
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < NS; ++q) sred[q][warp] = v[q];
    sred[NS][warp] = mx;
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int q = 0; q < NS; ++q) v[q] = warp_sum(lane < nw ? sred[q][lane] : 0.0);
    mx = warp_max(lane < nw ? sred[NS][lane] : -INFINITY);
    if (lane == 0) {
#pragma unroll
      for (int q = 0; q < NS; ++q) part[q * kRedSlots + blockIdx.x] = v[q];
      part[NS * kRedSlots + blockIdx.x] = mx;
      __threadfence();
      s_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  // the last block: every thread takes a fixed stride of the block partials,
  // then the fixed block tree (the same order on every run)
  double fin[NS];
  double fmx = -INFINITY;
#pragma unroll
  for (int q = 0; q < NS; ++q) fin[q] = 0.0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
#pragma unroll
    for (int q = 0; q < NS; ++q) fin[q] += __ldcg(part + q * kRedSlots + b);
    fmx = fmax(fmx, __ldcg(part + NS * kRedSlots + b));
  }
#pragma unroll
  for (int q = 0; q < NS; ++q) fin[q] = warp_sum(fin[q]);
  fmx = warp_max(fmx);
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < NS; ++q) sred[q][warp] = fin[q];
    sred[NS][warp] = fmx;
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int q = 0; q < NS; ++q) fin[q] = warp_sum(lane < nw ? sred[q][lane] : 0.0);
    fmx = warp_max(lane < nw ? sred[NS][lane] : -INFINITY);
    if (lane == 0) {
#pragma unroll
      for (int q = 0; q < NS; ++q) out[q] = fin[q];
      out[NS] = fmx;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    *ticket = 0;
    __threadfence();
  }
}

struct Vecs {
  double *low, *upp, *alpha, *beta, *p0, *q0, *P, *Q, *xmin, *xmax, *xold1, *xold2;
  double *x, *xsi, *eta, *dx, *dxsi, *deta, *x0, *xsi0, *eta0, *tdx, *diagx;
};

struct Red {
  double* part;
  unsigned* ticket;
  double* out;
};

// mma_gensub_cpu (mma_cpu.f90:8-184) + the subsolve's starting point (:236-246)
template <int M>
__global__ void __launch_bounds__(NT)
    k_gensub(Vecs V, const double* __restrict__ xval, const double* __restrict__ df0dx,
             const double* __restrict__ dfdx, int early, double asyinit, double asyincr, double asydecr, int64_t n,
             Red R) {
  double bi[M];
#pragma unroll
  for (int i = 0; i < M; ++i) bi[i] = 0.0;
  for (int64_t j = blockIdx.x * (int64_t)NT + threadIdx.x; j < n; j += (int64_t)gridDim.x * NT) {
    const double x = xval[j], xr = V.xmax[j] - V.xmin[j];
    double low, upp;
    if (early) {
      low = x - asyinit * xr;
      upp = x + asyinit * xr;
    } else {
      const double o1 = V.xold1[j], o2 = V.xold2[j], sg = (x - o1) * (o1 - o2);
      const double fac = sg < 0 ? asydecr : (sg > 0 ? asyincr : 1.0);
      low = x - fac * (o1 - V.low[j]);
      upp = x + fac * (V.upp[j] - o1);
      low = fmax(low, x - 10.0 * xr);
      low = fmin(low, x - C001 * xr);
      upp = fmin(upp, x + 10.0 * xr);
      upp = fmax(upp, x + C001 * xr);
    }
    V.low[j] = low;
    V.upp[j] = upp;
    const double al = fmax(fmax(V.xmin[j], low + 0.1 * (x - low)), x - 0.5 * xr);
    const double be = fmin(fmin(V.xmax[j], upp - C01 * (upp - x)), x + 0.5 * xr);
    V.alpha[j] = al;
    V.beta[j] = be;
    const double r = 0.00001 / fmax(0.00001, xr), ux = upp - x, xl = x - low, ux2 = ux * ux, xl2 = xl * xl;
    const double g0 = df0dx[j];
    V.p0[j] = ux2 * (1.001 * fmax(g0, 0.0) + 0.001 * fmax(-g0, 0.0) + r);
    V.q0[j] = xl2 * (0.001 * fmax(g0, 0.0) + 1.001 * fmax(-g0, 0.0) + r);
#pragma unroll
    for (int i = 0; i < M; ++i) {
      const double g = dfdx[i + M * j];
      const double p = ux2 * (1.001 * fmax(g, 0.0) + 0.001 * fmax(-g, 0.0) + r);
      const double q = xl2 * (0.001 * fmax(g, 0.0) + 1.001 * fmax(-g, 0.0) + r);
      V.P[i * n + j] = p;
      V.Q[i * n + j] = q;
      bi[i] += p / ux + q / xl;
    }
    const double xs = 0.5 * (al + be);
    V.x[j] = xs;
    V.xsi[j] = fmax(1.0, 1.0 / (xs - al));
    V.eta[j] = fmax(1.0, 1.0 / (be - xs));
  }
  reduce_out<M>(bi, -INFINITY, R.part, R.ticket, R.out);
}

struct Dual {
  double lam[MMAX];
  double dlam[MMAX];
  double epsi, steg;
};

// Residual of the perturbed KKT system at (x, xsi, eta; lambda): sums
// g_i(x) = sum_j P_ij/(u-x) + Q_ij/(x-l), sum of rex^2 + rexsi^2 + reeta^2
// and max |rex|, |rexsi|, |reeta|.  TRIAL: first step from the line-search
// origin: x = x0 + steg dx (likewise xsi, eta).
template <int M, bool TRIAL>
__global__ void __launch_bounds__(NT) k_resid(Vecs V, Dual D, int64_t n, Red R) {
  double acc[M + 1];
#pragma unroll
  for (int i = 0; i <= M; ++i) acc[i] = 0.0;
  double mx = 0.0;
  for (int64_t j = blockIdx.x * (int64_t)NT + threadIdx.x; j < n; j += (int64_t)gridDim.x * NT) {
    double x, xsi, eta;
    if (TRIAL) {
      x = V.x0[j] + D.steg * V.dx[j];
      xsi = V.xsi0[j] + D.steg * V.dxsi[j];
      eta = V.eta0[j] + D.steg * V.deta[j];
      V.x[j] = x;
      V.xsi[j] = xsi;
      V.eta[j] = eta;
    } else {
      x = V.x[j];
      xsi = V.xsi[j];
      eta = V.eta[j];
    }
    double rux, rxl;
    rcp2(V.upp[j] - x, x - V.low[j], rux, rxl);
    double pl = V.p0[j], ql = V.q0[j];
#pragma unroll
    for (int i = 0; i < M; ++i) {
      const double p = V.P[i * n + j], q = V.Q[i * n + j];
      pl += p * D.lam[i];
      ql += q * D.lam[i];
      acc[i] += p * rux + q * rxl;
    }
    const double rex = pl * (rux * rux) - ql * (rxl * rxl) - xsi + eta;
    const double rexsi = xsi * (x - V.alpha[j]) - D.epsi;
    const double reeta = eta * (V.beta[j] - x) - D.epsi;
    acc[M] += rex * rex + rexsi * rexsi + reeta * reeta;
    mx = fmax(mx, fmax(fabs(rex), fmax(fabs(rexsi), fabs(reeta))));
  }
  reduce_out<M + 1>(acc, mx, R.part, R.ticket, R.out);
}

// Newton assembly (mma_cpu.f90:307-405): delx, diagx per j (delx/diagx and
// 1/diagx kept), and the sums g_i(x), b_i = sum_j GG_ij delx_j/diagx_j,
// A_ik = sum_j GG_ij GG_kj / diagx_j (upper triangle).  FP64 division is
// costly on this GPU's narrow FP64 pipe, so each kernel forms the few
// reciprocals it needs (1/(u-x), 1/(x-l), 1/(x-alpha), 1/(beta-x),
// 1/diagx) once and multiplies: the reference's quotients to within an ulp.
template <int M>
__global__ void __launch_bounds__(NT) k_newton(Vecs V, Dual D, int64_t n, Red R) {
  constexpr int NS = 2 * M + M * (M + 1) / 2;
  double acc[NS];
#pragma unroll
  for (int q = 0; q < NS; ++q) acc[q] = 0.0;
  for (int64_t j = blockIdx.x * (int64_t)NT + threadIdx.x; j < n; j += (int64_t)gridDim.x * NT) {
    const double x = V.x[j], al = V.alpha[j], be = V.beta[j];
    double rux, rxl, ral, rbe;
    rcp4(V.upp[j] - x, x - V.low[j], x - al, be - x, rux, rxl, ral, rbe);
    const double rux2 = rux * rux, rxl2 = rxl * rxl;
    double pl = V.p0[j], ql = V.q0[j], gg[M];
#pragma unroll
    for (int i = 0; i < M; ++i) {
      const double p = V.P[i * n + j], q = V.Q[i * n + j];
      pl += p * D.lam[i];
      ql += q * D.lam[i];
      acc[i] += p * rux + q * rxl;
      gg[i] = p * rux2 - q * rxl2;
    }
    const double delx = pl * rux2 - ql * rxl2 - D.epsi * ral + D.epsi * rbe;
    double diagx = pl * (rux2 * rux) + ql * (rxl2 * rxl);
    diagx = 2.0 * diagx + V.xsi[j] * ral + V.eta[j] * rbe;
    const double rdg = 1.0 / diagx, t = delx * rdg;
    V.tdx[j] = t;
    V.diagx[j] = rdg;  // kept as its reciprocal
    int q = 2 * M;
#pragma unroll
    for (int i = 0; i < M; ++i) {
      acc[M + i] += gg[i] * t;
#pragma unroll
      for (int k = i; k < M; ++k) acc[q++] += gg[i] * rdg * gg[k];
    }
  }
  reduce_out<NS>(acc, -INFINITY, R.part, R.ticket, R.out);
}

// Directions (mma_cpu.f90:418-433) and the largest step ratio (:436-439);
// the line-search origin is saved.
template <int M>
__global__ void __launch_bounds__(NT) k_dir(Vecs V, Dual D, int64_t n, Red R) {
  double none[1] = {0.0};
  double mx = -INFINITY;
  for (int64_t j = blockIdx.x * (int64_t)NT + threadIdx.x; j < n; j += (int64_t)gridDim.x * NT) {
    const double x = V.x[j], al = V.alpha[j], be = V.beta[j], xsi = V.xsi[j], eta = V.eta[j];
    double rux, rxl, ral, rbe, rxs, ret;
    rcp4(V.upp[j] - x, x - V.low[j], x - al, be - x, rux, rxl, ral, rbe);
    rcp2(xsi, eta, rxs, ret);
    const double rux2 = rux * rux, rxl2 = rxl * rxl, rdg = V.diagx[j];
    double gl = 0.0;
#pragma unroll
    for (int i = 0; i < M; ++i) gl += (V.P[i * n + j] * rux2 - V.Q[i * n + j] * rxl2) * D.dlam[i];
    const double dx = -V.tdx[j] - gl * rdg;
    const double dxsi = -xsi + (D.epsi - dx * xsi) * ral;
    const double deta = -eta + (D.epsi + dx * eta) * rbe;
    V.dx[j] = dx;
    V.dxsi[j] = dxsi;
    V.deta[j] = deta;
    V.x0[j] = x;
    V.xsi0[j] = xsi;
    V.eta0[j] = eta;
    mx = fmax(mx, fmax(fmax(-C101 * dxsi * rxs, -C101 * deta * ret), fmax(-C101 * dx * ral, C101 * dx * rbe)));
  }
  reduce_out<1>(none, mx, R.part, R.ticket, R.out);
}

// mma_KKT_cpu (:581-641), the n-sized part
template <int M>
__global__ void __launch_bounds__(NT)
    k_kkt(Vecs V, Dual D, const double* __restrict__ xval, const double* __restrict__ df0dx,
          const double* __restrict__ dfdx, int64_t n, Red R) {
  double acc[1] = {0.0};
  double mx = 0.0;
  for (int64_t j = blockIdx.x * (int64_t)NT + threadIdx.x; j < n; j += (int64_t)gridDim.x * NT) {
    double rex = df0dx[j] - V.xsi[j] + V.eta[j];
#pragma unroll
    for (int i = 0; i < M; ++i) rex += dfdx[i + M * j] * D.lam[i];
    const double rexsi = V.xsi[j] * (xval[j] - V.xmin[j]);
    const double reeta = V.eta[j] * (V.xmax[j] - xval[j]);
    acc[0] += rex * rex + rexsi * rexsi + reeta * reeta;
    mx = fmax(mx, fmax(fabs(rex), fmax(fabs(rexsi), fabs(reeta))));
  }
  reduce_out<1>(acc, mx, R.part, R.ticket, R.out);
}

// max_j x_j (in the max lane)
__global__ void __launch_bounds__(NT) k_max(const double* __restrict__ x, int64_t n, Red R) {
  double none[1] = {0.0};
  double mx = -INFINITY;
  for (int64_t j = blockIdx.x * (int64_t)NT + threadIdx.x; j < n; j += (int64_t)gridDim.x * NT) mx = fmax(mx, x[j]);
  reduce_out<1>(none, mx, R.part, R.ticket, R.out);
}

__global__ void __launch_bounds__(NT) k_fill(double* __restrict__ a, double v, int64_t n) {
  for (int64_t j = blockIdx.x * (int64_t)NT + threadIdx.x; j < n; j += (int64_t)gridDim.x * NT) a[j] = v;
}

__global__ void __launch_bounds__(NT) k_neg(double* __restrict__ o, const double* __restrict__ a, int64_t n) {
  for (int64_t j = blockIdx.x * (int64_t)NT + threadIdx.x; j < n; j += (int64_t)gridDim.x * NT) o[j] = -a[j];
}

// Gaussian elimination with partial pivoting (DGESV's factorisation) of the
// (m+1) x (m+1) Newton system; returns false if a pivot is zero
bool solve_small(int k, std::vector<double> A, std::vector<double>& b) {
  for (int c = 0; c < k; ++c) {
    int p = c;
    for (int r = c + 1; r < k; ++r)
      if (fabs(A[r * k + c]) > fabs(A[p * k + c])) p = r;
    if (A[p * k + c] == 0.0) return false;
    if (p != c) {
      for (int q = 0; q < k; ++q) std::swap(A[c * k + q], A[p * k + q]);
      std::swap(b[c], b[p]);
    }
    for (int r = c + 1; r < k; ++r) {
      const double f = A[r * k + c] / A[c * k + c];
      for (int q = c; q < k; ++q) A[r * k + q] -= f * A[c * k + q];
      b[r] -= f * b[c];
    }
  }
  for (int c = k - 1; c >= 0; --c) {
    double s = b[c];
    for (int q = c + 1; q < k; ++q) s -= A[c * k + q] * b[q];
    b[c] = s / A[c * k + c];
  }
  return true;
}

}  // namespace mm
}  // namespace ntg

struct ntg_mma {
  int64_t n = 0;
  int m = 0;
  cudaStream_t stream = 0;
  double a0 = 1.0;
  std::vector<double> a, c, d, y, lam, s, mu, bi;
  double z = 1.0, zeta = 1.0;
  int max_iter = 100;
  double epsimin = 0.0, asyinit = 0.5, asyincr = 1.2, asydecr = 0.7;
  double residumax = 0.0, residunorm = 0.0;
  long long newton_steps = 0, trials = 0, levels = 0;
  ntg::mm::Vecs V{};
  double* part = nullptr;
  unsigned* ticket = nullptr;
  double* out_d = nullptr;
  double* out_h = nullptr;  // pinned
  int grid = 1;
};

using namespace ntg;

namespace {

mm::Red red(ntg_mma* o) { return mm::Red{o->part, o->ticket, o->out_d}; }

int fetch(ntg_mma* o, int count) {
  NTG_CUDA_TRY(cudaGetLastError());
  NTG_CUDA_TRY(cudaMemcpyAsync(o->out_h, o->out_d, sizeof(double) * count, cudaMemcpyDeviceToHost, o->stream));
  NTG_CUDA_TRY(cudaStreamSynchronize(o->stream));
  return NTG_OK;
}

template <typename F>
int with_m(int m, F&& f) {
  switch (m) {
    case 1: return f(std::integral_constant<int, 1>{});
    case 2: return f(std::integral_constant<int, 2>{});
    case 3: return f(std::integral_constant<int, 3>{});
    case 4: return f(std::integral_constant<int, 4>{});
    default: set_error("MMA: m=%d constraints not compiled (1..4)", m); return NTG_ERR_UNSUPPORTED;
  }
}

mm::Dual dual(const ntg_mma* o, double epsi) {
  mm::Dual D{};
  for (int i = 0; i < o->m; ++i) D.lam[i] = o->lam[i];
  D.epsi = epsi;
  return D;
}

// residual of the full perturbed KKT system from the device partial sums
// (out: m sums g_i, the x-part sum of squares, the x-part max)
void combine(const ntg_mma* o, const double* out, const std::vector<double>& y, double z,
             const std::vector<double>& lam, const std::vector<double>& s, const std::vector<double>& mu, double zeta,
             double epsi, double& norm, double& mx) {
  const int m = o->m;
  double sq = out[m], big = out[m + 1];
  double rez = o->a0 - zeta, rezeta = zeta * z - epsi;
  for (int i = 0; i < m; ++i) rez -= lam[i] * o->a[i];
  sq += rez * rez + rezeta * rezeta;
  big = std::max(big, std::max(fabs(rez), fabs(rezeta)));
  for (int i = 0; i < m; ++i) {
    const double rey = o->c[i] + o->d[i] * y[i] - lam[i] - mu[i];
    const double relam = out[i] - o->a[i] * z - y[i] + s[i] - o->bi[i];
    const double remu = mu[i] * y[i] - epsi;
    const double res = lam[i] * s[i] - epsi;
    sq += rey * rey + relam * relam + remu * remu + res * res;
    big = std::max(big, std::max(std::max(fabs(rey), fabs(relam)), std::max(fabs(remu), fabs(res))));
  }
  norm = sqrt(sq);
  mx = big;
}

template <int M>
int subsolve(ntg_mma* o, double* designx) {
  const int m = M;
  const int64_t n = o->n;
  const int g = o->grid;
  cudaStream_t st = o->stream;
  double epsi = 1.0;
  std::vector<double> y(m, 1.0), lam(m, 1.0), s(m, 1.0), mu(m);
  double z = 1.0, zeta = 1.0;
  for (int i = 0; i < m; ++i) mu[i] = std::max(1.0, 0.5 * o->c[i]);
  while (epsi > mm::C09 * o->epsimin) {
    ++o->levels;
    o->lam = lam;
    mm::k_resid<M, false><<<g, mm::NT, 0, st>>>(o->V, dual(o, epsi), n, red(o));
    NTG_COUNT_LAUNCH();
    NTG_TRY(fetch(o, m + 2));
    double residunorm, residumax;
    combine(o, o->out_h, y, z, lam, s, mu, zeta, epsi, residunorm, residumax);
    for (int it = 0; it < o->max_iter; ++it) {
      if (residumax < epsi) break;
      ++o->newton_steps;
      o->lam = lam;
      mm::k_newton<M><<<g, mm::NT, 0, st>>>(o->V, dual(o, epsi), n, red(o));
      NTG_COUNT_LAUNCH();
      constexpr int NS = 2 * M + M * (M + 1) / 2;
      NTG_TRY(fetch(o, NS));
      const double* out = o->out_h;
      std::vector<double> dely(m), dellam(m), bb(m + 1), AA((m + 1) * (m + 1));
      double delz = o->a0 - epsi / z;
      for (int i = 0; i < m; ++i) delz -= lam[i] * o->a[i];
      for (int i = 0; i < m; ++i) {
        dely[i] = o->c[i] + o->d[i] * y[i] - lam[i] - epsi / y[i];
        dellam[i] = out[i] - o->a[i] * z - y[i] - o->bi[i] + epsi / lam[i];
        bb[i] = dellam[i] + dely[i] / (o->d[i] + mu[i] / y[i]) - out[m + i];
      }
      bb[m] = delz;
      int q = 2 * m;
      for (int i = 0; i < m; ++i)
        for (int k = i; k < m; ++k) {
          AA[i * (m + 1) + k] = out[q];
          AA[k * (m + 1) + i] = out[q];
          ++q;
        }
      for (int i = 0; i < m; ++i) {
        AA[i * (m + 1) + i] += s[i] / lam[i] + 1.0 / (o->d[i] + mu[i] / y[i]);
        AA[i * (m + 1) + m] = o->a[i];
        AA[m * (m + 1) + i] = o->a[i];
      }
      AA[m * (m + 1) + m] = -zeta / z;
      if (!mm::solve_small(m + 1, AA, bb)) {
        set_error("MMA: singular Newton system in the subproblem solve");
        return NTG_BREAKDOWN;
      }
      std::vector<double> dlam(bb.begin(), bb.begin() + m), dy(m), dmu(m), ds(m);
      const double dz = bb[m];
      for (int i = 0; i < m; ++i) {
        dy[i] = (-dely[i] + dlam[i]) / (o->d[i] + mu[i] / y[i]);
        dmu[i] = -mu[i] + (epsi - mu[i] * dy[i]) / y[i];
        ds[i] = -s[i] + (epsi - dlam[i] * s[i]) / lam[i];
      }
      const double dzeta = -zeta + (epsi - zeta * dz) / z;
      mm::Dual D = dual(o, epsi);
      for (int i = 0; i < m; ++i) D.dlam[i] = dlam[i];
      mm::k_dir<M><<<g, mm::NT, 0, st>>>(o->V, D, n, red(o));
      NTG_COUNT_LAUNCH();
      NTG_TRY(fetch(o, 2));
      double steg = std::max(1.0, o->out_h[1]);
      auto ratio = [&](double dv, double v) { steg = std::max(steg, -mm::C101 * dv / v); };
      for (int i = 0; i < m; ++i) {
        ratio(dy[i], y[i]);
        ratio(dlam[i], lam[i]);
        ratio(dmu[i], mu[i]);
        ratio(ds[i], s[i]);
      }
      ratio(dz, z);
      ratio(dzeta, zeta);
      steg = 1.0 / steg;
      const std::vector<double> y0 = y, lam0 = lam, mu0 = mu, s0 = s;
      const double z0 = z, zeta0 = zeta;
      double newres = 2.0 * residunorm;
      int itto = 0;
      while (newres > residunorm && itto < 50) {
        ++itto;
        ++o->trials;
        for (int i = 0; i < m; ++i) {
          y[i] = y0[i] + steg * dy[i];
          lam[i] = lam0[i] + steg * dlam[i];
          mu[i] = mu0[i] + steg * dmu[i];
          s[i] = s0[i] + steg * ds[i];
        }
        z = z0 + steg * dz;
        zeta = zeta0 + steg * dzeta;
        o->lam = lam;
        mm::Dual Dt = dual(o, epsi);
        Dt.steg = steg;
        mm::k_resid<M, true><<<g, mm::NT, 0, st>>>(o->V, Dt, n, red(o));
        NTG_COUNT_LAUNCH();
        NTG_TRY(fetch(o, m + 2));
        combine(o, o->out_h, y, z, lam, s, mu, zeta, epsi, newres, residumax);
        steg = steg / 2.0;
      }
      residunorm = newres;
    }
    epsi = 0.1 * epsi;
  }
  // xold2 <- xold1 <- the design the step started from; design <- x
  NTG_CUDA_TRY(cudaMemcpyAsync(o->V.xold2, o->V.xold1, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  NTG_CUDA_TRY(cudaMemcpyAsync(o->V.xold1, designx, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  NTG_CUDA_TRY(cudaMemcpyAsync(designx, o->V.x, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  o->y = y;
  o->z = z;
  o->lam = lam;
  o->zeta = zeta;
  o->mu = mu;
  o->s = s;
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

void mma_free(ntg_mma* o) {
  double** all[] = {&o->V.low, &o->V.upp, &o->V.alpha, &o->V.beta, &o->V.p0, &o->V.q0, &o->V.P, &o->V.Q,
                    &o->V.xmin, &o->V.xmax, &o->V.xold1, &o->V.xold2, &o->V.x, &o->V.xsi, &o->V.eta, &o->V.dx,
                    &o->V.dxsi, &o->V.deta, &o->V.x0, &o->V.xsi0, &o->V.eta0, &o->V.tdx, &o->V.diagx,
                    &o->part, &o->out_d};
  for (double** p : all) dev_free(*p);
  dev_free(o->ticket);
  if (o->out_h) cudaFreeHost(o->out_h);
  o->out_h = nullptr;
}

}  // namespace

extern "C" {

int ntg_mma_create(ntg_mma** out, int64_t n, int m, const double* x_d, double a0, const double* a, const double* c,
                   const double* d, const double* xmin_d, const double* xmax_d, int max_iter, double epsimin,
                   double asyinit, double asyincr, double asydecr, void* stream) {
  clear_error();
  NTG_CHECK_ARG(out && x_d && a && c && d && xmin_d && xmax_d && n > 0, "ntg_mma_create: bad argument");
  NTG_CHECK_ARG(m >= 1 && m <= mm::MMAX, "ntg_mma_create: m must be in [1, 4]");
  ntg_mma* o = new ntg_mma();
  o->n = n;
  o->m = m;
  o->stream = (cudaStream_t)stream;
  o->a0 = a0;
  o->a.assign(a, a + m);
  o->c.assign(c, c + m);
  o->d.assign(d, d + m);
  o->y.assign(m, 0.0);
  o->lam.assign(m, 0.0);
  o->s.assign(m, 0.0);
  o->mu.assign(m, 0.0);
  o->bi.assign(m, 0.0);
  o->z = o->zeta = 0.0;
  // defaults of mma_init_attributes (mma.f90:275-283)
  o->max_iter = max_iter > 0 ? max_iter : 100;
  o->epsimin = epsimin > 0 ? epsimin : 1.0e-9 * sqrt((double)(m + n));
  o->asyinit = asyinit > 0 ? asyinit : 0.5;
  o->asyincr = asyincr > 0 ? asyincr : 1.2;
  o->asydecr = asydecr > 0 ? asydecr : 0.7;
  o->residumax = o->residunorm = 1.79769313486231570e308;
  const int64_t g = (n + mm::NT - 1) / mm::NT, cap = std::min<int64_t>((int64_t)num_sms() * 8, kRedSlots);
  o->grid = (int)std::max<int64_t>(1, std::min(g, cap));
  int st = NTG_OK;
  double** vecs[] = {&o->V.low, &o->V.upp, &o->V.alpha, &o->V.beta, &o->V.p0, &o->V.q0, &o->V.xmin, &o->V.xmax,
                     &o->V.xold1, &o->V.xold2, &o->V.x, &o->V.xsi, &o->V.eta, &o->V.dx, &o->V.dxsi, &o->V.deta,
                     &o->V.x0, &o->V.xsi0, &o->V.eta0, &o->V.tdx, &o->V.diagx};
  for (double** p : vecs)
    if (!st) st = dev_alloc(p, (size_t)n);
  if (!st) st = dev_alloc(&o->V.P, (size_t)(m * n));
  if (!st) st = dev_alloc(&o->V.Q, (size_t)(m * n));
  if (!st) st = dev_alloc(&o->part, (size_t)mm::LANES * kRedSlots);
  if (!st) st = dev_alloc(&o->out_d, (size_t)mm::LANES);
  if (!st) st = dev_alloc(&o->ticket, 1);
  if (!st && cudaMallocHost(&o->out_h, sizeof(double) * mm::LANES) != cudaSuccess) {
    set_error("ntg_mma_create: pinned allocation failed");
    st = NTG_ERR_ALLOC;
  }
  if (!st) {
    cudaStream_t s = o->stream;
    const size_t b = sizeof(double) * n;
    if (cudaMemsetAsync(o->ticket, 0, sizeof(unsigned), s) != cudaSuccess ||
        cudaMemcpyAsync(o->V.xold1, x_d, b, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(o->V.xold2, x_d, b, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(o->V.xmin, xmin_d, b, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(o->V.xmax, xmax_d, b, cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
      set_error("ntg_mma_create: copy failed");
      st = NTG_ERR_CUDA;
    }
  }
  if (!st) {
    // low = min(x), upp = max(x) as the reference initialises them
    mm::k_max<<<o->grid, mm::NT, 0, o->stream>>>(x_d, n, red(o));
    NTG_COUNT_LAUNCH();
    st = fetch(o, 2);
    const double xmax = o->out_h[1];
    if (!st) {
      mm::k_neg<<<o->grid, mm::NT, 0, o->stream>>>(o->V.x0, x_d, n);
      mm::k_max<<<o->grid, mm::NT, 0, o->stream>>>(o->V.x0, n, red(o));
      NTG_COUNT_LAUNCH();
      NTG_COUNT_LAUNCH();
      st = fetch(o, 2);
    }
    if (!st) {
      const double xmin = -o->out_h[1];
      mm::k_fill<<<o->grid, mm::NT, 0, o->stream>>>(o->V.low, xmin, n);
      mm::k_fill<<<o->grid, mm::NT, 0, o->stream>>>(o->V.upp, xmax, n);
      NTG_COUNT_LAUNCH();
      NTG_COUNT_LAUNCH();
      if (cudaGetLastError() != cudaSuccess) st = NTG_ERR_CUDA;
    }
  }
  if (st) {
    mma_free(o);
    delete o;
    return st;
  }
  *out = o;
  return NTG_OK;
}

int ntg_mma_destroy(ntg_mma* o) {
  if (!o) return NTG_OK;
  cudaStreamSynchronize(o->stream);
  mma_free(o);
  delete o;
  return NTG_OK;
}

int ntg_mma_update(ntg_mma* o, int iter, double* x_d, const double* df0dx_d, const double* fval,
                   const double* dfdx_d) {
  clear_error();
  NTG_CHECK_ARG(o && x_d && df0dx_d && fval && dfdx_d, "ntg_mma_update: null argument");
  return with_m(o->m, [&](auto MC) -> int {
    constexpr int M = decltype(MC)::value;
    mm::k_gensub<M><<<o->grid, mm::NT, 0, o->stream>>>(o->V, x_d, df0dx_d, dfdx_d, iter < 3 ? 1 : 0, o->asyinit,
                                                        o->asyincr, o->asydecr, o->n, red(o));
    NTG_COUNT_LAUNCH();
    NTG_TRY(fetch(o, M));
    for (int i = 0; i < M; ++i) o->bi[i] = o->out_h[i] - fval[i];
    return subsolve<M>(o, x_d);
  });
}

int ntg_mma_kkt(ntg_mma* o, const double* x_d, const double* df0dx_d, const double* fval, const double* dfdx_d,
                double* residumax, double* residunorm) {
  clear_error();
  NTG_CHECK_ARG(o && x_d && df0dx_d && fval && dfdx_d, "ntg_mma_kkt: null argument");
  return with_m(o->m, [&](auto MC) -> int {
    constexpr int M = decltype(MC)::value;
    mm::k_kkt<M><<<o->grid, mm::NT, 0, o->stream>>>(o->V, dual(o, 0.0), x_d, df0dx_d, dfdx_d, o->n, red(o));
    NTG_COUNT_LAUNCH();
    NTG_TRY(fetch(o, 2));
    double sq = o->out_h[0], big = o->out_h[1];
    double rez = o->a0 - o->zeta, rezeta = o->zeta * o->z;
    for (int i = 0; i < M; ++i) rez -= o->lam[i] * o->a[i];
    sq += rez * rez + rezeta * rezeta;
    big = std::max(big, std::max(fabs(rez), fabs(rezeta)));
    for (int i = 0; i < M; ++i) {
      const double rey = o->c[i] + o->d[i] * o->y[i] - o->lam[i] - o->mu[i];
      const double relam = fval[i] - o->a[i] * o->z - o->y[i] + o->s[i];
      const double remu = o->mu[i] * o->y[i], res = o->lam[i] * o->s[i];
      sq += rey * rey + relam * relam + remu * remu + res * res;
      big = std::max(big, std::max(std::max(fabs(rey), fabs(relam)), std::max(fabs(remu), fabs(res))));
    }
    o->residumax = big;
    o->residunorm = sqrt(sq);
    if (residumax) *residumax = big;
    if (residunorm) *residunorm = o->residunorm;
    return NTG_OK;
  });
}

int ntg_mma_info(const ntg_mma* o, long long* counts, double* residumax, double* residunorm) {
  clear_error();
  NTG_CHECK_ARG(o, "ntg_mma_info: null handle");
  if (counts) {
    counts[0] = o->newton_steps;
    counts[1] = o->trials;
    counts[2] = o->levels;
  }
  if (residumax) *residumax = o->residumax;
  if (residunorm) *residunorm = o->residunorm;
  return NTG_OK;
}

}  // extern "C"
