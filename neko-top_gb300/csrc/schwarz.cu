// Overlapping additive Schwarz preconditioner with fast-diagonalisation (FDM)
// local solves, in FP32, for structured box meshes.
//
//   z = sum_e R_e^T  A~_e^{-1}  R_e r
//
// R_e gathers the assembled residual on element e extended by one node layer
// into each neighbour ((lx+2)^3 nodes); A~_e is the separable approximation of
// the local operator on that extended box,
//   h1 (Bz x By x Kx + Bz x Ky x Bx + Kz x By x Bx) + h2 (Bz x By x Bx),
// with 1D stiffness/mass matrices assembled from the element and the adjacent
// GLL interval of each neighbour (homogeneous Dirichlet one node further out),
// inverted through the generalised eigenvectors of each 1D pair
// (Lynch, Rice & Thomas 1964; Fischer 1997, "An overlapping Schwarz method for
// spectral element solution of the incompressible Navier-Stokes equations").
// Element lengths come from the node coordinates; h1/h2 are element means.
//
// Reference context: Neko's pressure solves use a Schwarz-multigrid
// preconditioner ('hsmg', examples/rugby_ball/rugby_ball.case:46-52); this is
// its one-level Schwarz part on the GLL grid.
//
// Determinism: the prolongation is a pull -- every local node sums, in a fixed
// order, the extended results of the elements whose extended box covers it --
// followed by the ordinary gather-scatter, so no atomics are involved.
#include <cmath>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

#include "common.cuh"
#include "reduce.cuh"

namespace ntg {

namespace sw {

// mean distance between opposite faces of each element along r, s, t
__global__ void k_lengths(const double* __restrict__ x, const double* __restrict__ y, const double* __restrict__ z,
                          int64_t nelv, int lx, double* __restrict__ hl) {
  const int lx2 = lx * lx, lx3 = lx2 * lx, N = lx - 1;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nelv; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e * lx3;
    double s[3] = {0, 0, 0};
    for (int p = 0; p < lx; ++p)
      for (int q = 0; q < lx; ++q) {
        int64_t a0[3] = {b + 0 + lx * p + lx2 * q, b + p + lx * 0 + lx2 * q, b + p + lx * q + lx2 * 0};
        int64_t a1[3] = {b + N + lx * p + lx2 * q, b + p + lx * N + lx2 * q, b + p + lx * q + lx2 * N};
        for (int d = 0; d < 3; ++d) {
          const double dx = x[a1[d]] - x[a0[d]], dy = y[a1[d]] - y[a0[d]], dz = z[a1[d]] - z[a0[d]];
          s[d] += sqrt(dx * dx + dy * dy + dz * dz);
        }
      }
    for (int d = 0; d < 3; ++d) hl[3 * e + d] = s[d] / (double)lx2;
  }
}

// element means of h1 and h2 (h2 may be null -> 0; h1 null -> h1c)
__global__ void k_coef_means(const double* __restrict__ h1, double h1c, const double* __restrict__ hB,
                             const double* __restrict__ B, int64_t nelv, int lx3, float* __restrict__ hc) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nelv; e += (int64_t)gridDim.x * blockDim.x) {
    double a = 0, c = 0;
    for (int q = 0; q < lx3; ++q) {
      const int64_t l = e * lx3 + q;
      a += h1 ? h1[l] : h1c;
      if (hB) c += hB[l] / B[l];
    }
    hc[2 * e] = (float)(a / lx3);
    hc[2 * e + 1] = (float)(c / lx3);
  }
}

template <int LX>
struct Ext {
  static constexpr int N = LX - 1, LE = LX + 2, LE2 = LE * LE, LE3 = LE * LE * LE;
};

// extended residual -> FDM solve -> extended result (one block per element)
template <int LX>
__global__ void __launch_bounds__(128)
    k_fdm(const float* __restrict__ r, float* __restrict__ ze, const float* __restrict__ S,
          const float* __restrict__ lam, const float* __restrict__ hc, int Ex, int Ey, int Ez, const Scalars* sc) {
  using X = Ext<LX>;
  constexpr int LE = X::LE, LE2 = X::LE2, LE3 = X::LE3, N = X::N;
  constexpr int LX2 = LX * LX, LX3 = LX * LX * LX;
  if (sc && sc->done) return;
  __shared__ float A[LE3], Bt[LE3], sS[3][LE2], sL[3][LE];
  const int64_t nelv = (int64_t)Ex * Ey * Ez;
  for (int64_t e = blockIdx.x; e < nelv; e += gridDim.x) {
    const int ex = (int)(e % Ex), ey = (int)((e / Ex) % Ey), ez = (int)(e / ((int64_t)Ex * Ey));
    for (int q = threadIdx.x; q < 3 * LE2; q += blockDim.x) sS[q / LE2][q % LE2] = S[e * 3 * LE2 + q];
    for (int q = threadIdx.x; q < 3 * LE; q += blockDim.x) sL[q / LE][q % LE] = lam[e * 3 * LE + q];
    const float h1 = hc[2 * e], h2 = hc[2 * e + 1];
    // gather R_e r
    for (int q = threadIdx.x; q < LE3; q += blockDim.x) {
      const int a = q % LE, b = (q / LE) % LE, c = q / LE2;
      int i = a - 1, j = b - 1, k = c - 1;
      int dx = 0, dy = 0, dz = 0;
      if (i < 0) { dx = -1; i = N - 1; } else if (i > N) { dx = 1; i = 1; }
      if (j < 0) { dy = -1; j = N - 1; } else if (j > N) { dy = 1; j = 1; }
      if (k < 0) { dz = -1; k = N - 1; } else if (k > N) { dz = 1; k = 1; }
      const int nx = ex + dx, ny = ey + dy, nz = ez + dz;
      float v = 0.f;
      if (nx >= 0 && nx < Ex && ny >= 0 && ny < Ey && nz >= 0 && nz < Ez) {
        const int64_t en = nx + (int64_t)Ex * (ny + (int64_t)Ey * nz);
        v = r[en * LX3 + i + LX * j + LX2 * k];
      }
      A[q] = v;
    }
    __syncthreads();
    // transform: Bt = (Sz x Sy x Sx)^T A   (three passes, A <-> Bt)
    for (int q = threadIdx.x; q < LE3; q += blockDim.x) {
      const int a = q % LE, rest = q - a;
      float s = 0.f;
#pragma unroll
      for (int p = 0; p < LE; ++p) s = fmaf(sS[0][p * LE + a], A[rest + p], s);
      Bt[q] = s;
    }
    __syncthreads();
    for (int q = threadIdx.x; q < LE3; q += blockDim.x) {
      const int a = q % LE, b = (q / LE) % LE, c = q / LE2;
      float s = 0.f;
#pragma unroll
      for (int p = 0; p < LE; ++p) s = fmaf(sS[1][p * LE + b], Bt[a + LE * p + LE2 * c], s);
      A[q] = s;
    }
    __syncthreads();
    for (int q = threadIdx.x; q < LE3; q += blockDim.x) {
      const int a = q % LE, b = (q / LE) % LE, c = q / LE2;
      float s = 0.f;
#pragma unroll
      for (int p = 0; p < LE; ++p) s = fmaf(sS[2][p * LE + c], A[a + LE * b + LE2 * p], s);
      Bt[q] = s / (h1 * (sL[0][a] + sL[1][b] + sL[2][c]) + h2);
    }
    __syncthreads();
    // back: A = (Sz x Sy x Sx) Bt
    for (int q = threadIdx.x; q < LE3; q += blockDim.x) {
      const int a = q % LE, b = (q / LE) % LE, c = q / LE2;
      float s = 0.f;
#pragma unroll
      for (int p = 0; p < LE; ++p) s = fmaf(sS[2][c * LE + p], Bt[a + LE * b + LE2 * p], s);
      A[q] = s;
    }
    __syncthreads();
    for (int q = threadIdx.x; q < LE3; q += blockDim.x) {
      const int a = q % LE, b = (q / LE) % LE, c = q / LE2;
      float s = 0.f;
#pragma unroll
      for (int p = 0; p < LE; ++p) s = fmaf(sS[1][b * LE + p], A[a + LE * p + LE2 * c], s);
      Bt[q] = s;
    }
    __syncthreads();
    for (int q = threadIdx.x; q < LE3; q += blockDim.x) {
      const int a = q % LE, rest = q - a;
      float s = 0.f;
#pragma unroll
      for (int p = 0; p < LE; ++p) s = fmaf(sS[0][a * LE + p], Bt[rest + p], s);
      ze[e * LE3 + q] = s;
    }
    __syncthreads();
  }
}

// prolongation: every local node sums the extended results covering it
template <int LX>
__global__ void k_pull(const float* __restrict__ ze, float* __restrict__ z, int Ex, int Ey, int Ez,
                       const Scalars* sc) {
  using X = Ext<LX>;
  constexpr int LE = X::LE, LE2 = X::LE2, LE3 = X::LE3, N = X::N;
  constexpr int LX2 = LX * LX, LX3 = LX * LX * LX;
  if (sc && sc->done) return;
  const int64_t n = (int64_t)Ex * Ey * Ez * LX3;
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < n; l += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = l / LX3;
    const int m = (int)(l - e * LX3);
    const int i = m % LX, j = (m / LX) % LX, k = m / LX2;
    const int ex = (int)(e % Ex), ey = (int)((e / Ex) % Ey), ez = (int)(e / ((int64_t)Ex * Ey));
    // per dimension: (element offset, extended index) of the covering elements
    int ox[3], ax[3], nxc = 1, oy[3], ay[3], nyc = 1, oz[3], az[3], nzc = 1;
    ox[0] = 0; ax[0] = i + 1;
    oy[0] = 0; ay[0] = j + 1;
    oz[0] = 0; az[0] = k + 1;
    if (i == 1 && ex > 0) { ox[nxc] = -1; ax[nxc++] = N + 2; }
    if (i == N - 1 && ex < Ex - 1) { ox[nxc] = 1; ax[nxc++] = 0; }
    if (j == 1 && ey > 0) { oy[nyc] = -1; ay[nyc++] = N + 2; }
    if (j == N - 1 && ey < Ey - 1) { oy[nyc] = 1; ay[nyc++] = 0; }
    if (k == 1 && ez > 0) { oz[nzc] = -1; az[nzc++] = N + 2; }
    if (k == N - 1 && ez < Ez - 1) { oz[nzc] = 1; az[nzc++] = 0; }
    float acc = 0.f;
    for (int c = 0; c < nzc; ++c)
      for (int b = 0; b < nyc; ++b)
        for (int a = 0; a < nxc; ++a) {
          const int64_t en = (ex + ox[a]) + (int64_t)Ex * ((ey + oy[b]) + (int64_t)Ey * (ez + oz[c]));
          acc += ze[en * LE3 + ax[a] + LE * ay[b] + LE2 * az[c]];
        }
    z[l] = acc;
  }
}

// symmetric Jacobi eigen-decomposition (cyclic sweeps), n <= 16
static void jacobi_eig(int n, double* a, double* v, double* w) {
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) v[i * n + j] = (i == j);
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0;
    for (int i = 0; i < n; ++i)
      for (int j = i + 1; j < n; ++j) off += a[i * n + j] * a[i * n + j];
    if (off < 1e-30) break;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = a[p * n + q];
        if (std::fabs(apq) < 1e-300) continue;
        const double theta = (a[q * n + q] - a[p * n + p]) / (2 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1));
        const double c = 1 / std::sqrt(t * t + 1), s = t * c;
        for (int k = 0; k < n; ++k) {
          const double akp = a[k * n + p], akq = a[k * n + q];
          a[k * n + p] = c * akp - s * akq;
          a[k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          const double apk = a[p * n + k], aqk = a[q * n + k];
          a[p * n + k] = c * apk - s * aqk;
          a[q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double vkp = v[k * n + p], vkq = v[k * n + q];
          v[k * n + p] = c * vkp - s * vkq;
          v[k * n + q] = s * vkp + c * vkq;
        }
      }
  }
  for (int i = 0; i < n; ++i) w[i] = a[i * n + i];
}

}  // namespace sw

}  // namespace ntg

struct ntg_schwarz {
  ntg_plan* plan = nullptr;
  int Ex = 0, Ey = 0, Ez = 0, LE = 0;
  float* S = nullptr;    // E x 3 x LE^2 (column f = eigenvector f)
  float* lam = nullptr;  // E x 3 x LE
  float* hc = nullptr;   // E x 2 (h1, h2 element means)
  float* ze = nullptr;   // E x LE^3 extended results
  std::vector<double> hl;  // element lengths (host)
};

using namespace ntg;

// 1D extended operator for lengths (left, centre, right): the assembled
// stiffness / mass of the three intervals restricted to the nodes N-1 of the
// left element, all nodes of the centre one and node 1 of the right one.
static void fdm_1d(const ntg_plan* p, double hl, double hc, double hr, double* S, double* lam) {
  const int lx = p->lx, N = lx - 1, LE = lx + 2, ng = 3 * N + 1;
  std::vector<double> Kg(ng * ng, 0.0), Bg(ng, 0.0);
  const double hs[3] = {hl, hc, hr};
  for (int el = 0; el < 3; ++el) {
    const double h = hs[el];
    for (int a = 0; a < lx; ++a) {
      Bg[el * N + a] += 0.5 * h * p->wq[a];
      for (int b = 0; b < lx; ++b) {
        double k = 0;
        for (int q = 0; q < lx; ++q) k += p->D[q * lx + a] * p->wq[q] * p->D[q * lx + b];
        Kg[(el * N + a) * ng + (el * N + b)] += (2.0 / h) * k;
      }
    }
  }
  // extended unknowns: global 1D nodes N-1 .. 2N+1
  std::vector<double> C(LE * LE), V(LE * LE), w(LE), bi(LE);
  for (int a = 0; a < LE; ++a) bi[a] = 1.0 / std::sqrt(Bg[N - 1 + a]);
  for (int a = 0; a < LE; ++a)
    for (int b = 0; b < LE; ++b) C[a * LE + b] = bi[a] * Kg[(N - 1 + a) * ng + (N - 1 + b)] * bi[b];
  sw::jacobi_eig(LE, C.data(), V.data(), w.data());
  for (int a = 0; a < LE; ++a)
    for (int f = 0; f < LE; ++f) S[a * LE + f] = bi[a] * V[a * LE + f];
  for (int f = 0; f < LE; ++f) lam[f] = w[f];
}

static void schwarz_free(ntg_schwarz* s) {
  dev_free(s->S); dev_free(s->lam); dev_free(s->hc); dev_free(s->ze);
}

int ntg::schwarz_apply(ntg_schwarz* w, float* z, const float* r, cudaStream_t s, const Scalars* sc) {
  ntg_plan* p = w->plan;
  const int64_t nelv = p->nelv;
  int grid = (int)(nelv < (int64_t)num_sms() * 16 ? nelv : (int64_t)num_sms() * 16);
  switch (p->lx) {
    case 4:
      { sw::k_fdm<4><<<grid, 128, 0, s>>>(r, w->ze, w->S, w->lam, w->hc, w->Ex, w->Ey, w->Ez, sc); NTG_COUNT_LAUNCH(); }
      { sw::k_pull<4><<<grid_for(p->n, 256), 256, 0, s>>>(w->ze, z, w->Ex, w->Ey, w->Ez, sc); NTG_COUNT_LAUNCH(); }
      break;
    case 6:
      { sw::k_fdm<6><<<grid, 128, 0, s>>>(r, w->ze, w->S, w->lam, w->hc, w->Ex, w->Ey, w->Ez, sc); NTG_COUNT_LAUNCH(); }
      { sw::k_pull<6><<<grid_for(p->n, 256), 256, 0, s>>>(w->ze, z, w->Ex, w->Ey, w->Ez, sc); NTG_COUNT_LAUNCH(); }
      break;
    case 8:
      { sw::k_fdm<8><<<grid, 128, 0, s>>>(r, w->ze, w->S, w->lam, w->hc, w->Ex, w->Ey, w->Ez, sc); NTG_COUNT_LAUNCH(); }
      { sw::k_pull<8><<<grid_for(p->n, 256), 256, 0, s>>>(w->ze, z, w->Ex, w->Ey, w->Ez, sc); NTG_COUNT_LAUNCH(); }
      break;
    default:
      set_error("schwarz: lx=%d not compiled (4, 6, 8)", p->lx);
      return NTG_ERR_UNSUPPORTED;
  }
  NTG_CUDA_TRY(cudaGetLastError());
  NTG_TRY(gs_add_guarded_f32(p, z, s, sc));
  return mask_guarded_f32(p, z, s, sc);
}

extern "C" {

int ntg_schwarz_create(ntg_plan* p, int ex, int ey, int ez, const double* x_d, const double* y_d, const double* z_d,
                       ntg_schwarz** out) {
  clear_error();
  NTG_CHECK_ARG(p && out && x_d && y_d && z_d, "ntg_schwarz_create: null argument");
  NTG_CHECK_ARG(ex > 0 && ey > 0 && ez > 0 && (int64_t)ex * ey * ez == p->nelv,
                "ntg_schwarz_create: ex*ey*ez must equal the plan's element count (structured box, x fastest)");
  NTG_CHECK_ARG(p->lx == 4 || p->lx == 6 || p->lx == 8, "ntg_schwarz_create: lx must be 4, 6 or 8");
  *out = nullptr;
  ntg_schwarz* s = new ntg_schwarz();
  s->plan = p;
  s->Ex = ex; s->Ey = ey; s->Ez = ez;
  s->LE = p->lx + 2;
  const int LE = s->LE, LE2 = LE * LE;
  const int64_t E = p->nelv;
  int st = NTG_OK;
  double* dl = nullptr;
  do {
    if ((st = dev_alloc(&s->S, (size_t)E * 3 * LE2)) || (st = dev_alloc(&s->lam, (size_t)E * 3 * LE)) ||
        (st = dev_alloc(&s->hc, (size_t)E * 2)) || (st = dev_alloc(&s->ze, (size_t)E * LE2 * LE)) ||
        (st = dev_alloc(&dl, (size_t)E * 3)))
      break;
    { sw::k_lengths<<<grid_for(E, 128), 128, 0, p->stream>>>(x_d, y_d, z_d, E, p->lx, dl); NTG_COUNT_LAUNCH(); }
    s->hl.resize((size_t)E * 3);
    if (cudaMemcpyAsync(s->hl.data(), dl, sizeof(double) * E * 3, cudaMemcpyDeviceToHost, p->stream) != cudaSuccess ||
        cudaStreamSynchronize(p->stream) != cudaSuccess) {
      st = NTG_ERR_CUDA;
      set_error("ntg_schwarz_create: lengths");
      break;
    }
    // 1D operators per element and direction; repeated length triples reuse
    // one decomposition (lengths rounded to 6 significant digits)
    std::vector<float> hS((size_t)E * 3 * LE2), hL((size_t)E * 3 * LE);
    std::map<std::tuple<long long, long long, long long>, std::pair<std::vector<double>, std::vector<double>>> cache;
    auto key = [](double v) { return (long long)std::llround(v * 1e6 / std::pow(10.0, std::floor(std::log10(v)))) +
                                     (long long)(std::floor(std::log10(v)) + 400) * 100000000LL; };
    const int dims[3] = {ex, ey, ez};
    for (int64_t e = 0; e < E; ++e) {
      const int c[3] = {(int)(e % ex), (int)((e / ex) % ey), (int)(e / ((int64_t)ex * ey))};
      const int64_t stride[3] = {1, ex, (int64_t)ex * ey};
      for (int d = 0; d < 3; ++d) {
        const double hc = s->hl[3 * e + d];
        const double hlft = c[d] > 0 ? s->hl[3 * (e - stride[d]) + d] : hc;
        const double hrgt = c[d] < dims[d] - 1 ? s->hl[3 * (e + stride[d]) + d] : hc;
        auto kk = std::make_tuple(key(hlft), key(hc), key(hrgt));
        auto it = cache.find(kk);
        if (it == cache.end()) {
          std::vector<double> Sv(LE2), Lv(LE);
          fdm_1d(p, hlft, hc, hrgt, Sv.data(), Lv.data());
          it = cache.emplace(kk, std::make_pair(Sv, Lv)).first;
        }
        for (int q = 0; q < LE2; ++q) hS[(size_t)e * 3 * LE2 + d * LE2 + q] = (float)it->second.first[q];
        for (int q = 0; q < LE; ++q) hL[(size_t)e * 3 * LE + d * LE + q] = (float)it->second.second[q];
      }
    }
    if (cudaMemcpy(s->S, hS.data(), sizeof(float) * hS.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(s->lam, hL.data(), sizeof(float) * hL.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
      st = NTG_ERR_CUDA;
      set_error("ntg_schwarz_create: upload");
      break;
    }
    st = ntg_schwarz_update(s);
  } while (0);
  dev_free(dl);
  if (st) {
    schwarz_free(s);
    delete s;
    return st;
  }
  *out = s;
  return NTG_OK;
}

// refresh the element means of h1 / h2 after ntg_coef_set
int ntg_schwarz_update(ntg_schwarz* s) {
  clear_error();
  NTG_CHECK_ARG(s, "ntg_schwarz_update: null argument");
  ntg_plan* p = s->plan;
  const int lx3 = p->lx * p->lx * p->lx;
  { sw::k_coef_means<<<grid_for(p->nelv, 128), 128, 0, p->stream>>>(p->h1_const ? nullptr : p->h1, p->h1c, p->ifh2 ? p->hB : nullptr, p->B, p->nelv, lx3, s->hc); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

int ntg_schwarz_destroy(ntg_schwarz* s) {
  clear_error();
  if (!s) return NTG_OK;
  cudaStreamSynchronize(s->plan->stream);
  schwarz_free(s);
  delete s;
  return NTG_OK;
}

// z = M r (FP32, assembled and masked), for tests and external Krylov methods
int ntg_schwarz_apply(ntg_schwarz* s, float* z_d, const float* r_d) {
  clear_error();
  NTG_CHECK_ARG(s && z_d && r_d, "ntg_schwarz_apply: null argument");
  NTG_TRY(ensure_fp32(s->plan));
  return schwarz_apply(s, z_d, r_d, s->plan->stream, nullptr);
}

}  // extern "C"
