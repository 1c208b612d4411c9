// Plan (mesh + coef_t + gs_t) construction: GLL basis, synthetic box mesh,
// geometric factors, gather-scatter maps, coefficients and masks.
//
// The reference builds these inside Neko (coef_t init and gs_t init at
// sources/adjoint/adjoint_scheme.f90:341-343; dofmap global ids).  Here
// every array is built on the device from coordinates and global ids.
#include <cub/cub.cuh>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <atomic>
#include <mutex>

#include <vector>

#include "common.cuh"

namespace ntg {

static thread_local std::string g_err;

void set_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
}
void clear_error() { g_err.clear(); }
const char* last_error() { return g_err.c_str(); }

static std::atomic<unsigned long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

// Device timers: one open (start) event per id; stopped pairs wait in a
// list until ntg_timer_read resolves them.
struct TimerState {
  bool enabled = false;
  cudaEvent_t open[TM_COUNT] = {};
  struct Pair { int id; cudaEvent_t a, b; };
  std::vector<Pair> pending;
  std::vector<cudaEvent_t> pool;
  double total_ms[TM_COUNT] = {};
  long long count[TM_COUNT] = {};
  std::mutex mu;
  cudaEvent_t get() {
    if (!pool.empty()) { cudaEvent_t e = pool.back(); pool.pop_back(); return e; }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
  }
};
static TimerState g_tm;

void timer_start(int id, cudaStream_t s) {
  if (!g_tm.enabled || id < 0 || id >= TM_COUNT) return;
  std::lock_guard<std::mutex> lk(g_tm.mu);
  if (!g_tm.open[id]) g_tm.open[id] = g_tm.get();
  cudaEventRecord(g_tm.open[id], s);
}
void timer_stop(int id, cudaStream_t s) {
  if (!g_tm.enabled || id < 0 || id >= TM_COUNT) return;
  std::lock_guard<std::mutex> lk(g_tm.mu);
  if (!g_tm.open[id]) return;
  cudaEvent_t b = g_tm.get();
  cudaEventRecord(b, s);
  g_tm.pending.push_back({id, g_tm.open[id], b});
  g_tm.open[id] = nullptr;
}
static void timer_resolve() {
  for (auto& p : g_tm.pending) {
    float ms = 0.f;
    cudaEventSynchronize(p.b);
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      g_tm.total_ms[p.id] += ms;
      g_tm.count[p.id] += 1;
    }
    g_tm.pool.push_back(p.a);
    g_tm.pool.push_back(p.b);
  }
  g_tm.pending.clear();
}

// SM count of the current device, looked up once per device ordinal.
int num_sms() {
  static std::atomic<int> cache[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) dev = 0;
  if (dev >= 64) {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 152;
    return sms;
  }
  int sms = cache[dev].load(std::memory_order_relaxed);
  if (sms <= 0) {
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 152;
    cache[dev].store(sms, std::memory_order_relaxed);
  }
  return sms;
}

// Grid for a grid-stride loop over `work` items: 16 blocks per SM at most,
// and never more than kRedSlots blocks, since the reducing kernels write one
// partial per block into kRedSlots slots per lane.
int grid_for(int64_t work, int threads) {
  int64_t g = (work + threads - 1) / threads;
  int64_t cap = (int64_t)num_sms() * 16;
  if (cap > kRedSlots) cap = kRedSlots;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

// GLL nodes and weights of order N = lx-1 (Newton on (1-x^2)P_N'(x) from
// Chebyshev-Gauss-Lobatto starting points), and the derivative matrix
// D[i*lx+j] = phi_j'(xi_i).
static void legendre(int N, double x, double* pN, double* pNm1) {
  double p0 = 1.0, p1 = x;
  for (int k = 2; k <= N; ++k) {
    double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
    p0 = p1;
    p1 = p2;
  }
  *pN = (N == 0) ? 1.0 : p1;
  *pNm1 = (N == 0) ? 0.0 : p0;
}

void gll_basis(int lx, double* xi, double* w, double* D) {
  const int N = lx - 1;
  for (int j = 0; j <= N; ++j) {
    double x = -std::cos(M_PI * j / N);
    for (int it = 0; it < 100; ++it) {
      double pN, pNm1;
      legendre(N, x, &pN, &pNm1);
      double dx = (x * pN - pNm1) / ((N + 1) * pN);
      x -= dx;
      if (std::fabs(dx) < 1e-17) break;
    }
    xi[j] = x;
  }
  xi[0] = -1.0;
  xi[N] = 1.0;
  for (int j = 0; j < lx / 2; ++j) {
    double a = 0.5 * (xi[N - j] - xi[j]);
    xi[j] = -a;
    xi[N - j] = a;
  }
  if (lx % 2 == 1) xi[N / 2] = 0.0;
  double pn[NTG_LXMAX];
  for (int j = 0; j <= N; ++j) {
    double q;
    legendre(N, xi[j], &pn[j], &q);
    w[j] = 2.0 / (N * (N + 1.0) * pn[j] * pn[j]);
  }
  for (int i = 0; i <= N; ++i)
    for (int j = 0; j <= N; ++j) {
      double v;
      if (i != j) v = pn[i] / (pn[j] * (xi[i] - xi[j]));
      else if (i == 0) v = -0.25 * N * (N + 1.0);
      else if (i == N) v = 0.25 * N * (N + 1.0);
      else v = 0.0;
      D[i * lx + j] = v;
    }
}

struct Basis {
  double D[NTG_LXMAX * NTG_LXMAX];
  double w[NTG_LXMAX];
  double t[NTG_LXMAX];  // (xi+1)/2 with exact end points
};

// ---------------------------------------------------------------------------
// SplitMix64 keyed by (seed, stream, index) -- the generator the synthetic
// inputs use.
// ---------------------------------------------------------------------------
__host__ __device__ inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
__host__ __device__ inline uint64_t rng_u64(uint64_t seed, uint64_t stream, uint64_t idx) {
  uint64_t key = mix64(seed * 0x9E3779B97F4A7C15ULL + stream * 0xD1B54A32D192ED03ULL + 0x632BE59BD9B4E019ULL);
  return mix64(key + (idx + 1) * 0x9E3779B97F4A7C15ULL);
}
__host__ __device__ inline double rng_unif(uint64_t seed, uint64_t stream, uint64_t idx) {
  return (double)(rng_u64(seed, stream, idx) >> 11) * (1.0 / 9007199254740992.0);
}

struct Deform {
  int abc[9];
  double ph[3];
  double amp, h[3], lo[3], hi[3];
};

__global__ void k_mesh_box(int Ex, int Ey, int Ez, int lx, Basis bs, Deform df, double* __restrict__ x,
                           double* __restrict__ y, double* __restrict__ z, int64_t* __restrict__ gid) {
  const int64_t lx3 = (int64_t)lx * lx * lx;
  const int64_t n = (int64_t)Ex * Ey * Ez * lx3;
  const int N = lx - 1;
  const int64_t nx = (int64_t)Ex * N + 1, ny = (int64_t)Ey * N + 1;
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < n; l += (int64_t)gridDim.x * blockDim.x) {
    int64_t e = l / lx3;
    int m = (int)(l - e * lx3);
    int i = m % lx, j = (m / lx) % lx, k = m / (lx * lx);
    int ex = (int)(e % Ex), ey = (int)((e / Ex) % Ey), ez = (int)(e / ((int64_t)Ex * Ey));
    double X = (ex + bs.t[i]) / Ex, Y = (ey + bs.t[j]) / Ey, Z = (ez + bs.t[k]) / Ez;
    double px = df.lo[0] + X * (df.hi[0] - df.lo[0]);
    double py = df.lo[1] + Y * (df.hi[1] - df.lo[1]);
    double pz = df.lo[2] + Z * (df.hi[2] - df.lo[2]);
    if (df.amp != 0.0) {
      // wavelength 16/a elements, independent of the mesh size
      const double tp = 2.0 * 3.14159265358979323846;
      double S = (ex + bs.t[i]) / 16.0, T = (ey + bs.t[j]) / 16.0, U = (ez + bs.t[k]) / 16.0;
      px += df.amp * df.h[0] * sin(tp * (df.abc[0] * S + df.abc[1] * T + df.abc[2] * U) + df.ph[0]);
      py += df.amp * df.h[1] * sin(tp * (df.abc[3] * S + df.abc[4] * T + df.abc[5] * U) + df.ph[1]);
      pz += df.amp * df.h[2] * sin(tp * (df.abc[6] * S + df.abc[7] * T + df.abc[8] * U) + df.ph[2]);
    }
    x[l] = px;
    y[l] = py;
    z[l] = pz;
    int64_t gx = (int64_t)ex * N + i, gy = (int64_t)ey * N + j, gz = (int64_t)ez * N + k;
    gid[l] = gx + nx * (gy + ny * gz);
  }
}

__global__ void k_mask_face_xmax(int Ex, int Ey, int Ez, int lx, int32_t* __restrict__ mask) {
  // entry q enumerates (element column ey,ez) x (j,k) of the face i = N of
  // element ex = Ex-1, ordered by element then by k, j (ascending local index)
  const int64_t per = (int64_t)lx * lx;
  const int64_t total = (int64_t)Ey * Ez * per;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    int64_t c = q / per;
    int r = (int)(q - c * per);
    int j = r % lx, k = r / lx;
    int64_t e = (Ex - 1) + (int64_t)Ex * c;
    int64_t l = (lx - 1) + lx * (j + lx * (k + (int64_t)lx * e));
    mask[q] = (int32_t)(l + 1);
  }
}

// Geometric factors, one thread per node.
__global__ void k_geom(int64_t nelv, int lx, Basis bs, const double* __restrict__ x, const double* __restrict__ y,
                       const double* __restrict__ z, double* __restrict__ g11, double* __restrict__ g12,
                       double* __restrict__ g13, double* __restrict__ g22, double* __restrict__ g23,
                       double* __restrict__ g33, double* __restrict__ B) {
  const int64_t lx3 = (int64_t)lx * lx * lx;
  const int64_t n = nelv * lx3;
  for (int64_t gm = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; gm < n; gm += (int64_t)gridDim.x * blockDim.x) {
    int64_t e = gm / lx3;
    int m = (int)(gm - e * lx3);
    int i = m % lx, j = (m / lx) % lx, k = m / (lx * lx);
    const double* xe = x + e * lx3;
    const double* ye = y + e * lx3;
    const double* ze = z + e * lx3;
    double xr = 0, xs = 0, xt = 0, yr = 0, ys = 0, yt = 0, zr = 0, zs = 0, zt = 0;
    for (int l = 0; l < lx; ++l) {
      int ir = l + lx * (j + lx * k), is = i + lx * (l + lx * k), it = i + lx * (j + lx * l);
      double dr = bs.D[i * lx + l], ds = bs.D[j * lx + l], dt = bs.D[k * lx + l];
      xr += dr * xe[ir]; yr += dr * ye[ir]; zr += dr * ze[ir];
      xs += ds * xe[is]; ys += ds * ye[is]; zs += ds * ze[is];
      xt += dt * xe[it]; yt += dt * ye[it]; zt += dt * ze[it];
    }
    double J = xr * (ys * zt - yt * zs) - xs * (yr * zt - yt * zr) + xt * (yr * zs - ys * zr);
    double iJ = 1.0 / J;
    double rx = (ys * zt - yt * zs) * iJ, ry = (xt * zs - xs * zt) * iJ, rz = (xs * yt - xt * ys) * iJ;
    double sx = (yt * zr - yr * zt) * iJ, sy = (xr * zt - xt * zr) * iJ, sz = (xt * yr - xr * yt) * iJ;
    double tx = (yr * zs - ys * zr) * iJ, ty = (xs * zr - xr * zs) * iJ, tz = (xr * ys - xs * yr) * iJ;
    double wJ = bs.w[i] * bs.w[j] * bs.w[k] * J;
    g11[gm] = wJ * (rx * rx + ry * ry + rz * rz);
    g12[gm] = wJ * (rx * sx + ry * sy + rz * sz);
    g13[gm] = wJ * (rx * tx + ry * ty + rz * tz);
    g22[gm] = wJ * (sx * sx + sy * sy + sz * sz);
    g23[gm] = wJ * (sx * tx + sy * ty + sz * tz);
    g33[gm] = wJ * (tx * tx + ty * ty + tz * tz);
    B[gm] = wJ;
  }
}

__global__ void k_iota(int32_t* __restrict__ v, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    v[i] = (int32_t)i;
}
__global__ void k_iota64(int64_t* __restrict__ v, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    v[i] = i;
}
__global__ void k_head_flags(const int64_t* __restrict__ key, int64_t n, uint8_t* __restrict__ flag) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x)
    flag[p] = (p == 0 || key[p] != key[p - 1]) ? 1 : 0;
}
// per segment: count, multiplicity and shared flag
__global__ void k_seg_info(const int64_t* __restrict__ offs, int64_t nu, const int32_t* __restrict__ perm,
                           double* __restrict__ mult, int32_t* __restrict__ cnt, uint8_t* __restrict__ shflag) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < nu; s += (int64_t)gridDim.x * blockDim.x) {
    int64_t a = offs[s], b = offs[s + 1];
    double m = 1.0 / (double)(b - a);
    for (int64_t p = a; p < b; ++p) mult[perm[p]] = m;
    cnt[s] = (int32_t)(b - a);
    shflag[s] = (b - a) > 1;
  }
}
__global__ void k_fill_shared(const int64_t* __restrict__ sh_start, const int32_t* __restrict__ sh_off,
                              int64_t nsh, const int32_t* __restrict__ perm, int32_t* __restrict__ sh_idx) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nsh; t += (int64_t)gridDim.x * blockDim.x) {
    int64_t a = sh_start[t];
    int c = sh_off[t + 1] - sh_off[t];
    for (int q = 0; q < c; ++q) sh_idx[sh_off[t] + q] = perm[a + q];
  }
}
__global__ void k_d2f(const double* __restrict__ a, float* __restrict__ b, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}
__global__ void k_mul(const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ c,
                      double bc, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    c[i] = (a ? a[i] : bc) * b[i];
}
__global__ void k_copy_mask(const int32_t* __restrict__ in, int32_t* __restrict__ out, int64_t m, int base,
                            int64_t n, int* __restrict__ bad) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t v = (int64_t)in[i] - base;
    if (v < 0 || v >= n) {
      *bad = 1;
      v = 0;
    }
    out[i] = (int32_t)v;
  }
}

static Basis make_basis(int lx) {
  Basis b;
  double xi[NTG_LXMAX];
  gll_basis(lx, xi, b.w, b.D);
  for (int i = 0; i < lx; ++i) b.t[i] = 0.5 * (xi[i] + 1.0);
  b.t[0] = 0.0;
  b.t[lx - 1] = 1.0;
  return b;
}

// the Dirichlet mask as one bit per node, a byte per row of lx <= 8 nodes
// (rows x fastest, n / lx bytes), for kernels that assemble and mask a row
// in one pass; built on the host from the mask list
int ensure_maskrow(ntg_plan* p) {
  if (p->maskrow) return NTG_OK;
  if (p->lx > 8) {
    set_error("mask rows: lx=%d above 8", p->lx);
    return NTG_ERR_UNSUPPORTED;
  }
  const int64_t rows = p->n / p->lx;
  std::vector<uint8_t> bits((size_t)rows, 0);
  if (p->nmask > 0) {
    std::vector<int32_t> mk((size_t)p->nmask);
    NTG_CUDA_TRY(cudaMemcpyAsync(mk.data(), p->mask, sizeof(int32_t) * mk.size(), cudaMemcpyDeviceToHost, p->stream));
    NTG_CUDA_TRY(cudaStreamSynchronize(p->stream));
    for (int32_t l : mk) bits[l / p->lx] |= (uint8_t)(1u << (l % p->lx));
  }
  NTG_TRY(dev_alloc(&p->maskrow, (size_t)rows));
  NTG_CUDA_TRY(cudaMemcpy(p->maskrow, bits.data(), (size_t)rows, cudaMemcpyHostToDevice));
  return NTG_OK;
}

int ensure_fp32(ntg_plan* p) {
  if (p->gf[0]) return NTG_OK;
  const int T = 256;
  int G = grid_for(p->n, T);
  for (int a = 0; a < 6; ++a) {
    NTG_TRY(dev_alloc(&p->gf[a], p->n));
    { k_d2f<<<G, T, 0, p->stream>>>(p->g[a], p->gf[a], p->n); NTG_COUNT_LAUNCH(); }
  }
  NTG_TRY(dev_alloc(&p->multf, p->n));
  { k_d2f<<<G, T, 0, p->stream>>>(p->mult, p->multf, p->n); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

static void plan_free(ntg_plan* p) {
  for (int a = 0; a < 6; ++a) {
    dev_free(p->g[a]);
    dev_free(p->gf[a]);
  }
  dev_free(p->B); dev_free(p->mult); dev_free(p->multf);
  dev_free(p->perm); dev_free(p->offs); dev_free(p->sh_idx); dev_free(p->sh_off);
  dev_free(p->h1); dev_free(p->h1f); dev_free(p->hB); dev_free(p->hBf);
  dev_free(p->mask); dev_free(p->maskrow); dev_free(p->dinv); dev_free(p->dinvf);
  dev_free(p->red_part); dev_free(p->scal); dev_free(p->dev_err);
  dev_free(p->gs2); dev_free(p->gs4); dev_free(p->gs8); dev_free(p->gsx_idx); dev_free(p->gsx_off);
  dev_free(p->met); dev_free(p->binv); dev_free(p->dscr);
  if (p->host_red) cudaFreeHost(p->host_red);
  p->host_red = nullptr;
}

static int build_gs(ntg_plan* p, const int64_t* glb) {
  const int64_t n = p->n;
  const int T = 256;
  const int G = grid_for(n, T);
  cudaStream_t s = p->stream;
  int st = NTG_OK;
  int64_t *keys_sorted = nullptr, *pos = nullptr, *offs_tmp = nullptr, *sh_start = nullptr, *d_num = nullptr;
  int32_t *vals = nullptr, *cnt = nullptr, *sh_cnt = nullptr;
  uint8_t *flag = nullptr, *shflag = nullptr;
  void* tmp = nullptr;
  size_t tmp_bytes = 0, need = 0;
  int64_t nu = 0, nsh = 0;
  // key range for the radix sort
  int64_t gmax = 0;
  {
    int64_t* d_max = nullptr;
    if ((st = dev_alloc(&d_max, 1))) return st;
    size_t tb = 0;
    cub::DeviceReduce::Max(nullptr, tb, glb, d_max, n, s);
    void* t2 = nullptr;
    if (cudaMalloc(&t2, tb) != cudaSuccess) { dev_free(d_max); set_error("alloc"); return NTG_ERR_ALLOC; }
    cub::DeviceReduce::Max(t2, tb, glb, d_max, n, s);
    cudaMemcpyAsync(&gmax, d_max, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    cudaFree(t2);
    dev_free(d_max);
  }
  int end_bit = 1;
  while (end_bit < 63 && (int64_t(1) << end_bit) <= gmax) ++end_bit;

#define GS_ALLOC(ptr, cnt_)                      \
  if ((st = dev_alloc(&ptr, (size_t)(cnt_)))) goto done;
  GS_ALLOC(keys_sorted, n);
  GS_ALLOC(vals, n);
  GS_ALLOC(p->perm, n);
  GS_ALLOC(flag, n);
  GS_ALLOC(pos, n);
  GS_ALLOC(offs_tmp, n + 1);
  GS_ALLOC(d_num, 1);
  { k_iota<<<G, T, 0, s>>>(vals, n); NTG_COUNT_LAUNCH(); }
  { k_iota64<<<G, T, 0, s>>>(pos, n); NTG_COUNT_LAUNCH(); }
  // stable radix sort of (global id, local index)
  cub::DeviceRadixSort::SortPairs(nullptr, need, glb, keys_sorted, vals, p->perm, n, 0, end_bit, s);
  tmp_bytes = need;
  cub::DeviceSelect::Flagged(nullptr, need, pos, flag, offs_tmp, d_num, n, s);
  if (need > tmp_bytes) tmp_bytes = need;
  if (cudaMalloc(&tmp, tmp_bytes) != cudaSuccess) { st = NTG_ERR_ALLOC; set_error("gs tmp alloc"); goto done; }
  cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, glb, keys_sorted, vals, p->perm, n, 0, end_bit, s);
  { k_head_flags<<<G, T, 0, s>>>(keys_sorted, n, flag); NTG_COUNT_LAUNCH(); }
  cub::DeviceSelect::Flagged(tmp, tmp_bytes, pos, flag, offs_tmp, d_num, n, s);
  if (cudaMemcpyAsync(&nu, d_num, sizeof(int64_t), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess) {
    st = NTG_ERR_CUDA; set_error("gs build: %s", cudaGetErrorString(cudaGetLastError())); goto done;
  }
  p->nu = nu;
  GS_ALLOC(p->offs, nu + 1);
  cudaMemcpyAsync(p->offs, offs_tmp, sizeof(int64_t) * nu, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(p->offs + nu, &p->n, sizeof(int64_t), cudaMemcpyHostToDevice, s);
  GS_ALLOC(p->mult, n);
  GS_ALLOC(cnt, nu);
  GS_ALLOC(shflag, nu);
  { k_seg_info<<<grid_for(nu, T), T, 0, s>>>(p->offs, nu, p->perm, p->mult, cnt, shflag); NTG_COUNT_LAUNCH(); }
  // shared segments: starts and counts
  GS_ALLOC(sh_start, nu);
  GS_ALLOC(sh_cnt, nu + 1);
  {
    size_t n1 = 0, n2 = 0, n3 = 0;
    cub::DeviceSelect::Flagged(nullptr, n1, p->offs, shflag, sh_start, d_num, nu, s);
    cub::DeviceSelect::Flagged(nullptr, n2, cnt, shflag, sh_cnt, d_num, nu, s);
    cub::DeviceScan::ExclusiveSum(nullptr, n3, sh_cnt, sh_cnt, nu + 1, s);
    size_t mx = n1 > n2 ? n1 : n2;
    if (n3 > mx) mx = n3;
    if (mx > tmp_bytes) {
      cudaFree(tmp);
      tmp = nullptr;
      tmp_bytes = mx;
      if (cudaMalloc(&tmp, tmp_bytes) != cudaSuccess) { st = NTG_ERR_ALLOC; set_error("gs tmp alloc"); goto done; }
    }
    cub::DeviceSelect::Flagged(tmp, tmp_bytes, p->offs, shflag, sh_start, d_num, nu, s);
    cub::DeviceSelect::Flagged(tmp, tmp_bytes, cnt, shflag, sh_cnt, d_num, nu, s);
    if (cudaMemcpyAsync(&nsh, d_num, sizeof(int64_t), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
      st = NTG_ERR_CUDA; set_error("gs build (shared)"); goto done;
    }
    p->nshared = nsh;
    // sh_cnt[nsh] = 0 so the exclusive scan yields the total at [nsh]
    cudaMemsetAsync(sh_cnt + nsh, 0, sizeof(int32_t), s);
    cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, sh_cnt, sh_cnt, nsh + 1, s);
    int32_t total = 0;
    cudaMemcpyAsync(&total, sh_cnt + nsh, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    p->nshared_idx = total;
    GS_ALLOC(p->sh_off, nsh + 1);
    cudaMemcpyAsync(p->sh_off, sh_cnt, sizeof(int32_t) * (nsh + 1), cudaMemcpyDeviceToDevice, s);
    GS_ALLOC(p->sh_idx, total > 0 ? total : 1);
    if (nsh > 0) { k_fill_shared<<<grid_for(nsh, T), T, 0, s>>>(sh_start, p->sh_off, nsh, p->perm, p->sh_idx); NTG_COUNT_LAUNCH(); }
  }
  if (cudaStreamSynchronize(s) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
    st = NTG_ERR_CUDA;
    set_error("gs build kernels failed");
  }
#undef GS_ALLOC
done:
  if (tmp) cudaFree(tmp);
  dev_free(keys_sorted); dev_free(vals); dev_free(flag); dev_free(pos); dev_free(offs_tmp);
  dev_free(d_num); dev_free(cnt); dev_free(shflag); dev_free(sh_start); dev_free(sh_cnt);
  return st;
}

}  // namespace ntg

using namespace ntg;

extern "C" {

const char* ntg_version(void) { return "ntgb300 0.1 (sm_103a)"; }
const char* ntg_last_error(void) { return ntg::last_error(); }

unsigned long long ntg_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

int ntg_timer_enable(int on) {
  std::lock_guard<std::mutex> lk(g_tm.mu);
  g_tm.enabled = on != 0;
  return NTG_OK;
}

int ntg_timer_read(int id, double* total_ms, long long* count) {
  clear_error();
  NTG_CHECK_ARG(id >= 0 && id < TM_COUNT && total_ms && count, "ntg_timer_read: bad argument");
  std::lock_guard<std::mutex> lk(g_tm.mu);
  timer_resolve();
  *total_ms = g_tm.total_ms[id];
  *count = g_tm.count[id];
  return NTG_OK;
}

int ntg_timer_reset(void) {
  std::lock_guard<std::mutex> lk(g_tm.mu);
  timer_resolve();
  for (int i = 0; i < TM_COUNT; ++i) {
    g_tm.total_ms[i] = 0.0;
    g_tm.count[i] = 0;
  }
  return NTG_OK;
}

int ntg_supported_lx(int* lx, int cap) {
  static const int L[] = {2, 3, 4, 5, 6, 7, 8, 9, 10};
  int c = 0;
  for (int v : L) {
    if (lx && c < cap) lx[c] = v;
    ++c;
  }
  return c;
}

int ntg_mesh_box(int ex, int ey, int ez, int lx, const double* lo3, const double* hi3, double amp, uint64_t seed,
                 double* x_d, double* y_d, double* z_d, int64_t* glb_d, void* stream) {
  clear_error();
  NTG_CHECK_ARG(ex > 0 && ey > 0 && ez > 0, "ntg_mesh_box: element counts must be positive");
  NTG_CHECK_ARG(lx >= 2 && lx <= NTG_LXMAX, "ntg_mesh_box: lx out of range");
  NTG_CHECK_ARG(x_d && y_d && z_d && glb_d && lo3 && hi3, "ntg_mesh_box: null pointer");
  Basis bs = make_basis(lx);
  Deform df;
  for (int d = 0; d < 3; ++d) {
    for (int q = 0; q < 3; ++q) df.abc[3 * d + q] = 1 + (int)(rng_u64(seed, 1, 4 * d + q) % 3ULL);
    df.ph[d] = 2.0 * M_PI * rng_unif(seed, 1, 4 * d + 3);
    df.lo[d] = lo3[d];
    df.hi[d] = hi3[d];
  }
  df.h[0] = (hi3[0] - lo3[0]) / ex;
  df.h[1] = (hi3[1] - lo3[1]) / ey;
  df.h[2] = (hi3[2] - lo3[2]) / ez;
  df.amp = amp;
  int64_t n = (int64_t)ex * ey * ez * lx * lx * lx;
  { k_mesh_box<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(ex, ey, ez, lx, bs, df, x_d, y_d, z_d, glb_d); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

int ntg_mask_face_xmax(int ex, int ey, int ez, int lx, int32_t* mask_d, int64_t* nmask, void* stream) {
  clear_error();
  NTG_CHECK_ARG(ex > 0 && ey > 0 && ez > 0 && lx >= 2 && nmask, "ntg_mask_face_xmax: bad arguments");
  int64_t total = (int64_t)ey * ez * lx * lx;
  *nmask = total;
  if (mask_d) {
    { k_mask_face_xmax<<<grid_for(total, 256), 256, 0, (cudaStream_t)stream>>>(ex, ey, ez, lx, mask_d); NTG_COUNT_LAUNCH(); }
    NTG_CUDA_TRY(cudaGetLastError());
  }
  return NTG_OK;
}

int ntg_plan_create(ntg_plan** plan, int64_t nelv, int lx, const double* x_d, const double* y_d, const double* z_d,
                    const int64_t* glb_d) {
  clear_error();
  NTG_CHECK_ARG(plan, "ntg_plan_create: null plan pointer");
  *plan = nullptr;
  NTG_CHECK_ARG(nelv > 0, "ntg_plan_create: nelv must be positive");
  NTG_CHECK_ARG(lx >= 2 && lx <= 10, "ntg_plan_create: lx must be in [2, 10]");
  NTG_CHECK_ARG(x_d && y_d && z_d && glb_d, "ntg_plan_create: null coordinate or id pointer");
  NTG_CHECK_ARG(nelv * (int64_t)lx * lx * lx < ((int64_t)1 << 31), "ntg_plan_create: n must be < 2^31");
  ntg_plan* p = new ntg_plan();
  p->lx = lx;
  p->nelv = nelv;
  p->n = nelv * (int64_t)lx * lx * lx;
  Basis bs = make_basis(lx);
  memcpy(p->D, bs.D, sizeof(double) * lx * lx);
  memcpy(p->wq, bs.w, sizeof(double) * lx);
  for (int q = 0; q < lx * lx; ++q) p->Df[q] = (float)p->D[q];
  int st = NTG_OK;
  do {
    for (int a = 0; a < 6 && !st; ++a) st = dev_alloc(&p->g[a], p->n);
    if (st) break;
    if ((st = dev_alloc(&p->B, p->n))) break;
    if ((st = dev_alloc(&p->red_part, (size_t)kRedSlots * kRedLanes))) break;
    if ((st = dev_alloc(&p->scal, 1))) break;
    if ((st = dev_alloc(&p->dev_err, 1))) break;
    if (cudaMemset(p->dev_err, 0, sizeof(int)) != cudaSuccess) { st = NTG_ERR_CUDA; break; }
    if (cudaMemset(p->scal, 0, sizeof(Scalars)) != cudaSuccess) { st = NTG_ERR_CUDA; break; }
    if (cudaMallocHost(&p->host_red, sizeof(double) * 16) != cudaSuccess) { st = NTG_ERR_ALLOC; break; }
    { k_geom<<<grid_for(p->n, 128), 128, 0, p->stream>>>(nelv, lx, bs, x_d, y_d, z_d, p->g[0], p->g[1], p->g[2],
                                                        p->g[3], p->g[4], p->g[5], p->B); NTG_COUNT_LAUNCH(); }
    if (cudaGetLastError() != cudaSuccess) { st = NTG_ERR_CUDA; set_error("k_geom launch failed"); break; }
    if ((st = build_gs(p, glb_d))) break;
    if ((st = build_gs_classes(p))) break;
  } while (0);
  if (st) {
    plan_free(p);
    delete p;
    return st;
  }
  *plan = p;
  return NTG_OK;
}

int ntg_plan_destroy(ntg_plan* plan) {
  clear_error();
  if (!plan) return NTG_OK;
  cudaStreamSynchronize(plan->stream);
  plan_free(plan);
  delete plan;
  return NTG_OK;
}

int ntg_plan_set_stream(ntg_plan* plan, void* stream) {
  clear_error();
  NTG_CHECK_ARG(plan, "ntg_plan_set_stream: null plan");
  plan->stream = (cudaStream_t)stream;
  return NTG_OK;
}

int ntg_plan_info(const ntg_plan* plan, int64_t* nelv, int* lx, int64_t* n, int64_t* nu, int64_t* nshared) {
  clear_error();
  NTG_CHECK_ARG(plan, "ntg_plan_info: null plan");
  if (nelv) *nelv = plan->nelv;
  if (lx) *lx = plan->lx;
  if (n) *n = plan->n;
  if (nu) *nu = plan->nu;
  if (nshared) *nshared = plan->nshared;
  return NTG_OK;
}

int ntg_coef_get(const ntg_plan* p, double* g11_d, double* g12_d, double* g13_d, double* g22_d, double* g23_d,
                 double* g33_d, double* B_d, double* mult_d) {
  clear_error();
  NTG_CHECK_ARG(p, "ntg_coef_get: null plan");
  double* outs[8] = {g11_d, g12_d, g13_d, g22_d, g23_d, g33_d, B_d, mult_d};
  const double* ins[8] = {p->g[0], p->g[1], p->g[2], p->g[3], p->g[4], p->g[5], p->B, p->mult};
  for (int a = 0; a < 8; ++a)
    if (outs[a]) NTG_CUDA_TRY(cudaMemcpyAsync(outs[a], ins[a], sizeof(double) * p->n, cudaMemcpyDeviceToDevice, p->stream));
  return NTG_OK;
}

int ntg_gs_export(const ntg_plan* p, int32_t* perm_d, int64_t* offs_d) {
  clear_error();
  NTG_CHECK_ARG(p, "ntg_gs_export: null plan");
  if (perm_d) NTG_CUDA_TRY(cudaMemcpyAsync(perm_d, p->perm, sizeof(int32_t) * p->n, cudaMemcpyDeviceToDevice, p->stream));
  if (offs_d) NTG_CUDA_TRY(cudaMemcpyAsync(offs_d, p->offs, sizeof(int64_t) * (p->nu + 1), cudaMemcpyDeviceToDevice, p->stream));
  return NTG_OK;
}

int ntg_coef_set(ntg_plan* p, const double* h1_d, double h1c, const double* h2_d, double h2c, int ifh2) {
  clear_error();
  NTG_CHECK_ARG(p, "ntg_coef_set: null plan");
  const int T = 256;
  const int G = grid_for(p->n, T);
  if (h1_d) {
    if (!p->h1) NTG_TRY(dev_alloc(&p->h1, p->n));
    if (!p->h1f) NTG_TRY(dev_alloc(&p->h1f, p->n));
    NTG_CUDA_TRY(cudaMemcpyAsync(p->h1, h1_d, sizeof(double) * p->n, cudaMemcpyDeviceToDevice, p->stream));
    { k_d2f<<<G, T, 0, p->stream>>>(p->h1, p->h1f, p->n); NTG_COUNT_LAUNCH(); }
    p->h1_const = 0;
  } else {
    p->h1_const = 1;
    p->h1c = h1c;
  }
  p->ifh2 = ifh2 ? 1 : 0;
  if (p->ifh2) {
    if (!p->hB) NTG_TRY(dev_alloc(&p->hB, p->n));
    if (!p->hBf) NTG_TRY(dev_alloc(&p->hBf, p->n));
    { k_mul<<<G, T, 0, p->stream>>>(h2_d, p->B, p->hB, h2c, p->n); NTG_COUNT_LAUNCH(); }
    { k_d2f<<<G, T, 0, p->stream>>>(p->hB, p->hBf, p->n); NTG_COUNT_LAUNCH(); }
  }
  p->jacobi_ready = 0;
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

int ntg_plan_set_mask(ntg_plan* p, const int32_t* mask_d, int64_t nmask, int base) {
  clear_error();
  NTG_CHECK_ARG(p, "ntg_plan_set_mask: null plan");
  NTG_CHECK_ARG(nmask >= 0 && (nmask == 0 || mask_d), "ntg_plan_set_mask: bad mask");
  dev_free(p->mask);
  dev_free(p->maskrow);
  p->maskrow = nullptr;
  p->nmask = 0;
  p->jacobi_ready = 0;
  if (nmask == 0) return NTG_OK;
  NTG_TRY(dev_alloc(&p->mask, nmask));
  int* bad = nullptr;
  NTG_TRY(dev_alloc(&bad, 1));
  cudaMemsetAsync(bad, 0, sizeof(int), p->stream);
  { k_copy_mask<<<grid_for(nmask, 256), 256, 0, p->stream>>>(mask_d, p->mask, nmask, base, p->n, bad); NTG_COUNT_LAUNCH(); }
  int hbad = 0;
  cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, p->stream);
  cudaError_t e = cudaStreamSynchronize(p->stream);
  dev_free(bad);
  if (e != cudaSuccess) {
    set_error("ntg_plan_set_mask: %s", cudaGetErrorString(e));
    return NTG_ERR_CUDA;
  }
  if (hbad) {
    dev_free(p->mask);
    set_error("ntg_plan_set_mask: mask entry out of range for base %d", base);
    return NTG_ERR_INVALID;
  }
  p->nmask = nmask;
  return NTG_OK;
}

}  // extern "C"
