// Pointwise coefficient kernels of neko-top on sm_103a: the masked vector
// ops of sources/neko_ext/math (same extern "C" names and argument
// conventions as the reference's math_ext.cu:49-108), the RAMP mapping,
// the Brinkman source term, the permeability build and the FP64
// minimum-dissipation sensitivity.
//
// All are HBM-bound streams: grid-stride loops over a grid sized to a
// multiple of the SM count, 64-bit indices, no atomics.
#include <cmath>

#include <mutex>

#include "common.cuh"
#include "reduce.cuh"

namespace ntg {

static cudaStream_t g_glb_queue = 0;  // Neko's glb_cmd_queue

#define GRID_LOOP(i, n) \
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

// masks are 1-based, as in math_ext_kernel.h:41-114 of the reference
__global__ void k_cadd_mask(double* __restrict__ a, double c, const int* __restrict__ mask, int m) {
  GRID_LOOP(i, m) { a[mask[i] - 1] += c; }
}
__global__ void k_invcol1_mask(double* __restrict__ a, const int* __restrict__ mask, int m) {
  GRID_LOOP(i, m) { a[mask[i] - 1] = 1.0 / a[mask[i] - 1]; }
}
__global__ void k_cmult_mask(double* __restrict__ a, double c, const int* __restrict__ mask, int m) {
  GRID_LOOP(i, m) { a[mask[i] - 1] = c * a[mask[i] - 1]; }
}
__global__ void k_col2_mask(double* __restrict__ a, const double* __restrict__ b, const int* __restrict__ mask, int m) {
  GRID_LOOP(i, m) { a[mask[i] - 1] *= b[mask[i] - 1]; }
}
__global__ void k_col3_mask(double* __restrict__ a, const double* __restrict__ b, const double* __restrict__ c,
                            const int* __restrict__ mask, int m) {
  GRID_LOOP(i, m) { a[mask[i] - 1] = b[mask[i] - 1] * c[mask[i] - 1]; }
}
__global__ void k_sub3_mask(double* __restrict__ a, const double* __restrict__ b, const double* __restrict__ c,
                            const int* __restrict__ mask, int m) {
  GRID_LOOP(i, m) { a[mask[i] - 1] = b[mask[i] - 1] - c[mask[i] - 1]; }
}
// glsc2_mask: sum over the mask of a*b (math_ext.f90:99-116 accumulates in
// extended precision; here FP64 with a deterministic two-level tree).
struct FinStore0 {
  __device__ void operator()(const double* acc, Scalars* sc) const { sc->red[0] = acc[0]; }
};
__global__ void k_glsc2_mask(const double* __restrict__ a, const double* __restrict__ b, const int* __restrict__ mask,
                             int m, double* __restrict__ part, Scalars* sc) {
  double s = 0;
  GRID_LOOP(i, m) { s += a[mask[i] - 1] * b[mask[i] - 1]; }
  double v[1] = {s};
  grid_reduce<1>(v, part, sc, FinStore0());
}

// RAMP_mapping.f90:182-196 / :227-245
__global__ void k_ramp_fwd(double* __restrict__ out, const double* __restrict__ x, int64_t n, double fmin,
                           double fmax, double q, int convex_up) {
  GRID_LOOP(i, n) {
    double v = x[i];
    out[i] = convex_up ? fmin + (fmax - fmin) * v * (1.0 + q) / (v + q)
                       : fmin + (fmax - fmin) * v / (1.0 + q * (1.0 - v));
  }
}
// RAMP_mapping.f90:203-222 / :250-267
__global__ void k_ramp_bwd(double* __restrict__ din, const double* __restrict__ dout, const double* __restrict__ x,
                           int64_t n, double fmin, double fmax, double q, int convex_up) {
  GRID_LOOP(i, n) {
    double v = x[i];
    double d;
    if (convex_up) d = (fmax - fmin) * (q + 1.0) / ((v + q) * (v + q));
    else {
      double t = 1.0 - q * (v - 1.0);
      d = (fmax - fmin) * (q + 1.0) / (t * t);
    }
    din[i] = d * dout[i];
  }
}
// simple_brinkman_source_term.f90:139-153: f -= u * chi, three components
__global__ void k_brinkman(double* __restrict__ fx, double* __restrict__ fy, double* __restrict__ fz,
                           const double* __restrict__ u, const double* __restrict__ v, const double* __restrict__ w,
                           const double* __restrict__ chi, int64_t n) {
  GRID_LOOP(i, n) {
    double c = chi[i];
    fx[i] -= u[i] * c;
    fy[i] -= v[i] * c;
    fz[i] -= w[i] * c;
  }
}
__global__ void k_brinkman_mask(double* __restrict__ fx, double* __restrict__ fy, double* __restrict__ fz,
                                const double* __restrict__ u, const double* __restrict__ v,
                                const double* __restrict__ w, const double* __restrict__ chi,
                                const int32_t* __restrict__ mask, int64_t m, int base) {
  GRID_LOOP(q, m) {
    int64_t i = (int64_t)mask[q] - base;
    double c = chi[i];
    fx[i] -= u[i] * c;
    fy[i] -= v[i] * c;
    fz[i] -= w[i] * c;
  }
}
// design.f90:327-335: kappa = -(perm1 + (perm0-perm1)(pen+1) * phi/(pen+phi))
__global__ void k_permeability(double* __restrict__ kappa, const double* __restrict__ phi, int64_t n, double c,
                               double perm1, double pen) {
  GRID_LOOP(i, n) {
    double r = 1.0 / (pen + phi[i]);
    r = r * phi[i];
    r = r * c;
    r = r + perm1;
    kappa[i] = -1.0 * r;
  }
}
// minimum_dissipation_objective_function.f90:272-296
__global__ void k_sens_md(double* __restrict__ s, const double* __restrict__ u, const double* __restrict__ v,
                          const double* __restrict__ w, const double* __restrict__ ua, const double* __restrict__ va,
                          const double* __restrict__ wa, int64_t n, int if_lube, double K) {
  GRID_LOOP(i, n) {
    double t = u[i] * ua[i];
    t += v[i] * va[i];
    t += w[i] * wa[i];
    t *= -1.0;
    if (if_lube) {
      double l = u[i] * u[i];
      l += v[i] * v[i];
      l += w[i] * w[i];
      t += K * l;
    }
    s[i] = t;
  }
}

// Scratch of the standalone masked dot (device partials + scalars + a
// pinned result slot), allocated on the first call made with each device
// current and kept per device ordinal until the process exits; a mutex
// serialises the first calls of concurrent host threads.
struct GlscScratch {
  double* part = nullptr;
  Scalars* scal = nullptr;
  double* host = nullptr;
};
static std::mutex g_glsc_mu;
static GlscScratch g_glsc[64];

static int glsc_scratch(GlscScratch** out) {
  int dev = 0;
  NTG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    set_error("cuda_glsc2_mask: device ordinal %d out of range", dev);
    return NTG_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(g_glsc_mu);
  GlscScratch& g = g_glsc[dev];
  if (!g.host) {
    GlscScratch t;
    int st = NTG_OK;
    do {
      if ((st = dev_alloc(&t.part, (size_t)kRedSlots * kRedLanes))) break;
      if ((st = dev_alloc(&t.scal, 1))) break;
      if (cudaMemset(t.scal, 0, sizeof(Scalars)) != cudaSuccess) { st = NTG_ERR_CUDA; set_error("cuda_glsc2_mask: memset"); break; }
      if (cudaMallocHost(&t.host, sizeof(double)) != cudaSuccess) { st = NTG_ERR_ALLOC; set_error("cuda_glsc2_mask: pinned slot"); t.host = nullptr; break; }
    } while (0);
    if (st) {
      dev_free(t.part);
      dev_free(t.scal);
      return st;
    }
    g = t;
  }
  *out = &g;
  return NTG_OK;
}

static int grid1(int64_t n) { return grid_for(n, 256); }

}  // namespace ntg

using namespace ntg;

extern "C" {

void ntg_set_glb_queue(void* stream) { g_glb_queue = (cudaStream_t)stream; }

static void report_launch(const char* name) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) set_error("%s: %s", name, cudaGetErrorString(e));
}

void cuda_cadd_mask(void* a, double* c, int* size, int* mask, int* mask_size) {
  clear_error();
  (void)size;
  if (*mask_size <= 0) return;
  { k_cadd_mask<<<grid1(*mask_size), 256, 0, g_glb_queue>>>((double*)a, *c, mask, *mask_size); NTG_COUNT_LAUNCH(); }
  report_launch("cuda_cadd_mask");
}
void cuda_invcol1_mask(void* a, int* size, int* mask, int* mask_size) {
  clear_error();
  (void)size;
  if (*mask_size <= 0) return;
  { k_invcol1_mask<<<grid1(*mask_size), 256, 0, g_glb_queue>>>((double*)a, mask, *mask_size); NTG_COUNT_LAUNCH(); }
  report_launch("cuda_invcol1_mask");
}
void cuda_cmult_mask(void* a, double* c, int* size, int* mask, int* mask_size) {
  clear_error();
  (void)size;
  if (*mask_size <= 0) return;
  { k_cmult_mask<<<grid1(*mask_size), 256, 0, g_glb_queue>>>((double*)a, *c, mask, *mask_size); NTG_COUNT_LAUNCH(); }
  report_launch("cuda_cmult_mask");
}
void cuda_col2_mask(void* a, void* b, int* size, int* mask, int* mask_size) {
  clear_error();
  (void)size;
  if (*mask_size <= 0) return;
  { k_col2_mask<<<grid1(*mask_size), 256, 0, g_glb_queue>>>((double*)a, (const double*)b, mask, *mask_size); NTG_COUNT_LAUNCH(); }
  report_launch("cuda_col2_mask");
}
void cuda_col3_mask(void* a, void* b, void* c, int* size, int* mask, int* mask_size) {
  clear_error();
  (void)size;
  if (*mask_size <= 0) return;
  { k_col3_mask<<<grid1(*mask_size), 256, 0, g_glb_queue>>>((double*)a, (const double*)b, (const double*)c, mask,
                                                          *mask_size); NTG_COUNT_LAUNCH(); }
  report_launch("cuda_col3_mask");
}
void cuda_sub3_mask(void* a, void* b, void* c, int* size, int* mask, int* mask_size) {
  clear_error();
  (void)size;
  if (*mask_size <= 0) return;
  { k_sub3_mask<<<grid1(*mask_size), 256, 0, g_glb_queue>>>((double*)a, (const double*)b, (const double*)c, mask,
                                                          *mask_size); NTG_COUNT_LAUNCH(); }
  report_launch("cuda_sub3_mask");
}
double cuda_glsc2_mask(void* a, void* b, int* size, int* mask, int* mask_size) {
  clear_error();
  (void)size;
  if (*mask_size <= 0) return 0.0;
  GlscScratch* g = nullptr;
  if (glsc_scratch(&g) != NTG_OK) return NAN;
  { k_glsc2_mask<<<grid1(*mask_size), 256, 0, g_glb_queue>>>((const double*)a, (const double*)b, mask, *mask_size,
                                                           g->part, g->scal); NTG_COUNT_LAUNCH(); }
  report_launch("cuda_glsc2_mask");
  cudaMemcpyAsync(g->host, &g->scal->red[0], sizeof(double), cudaMemcpyDeviceToHost, g_glb_queue);
  if (cudaStreamSynchronize(g_glb_queue) != cudaSuccess) {
    set_error("cuda_glsc2_mask: %s", cudaGetErrorString(cudaGetLastError()));
    return NAN;
  }
  return *g->host;
}

int ntg_ramp_forward(double* xout_d, const double* xin_d, int64_t n, double fmin, double fmax, double q,
                     int convex_up, void* stream) {
  clear_error();
  NTG_CHECK_ARG(xout_d && xin_d && n >= 0, "ntg_ramp_forward: bad argument");
  if (n == 0) return NTG_OK;
  { k_ramp_fwd<<<grid1(n), 256, 0, (cudaStream_t)stream>>>(xout_d, xin_d, n, fmin, fmax, q, convex_up); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

int ntg_ramp_backward(double* dF_din_d, const double* dF_dout_d, const double* xin_d, int64_t n, double fmin,
                      double fmax, double q, int convex_up, void* stream) {
  clear_error();
  NTG_CHECK_ARG(dF_din_d && dF_dout_d && xin_d && n >= 0, "ntg_ramp_backward: bad argument");
  if (n == 0) return NTG_OK;
  { k_ramp_bwd<<<grid1(n), 256, 0, (cudaStream_t)stream>>>(dF_din_d, dF_dout_d, xin_d, n, fmin, fmax, q, convex_up); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

int ntg_brinkman_compute(double* fx_d, double* fy_d, double* fz_d, const double* u_d, const double* v_d,
                         const double* w_d, const double* chi_d, int64_t n, const int32_t* mask_d, int64_t nmask,
                         int base, void* stream) {
  clear_error();
  NTG_CHECK_ARG(fx_d && fy_d && fz_d && u_d && v_d && w_d && chi_d && n >= 0, "ntg_brinkman_compute: bad argument");
  cudaStream_t s = (cudaStream_t)stream;
  if (mask_d) {
    if (nmask <= 0) return NTG_OK;
    { k_brinkman_mask<<<grid1(nmask), 256, 0, s>>>(fx_d, fy_d, fz_d, u_d, v_d, w_d, chi_d, mask_d, nmask, base); NTG_COUNT_LAUNCH(); }
  } else {
    if (n == 0) return NTG_OK;
    { k_brinkman<<<grid1(n), 256, 0, s>>>(fx_d, fy_d, fz_d, u_d, v_d, w_d, chi_d, n); NTG_COUNT_LAUNCH(); }
  }
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

int ntg_permeability(double* kappa_d, const double* phi_d, int64_t n, double perm0, double perm1, double penalty,
                     void* stream) {
  clear_error();
  NTG_CHECK_ARG(kappa_d && phi_d && n >= 0, "ntg_permeability: bad argument");
  if (n == 0) return NTG_OK;
  double c = (perm0 - perm1) * (penalty + 1.0);
  { k_permeability<<<grid1(n), 256, 0, (cudaStream_t)stream>>>(kappa_d, phi_d, n, c, perm1, penalty); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

int ntg_sens_min_dissipation(double* s_d, const double* u_d, const double* v_d, const double* w_d,
                             const double* ua_d, const double* va_d, const double* wa_d, int64_t n, int if_lube,
                             double K_scale, void* stream) {
  clear_error();
  NTG_CHECK_ARG(s_d && u_d && v_d && w_d && ua_d && va_d && wa_d && n >= 0, "ntg_sens_min_dissipation: bad argument");
  if (n == 0) return NTG_OK;
  { k_sens_md<<<grid1(n), 256, 0, (cudaStream_t)stream>>>(s_d, u_d, v_d, w_d, ua_d, va_d, wa_d, n, if_lube, K_scale); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

}  // extern "C"
