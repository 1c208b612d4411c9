// Seeded synthetic fields for the benchmark workloads (the same generators
// as the oracle's, from the same SplitMix64 counter-based stream), and the
// weak right-hand side b = mask(gs(B f)).
//
// Fields are functions of the global node id or of the node coordinates,
// so they are continuous across element faces.
#include <cmath>

#include "common.cuh"

namespace ntg {

__host__ __device__ inline uint64_t smix(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
__host__ __device__ inline uint64_t srng_u64(uint64_t seed, uint64_t stream, uint64_t idx) {
  uint64_t key = smix(seed * 0x9E3779B97F4A7C15ULL + stream * 0xD1B54A32D192ED03ULL + 0x632BE59BD9B4E019ULL);
  return smix(key + (idx + 1) * 0x9E3779B97F4A7C15ULL);
}
__host__ __device__ inline double srng_unif(uint64_t seed, uint64_t stream, uint64_t idx) {
  return (double)(srng_u64(seed, stream, idx) >> 11) * (1.0 / 9007199254740992.0);
}

constexpr int kMaxModes = 64;
constexpr int kStreamModes = 4, kStreamBlobs = 5;

struct Modes {
  int k[3 * kMaxModes];
  double a[kMaxModes], ph[kMaxModes];
  int nm;
  double lo[3], hi[3];
};
struct Blobs {
  double c[3 * kMaxModes];
  int nb;
  double inv2w2;
};

__global__ void k_uniform(const int64_t* __restrict__ gid, int64_t n, uint64_t seed, uint64_t stream, double lo,
                          double hi, double* __restrict__ f) {
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < n; l += (int64_t)gridDim.x * blockDim.x)
    f[l] = lo + (hi - lo) * srng_unif(seed, stream, (uint64_t)gid[l]);
}

__global__ void k_fourier(const double* __restrict__ x, const double* __restrict__ y, const double* __restrict__ z,
                          int64_t n, const __grid_constant__ Modes md, double* __restrict__ f) {
  const double tp = 2.0 * 3.14159265358979323846;
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < n; l += (int64_t)gridDim.x * blockDim.x) {
    double X = (x[l] - md.lo[0]) / (md.hi[0] - md.lo[0]);
    double Y = (y[l] - md.lo[1]) / (md.hi[1] - md.lo[1]);
    double Z = (z[l] - md.lo[2]) / (md.hi[2] - md.lo[2]);
    double s = 0;
    for (int m = 0; m < md.nm; ++m)
      s += md.a[m] * cos(tp * (md.k[3 * m] * X + md.k[3 * m + 1] * Y + md.k[3 * m + 2] * Z) + md.ph[m]);
    f[l] = s;
  }
}

__global__ void k_blobs(const double* __restrict__ x, const double* __restrict__ y, const double* __restrict__ z,
                        int64_t n, const __grid_constant__ Blobs bl, double* __restrict__ f) {
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < n; l += (int64_t)gridDim.x * blockDim.x) {
    double s = 0;
    for (int b = 0; b < bl.nb; ++b) {
      double dx = x[l] - bl.c[3 * b], dy = y[l] - bl.c[3 * b + 1], dz = z[l] - bl.c[3 * b + 2];
      s += exp(-(dx * dx + dy * dy + dz * dz) * bl.inv2w2);
    }
    f[l] = s < 0 ? 0 : (s > 1 ? 1 : s);
  }
}

__global__ void k_mulB2(double* __restrict__ o, const double* __restrict__ f, const double* __restrict__ B, int64_t n) {
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < n; l += (int64_t)gridDim.x * blockDim.x)
    o[l] = f[l] * B[l];
}

}  // namespace ntg

using namespace ntg;

extern "C" {

int ntg_field_uniform(const int64_t* gid_d, int64_t n, uint64_t seed, uint64_t stream_id, double lo, double hi,
                      double* f_d, void* stream) {
  clear_error();
  NTG_CHECK_ARG(gid_d && f_d && n >= 0, "ntg_field_uniform: bad argument");
  if (n == 0) return NTG_OK;
  { k_uniform<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(gid_d, n, seed, stream_id, lo, hi, f_d); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

int ntg_field_fourier(const double* x_d, const double* y_d, const double* z_d, int64_t n, const double* lo3,
                      const double* hi3, int nmodes, int kmax, uint64_t seed, double* f_d, void* stream) {
  clear_error();
  NTG_CHECK_ARG(x_d && y_d && z_d && f_d && lo3 && hi3 && n >= 0, "ntg_field_fourier: bad argument");
  NTG_CHECK_ARG(nmodes >= 1 && nmodes <= kMaxModes && kmax >= 1, "ntg_field_fourier: 1 <= nmodes <= 64");
  Modes md;
  md.nm = nmodes;
  for (int m = 0; m < nmodes; ++m) {
    double kk = 0;
    for (int d = 0; d < 3; ++d) {
      md.k[3 * m + d] = 1 + (int)(srng_u64(seed, kStreamModes, 8 * m + d) % (uint64_t)kmax);
      kk += (double)md.k[3 * m + d] * md.k[3 * m + d];
    }
    md.a[m] = (2.0 * srng_unif(seed, kStreamModes, 8 * m + 3) - 1.0) / kk;
    md.ph[m] = 2.0 * M_PI * srng_unif(seed, kStreamModes, 8 * m + 4);
  }
  for (int d = 0; d < 3; ++d) {
    md.lo[d] = lo3[d];
    md.hi[d] = hi3[d];
  }
  if (n == 0) return NTG_OK;
  { k_fourier<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(x_d, y_d, z_d, n, md, f_d); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

// Fourier modes with explicit parameters (host arrays): k (3*nmodes ints),
// amplitudes and phases; used for right-hand-side sequences whose mode
// amplitudes evolve between solves.
int ntg_field_modes(const double* x_d, const double* y_d, const double* z_d, int64_t n, const double* lo3,
                    const double* hi3, int nmodes, const int* k, const double* amp, const double* ph, double* f_d,
                    void* stream) {
  clear_error();
  NTG_CHECK_ARG(x_d && y_d && z_d && f_d && lo3 && hi3 && k && amp && ph && n >= 0, "ntg_field_modes: bad argument");
  NTG_CHECK_ARG(nmodes >= 1 && nmodes <= kMaxModes, "ntg_field_modes: 1 <= nmodes <= 64");
  Modes md;
  md.nm = nmodes;
  for (int m = 0; m < nmodes; ++m) {
    for (int d = 0; d < 3; ++d) md.k[3 * m + d] = k[3 * m + d];
    md.a[m] = amp[m];
    md.ph[m] = ph[m];
  }
  for (int d = 0; d < 3; ++d) {
    md.lo[d] = lo3[d];
    md.hi[d] = hi3[d];
  }
  if (n == 0) return NTG_OK;
  { k_fourier<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(x_d, y_d, z_d, n, md, f_d); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

int ntg_field_blobs(const double* x_d, const double* y_d, const double* z_d, int64_t n, const double* lo3,
                    const double* hi3, uint64_t seed, int nblobs, double width, double* f_d, void* stream) {
  clear_error();
  NTG_CHECK_ARG(x_d && y_d && z_d && f_d && lo3 && hi3 && n >= 0 && width > 0, "ntg_field_blobs: bad argument");
  NTG_CHECK_ARG(nblobs >= 1 && nblobs <= kMaxModes, "ntg_field_blobs: 1 <= nblobs <= 64");
  Blobs bl;
  bl.nb = nblobs;
  bl.inv2w2 = 1.0 / (2.0 * width * width);
  for (int b = 0; b < nblobs; ++b)
    for (int d = 0; d < 3; ++d) bl.c[3 * b + d] = lo3[d] + (hi3[d] - lo3[d]) * srng_unif(seed, kStreamBlobs, 4 * b + d);
  if (n == 0) return NTG_OK;
  { k_blobs<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(x_d, y_d, z_d, n, bl, f_d); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

int ntg_rhs_assemble(ntg_plan* p, const double* f_d, double* b_d) {
  clear_error();
  NTG_CHECK_ARG(p && f_d && b_d, "ntg_rhs_assemble: null argument");
  { k_mulB2<<<grid_for(p->n, 256), 256, 0, p->stream>>>(b_d, f_d, p->B, p->n); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  NTG_TRY(gs_launch(p, b_d, NTG_GS_ADD, p->stream));
  return mask_launch(p, b_d, p->stream);
}

}  // extern "C"
