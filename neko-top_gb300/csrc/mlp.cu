// Learned initial guess: a per-element MLP trained online on the solver's own
// solutions.  Forward, backward and Adam are hand-written; every GEMM runs
// on the tensor cores (tcgen05, BF16 operands, FP32 accumulation in TMEM;
// tc_gemm.cu).
//
// Insertion points in the reference: the initial guess of the pressure /
// filter solves -- projection pre_solving at sources/adjoint/adjoint_pnpn.f90:729
// and the filter's guess copy at sources/mapping_functions/PDE_filter_mapping.f90:246,332.
// The reference has no learned part; this is new.
//
// Network (per element, rows = elements, lx^3 = 512 nodes):
//   X  [E x 5*512] = the last 4 solutions / s_x and the right-hand side / s_b
//                    on the element's nodes (BF16; s = RMS values)
//   H1 = relu(X W1 + b1)   [E x 64]
//   H2 = relu(H1 W2 + b2)  [E x 64]
//   Y  = H2 W3 + b3        [E x 512]  a nodal correction: the element's guess
//                                     is x_{k-1} + s_x Y (W3 starts at zero,
//                                     so the untrained net returns the newest
//                                     solution), made continuous by the
//                                     mult-weighted gather-scatter and masked.
// Loss (online training): relative energy error (D, A D)/(x, A x) plus
// relative L2 error of the assembled guess D = g - x; the gradient flows
// back through the averaging (mult * gs).  The raw test entry points use
// the MSE of Y.
//
// GEMM layout: every operand is K-major (C = A B^T with A [M x K], B
// [N x K]).  The forward pass keeps BF16 copies of the weights transposed
// (W1T [64 x 2560], W2T, W3T [512 x 64]); the backward pass uses W2 and W3
// as stored; the weight gradients are X^T dZ1, H1^T dZ2, H2^T dY with the
// element index as K, so the forward epilogues also write H1 and H2
// transposed (element index contiguous) and X, dZ and dY get transposed
// copies.  Transposed buffers have a leading dimension rounded up to 8
// elements (16-byte rows for the TMA engine).  Weight gradients split the
// element range over CTAs and add the partials in a fixed order, so a
// training step is deterministic.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include <cuda_bf16.h>

#include "common.cuh"
#include "reduce.cuh"
#include "tc.cuh"

namespace ntg {

namespace mlp {

// X[m][f*lx3 + node] = bf16(field_f[m*lx3 + node] * scale_f), f < nhist; the
// right-hand side last
struct PrepArgs {
  const float* hist[8];
  const double* b;
  float scale[8];
  float bscale;
  int nhist;
};
__global__ void k_prep_x(PrepArgs pa, int64_t E, int lx3, __nv_bfloat16* __restrict__ X) {
  const int F = (pa.nhist + 1) * lx3;
  const int64_t total = E * F;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t m = i / F;
    const int k = (int)(i - m * F);
    const int f = k / lx3, node = k - f * lx3;
    const int64_t l = m * lx3 + node;
    float v = f < pa.nhist ? pa.hist[f][l] * pa.scale[f] : (float)(pa.b[l] * pa.bscale);
    X[i] = __float2bfloat16(v);
  }
}

// T [cols x ldt] = S^T for S [rows x cols] (BF16), 32 x 32 tiles through
// shared memory (coalesced on both sides)
__global__ void k_transpose_bf16(const __nv_bfloat16* __restrict__ S, int64_t rows, int64_t cols,
                                 __nv_bfloat16* __restrict__ T, int64_t ldt) {
  __shared__ __nv_bfloat16 tile[32][34];
  const int64_t ntc = (cols + 31) / 32, ntr = (rows + 31) / 32;
  for (int64_t t = blockIdx.x; t < ntc * ntr; t += gridDim.x) {
    const int64_t r0 = (t / ntc) * 32, c0 = (t % ntc) * 32;
    for (int q = threadIdx.y; q < 32; q += blockDim.y) {
      const int64_t r = r0 + q, c = c0 + threadIdx.x;
      tile[q][threadIdx.x] = (r < rows && c < cols) ? S[r * cols + c] : __float2bfloat16(0.f);
    }
    __syncthreads();
    for (int q = threadIdx.y; q < 32; q += blockDim.y) {
      const int64_t c = c0 + q, r = r0 + threadIdx.x;
      if (c < cols && r < rows) T[c * ldt + r] = tile[threadIdx.x][q];
    }
    __syncthreads();
  }
}

// Activation gradient of a row-major [M x N] block: dZ = dH * (Hact > 0)
// (no mask when Hact is null).  Writes any of: FP32 dZ, BF16 dZb (both
// row-major), BF16 dZT (transposed, leading dimension ldt).  A block takes
// 32 rows; the transposed write goes through shared memory.
template <int N>
__global__ void __launch_bounds__(256) k_act_back(const float* __restrict__ dH, const __nv_bfloat16* __restrict__ Hact,
                                                  int64_t M, float* __restrict__ dZ, __nv_bfloat16* __restrict__ dZb,
                                                  __nv_bfloat16* __restrict__ dZT, int64_t ldt) {
  __shared__ __nv_bfloat16 tile[32][N + 2];
  for (int64_t r0 = (int64_t)blockIdx.x * 32; r0 < M; r0 += (int64_t)gridDim.x * 32) {
    for (int q = threadIdx.x; q < 32 * N; q += blockDim.x) {
      const int rr = q / N, c = q - rr * N;
      const int64_t r = r0 + rr;
      float v = 0.f;
      if (r < M) {
        v = dH[r * N + c];
        if (Hact && !(__bfloat162float(Hact[r * N + c]) > 0.f)) v = 0.f;
        if (dZ) dZ[r * N + c] = v;
        if (dZb) dZb[r * N + c] = __float2bfloat16(v);
      }
      tile[rr][c] = __float2bfloat16(v);
    }
    __syncthreads();
    if (dZT) {
      for (int q = threadIdx.x; q < 32 * N; q += blockDim.x) {
        const int c = q / 32, rr = q - c * 32;
        const int64_t r = r0 + rr;
        if (r < M) dZT[c * ldt + r] = tile[rr][c];
      }
    }
    __syncthreads();
  }
}

// column sums of a row-major [M x N] FP32 matrix, deterministic: a block per
// 32 columns, fixed row partition, fixed tree
__global__ void k_colsum(const float* __restrict__ a, int64_t M, int N, float* __restrict__ out) {
  __shared__ float red[8][32];
  const int col = blockIdx.x * 32 + (threadIdx.x & 31);
  const int rw = threadIdx.x >> 5;
  float s = 0.f;
  if (col < N)
    for (int64_t r = rw; r < M; r += 8) s += a[r * N + col];
  red[rw][threadIdx.x & 31] = s;
  __syncthreads();
  if (rw == 0 && col < N) {
    float t = 0.f;
    for (int q = 0; q < 8; ++q) t += red[q][threadIdx.x & 31];
    out[col] = t;
  }
}

// dY = (Y - T) * g (MSE gradient), loss partials
struct FinLoss {
  __device__ void operator()(const double* acc, Scalars* sc) const { sc->red[1] = acc[0]; }
};
__global__ void k_loss_grad(const float* __restrict__ Y, const float* __restrict__ T, int64_t len, float g,
                            float* __restrict__ dY, double* __restrict__ part, Scalars* sc) {
  float s = 0.f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < len; i += (int64_t)gridDim.x * blockDim.x) {
    const float d = Y[i] - T[i];
    s += d * d;
    dY[i] = d * g;
  }
  double v[1] = {(double)s};
  grid_reduce<1>(v, part, sc, FinLoss());
}

// D = (x_{k-1} + s Y) * mult, the element-local guess before averaging
__global__ void k_head(const float* __restrict__ Y, const float* __restrict__ hnew, float s,
                       const float* __restrict__ mult, int64_t n, float* __restrict__ D) {
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < n; l += (int64_t)gridDim.x * blockDim.x)
    D[l] = (hnew[l] + s * Y[l]) * mult[l];
}
// the same in FP64 for the guess itself
__global__ void k_head64(const float* __restrict__ Y, const float* __restrict__ hnew, double s,
                         const double* __restrict__ mult, int64_t n, double* __restrict__ out) {
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < n; l += (int64_t)gridDim.x * blockDim.x)
    out[l] = ((double)hnew[l] + s * (double)Y[l]) * mult[l];
}
__global__ void k_sub_inplace(float* __restrict__ D, const float* __restrict__ T, int64_t n) {
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < n; l += (int64_t)gridDim.x * blockDim.x)
    D[l] -= T[l];
}
// AD <- ge A D + gl D, loss = sum 0.5 (ge D.AD + gl D.D) (local sums)
__global__ void k_energy_grad_field(const float* __restrict__ D, float* __restrict__ AD, int64_t n, float ge, float gl,
                                    double* __restrict__ part, Scalars* sc) {
  float s = 0.f;
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < n; l += (int64_t)gridDim.x * blockDim.x) {
    const float d = D[l], ad = AD[l];
    s += 0.5f * (ge * d * ad + gl * d * d);
    AD[l] = ge * ad + gl * d;
  }
  double v[1] = {(double)s};
  grid_reduce<1>(v, part, sc, FinLoss());
}
// dY = s * mult * gG (the gradient w.r.t. the nodal output; nodal layout =
// row-major [E x lx3])
__global__ void k_head_grad(const float* __restrict__ gG, const float* __restrict__ mult, float s, int64_t n,
                            float* __restrict__ dY) {
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < n; l += (int64_t)gridDim.x * blockDim.x)
    dY[l] = s * mult[l] * gG[l];
}

// (a, b) in FP32 per thread, FP64 across blocks -> red[3]
struct FinSlot3 {
  __device__ void operator()(const double* acc, Scalars* sc) const { sc->red[3] = acc[0]; }
};
__global__ void k_dot_f(const float* __restrict__ a, const float* __restrict__ b, int64_t n, double* __restrict__ part,
                        Scalars* sc) {
  float s = 0.f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s += a[i] * b[i];
  double v[1] = {(double)s};
  grid_reduce<1>(v, part, sc, FinSlot3());
}

// Adam (bias-corrected) on FP32 master weights
__global__ void k_adam(float* __restrict__ w, const float* __restrict__ gr, float* __restrict__ m1,
                       float* __restrict__ m2, int64_t len, float lr, float b1, float b2, float c1, float c2,
                       float eps) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < len; i += (int64_t)gridDim.x * blockDim.x) {
    const float gg = gr[i];
    const float a = b1 * m1[i] + (1.f - b1) * gg;
    const float b = b2 * m2[i] + (1.f - b2) * gg * gg;
    m1[i] = a;
    m2[i] = b;
    w[i] = w[i] - lr * (a * c1) / (sqrtf(b * c2) + eps);
  }
}

// BF16 weight copies for the GEMMs: W (as stored, [rows x cols]) and/or its
// transpose WT [cols x rows]
__global__ void k_wcopy(const float* __restrict__ W, int64_t rows, int64_t cols, __nv_bfloat16* __restrict__ Wb,
                        __nv_bfloat16* __restrict__ WT) {
  const int64_t len = rows * cols;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < len; i += (int64_t)gridDim.x * blockDim.x) {
    const __nv_bfloat16 v = __float2bfloat16(W[i]);
    if (Wb) Wb[i] = v;
    if (WT) {
      const int64_t r = i / cols, c = i - r * cols;
      WT[c * rows + r] = v;
    }
  }
}

// T = x (float); history push h = x
__global__ void k_target(const double* __restrict__ x, int64_t n, float* __restrict__ T, float* __restrict__ h) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (T) T[i] = (float)x[i];
    if (h) h[i] = (float)x[i];
  }
}
// sum of squares, deterministic -> red[2]
struct FinSlot2 {
  __device__ void operator()(const double* acc, Scalars* sc) const { sc->red[2] = acc[0]; }
};
template <typename T>
__global__ void k_sumsq(const T* __restrict__ a, int64_t n, double* __restrict__ part, Scalars* sc) {
  float s = 0.f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float v = (float)a[i];
    s += v * v;
  }
  double v[1] = {(double)s};
  grid_reduce<1>(v, part, sc, FinSlot2());
}

}  // namespace mlp

}  // namespace ntg

struct ntg_guess {
  ntg_plan* plan = nullptr;
  int nhist = 4, H = 64, F = 0, O = 0, lx3 = 0;
  int64_t E = 0, n = 0, ldt = 0;
  // parameters: flat FP32 [W1 F*H | b1 H | W2 H*H | b2 H | W3 H*O | b3 O], W row-major [in x out]
  int64_t oW1 = 0, ob1 = 0, oW2 = 0, ob2 = 0, oW3 = 0, ob3 = 0, np = 0;
  float *P = nullptr, *G = nullptr, *m1 = nullptr, *m2 = nullptr;
  // BF16 weight copies: forward (transposed) and backward (as stored)
  __nv_bfloat16 *W1T = nullptr, *W2T = nullptr, *W3T = nullptr, *W2b = nullptr, *W3b = nullptr;
  // activations (row-major [E x .]) and transposed copies ([. x ldt])
  __nv_bfloat16 *X = nullptr, *XT = nullptr, *H1b = nullptr, *H2b = nullptr, *H1T = nullptr, *H2T = nullptr;
  __nv_bfloat16 *dYb = nullptr, *dYT = nullptr, *dZb = nullptr, *dZT = nullptr;
  float *Y = nullptr, *T = nullptr, *dY = nullptr, *dH = nullptr, *dZ = nullptr, *split = nullptr;
  int64_t split_len = 0;
  float *D = nullptr, *AD = nullptr;  // energy loss: error and its element-local A image
  double tat = 1.0, tt = 1.0;         // (T, A T) and (T, T) of the current target
  int loss_mode = 1;                  // 1: relative energy + L2 (online training); 0: MSE
  float hscale = 1.f;                 // s_x of the current input (output scale)
  // history ring of solutions (FP32), newest at hist[(head - 1) mod nhist]
  float* hist[8] = {};
  double hrms[8] = {};
  int hcount = 0, head = 0;
  ntg::Scalars* sc = nullptr;
  ntg::Scalars* hs = nullptr;  // pinned
  long long t = 0;
  float lr = 1e-3f, beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
};

using namespace ntg;
using namespace ntg::mlp;

static const float* newest(const ntg_guess* g) { return g->hist[(g->head - 1 + g->nhist) % g->nhist]; }

static void guess_free(ntg_guess* g) {
  dev_free(g->P); dev_free(g->G); dev_free(g->m1); dev_free(g->m2);
  dev_free(g->W1T); dev_free(g->W2T); dev_free(g->W3T); dev_free(g->W2b); dev_free(g->W3b);
  dev_free(g->X); dev_free(g->XT); dev_free(g->H1b); dev_free(g->H2b); dev_free(g->H1T); dev_free(g->H2T);
  dev_free(g->dYb); dev_free(g->dYT); dev_free(g->dZb); dev_free(g->dZT);
  dev_free(g->Y); dev_free(g->T); dev_free(g->dY); dev_free(g->dH); dev_free(g->dZ); dev_free(g->split);
  dev_free(g->D); dev_free(g->AD);
  for (int i = 0; i < 8; ++i) dev_free(g->hist[i]);
  dev_free(g->sc);
  if (g->hs) cudaFreeHost(g->hs);
  g->hs = nullptr;
}

// refresh the BF16 weight copies from the FP32 master weights
static int refresh_weights(ntg_guess* g) {
  cudaStream_t s = g->plan->stream;
  const int64_t F = g->F, H = g->H, O = g->O;
  { k_wcopy<<<grid_for(F * H, 256), 256, 0, s>>>(g->P + g->oW1, F, H, nullptr, g->W1T); NTG_COUNT_LAUNCH(); }
  { k_wcopy<<<grid_for(H * H, 256), 256, 0, s>>>(g->P + g->oW2, H, H, g->W2b, g->W2T); NTG_COUNT_LAUNCH(); }
  { k_wcopy<<<grid_for(H * O, 256), 256, 0, s>>>(g->P + g->oW3, H, O, g->W3b, g->W3T); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

// splits of the element range (K) for a weight gradient of M x N outputs:
// about two CTAs per SM, the partials within the split buffer
static int wsplits(const ntg_guess* g, int64_t M, int64_t N) {
  const int64_t bn = N <= 64 ? 64 : (N <= 128 ? 128 : 256);
  const int64_t tiles = ((M + 127) / 128) * ((N + bn - 1) / bn);
  int64_t sp = (2 * (int64_t)num_sms() + tiles - 1) / tiles;
  sp = std::min<int64_t>(sp, g->split_len / (M * N));
  return (int)std::max<int64_t>(sp, 1);
}

// forward on E rows of X -> Y (FP32); keeps H1/H2 (and their transposes)
static int guess_forward(ntg_guess* g, const __nv_bfloat16* X, int64_t E) {
  cudaStream_t s = g->plan->stream;
  int* err = g->plan->dev_err;
  const int64_t F = g->F, H = g->H, O = g->O, ldt = g->ldt;
  NTG_TRY(tc_gemm_bf16(X, F, g->W1T, F, E, H, F, nullptr, 0, g->H1b, H, g->H1T, ldt, g->P + g->ob1, 1, 1, nullptr,
                       0, err, s));
  NTG_TRY(tc_gemm_bf16(g->H1b, H, g->W2T, H, E, H, H, nullptr, 0, g->H2b, H, g->H2T, ldt, g->P + g->ob2, 1, 1,
                       nullptr, 0, err, s));
  NTG_TRY(tc_gemm_bf16(g->H2b, H, g->W3T, H, E, O, H, g->Y, O, nullptr, 0, nullptr, 0, g->P + g->ob3, 0, 1, nullptr,
                       0, err, s));
  return NTG_OK;
}

// Gradients into G, given dY (FP32, [E x O]) after guess_forward on X; XT
// (the transpose of X) must be current.
static int guess_backward(ntg_guess* g, int64_t E) {
  cudaStream_t s = g->plan->stream;
  int* err = g->plan->dev_err;
  const int64_t F = g->F, H = g->H, O = g->O, ldt = g->ldt;
  const int ab = (int)std::min<int64_t>((E + 31) / 32, 4096);
  // dY -> BF16 row-major (A of dH2) and transposed (B of dW3)
  { k_act_back<512><<<ab, 256, 0, s>>>(g->dY, nullptr, E, nullptr, g->dYb, g->dYT, ldt); NTG_COUNT_LAUNCH(); }
  { k_colsum<<<(int)((O + 31) / 32), 256, 0, s>>>(g->dY, E, (int)O, g->G + g->ob3); NTG_COUNT_LAUNCH(); }
  // dW3 [H x O] = H2^T dY
  NTG_TRY(tc_gemm_bf16(g->H2T, ldt, g->dYT, ldt, H, O, E, g->G + g->oW3, O, nullptr, 0, nullptr, 0, nullptr, 0,
                       wsplits(g, H, O), g->split, 0, err, s));
  // dH2 = dY W3^T ; dZ2 = dH2 * (H2 > 0)
  NTG_TRY(tc_gemm_bf16(g->dYb, O, g->W3b, O, E, H, O, g->dH, H, nullptr, 0, nullptr, 0, nullptr, 0, 1, nullptr, 0,
                       err, s));
  { k_act_back<64><<<ab, 256, 0, s>>>(g->dH, g->H2b, E, g->dZ, g->dZb, g->dZT, ldt); NTG_COUNT_LAUNCH(); }
  { k_colsum<<<(int)((H + 31) / 32), 256, 0, s>>>(g->dZ, E, (int)H, g->G + g->ob2); NTG_COUNT_LAUNCH(); }
  // dW2 [H x H] = H1^T dZ2
  NTG_TRY(tc_gemm_bf16(g->H1T, ldt, g->dZT, ldt, H, H, E, g->G + g->oW2, H, nullptr, 0, nullptr, 0, nullptr, 0,
                       wsplits(g, H, H), g->split, 0, err, s));
  // dH1 = dZ2 W2^T ; dZ1 = dH1 * (H1 > 0)
  NTG_TRY(tc_gemm_bf16(g->dZb, H, g->W2b, H, E, H, H, g->dH, H, nullptr, 0, nullptr, 0, nullptr, 0, 1, nullptr, 0,
                       err, s));
  { k_act_back<64><<<ab, 256, 0, s>>>(g->dH, g->H1b, E, g->dZ, nullptr, g->dZT, ldt); NTG_COUNT_LAUNCH(); }
  { k_colsum<<<(int)((H + 31) / 32), 256, 0, s>>>(g->dZ, E, (int)H, g->G + g->ob1); NTG_COUNT_LAUNCH(); }
  // dW1 [F x H] = X^T dZ1
  NTG_TRY(tc_gemm_bf16(g->XT, ldt, g->dZT, ldt, F, H, E, g->G + g->oW1, H, nullptr, 0, nullptr, 0, nullptr, 0,
                       wsplits(g, F, H), g->split, 0, err, s));
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

static int transpose_x(ntg_guess* g, const __nv_bfloat16* X, int64_t E) {
  const int64_t tiles = ((E + 31) / 32) * ((g->F + 31) / 32);
  const int grid = (int)std::min<int64_t>(tiles, (int64_t)num_sms() * 8);
  { k_transpose_bf16<<<grid, dim3(32, 8), 0, g->plan->stream>>>(X, E, g->F, g->XT, g->ldt); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

// dY of the online loss: the relative energy + L2 error of the assembled
// guess against the target T (after guess_forward on all elements)
static int energy_grad(ntg_guess* g) {
  ntg_plan* p = g->plan;
  cudaStream_t s = p->stream;
  const int G = grid_for(g->n, 256);
  { k_head<<<G, 256, 0, s>>>(g->Y, newest(g), g->hscale, p->multf, g->n, g->D); NTG_COUNT_LAUNCH(); }
  NTG_TRY(gs_launch_f32(p, g->D, NTG_GS_ADD, s));
  NTG_TRY(mask_launch_f32(p, g->D, s));
  { k_sub_inplace<<<G, 256, 0, s>>>(g->D, g->T, g->n); NTG_COUNT_LAUNCH(); }
  NTG_TRY(ax_launch_f32(p, g->AD, g->D, nullptr, 0, s));
  const float ge = (float)(2.0 / g->tat), gl = (float)(2.0 / g->tt);
  { k_energy_grad_field<<<G, 256, 0, s>>>(g->D, g->AD, g->n, ge, gl, p->red_part, g->sc); NTG_COUNT_LAUNCH(); }
  NTG_TRY(gs_launch_f32(p, g->AD, NTG_GS_ADD, s));
  NTG_TRY(mask_launch_f32(p, g->AD, s));
  { k_head_grad<<<G, 256, 0, s>>>(g->AD, p->multf, g->hscale, g->n, g->dY); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

static int guess_adam(ntg_guess* g) {
  g->t += 1;
  const float c1 = 1.0f / (1.0f - powf(g->beta1, (float)g->t));
  const float c2 = 1.0f / (1.0f - powf(g->beta2, (float)g->t));
  { k_adam<<<grid_for(g->np, 256), 256, 0, g->plan->stream>>>(g->P, g->G, g->m1, g->m2, g->np, g->lr, g->beta1, g->beta2, c1, c2, g->eps); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  return refresh_weights(g);
}

static int poll_red(ntg_guess* g, int slot, double* out) {
  cudaStream_t s = g->plan->stream;
  NTG_CUDA_TRY(cudaMemcpyAsync(g->hs, g->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
  NTG_CUDA_TRY(cudaStreamSynchronize(s));
  *out = g->hs->red[slot];
  return NTG_OK;
}

// the bounded waits of the tensor-core kernels report through the plan's
// error flag
static int check_tc_error(ntg_guess* g) {
  cudaStream_t s = g->plan->stream;
  NTG_CUDA_TRY(cudaMemcpyAsync(&g->hs->status, g->plan->dev_err, sizeof(int), cudaMemcpyDeviceToHost, s));
  NTG_CUDA_TRY(cudaStreamSynchronize(s));
  if (g->hs->status) {
    NTG_CUDA_TRY(cudaMemsetAsync(g->plan->dev_err, 0, sizeof(int), s));
    set_error("learned guess: a tensor-core kernel's bounded wait ran out");
    return NTG_ERR_CUDA;
  }
  return NTG_OK;
}

// X from the history (newest first) and b, with RMS scalings
static int build_x(ntg_guess* g, const double* b) {
  cudaStream_t s = g->plan->stream;
  double bb = 0;
  { k_sumsq<double><<<grid_for(g->n, 256), 256, 0, s>>>(b, g->n, g->plan->red_part, g->sc); NTG_COUNT_LAUNCH(); }
  NTG_TRY(poll_red(g, 2, &bb));
  const double sb = sqrt(bb / (double)g->n);
  const int nw = (g->head - 1 + g->nhist) % g->nhist;
  double sx = g->hrms[nw];
  if (!(sx > 0)) sx = 1.0;
  PrepArgs pa;
  pa.nhist = g->nhist;
  for (int f = 0; f < g->nhist; ++f) {
    const int slot = (g->head - 1 - f + 2 * g->nhist) % g->nhist;
    pa.hist[f] = g->hist[slot];
    pa.scale[f] = (float)(1.0 / sx);
  }
  pa.b = b;
  pa.bscale = (float)(sb > 0 ? 1.0 / sb : 1.0);
  { k_prep_x<<<grid_for(g->E * g->F, 256), 256, 0, s>>>(pa, g->E, g->lx3, g->X); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  g->hscale = (float)sx;
  return NTG_OK;
}

extern "C" {

int ntg_guess_create(ntg_plan* plan, int history, int hidden, uint64_t seed, ntg_guess** out) {
  clear_error();
  NTG_CHECK_ARG(plan && out, "ntg_guess_create: null argument");
  NTG_CHECK_ARG(history >= 1 && history <= 7, "ntg_guess_create: history must be in [1, 7]");
  NTG_CHECK_ARG(hidden == 64, "ntg_guess_create: hidden must be 64");
  NTG_CHECK_ARG(plan->lx == 8, "ntg_guess_create: the nodal head is built for lx = 8 (512 nodes)");
  NTG_CHECK_ARG(plan->dev_err, "ntg_guess_create: plan without an error flag");
  *out = nullptr;
  ntg_guess* g = new ntg_guess();
  g->plan = plan;
  g->nhist = history;
  g->H = hidden;
  g->lx3 = plan->lx * plan->lx * plan->lx;
  g->F = (history + 1) * g->lx3;
  g->O = g->lx3;  // nodal output head
  g->E = plan->nelv;
  g->n = plan->n;
  g->ldt = (g->E + 7) / 8 * 8;
  const int64_t F = g->F, H = g->H, O = g->O, E = g->E, ldt = g->ldt;
  g->oW1 = 0; g->ob1 = F * H; g->oW2 = g->ob1 + H; g->ob2 = g->oW2 + H * H; g->oW3 = g->ob2 + H;
  g->ob3 = g->oW3 + H * O; g->np = g->ob3 + O;
  int st = NTG_OK;
  do {
    if ((st = dev_alloc(&g->P, g->np)) || (st = dev_alloc(&g->G, g->np)) || (st = dev_alloc(&g->m1, g->np)) ||
        (st = dev_alloc(&g->m2, g->np)))
      break;
    if ((st = dev_alloc(&g->W1T, F * H)) || (st = dev_alloc(&g->W2T, H * H)) || (st = dev_alloc(&g->W3T, H * O)) ||
        (st = dev_alloc(&g->W2b, H * H)) || (st = dev_alloc(&g->W3b, H * O)))
      break;
    if ((st = dev_alloc(&g->X, E * F)) || (st = dev_alloc(&g->XT, F * ldt)) || (st = dev_alloc(&g->H1b, E * H)) ||
        (st = dev_alloc(&g->H2b, E * H)) || (st = dev_alloc(&g->H1T, H * ldt)) || (st = dev_alloc(&g->H2T, H * ldt)))
      break;
    if ((st = dev_alloc(&g->dYb, E * O)) || (st = dev_alloc(&g->dYT, O * ldt)) || (st = dev_alloc(&g->dZb, E * H)) ||
        (st = dev_alloc(&g->dZT, H * ldt)))
      break;
    // Y, T, dY, D, AD hold nodal fields (E * lx^3 = n) or E * O raw values
    if ((st = dev_alloc(&g->Y, E * O)) || (st = dev_alloc(&g->T, std::max(g->n, E * O))) ||
        (st = dev_alloc(&g->dY, E * O)) || (st = dev_alloc(&g->dH, E * H)) || (st = dev_alloc(&g->dZ, E * H)) ||
        (st = dev_alloc(&g->D, g->n)) || (st = dev_alloc(&g->AD, g->n)))
      break;
    g->split_len = (int64_t)1 << 24;  // 64 MB of split-K partials
    if ((st = dev_alloc(&g->split, g->split_len))) break;
    for (int i = 0; i < history && !st; ++i) st = dev_alloc(&g->hist[i], g->n);
    if (st) break;
    if ((st = dev_alloc(&g->sc, 1))) break;
    if (cudaMemset(g->sc, 0, sizeof(Scalars)) != cudaSuccess) { st = NTG_ERR_CUDA; break; }
    // the transposed buffers' padding columns (ldt > E) stay zero
    if (cudaMemset(g->XT, 0, sizeof(__nv_bfloat16) * F * ldt) != cudaSuccess ||
        cudaMemset(g->H1T, 0, sizeof(__nv_bfloat16) * H * ldt) != cudaSuccess ||
        cudaMemset(g->H2T, 0, sizeof(__nv_bfloat16) * H * ldt) != cudaSuccess ||
        cudaMemset(g->dZT, 0, sizeof(__nv_bfloat16) * H * ldt) != cudaSuccess ||
        cudaMemset(g->dYT, 0, sizeof(__nv_bfloat16) * O * ldt) != cudaSuccess) { st = NTG_ERR_CUDA; break; }
    if (cudaMallocHost(&g->hs, sizeof(Scalars)) != cudaSuccess) { st = NTG_ERR_ALLOC; break; }
    // He-uniform weights from SplitMix64, zero biases; the output layer
    // starts at zero, so the untrained guess is exactly the newest solution
    std::vector<float> hp(g->np, 0.0f);
    auto fill = [&](int64_t off, int64_t cnt, int64_t fan_in, uint64_t stream_id) {
      const double lim = std::sqrt(6.0 / (double)fan_in);
      for (int64_t i = 0; i < cnt; ++i) {
        uint64_t z = seed * 0x9E3779B97F4A7C15ULL + stream_id * 0xD1B54A32D192ED03ULL + (uint64_t)(i + 1) * 0x632BE59BD9B4E019ULL;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        z ^= z >> 31;
        const double u = (double)(z >> 11) * (1.0 / 9007199254740992.0);
        hp[off + i] = (float)((2.0 * u - 1.0) * lim);
      }
    };
    fill(g->oW1, F * H, F, 11);
    fill(g->oW2, H * H, H, 12);
    if (cudaMemcpy(g->P, hp.data(), sizeof(float) * g->np, cudaMemcpyHostToDevice) != cudaSuccess) { st = NTG_ERR_CUDA; break; }
    cudaMemset(g->m1, 0, sizeof(float) * g->np);
    cudaMemset(g->m2, 0, sizeof(float) * g->np);
    if ((st = refresh_weights(g))) break;
    if (cudaStreamSynchronize(plan->stream) != cudaSuccess) { st = NTG_ERR_CUDA; break; }
  } while (0);
  if (st) {
    guess_free(g);
    delete g;
    return st;
  }
  *out = g;
  return NTG_OK;
}

int ntg_guess_destroy(ntg_guess* g) {
  clear_error();
  if (!g) return NTG_OK;
  cudaStreamSynchronize(g->plan->stream);
  guess_free(g);
  delete g;
  return NTG_OK;
}

int ntg_guess_set_lr(ntg_guess* g, double lr) {
  clear_error();
  NTG_CHECK_ARG(g && lr > 0, "ntg_guess_set_lr: bad argument");
  g->lr = (float)lr;
  return NTG_OK;
}

int64_t ntg_guess_num_params(const ntg_guess* g) { return g ? g->np : 0; }

int ntg_guess_params(ntg_guess* g, float* params_d, int set) {
  clear_error();
  NTG_CHECK_ARG(g && params_d, "ntg_guess_params: null argument");
  cudaStream_t s = g->plan->stream;
  if (set) {
    NTG_CUDA_TRY(cudaMemcpyAsync(g->P, params_d, sizeof(float) * g->np, cudaMemcpyDeviceToDevice, s));
    NTG_TRY(refresh_weights(g));
  } else {
    NTG_CUDA_TRY(cudaMemcpyAsync(params_d, g->P, sizeof(float) * g->np, cudaMemcpyDeviceToDevice, s));
  }
  return NTG_OK;
}

// Raw network access (rows of X are BF16 bit patterns, row length
// (history + 1) * lx^3, 16-byte aligned): Y = net(X) for E <= nelv rows,
// [E x lx^3].
int ntg_guess_forward_raw(ntg_guess* g, const uint16_t* X_d, int64_t E, float* Y_d) {
  clear_error();
  NTG_CHECK_ARG(g && X_d && Y_d && E >= 1 && E <= g->E, "ntg_guess_forward_raw: bad argument");
  NTG_TRY(guess_forward(g, reinterpret_cast<const __nv_bfloat16*>(X_d), E));
  NTG_CUDA_TRY(cudaMemcpyAsync(Y_d, g->Y, sizeof(float) * E * g->O, cudaMemcpyDeviceToDevice, g->plan->stream));
  return check_tc_error(g);
}

static int raw_step(ntg_guess* g, const uint16_t* X_d, const float* T_d, int64_t E, double* loss, int adam) {
  const __nv_bfloat16* X = reinterpret_cast<const __nv_bfloat16*>(X_d);
  cudaStream_t s = g->plan->stream;
  NTG_TRY(guess_forward(g, X, E));
  NTG_TRY(transpose_x(g, X, E));
  const int64_t len = E * g->O;
  { k_loss_grad<<<grid_for(len, 256), 256, 0, s>>>(g->Y, T_d, len, 2.0f / (float)len, g->dY, g->plan->red_part, g->sc); NTG_COUNT_LAUNCH(); }
  NTG_TRY(guess_backward(g, E));
  if (adam) NTG_TRY(guess_adam(g));
  double sse = 0;
  NTG_TRY(poll_red(g, 1, &sse));
  *loss = sse / (double)len;
  return check_tc_error(g);
}

// Gradients of the MSE loss mean((net(X) - T)^2) into grad_d (flat, the
// parameter layout), loss value in *loss.
int ntg_guess_grad_raw(ntg_guess* g, const uint16_t* X_d, const float* T_d, int64_t E, float* grad_d, double* loss) {
  clear_error();
  NTG_CHECK_ARG(g && X_d && T_d && grad_d && loss && E >= 1 && E <= g->E, "ntg_guess_grad_raw: bad argument");
  NTG_TRY(raw_step(g, X_d, T_d, E, loss, 0));
  NTG_CUDA_TRY(cudaMemcpyAsync(grad_d, g->G, sizeof(float) * g->np, cudaMemcpyDeviceToDevice, g->plan->stream));
  NTG_CUDA_TRY(cudaStreamSynchronize(g->plan->stream));
  return NTG_OK;
}

// One Adam step on explicit data (raw access, for tests).
int ntg_guess_train_raw(ntg_guess* g, const uint16_t* X_d, const float* T_d, int64_t E, double* loss) {
  clear_error();
  NTG_CHECK_ARG(g && X_d && T_d && loss && E >= 1 && E <= g->E, "ntg_guess_train_raw: bad argument");
  return raw_step(g, X_d, T_d, E, loss, 1);
}

int ntg_guess_predict(ntg_guess* g, const double* b_d, double* x_d, int* ready) {
  clear_error();
  NTG_CHECK_ARG(g && b_d && x_d && ready, "ntg_guess_predict: null argument");
  *ready = 0;
  if (g->hcount < g->nhist) return NTG_OK;
  NTG_TRY(build_x(g, b_d));
  NTG_TRY(guess_forward(g, g->X, g->E));
  cudaStream_t s = g->plan->stream;
  // x_{k-1} + s Y, averaged over shared nodes, then masked
  { k_head64<<<grid_for(g->n, 256), 256, 0, s>>>(g->Y, newest(g), (double)g->hscale, g->plan->mult, g->n, x_d); NTG_COUNT_LAUNCH(); }
  NTG_TRY(gs_launch(g->plan, x_d, NTG_GS_ADD, s));
  NTG_TRY(mask_launch(g->plan, x_d, s));
  NTG_TRY(check_tc_error(g));
  *ready = 1;
  return NTG_OK;
}

int ntg_guess_observe(ntg_guess* g, const double* b_d, const double* x_d, int train_steps, double* loss) {
  clear_error();
  NTG_CHECK_ARG(g && b_d && x_d, "ntg_guess_observe: null argument");
  cudaStream_t s = g->plan->stream;
  double last = -1.0;
  if (g->hcount >= g->nhist && train_steps > 0) {
    NTG_TRY(build_x(g, b_d));
    NTG_TRY(transpose_x(g, g->X, g->E));
    { k_target<<<grid_for(g->n, 256), 256, 0, s>>>(x_d, g->n, g->T, nullptr); NTG_COUNT_LAUNCH(); }
    const int energy = g->loss_mode == 1;
    if (energy) {
      // normalisers of the relative losses: (T, A T) with the element-local
      // operator, and (T, T)
      NTG_TRY(ax_launch_f32(g->plan, g->AD, g->T, nullptr, 0, s));
      { k_dot_f<<<grid_for(g->n, 256), 256, 0, s>>>(g->T, g->AD, g->n, g->plan->red_part, g->sc); NTG_COUNT_LAUNCH(); }
      NTG_TRY(poll_red(g, 3, &g->tat));
      { k_dot_f<<<grid_for(g->n, 256), 256, 0, s>>>(g->T, g->T, g->n, g->plan->red_part, g->sc); NTG_COUNT_LAUNCH(); }
      NTG_TRY(poll_red(g, 3, &g->tt));
      if (!(g->tat > 0)) g->tat = 1.0;
      if (!(g->tt > 0)) g->tt = 1.0;
    }
    for (int it = 0; it < train_steps; ++it) {
      NTG_TRY(guess_forward(g, g->X, g->E));
      if (energy) {
        NTG_TRY(energy_grad(g));
      } else {
        const int64_t len = g->E * g->O;
        { k_loss_grad<<<grid_for(len, 256), 256, 0, s>>>(g->Y, g->T, len, 2.0f / (float)len, g->dY, g->plan->red_part, g->sc); NTG_COUNT_LAUNCH(); }
      }
      NTG_TRY(guess_backward(g, g->E));
      NTG_TRY(guess_adam(g));
    }
    double sse = 0;
    NTG_TRY(poll_red(g, 1, &sse));
    last = energy ? sse : sse / (double)(g->E * g->O);
    NTG_TRY(check_tc_error(g));
  }
  // push x into the history ring
  float* slot = g->hist[g->head];
  { k_target<<<grid_for(g->n, 256), 256, 0, s>>>(x_d, g->n, nullptr, slot); NTG_COUNT_LAUNCH(); }
  double xx = 0;
  { k_sumsq<float><<<grid_for(g->n, 256), 256, 0, s>>>(slot, g->n, g->plan->red_part, g->sc); NTG_COUNT_LAUNCH(); }
  NTG_TRY(poll_red(g, 2, &xx));
  g->hrms[g->head] = sqrt(xx / (double)g->n);
  g->head = (g->head + 1) % g->nhist;
  if (g->hcount < g->nhist) g->hcount++;
  if (loss) *loss = last;
  return NTG_OK;
}

int ntg_guess_set_loss(ntg_guess* g, int energy) {
  clear_error();
  NTG_CHECK_ARG(g, "ntg_guess_set_loss: null argument");
  g->loss_mode = energy ? 1 : 0;
  return NTG_OK;
}

// Checkpoint of the whole network state: one FP32 device buffer of
// ntg_guess_state_len floats [P | Adam m1 | Adam m2 | history ring, slot by
// slot], the integers {Adam step, ring head, ring count, 0} and the ring's
// RMS scales (8 doubles).  dir = 0 stores, dir = 1 loads (the BF16 weight
// copies are rebuilt from P, so a restored network computes bit for bit as
// the saved one).
int64_t ntg_guess_state_len(const ntg_guess* g) { return g ? 3 * g->np + (int64_t)g->nhist * g->n : 0; }

int ntg_guess_state(ntg_guess* g, float* buf_d, long long* ints, double* hrms, int dir) {
  clear_error();
  NTG_CHECK_ARG(g && buf_d && ints && hrms && (dir == 0 || dir == 1), "ntg_guess_state: bad argument");
  cudaStream_t s = g->plan->stream;
  const int64_t np = g->np, n = g->n;
  float* parts[3] = {g->P, g->m1, g->m2};
  const cudaMemcpyKind k = cudaMemcpyDeviceToDevice;
  if (dir == 0) {
    for (int q = 0; q < 3; ++q) NTG_CUDA_TRY(cudaMemcpyAsync(buf_d + q * np, parts[q], sizeof(float) * np, k, s));
    for (int h = 0; h < g->nhist; ++h)
      NTG_CUDA_TRY(cudaMemcpyAsync(buf_d + 3 * np + h * n, g->hist[h], sizeof(float) * n, k, s));
    ints[0] = g->t;
    ints[1] = g->head;
    ints[2] = g->hcount;
    ints[3] = 0;
    for (int h = 0; h < 8; ++h) hrms[h] = g->hrms[h];
  } else {
    NTG_CHECK_ARG(ints[0] >= 0 && ints[1] >= 0 && ints[1] < g->nhist && ints[2] >= 0 && ints[2] <= g->nhist,
                  "ntg_guess_state: counters out of range");
    for (int q = 0; q < 3; ++q) NTG_CUDA_TRY(cudaMemcpyAsync(parts[q], buf_d + q * np, sizeof(float) * np, k, s));
    for (int h = 0; h < g->nhist; ++h)
      NTG_CUDA_TRY(cudaMemcpyAsync(g->hist[h], buf_d + 3 * np + h * n, sizeof(float) * n, k, s));
    NTG_TRY(refresh_weights(g));
    g->t = ints[0];
    g->head = (int)ints[1];
    g->hcount = (int)ints[2];
    for (int h = 0; h < 8; ++h) g->hrms[h] = hrms[h];
  }
  NTG_CUDA_TRY(cudaStreamSynchronize(s));
  return NTG_OK;
}

int ntg_guess_reset_history(ntg_guess* g) {
  clear_error();
  NTG_CHECK_ARG(g, "ntg_guess_reset_history: null argument");
  g->hcount = 0;
  g->head = 0;
  return NTG_OK;
}

}  // extern "C"
