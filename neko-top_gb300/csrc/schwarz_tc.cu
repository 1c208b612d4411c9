// Schwarz FDM local solves on the tensor cores (lx = 8, extended box 10^3).
//
// The local solve of element e is
//   w = c_e (S x S x S) D_e^-1 (S x S x S)^T x,   x the extended residual,
// with the one reference eigenvector matrix S (10 x 10, S[p][f]) shared by
// every element (see schwarz.cu).  The two in-plane directions together are
// one 100 x 100 matrix K = S x S, the same for all elements, so a batch of 8
// elements is two GEMMs on the tensor cores plus a per-line transform along
// the third direction:
//
//   1. Y1[fg][(e,c)] = sum_ab K[ab][fg] x_e[ab][c]       tcgen05, M = 128 (fg,
//      100 used), N = 80 (8 elements x 10 planes), K = 112 (ab, 100 used)
//   2. per (fg, e): y = S^T Y1[fg][e, .]; z_h = c_e y_h / D_e(f, g, h);
//      W1[fg][(e,c)] = sum_h S[c][h] z_h                CUDA cores, FP32,
//      one thread per TMEM lane fg, the line in registers
//   3. W[ab][(e,c)] = sum_fg K[ab][fg] W1[fg][(e,c)]     tcgen05, as step 1
//   4. ze[e][ab + 100 c] = W[ab][(e,c)]                  one thread per lane
//      ab: consecutive threads store consecutive addresses
//
// Precision.  The GEMM operands are BF16 with FP32 accumulation in TMEM.
// The data (x in step 1, W1 in step 3) are split as hi + lo (two BF16 terms,
// 16 significant bits) and both products accumulate into the same tile;
// K is rounded once to BF16.  The rounded K appears transposed in step 1 and
// as is in step 3 (the same rounded entries), so the preconditioner stays
// exactly symmetric: K~ D^-1 K~^T in the plane, with the third direction in
// FP32.  It is the same kind of approximate local solve as before, with K~
// in place of S x S to 2^-9 relative.
//
// Layout.  Every GEMM operand is K-major with the 128-byte swizzle of the
// tcgen05 shared-memory descriptors (8-row, 1024-byte atoms, 16-byte chunks
// XOR-permuted by the row within the atom), in chunks of 64 K values.  The
// constant K~ (both orientations, 2 x 32 KB) is prepared on the host in that
// image and copied into shared memory once per CTA; the data tiles are
// written by the threads with the same permutation.  K columns 100..127 of
// the data tiles are zeroed once and never written again, the constant's
// padding is zero, so the padded products vanish.
//
// Threads: 256 (8 warps).  Gather: warp w fetches element w of the batch
// (100 columns of 10 values, lanes on consecutive columns) and its coarse
// restriction (warp-shuffle sums in a fixed order).  Steps 2 and 4: warp w
// reads TMEM lanes 32 (w mod 4) .. +31 for elements 4 (w / 4) .. +3.  Thread
// 0 issues the MMAs; completion is signalled by tcgen05.commit on one
// mbarrier (two phases per batch), every wait bounded (on time-out the error
// flag is raised and the kernel drains and returns).  Two CTAs per SM
// (105 KB of shared memory and 256 TMEM columns each).
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "schwarz.cuh"
#include "tc.cuh"

namespace ntg {
namespace sw {
namespace ftc {

constexpr int LX = 8, N = 7, LE = 10, LE2 = 100, LE3 = 1000, LX2 = 64, LX3 = 512;
constexpr int EPB = 8, NCOL = EPB * LE;   // 80 GEMM columns per batch
constexpr int THREADS = 256;
constexpr int A_CHUNK = 128 * 128;         // 128 rows x 64 BF16 = 16 KB
constexpr int A_BYTES = 2 * A_CHUNK;       // K = 128 (two chunks)
constexpr int B_CHUNK = NCOL * 128;        // 80 rows x 64 BF16 = 10 KB
constexpr int B_BYTES = 2 * B_CHUNK;
constexpr int KSTEPS = 7;                  // K = 112 in steps of 16
// shared memory map (offsets from a 1024-aligned base)
constexpr int OFF_A1 = 0, OFF_A3 = A_BYTES, OFF_BH = 2 * A_BYTES, OFF_BL = OFF_BH + B_BYTES;
constexpr int OFF_S = OFF_BL + B_BYTES;             // S[p][f] fp32
constexpr int OFF_LAM = OFF_S + 4 * LE2;            // lam[10]
constexpr int OFF_ESC = OFF_LAM + 64;               // 8 elements x 8 scalars
constexpr int OFF_PH = OFF_ESC + 4 * EPB * 8;       // Q1 basis p[2][8]
constexpr int OFF_BAR = OFF_PH + 4 * 16;            // mbarrier
constexpr int OFF_SLOT = OFF_BAR + 8;               // TMEM base
constexpr int OFF_FLAG = OFF_SLOT + 4;
constexpr int SMEM_USED = OFF_FLAG + 4;
constexpr int SMEM = SMEM_USED + 1024;               // + alignment slack
constexpr uint32_t TMEM_COLS = 256;                  // D1 at column 0, D3 at 128
constexpr int IMG_BYTES = 2 * A_BYTES;               // the constant image: K~^T then K~

// byte offset of element (row, k) in a K-major, 128-byte-swizzled tile whose
// 64-wide K chunks are `chunk` bytes apart
__device__ __host__ __forceinline__ int swz(int row, int k, int chunk) {
  return (k >> 6) * chunk + (row >> 3) * 1024 + (row & 7) * 128 + ((((k & 63) >> 3) ^ (row & 7)) << 4) + (k & 7) * 2;
}

__device__ __forceinline__ void put_split(uint8_t* bh, uint8_t* bl, int off, float v) {
  const __nv_bfloat16 h = __float2bfloat16(v);
  const __nv_bfloat16 l = __float2bfloat16(v - __bfloat162float(h));
  *reinterpret_cast<__nv_bfloat16*>(bh + off) = h;
  *reinterpret_cast<__nv_bfloat16*>(bl + off) = l;
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__global__ void __launch_bounds__(THREADS, 2)
    k_fdm_tc(const float* __restrict__ r, float* __restrict__ ze, const float* __restrict__ esc, int Ex, int Ey,
             int Ez, const Scalars* sc, float* __restrict__ corner, CoarsePhi ph, const uint8_t* __restrict__ img,
             const float* __restrict__ Sg, const float* __restrict__ lamg, int* __restrict__ err) {
  if (sc && sc->done) return;
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = tc::smem_u32(smem_raw);
  uint8_t* sm = smem_raw + ((1024u - (raw & 1023u)) & 1023u);
  uint8_t* A1 = sm + OFF_A1;
  uint8_t* A3 = sm + OFF_A3;
  uint8_t* Bh = sm + OFF_BH;
  uint8_t* Bl = sm + OFF_BL;
  float* S = reinterpret_cast<float*>(sm + OFF_S);
  float* lam = reinterpret_cast<float*>(sm + OFF_LAM);
  float* es = reinterpret_cast<float*>(sm + OFF_ESC);
  float* sp = reinterpret_cast<float*>(sm + OFF_PH);
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + OFF_BAR);
  uint32_t* slot = reinterpret_cast<uint32_t*>(sm + OFF_SLOT);
  volatile int* flag = reinterpret_cast<volatile int*>(sm + OFF_FLAG);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // constants: the K~ image (64 KB), S, lam, the Q1 basis; zero the data tiles
  {
    const uint4* src = reinterpret_cast<const uint4*>(img);
    uint4* dst = reinterpret_cast<uint4*>(A1);
    for (int q = tid; q < IMG_BYTES / 16; q += THREADS) dst[q] = src[q];
    uint4* bz = reinterpret_cast<uint4*>(Bh);
    for (int q = tid; q < 2 * B_BYTES / 16; q += THREADS) bz[q] = make_uint4(0u, 0u, 0u, 0u);
    for (int q = tid; q < LE2; q += THREADS) S[q] = Sg[q];
    if (tid < LE) lam[tid] = lamg[tid];
    if (tid < 2 * LX) sp[tid] = ph.p[tid / LX][tid % LX];
  }
  if (tid == 0) {
    tc::mbar_init(bar, 1);
    *flag = 0;
    tc::fence_mbar_init();
  }
  if (warp == 0) tc::tmem_alloc(slot, TMEM_COLS);
  fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *slot;
  constexpr uint32_t idesc = tc::idesc_bf16_f32(128, NCOL);
  const uint32_t a1 = tc::smem_u32(A1), a3 = tc::smem_u32(A3), bh = tc::smem_u32(Bh), bl = tc::smem_u32(Bl);

  const int nelv = Ex * Ey * Ez;
  const int64_t zs = (int64_t)Ex * Ey * LX3;
  const int quarter = warp & 3, half = warp >> 2;
  const int lanerow = quarter * 32 + lane;  // TMEM lane of this thread: fg (step 2) / ab (step 4)
  bool failed = false;
  int fail_phase = 0;

  for (int e0 = blockIdx.x * EPB; e0 < nelv && !failed; e0 += gridDim.x * EPB) {
    // ---- gather: warp w fetches element e0 + w ----------------------------
    {
      const int el = warp, e = e0 + el;
      const bool live = e < nelv;
      if (lane < 8) es[el * 8 + lane] = live ? esc[(int64_t)e * 8 + lane] : 1.f;
      int ex = 0, ey = 0, ez = 0;
      if (live) {
        const int exy = e / Ex;
        ex = e - exy * Ex;
        ez = exy / Ey;
        ey = exy - ez * Ey;
      }
      float part[8];
#pragma unroll
      for (int v = 0; v < 8; ++v) part[v] = 0.f;
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const int q = lane + 32 * m;
        if (q >= LE2) break;
        const int a = q % LE, b = q / LE;
        int i = a - 1, dx = 0;
        if (i < 0) { dx = -1; i = N - 1; } else if (i > N) { dx = 1; i = 1; }
        int j = b - 1, dy = 0;
        if (j < 0) { dy = -1; j = N - 1; } else if (j > N) { dy = 1; j = 1; }
        const int nx = ex + dx, ny = ey + dy;
        const bool okxy = live && nx >= 0 && nx < Ex && ny >= 0 && ny < Ey;
        const float* rc = r + (int64_t)(nx + Ex * (ny + Ey * ez)) * LX3 + i + LX * j;
        float s0 = 0.f, s1 = 0.f;
#pragma unroll
        for (int c = 0; c < LE; ++c) {
          float val = 0.f;
          if (okxy) {
            if (c == 0) val = ez > 0 ? rc[(N - 1) * LX2 - zs] : 0.f;
            else if (c == LE - 1) val = ez < Ez - 1 ? rc[LX2 + zs] : 0.f;
            else val = rc[(c - 1) * LX2];
          }
          put_split(Bh, Bl, swz(el * LE + c, q, B_CHUNK), val);
          if (c >= 1 && c <= LX) {
            const int k = c - 1;
            const float wz = ((k == 0 && ez > 0) || (k == N && ez < Ez - 1)) ? 0.5f : 1.f;
            s0 = fmaf(sp[k] * wz, val, s0);
            s1 = fmaf(sp[LX + k] * wz, val, s1);
          }
        }
        if (corner && dx == 0 && dy == 0 && okxy) {
          const float wx = ((i == 0 && ex > 0) || (i == N && ex < Ex - 1)) ? 0.5f : 1.f;
          const float wy = ((j == 0 && ey > 0) || (j == N && ey < Ey - 1)) ? 0.5f : 1.f;
#pragma unroll
          for (int v = 0; v < 8; ++v)
            part[v] = fmaf(sp[(v & 1) * LX + i] * wx * (sp[((v >> 1) & 1) * LX + j] * wy), (v >> 2) ? s1 : s0, part[v]);
        }
      }
      if (corner) {
#pragma unroll
        for (int v = 0; v < 8; ++v) {
          float t = part[v];
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
          part[v] = t;
        }
        if (live && lane < 8) {
          float t = part[0];
#pragma unroll
          for (int v = 1; v < 8; ++v)
            if (lane == v) t = part[v];
          corner[(int64_t)e * 8 + lane] = t;
        }
      }
    }
    fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    // ---- step 1: Y1 = K~^T X (tensor cores) --------------------------------
    if (tid == 0) {
      tc::fence_after_sync();
#pragma unroll
      for (int s = 0; s < KSTEPS; ++s) {
        const uint32_t ao = (s >> 2) * A_CHUNK + (s & 3) * 32, bo = (s >> 2) * B_CHUNK + (s & 3) * 32;
        tc::mma_bf16(tmem, tc::desc_kmajor_sw128(a1 + ao), tc::desc_kmajor_sw128(bh + bo), idesc, s > 0 ? 1u : 0u);
        tc::mma_bf16(tmem, tc::desc_kmajor_sw128(a1 + ao), tc::desc_kmajor_sw128(bl + bo), idesc, 1u);
      }
      tc::mma_commit(bar);
    }
    if (!tc::mbar_wait(bar, 0)) failed = true;
    fail_phase = 0;
    if (__syncthreads_or(failed)) {
      failed = true;
      break;
    }
    tc::fence_after_sync();
    // ---- step 2: third direction per (fg, element), FP32 -------------------
    {
      float y[48];
      const uint32_t col = (uint32_t)(half * 40);
      const uint32_t ta = tmem + ((uint32_t)(quarter * 32) << 16) + col;
      tc::tmem_ld16(ta, *reinterpret_cast<float(*)[16]>(y));
      tc::tmem_ld16(ta + 16, *reinterpret_cast<float(*)[16]>(y + 16));
      tc::tmem_ld16(ta + 32, *reinterpret_cast<float(*)[16]>(y + 32));
      if (lanerow < LE2) {
        const int f = lanerow % LE, g = lanerow / LE;
#pragma unroll
        for (int el4 = 0; el4 < 4; ++el4) {
          const int el = half * 4 + el4;
          const float* ee = es + el * 8;
          const float sx = ee[0], sy = ee[1], sz = ee[2], ce = ee[3], h1 = ee[4], h2 = ee[5];
          const float base = h1 * (sx * lam[f] + sy * lam[g]) + h2;
          float z[LE];
#pragma unroll
          for (int h = 0; h < LE; ++h) {
            float t = 0.f;
#pragma unroll
            for (int c = 0; c < LE; ++c) t = fmaf(S[c * LE + h], y[el4 * LE + c], t);
            z[h] = __fdividef(ce * t, base + h1 * sz * lam[h]);
          }
#pragma unroll
          for (int c = 0; c < LE; ++c) {
            float w = 0.f;
#pragma unroll
            for (int h = 0; h < LE; ++h) w = fmaf(S[c * LE + h], z[h], w);
            put_split(Bh, Bl, swz(el * LE + c, lanerow, B_CHUNK), w);
          }
        }
      }
    }
    fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    // ---- step 3: W = K~ W1 (tensor cores) ----------------------------------
    if (tid == 0) {
      tc::fence_after_sync();
#pragma unroll
      for (int s = 0; s < KSTEPS; ++s) {
        const uint32_t ao = (s >> 2) * A_CHUNK + (s & 3) * 32, bo = (s >> 2) * B_CHUNK + (s & 3) * 32;
        tc::mma_bf16(tmem + 128, tc::desc_kmajor_sw128(a3 + ao), tc::desc_kmajor_sw128(bh + bo), idesc,
                     s > 0 ? 1u : 0u);
        tc::mma_bf16(tmem + 128, tc::desc_kmajor_sw128(a3 + ao), tc::desc_kmajor_sw128(bl + bo), idesc, 1u);
      }
      tc::mma_commit(bar);
    }
    if (!tc::mbar_wait(bar, 1)) failed = true;
    fail_phase = 1;
    if (__syncthreads_or(failed)) {
      failed = true;
      break;
    }
    tc::fence_after_sync();
    // ---- step 4: extended results to HBM ------------------------------------
    {
      float w[48];
      const uint32_t ta = tmem + ((uint32_t)(quarter * 32) << 16) + 128u + (uint32_t)(half * 40);
      tc::tmem_ld16(ta, *reinterpret_cast<float(*)[16]>(w));
      tc::tmem_ld16(ta + 16, *reinterpret_cast<float(*)[16]>(w + 16));
      tc::tmem_ld16(ta + 32, *reinterpret_cast<float(*)[16]>(w + 32));
      if (lanerow < LE2) {
#pragma unroll
        for (int el4 = 0; el4 < 4; ++el4) {
          const int e = e0 + half * 4 + el4;
          if (e >= nelv) break;
          float* out = ze + (int64_t)e * LE3 + lanerow;
#pragma unroll
          for (int c = 0; c < LE; ++c) out[LE2 * c] = w[el4 * LE + c];
        }
      }
    }
    tc::fence_before_sync();
    __syncthreads();
  }
  if (failed) {
    if (tid == 0) {
      atomicExch(err, 1);
      // the MMAs of the step that timed out: wait once more (bounded)
      tc::mbar_wait(bar, (uint32_t)fail_phase);
    }
    tc::fence_before_sync();
    __syncthreads();
  }
  if (warp == 0) tc::tmem_dealloc(tmem, TMEM_COLS);
}

// round to nearest even, FP32 -> BF16 bits
static uint16_t bf16_bits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  if ((u & 0x7F800000u) == 0x7F800000u) return (uint16_t)(u >> 16);
  const uint32_t r = ((u >> 16) & 1u) + 0x7FFFu;
  return (uint16_t)((u + r) >> 16);
}

}  // namespace ftc

int fdm_tc_prepare(const double* Sref, const double* lamref, FdmTc* t) {
  using namespace ftc;
  std::vector<uint8_t> img(IMG_BYTES, 0);
  for (int r = 0; r < LE2; ++r)
    for (int k = 0; k < LE2; ++k) {
      // A1 = K~^T: row (f, g) = r, column (a, b) = k; A3 = K~: row (a, b) = r, column (f, g) = k
      const int f1 = r % LE, g1 = r / LE, a1 = k % LE, b1 = k / LE;
      const uint16_t v1 = bf16_bits((float)(Sref[a1 * LE + f1] * Sref[b1 * LE + g1]));
      const int a3 = r % LE, b3 = r / LE, f3 = k % LE, g3 = k / LE;
      const uint16_t v3 = bf16_bits((float)(Sref[a3 * LE + f3] * Sref[b3 * LE + g3]));
      std::memcpy(&img[OFF_A1 + swz(r, k, A_CHUNK)], &v1, 2);
      std::memcpy(&img[OFF_A3 + swz(r, k, A_CHUNK)], &v3, 2);
    }
  std::vector<float> Sf(LE2), lf(LE);
  for (int q = 0; q < LE2; ++q) Sf[q] = (float)Sref[q];
  for (int q = 0; q < LE; ++q) lf[q] = (float)lamref[q];
  NTG_TRY(dev_alloc(&t->img, (size_t)IMG_BYTES));
  NTG_TRY(dev_alloc(&t->S, (size_t)LE2));
  NTG_TRY(dev_alloc(&t->lam, (size_t)LE));
  NTG_CUDA_TRY(cudaMemcpy(t->img, img.data(), IMG_BYTES, cudaMemcpyHostToDevice));
  NTG_CUDA_TRY(cudaMemcpy(t->S, Sf.data(), sizeof(float) * LE2, cudaMemcpyHostToDevice));
  NTG_CUDA_TRY(cudaMemcpy(t->lam, lf.data(), sizeof(float) * LE, cudaMemcpyHostToDevice));
  static bool attr[64] = {};
  int dev = 0;
  NTG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev >= 0 && dev < 64 && !attr[dev]) {
    NTG_CUDA_TRY(cudaFuncSetAttribute(k_fdm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM));
    attr[dev] = true;
  }
  int per_sm = 0;
  NTG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fdm_tc, THREADS, SMEM));
  t->per_sm = per_sm > 0 ? per_sm : 1;
  return NTG_OK;
}

void fdm_tc_free(FdmTc* t) {
  dev_free(t->img);
  dev_free(t->S);
  dev_free(t->lam);
}

int fdm_tc_launch(const FdmTc& t, const float* r, float* ze, const float* esc, int Ex, int Ey, int Ez,
                  const Scalars* sc, float* corner, const CoarsePhi& ph, int* err, cudaStream_t s) {
  using namespace ftc;
  const int64_t nelv = (int64_t)Ex * Ey * Ez;
  const int64_t batches = (nelv + EPB - 1) / EPB;
  const int64_t cap = (int64_t)num_sms() * t.per_sm;
  const int grid = (int)(batches < cap ? batches : cap);
  { k_fdm_tc<<<grid, THREADS, SMEM, s>>>(r, ze, esc, Ex, Ey, Ez, sc, corner, ph, t.img, t.S, t.lam, err); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

}  // namespace sw
}  // namespace ntg
