// BF16 GEMM on the 5th-generation tensor cores: C = A B^T with A [M x K]
// and B [N x K] both K-major (row-major, K contiguous), FP32 accumulation in
// tensor memory.  The learned guess's forward and backward passes run on it.
//
// One CTA computes a 128 x BN tile of C (BN = 64, 128 or 256 columns of
// TMEM).  Warp 0 (one thread) streams 64-wide K slices of A and B into a
// ring of shared-memory stages with 2D TMA tiled copies (128-byte swizzle);
// warp 1 (one thread) issues four tcgen05.mma (K = 16 each) per slice and
// frees the stage with tcgen05.commit on its "empty" mbarrier; after the
// last slice a commit on the "done" mbarrier releases the epilogue, in which
// all four warps read their 32 TMEM lanes (one output row per thread) with
// tcgen05.ld and write FP32, BF16 or transposed BF16 outputs with an
// optional bias and ReLU.  A split over K (grid.z) writes FP32 partial
// tiles that k_splitk_sum adds in a fixed order (deterministic).
//
// Rows and columns past M, N and K are read as zeros by the TMA engine (out-
// of-bounds fill) and not written.  Every wait is bounded: a wait that runs
// out raises *err, the CTA drains the copies it issued and the MMAs it
// started (bounded too), frees its TMEM and returns.
#include <cudaTypedefs.h>

#include <mutex>

#include "common.cuh"
#include "tc.cuh"

namespace ntg {
namespace tcg {

constexpr int BM = 128, BK = 64;
constexpr int kThreads = 128;

struct Epi {
  float* C;            // FP32 [M x ldc] (split: partial slab z at z * M * ldc)
  int64_t ldc;
  __nv_bfloat16* Cb;   // BF16 [M x ldcb]
  int64_t ldcb;
  __nv_bfloat16* CbT;  // BF16 transposed: (m, n) at n * ldt + m
  int64_t ldt;
  const float* bias;   // per column
  int relu;
  int split;           // 1: partial sums only
};

template <int BN, int ST>
struct Cfg {
  static constexpr int A_BYTES = BM * BK * 2;  // 16 KB
  static constexpr int B_BYTES = BN * BK * 2;
  static constexpr int STAGE = A_BYTES + B_BYTES;
  static constexpr int SMEM = 1024 + ST * STAGE + 256;
  static constexpr uint32_t TMEM_COLS = BN;
};

template <int BN, int ST>
__global__ void __launch_bounds__(kThreads, 1)
    k_tc_gemm(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, Epi ep, int64_t M,
              int64_t N, int kb_total, int kb_per_split, int* __restrict__ err) {
  using Cg = Cfg<BN, ST>;
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = tc::smem_u32(smem_raw);
  uint8_t* smem = smem_raw + ((1024u - (raw & 1023u)) & 1023u);
  uint8_t* sA = smem;
  uint8_t* sB = smem + ST * Cg::A_BYTES;
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + ST * Cg::STAGE);
  uint64_t* empty = full + ST;
  uint64_t* done = empty + ST;
  uint32_t* slot = reinterpret_cast<uint32_t*>(done + 1);
  volatile int* flags = reinterpret_cast<volatile int*>(slot + 1);  // [0] failed, [1] consumed, [2] issued

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t m0 = (int64_t)blockIdx.x * BM, n0 = (int64_t)blockIdx.y * BN;
  const int kb0 = (int)blockIdx.z * kb_per_split;
  const int kb1 = min(kb0 + kb_per_split, kb_total);
  const int nk = kb1 > kb0 ? kb1 - kb0 : 0;

  if (threadIdx.x == 0) {
    for (int s = 0; s < ST; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(done, 1);
    flags[0] = 0;
    flags[1] = 0;
    flags[2] = 0;
    tc::fence_mbar_init();
    tc::tma_prefetch_desc(&tmA);
    tc::tma_prefetch_desc(&tmB);
  }
  if (warp == 0) tc::tmem_alloc(slot, Cg::TMEM_COLS);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *slot;

  if (warp == 0 && lane == 0) {
    // producer: TMA copies of the K slices
    int issued = 0;
    for (int i = 0; i < nk; ++i) {
      const int s = i % ST;
      if (i >= ST && !tc::mbar_wait(&empty[s], (uint32_t)((i / ST) - 1) & 1u)) {
        flags[0] = 1;
        break;
      }
      if (flags[0]) break;
      tc::mbar_expect_tx(&full[s], (uint32_t)Cg::STAGE);
      tc::tma_load_2d(sA + s * Cg::A_BYTES, &tmA, (kb0 + i) * BK, (int)m0, &full[s]);
      tc::tma_load_2d(sB + s * Cg::B_BYTES, &tmB, (kb0 + i) * BK, (int)n0, &full[s]);
      ++issued;
    }
    flags[2] = issued;
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    constexpr uint32_t idesc = tc::idesc_bf16_f32(BM, BN);
    int consumed = 0;
    for (int i = 0; i < nk; ++i) {
      const int s = i % ST;
      if (!tc::mbar_wait(&full[s], (uint32_t)(i / ST) & 1u)) {
        flags[0] = 1;
        break;
      }
      tc::fence_after_sync();
      const uint32_t a0 = tc::smem_u32(sA + s * Cg::A_BYTES), b0 = tc::smem_u32(sB + s * Cg::B_BYTES);
#pragma unroll
      for (int k = 0; k < BK / 16; ++k)
        tc::mma_bf16(tmem, tc::desc_kmajor_sw128(a0 + 32u * k), tc::desc_kmajor_sw128(b0 + 32u * k), idesc,
                     (i > 0 || k > 0) ? 1u : 0u);
      tc::mma_commit(&empty[s]);
      ++consumed;
    }
    flags[1] = consumed;
    tc::mma_commit(done);  // arrives once every MMA above has completed
  }
  __syncwarp();
  const bool ok = tc::mbar_wait(done, 0);
  __syncthreads();
  const bool good = ok && !flags[0] && flags[1] == nk;
  tc::fence_after_sync();

  // epilogue: thread (warp w, lane l) owns row m0 + 32 w + l
  const int64_t row = m0 + warp * 32 + lane;
#pragma unroll 1
  for (int c = 0; c < BN; c += 16) {
    float v[16];
    if (nk > 0) {
      tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
    } else {
#pragma unroll
      for (int q = 0; q < 16; ++q) v[q] = 0.f;
    }
    if (!good || row >= M) continue;
    // whole 16-column chunks go out as 16-byte stores (a thread owns a row)
    const int64_t col0 = n0 + c;
    if (!ep.split && col0 + 16 <= N && ((!ep.C || (ep.ldc % 4 == 0 && (reinterpret_cast<uintptr_t>(ep.C) & 15) == 0)) &&
                                                   (!ep.Cb || (ep.ldcb % 8 == 0 && (reinterpret_cast<uintptr_t>(ep.Cb) & 15) == 0)))) {
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        float x = v[q];
        if (ep.bias) x += ep.bias[col0 + q];
        if (ep.relu) x = x > 0.f ? x : 0.f;
        v[q] = x;
      }
      if (ep.C) {
        float4* dst = reinterpret_cast<float4*>(ep.C + row * ep.ldc + col0);
#pragma unroll
        for (int q = 0; q < 4; ++q) dst[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
      }
      if (ep.Cb) {
        uint4 pk[2];
        uint32_t* w = reinterpret_cast<uint32_t*>(pk);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const __nv_bfloat162 h2 = __floats2bfloat162_rn(v[2 * q], v[2 * q + 1]);
          w[q] = *reinterpret_cast<const uint32_t*>(&h2);
        }
        uint4* dst = reinterpret_cast<uint4*>(ep.Cb + row * ep.ldcb + col0);
        dst[0] = pk[0];
        dst[1] = pk[1];
      }
      if (ep.CbT) {  // consecutive lanes hold consecutive rows: coalesced per column
#pragma unroll
        for (int q = 0; q < 16; ++q) ep.CbT[(col0 + q) * ep.ldt + row] = __float2bfloat16(v[q]);
      }
      continue;
    }
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int64_t col = n0 + c + q;
      if (col >= N) break;
      float x = v[q];
      if (ep.split) {
        ep.C[(int64_t)blockIdx.z * M * ep.ldc + row * ep.ldc + col] = x;
        continue;
      }
      if (ep.bias) x += ep.bias[col];
      if (ep.relu) x = x > 0.f ? x : 0.f;
      if (ep.C) ep.C[row * ep.ldc + col] = x;
      const __nv_bfloat16 xb = __float2bfloat16(x);
      if (ep.Cb) ep.Cb[row * ep.ldcb + col] = xb;
      if (ep.CbT) ep.CbT[col * ep.ldt + row] = xb;
    }
  }
  if (!good && threadIdx.x == 0) {
    atomicExch(err, 1);
    // drain the copies issued but not consumed (bounded)
    for (int i = flags[1]; i < flags[2]; ++i) tc::mbar_wait(&full[i % ST], (uint32_t)(i / ST) & 1u);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, Cg::TMEM_COLS);
}

// out = sum over z of S partial [M x N] slabs in order z = 0..S-1, then
// bias / ReLU; FP32 row-major (ldc) or transposed ((m, n) at n * ldc + m)
__global__ void k_splitk_sum(const float* __restrict__ part, int S, int64_t M, int64_t N, float* __restrict__ C,
                             int64_t ldc, int transpose, const float* __restrict__ bias, int relu) {
  const int64_t MN = M * N;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < MN; i += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int z = 0; z < S; ++z) s += part[(int64_t)z * MN + i];
    const int64_t m = i / N, n = i - m * N;
    if (bias) s += bias[n];
    if (relu) s = s > 0.f ? s : 0.f;
    C[transpose ? n * ldc + m : m * ldc + n] = s;
  }
}

// ---- host side -------------------------------------------------------------
static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
static std::once_flag g_encode_once;

static int encoder(PFN_cuTensorMapEncodeTiled_v12000* fn) {
  std::call_once(g_encode_once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  if (!g_encode) {
    set_error("tensor-core GEMM: cuTensorMapEncodeTiled is not available from the driver");
    return NTG_ERR_CUDA;
  }
  *fn = g_encode;
  return NTG_OK;
}

// Tensor map of a row-major BF16 matrix [rows x cols] with row stride ld
// elements, boxes of 64 columns x box_rows rows, 128-byte swizzle.
static int make_map(CUtensorMap* tm, const void* base, int64_t rows, int64_t cols, int64_t ld, int box_rows) {
  PFN_cuTensorMapEncodeTiled_v12000 enc;
  NTG_TRY(encoder(&enc));
  if ((reinterpret_cast<uintptr_t>(base) & 15u) || ((ld * 2) & 15) || rows < 1 || cols < 1 || ld < cols) {
    set_error("tensor-core GEMM: operand not 16-byte aligned or bad shape (rows %lld cols %lld ld %lld)",
              (long long)rows, (long long)cols, (long long)ld);
    return NTG_ERR_INVALID;
  }
  cuuint64_t gdim[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t gstride[1] = {(cuuint64_t)(ld * 2)};
  cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  const CUresult r = enc(tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), gdim, gstride, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("tensor-core GEMM: cuTensorMapEncodeTiled failed (%d)", (int)r);
    return NTG_ERR_CUDA;
  }
  return NTG_OK;
}

template <int BN, int ST>
static int launch(const CUtensorMap& ta, const CUtensorMap& tb, const Epi& ep, int64_t M, int64_t N, int kb_total,
                  int kb_per_split, int splits, int* err, cudaStream_t s) {
  using Cg = Cfg<BN, ST>;
  static bool attr[64] = {};
  int dev = 0;
  NTG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev >= 0 && dev < 64 && !attr[dev]) {
    NTG_CUDA_TRY(cudaFuncSetAttribute(k_tc_gemm<BN, ST>, cudaFuncAttributeMaxDynamicSharedMemorySize, Cg::SMEM));
    attr[dev] = true;
  }
  dim3 grid((unsigned)((M + BM - 1) / BM), (unsigned)((N + BN - 1) / BN), (unsigned)splits);
  { k_tc_gemm<BN, ST><<<grid, kThreads, Cg::SMEM, s>>>(ta, tb, ep, M, N, kb_total, kb_per_split, err); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

}  // namespace tcg

// C = A B^T on the tensor cores (see the top of this file).  A: [M x K]
// (row stride lda), B: [N x K] (row stride ldb), BF16, 16-byte aligned rows.
// Outputs (any subset): FP32 C [M x ldc], BF16 Cb [M x ldcb], BF16
// transposed CbT ((m, n) at n * ldt + m); bias per column and ReLU applied
// to all of them.  splits > 1 divides K over that many CTAs per tile and
// needs split_buf (splits * M * N floats); its sum goes to C only
// (row-major, or transposed with ldc the leading dimension when
// transpose_c != 0).
int tc_gemm_bf16(const __nv_bfloat16* A, int64_t lda, const __nv_bfloat16* B, int64_t ldb, int64_t M, int64_t N,
                 int64_t K, float* C, int64_t ldc, __nv_bfloat16* Cb, int64_t ldcb, __nv_bfloat16* CbT, int64_t ldt,
                 const float* bias, int relu, int splits, float* split_buf, int transpose_c, int* err,
                 cudaStream_t s) {
  using namespace tcg;
  if (M < 1 || N < 1 || K < 1) {
    set_error("tensor-core GEMM: empty shape");
    return NTG_ERR_INVALID;
  }
  const int BN = N <= 64 ? 64 : (N <= 128 ? 128 : 256);
  CUtensorMap ta, tb;
  NTG_TRY(make_map(&ta, A, M, K, lda, BM));
  NTG_TRY(make_map(&tb, B, N, K, ldb, BN));
  const int kb_total = (int)((K + BK - 1) / BK);
  if (splits < 1) splits = 1;
  if (splits > kb_total) splits = kb_total;
  const int kb_per_split = (kb_total + splits - 1) / splits;
  splits = (kb_total + kb_per_split - 1) / kb_per_split;
  Epi ep{};
  if (splits > 1) {
    if (!split_buf || !C || Cb || CbT) {
      set_error("tensor-core GEMM: a split over K needs split_buf and an FP32 output only");
      return NTG_ERR_INVALID;
    }
    ep.C = split_buf;
    ep.ldc = N;
    ep.split = 1;
  } else {
    if (transpose_c) {
      set_error("tensor-core GEMM: transposed FP32 output needs a split over K");
      return NTG_ERR_INVALID;
    }
    ep.C = C;
    ep.ldc = ldc;
    ep.Cb = Cb;
    ep.ldcb = ldcb;
    ep.CbT = CbT;
    ep.ldt = ldt;
    ep.bias = bias;
    ep.relu = relu;
  }
  if (BN == 64) NTG_TRY((launch<64, 4>(ta, tb, ep, M, N, kb_total, kb_per_split, splits, err, s)));
  else if (BN == 128) NTG_TRY((launch<128, 3>(ta, tb, ep, M, N, kb_total, kb_per_split, splits, err, s)));
  else NTG_TRY((launch<256, 2>(ta, tb, ep, M, N, kb_total, kb_per_split, splits, err, s)));
  if (splits > 1) {
    { k_splitk_sum<<<grid_for(M * N, 256), 256, 0, s>>>(split_buf, splits, M, N, C, ldc, transpose_c, bias, relu); NTG_COUNT_LAUNCH(); }
    NTG_CUDA_TRY(cudaGetLastError());
  }
  return NTG_OK;
}

// error flag of the public entry point when the caller passes none: one
// static device int per GPU, its address looked up per device
static __device__ int g_tc_err;
static std::mutex g_tc_mu;
static int* g_tc_err_addr[64] = {};

static int tc_err_ptr(int** out) {
  int dev = 0;
  NTG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    set_error("ntg_gemm_bf16: device ordinal %d out of range", dev);
    return NTG_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(g_tc_mu);
  if (!g_tc_err_addr[dev]) {
    void* p = nullptr;
    NTG_CUDA_TRY(cudaGetSymbolAddress(&p, g_tc_err));
    g_tc_err_addr[dev] = static_cast<int*>(p);
  }
  *out = g_tc_err_addr[dev];
  return NTG_OK;
}

}  // namespace ntg

using namespace ntg;

extern "C" int ntg_gemm_bf16(const uint16_t* A_d, int64_t lda, const uint16_t* B_d, int64_t ldb, float* C_d,
                             int64_t ldc, int64_t M, int64_t N, int64_t K, int* err_d, void* stream) {
  clear_error();
  NTG_CHECK_ARG(A_d && B_d && C_d && ldc >= N, "ntg_gemm_bf16: bad argument");
  int* err = err_d;
  if (!err) NTG_TRY(tc_err_ptr(&err));
  return tc_gemm_bf16(reinterpret_cast<const __nv_bfloat16*>(A_d), lda, reinterpret_cast<const __nv_bfloat16*>(B_d),
                      ldb, M, N, K, C_d, ldc, nullptr, 0, nullptr, 0, nullptr, 0, 1, nullptr, 0, err,
                      (cudaStream_t)stream);
}
