// Overlapping additive Schwarz preconditioner with fast-diagonalisation (FDM)
// local solves, in FP32, for structured box meshes.
//
//   z = sum_e R_e^T  A~_e^{-1}  R_e r
//
// R_e gathers the assembled residual on element e extended by one node layer
// into each neighbour ((lx+2)^3 nodes); A~_e is the separable approximation of
// the local operator on that extended box,
//   h1 (Bz x By x Kx + Bz x Ky x Bx + Kz x By x Bx) + h2 (Bz x By x Bx),
// with 1D stiffness/mass matrices assembled from the element's GLL interval
// and one interval of the element's own length on each side (homogeneous
// Dirichlet one node further out), inverted through the generalised
// eigenvectors of each 1D pair (Lynch, Rice & Thomas 1964; Fischer 1997, "An
// overlapping Schwarz method for spectral element solution of the
// incompressible Navier-Stokes equations").  With the element's own length on
// all three intervals every element shares the reference pair (S^, lam^),
// scaled by its lengths.  Element lengths come from the node coordinates;
// h1/h2 are element means.
//
// Optional coarse level (two-level Schwarz): z += P A_c^{-1} P^T r on the
// element vertices (Q1), solved by fast diagonalisation; see the coarse-level
// section below.
//
// Reference context: Neko's pressure solves use a Schwarz-multigrid
// preconditioner ('hsmg', examples/rugby_ball/rugby_ball.case:46-52); this is
// its Schwarz part on the GLL grid and its coarse-grid part.
//
// Kernels per application: k_fdm (gather, six 1D transforms, coarse
// restriction), k_crs_restrict + six k_crs_mode directions (coarse solve), k_pull
// (prolongation of both levels, optional (r, z)), then the Dirichlet mask.
//
// Determinism: the prolongation is a pull -- every local node sums, in a fixed
// order, the extended results of the elements whose extended box covers it --
// so every copy of a shared node is bit-identical without a gather-scatter
// pass, and no atomics are involved.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

#include "common.cuh"
#include "reduce.cuh"
#include "schwarz.cuh"

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


// Extended residual -> FDM solve -> extended result for a batch of EPB
// elements per block.
//
// The local model of element e is the separable operator on its extended
// box with the element's own length h_d in each direction for the adjacent
// intervals too.  Then every element shares one pair of 1D generalised
// eigenvectors and eigenvalues, those of the reference interval (h = 2):
// S_d = S^ sqrt(2 / h_d) and lam_d = (4 / h_d^2) lam^, so
//   A_e^-1 = 8 / (hx hy hz) (S^ x S^ x S^) D_e^-1 (S^ x S^ x S^)^T,
//   D_e(a, b, c) = h1 (4 lam^_a / hx^2 + 4 lam^_b / hy^2 + 4 lam^_c / hz^2) + h2.
// (Using the neighbours' own lengths instead changed no iteration count on
// the deformed boxes measured.)  S^ sits in the kernel-parameter bank and is
// read at compile-time indices, so the transforms load no operator from
// memory; an element brings only its six scalars.
//
// A thread owns two 1D lines of an element's extended box, (u, v) and
// (u, v + LE/2).  Each direction pass loads a line from the shared tile,
// applies S^ (or its transpose) two outputs at a time with packed FP32 FMAs
// (__ffma2_rn: rows f, f+1 of S^ against the duplicated line value) and
// writes the line back in place, so a pass needs one buffer and one barrier.
//   per element: scalars (sx, sy, sz, c, h1, h2) = (4/hx^2, 4/hy^2, 4/hz^2,
//                8/(hx hy hz), h1, h2); tile A[a + RS b + PS c]
// Tile strides: lines of a warp are consecutive (u fastest).  (RS, PS) make
// the r and s passes (two each) free of bank conflicts and the tile stride
// TPER keeps warps that span two elements free as well; the single t pass
// takes two-way conflicts (no stride choice avoids all three passes).
// the reference interval's extended 1D eigenvectors, as output pairs
template <int LE>
struct FdmRef {
  float P[LE / 2][LE][2];  // forward:  P[f/2][p][f&1] = S^[p][f]
  float Q[LE / 2][LE][2];  // backward: Q[a/2][f][a&1] = S^[a][f]
  float lam[LE];
};

template <int LX>
struct FdmCfg {
  static constexpr int LE = LX + 2, LE2 = LE * LE, LE3 = LE2 * LE, TPE = LE2 / 2;
  static constexpr int RS = LX == 8 ? 17 : LX == 6 ? 9 : 7;
  static constexpr int PS = LX == 8 ? 170 : LX == 6 ? 72 : 43;
  static constexpr int SPAN = (LE - 1) * (1 + RS + PS) + 1;
  static constexpr int TPER = LX == 8 ? 1714 : LX == 6 ? 576 : 257;
  static constexpr int NSC = 8;  // per-element scalars (six used)
  static constexpr int EPB = LX == 4 ? 16 : LX == 8 ? 4 : 8, THREADS = EPB * TPE, MINB = 4;
  static constexpr int MINB_EO = LX == 8 ? 4 : 3;  // the even-odd form keeps the folded lines in registers
  // (lx = 8: four elements per block measured 4% faster at 64^3 than eight, 1.14 vs 1.19 ms)
  // coarse restriction partials (8 per thread): in the tile rows' padding
  // (a in [LE, RS), two rows per thread) when it is wide enough, else after the tiles
  static constexpr bool HOLES = 2 * (RS - LE) >= 8;
  static constexpr int RED = HOLES ? 0 : EPB * TPE * 8;
  static constexpr size_t SMEM = ((size_t)EPB * (NSC + TPER) + RED) * sizeof(float);
  static_assert(LE % 2 == 0 && TPER >= SPAN && THREADS <= 1024, "layout");
};

// slot v of thread tl's coarse partials (A: the element's tile, red: the
// block's partial region, el: element slot)
template <int LX>
__device__ __forceinline__ float* crs_slot(float* A, float* red, int el, int tl, int v) {
  using C = FdmCfg<LX>;
  if constexpr (C::HOLES) {
    constexpr int W = C::RS - C::LE;
    const int b = tl % C::LE, c = tl / C::LE + (v < W ? 0 : C::LE / 2);
    return A + C::LE + (v < W ? v : v - W) + C::RS * b + C::PS * c;
  } else {
    return red + (el * C::TPE + tl) * 8 + v;
  }
}

template <int LE>
__device__ __forceinline__ float2 dup(float v) { return make_float2(v, v); }

// out(line1, line2)[f * ST] = sum_p M[f][p] in2[p] for both lines of the
// thread; M as interleaved output pairs in shared memory (row pair fp:
// M[fp*2LE + 2p + k] = M[2fp + k][p]), read as float4 broadcasts
template <int LE, int ST>
__device__ __forceinline__ void fdm_pair(const float* __restrict__ M, const float2 (&in)[LE], float* d1, float* d2) {
#pragma unroll
  for (int fp = 0; fp < LE / 2; ++fp) {
    const float* row = M + fp * 2 * LE;
    float2 a0 = make_float2(0.f, 0.f), a1 = make_float2(0.f, 0.f);
#pragma unroll
    for (int p = 0; p < LE; p += 2) {
      const float4 m4 = *reinterpret_cast<const float4*>(row + 2 * p);
      a0 = __ffma2_rn(dup<LE>(m4.x), in[p], a0);
      a1 = __ffma2_rn(dup<LE>(m4.y), in[p], a1);
      a0 = __ffma2_rn(dup<LE>(m4.z), in[p + 1], a0);
      a1 = __ffma2_rn(dup<LE>(m4.w), in[p + 1], a1);
    }
    d1[(2 * fp) * ST] = a0.x;
    d2[(2 * fp) * ST] = a0.y;
    d1[(2 * fp + 1) * ST] = a1.x;
    d2[(2 * fp + 1) * ST] = a1.y;
  }
}

// the same into registers
template <int LE>
__device__ __forceinline__ void fdm_pair_reg(const float* __restrict__ M, const float2 (&in)[LE], float2 (&out)[LE]) {
#pragma unroll
  for (int fp = 0; fp < LE / 2; ++fp) {
    const float* row = M + fp * 2 * LE;
    float2 a0 = make_float2(0.f, 0.f), a1 = make_float2(0.f, 0.f);
#pragma unroll
    for (int p = 0; p < LE; p += 2) {
      const float4 m4 = *reinterpret_cast<const float4*>(row + 2 * p);
      a0 = __ffma2_rn(dup<LE>(m4.x), in[p], a0);
      a1 = __ffma2_rn(dup<LE>(m4.y), in[p], a1);
      a0 = __ffma2_rn(dup<LE>(m4.z), in[p + 1], a0);
      a1 = __ffma2_rn(dup<LE>(m4.w), in[p + 1], a1);
    }
    out[2 * fp] = a0;
    out[2 * fp + 1] = a1;
  }
}

// Even-odd forms of the same transforms.  The reference extended interval
// is symmetric about its centre, so its eigenvectors alternate between
// symmetric (f even) and antisymmetric (f odd): S[LE-1-p][f] = (-1)^f S[p][f]
// (checked on the host before this path is chosen).  Then
//   forward  y_f = sum_{p<H} S[p][f] (x_p + (-1)^f x_{LE-1-p}),
//   backward x_p = E_p + O_p, x_{LE-1-p} = E_p - O_p with
//            E_p = sum_{f even} S[p][f] z_f, O_p = sum_{f odd} S[p][f] z_f,
// half the FMAs of the full LE x LE products.  Both read the forward pair
// table M = P (M[fp*2LE + 2p + k] = S[p][2fp + k]) at p < H only.
template <int LE>
__device__ __forceinline__ void eo_fold(float2 (&in)[LE]) {  // in[p] <- x_p + x_q, in[q] <- x_p - x_q (q = LE-1-p)
#pragma unroll
  for (int p = 0; p < LE / 2; ++p) {
    const float2 a = in[p], b = in[LE - 1 - p];
    in[p] = make_float2(a.x + b.x, a.y + b.y);
    in[LE - 1 - p] = make_float2(a.x - b.x, a.y - b.y);
  }
}
template <int LE, int ST>
__device__ __forceinline__ void fdm_fwd_eo(const float* __restrict__ M, float2 (&in)[LE], float* d1, float* d2) {
  constexpr int H = LE / 2;
  eo_fold<LE>(in);
#pragma unroll
  for (int fp = 0; fp < H; ++fp) {
    const float* row = M + fp * 2 * LE;
    float2 a0 = make_float2(0.f, 0.f), a1 = make_float2(0.f, 0.f);
#pragma unroll
    for (int p = 0; p < H; ++p) {
      const float2 m2 = *reinterpret_cast<const float2*>(row + 2 * p);
      a0 = __ffma2_rn(dup<LE>(m2.x), in[p], a0);
      a1 = __ffma2_rn(dup<LE>(m2.y), in[LE - 1 - p], a1);
    }
    d1[(2 * fp) * ST] = a0.x;
    d2[(2 * fp) * ST] = a0.y;
    d1[(2 * fp + 1) * ST] = a1.x;
    d2[(2 * fp + 1) * ST] = a1.y;
  }
}
template <int LE>
__device__ __forceinline__ void fdm_fwd_eo_reg(const float* __restrict__ M, float2 (&in)[LE], float2 (&out)[LE]) {
  constexpr int H = LE / 2;
  eo_fold<LE>(in);
#pragma unroll
  for (int fp = 0; fp < H; ++fp) {
    const float* row = M + fp * 2 * LE;
    float2 a0 = make_float2(0.f, 0.f), a1 = make_float2(0.f, 0.f);
#pragma unroll
    for (int p = 0; p < H; ++p) {
      const float2 m2 = *reinterpret_cast<const float2*>(row + 2 * p);
      a0 = __ffma2_rn(dup<LE>(m2.x), in[p], a0);
      a1 = __ffma2_rn(dup<LE>(m2.y), in[LE - 1 - p], a1);
    }
    out[2 * fp] = a0;
    out[2 * fp + 1] = a1;
  }
}
template <int LE, int ST>
__device__ __forceinline__ void fdm_bwd_eo(const float* __restrict__ M, const float2 (&in)[LE], float* d1, float* d2) {
  constexpr int H = LE / 2;
#pragma unroll
  for (int p = 0; p < H; ++p) {
    float2 e = make_float2(0.f, 0.f), o = make_float2(0.f, 0.f);
#pragma unroll
    for (int fp = 0; fp < H; ++fp) {
      const float2 m2 = *reinterpret_cast<const float2*>(M + fp * 2 * LE + 2 * p);
      e = __ffma2_rn(dup<LE>(m2.x), in[2 * fp], e);
      o = __ffma2_rn(dup<LE>(m2.y), in[2 * fp + 1], o);
    }
    d1[p * ST] = e.x + o.x;
    d2[p * ST] = e.y + o.y;
    d1[(LE - 1 - p) * ST] = e.x - o.x;
    d2[(LE - 1 - p) * ST] = e.y - o.y;
  }
}

// GEN: a general mesh (Ex = nelv, Ey = Ez = 1): the ghost layers come from
// the face-neighbour table (edge and corner positions stay zero) and the
// coarse restriction weighs nodes by minv = 1 / multiplicity.
template <int LX, bool EO, bool GEN>
__global__ void __launch_bounds__(FdmCfg<LX>::THREADS, EO ? FdmCfg<LX>::MINB_EO : FdmCfg<LX>::MINB)
    k_fdm(const float* __restrict__ r, float* __restrict__ ze, const float* __restrict__ esc, int Ex, int Ey,
          int Ez, const Scalars* sc, float* __restrict__ corner, CoarsePhi ph,
          const int32_t* __restrict__ ghost, const float* __restrict__ minv,
          const __grid_constant__ FdmRef<LX + 2> R) {
  using C = FdmCfg<LX>;
  constexpr int LE = C::LE, LE2 = C::LE2, LE3 = C::LE3, N = LX - 1, RS = C::RS, PS = C::PS, TPE = C::TPE;
  constexpr int EPB = C::EPB, NSC = C::NSC, LX2 = LX * LX, LX3 = LX2 * LX, H = LE / 2;
  if (sc && sc->done) return;
  extern __shared__ __align__(16) float smem[];
  const int nelv = Ex * Ey * Ez;
  const int tid = threadIdx.x, el = tid / TPE, tl = tid - el * TPE;
  const int u = tl % LE, v1 = tl / LE, v2 = v1 + H;  // lines (u, v1) and (u, v2); tl + TPE = u + LE v2
  float* es = smem + el * NSC;
  float* A = smem + EPB * NSC + el * C::TPER;
  float* red = smem + EPB * (NSC + C::TPER);
  __shared__ float sp[2][LX];  // Q1 basis at the GLL nodes
  __shared__ __align__(16) float sP[LE2], sQ[LE2];  // reference pairs (forward, backward)
  __shared__ float slam[LE];                        // reference eigenvalues
  if (tid == 0) {
#pragma unroll
    for (int t = 0; t < 2 * LX; ++t) sp[t / LX][t % LX] = ph.p[t / LX][t % LX];  // constant indices
  }
  for (int t = tid; t < LE2; t += blockDim.x) {
    sP[t] = (&R.P[0][0][0])[t];
    sQ[t] = (&R.Q[0][0][0])[t];
  }
  if (tid < LE) slam[tid] = R.lam[tid];
  __syncthreads();
  float2 in[LE];
  for (int e0 = blockIdx.x * EPB; e0 < nelv; e0 += gridDim.x * EPB) {
    const int e = e0 + el;
    const bool live = e < nelv;
    if (tl < NSC) es[tl] = live ? esc[(int64_t)e * NSC + tl] : 1.f;
    // gather R_e r: columns (a, b) = (u, v1), (u, v2) over c
    if (GEN && live) {
      const int64_t eb = (int64_t)e * LX3;
      const int32_t* gh = ghost + eb / LX * 6;  // (e * 6) * LX2
      const bool ia = u >= 1 && u <= LX;
      float part[8];
#pragma unroll
      for (int v = 0; v < 8; ++v) part[v] = 0.f;
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const int vb = q ? v2 : v1;
        const bool ib = vb >= 1 && vb <= LX;
        float* Ac = A + u + RS * vb;
        if (ia && ib) {
          // own column with the t-face ghosts at its ends
          const int i = u - 1, j = vb - 1;
          const int32_t g0 = gh[4 * LX2 + i + LX * j], g1 = gh[5 * LX2 + i + LX * j];
          Ac[0] = g0 >= 0 ? r[g0] : 0.f;
          Ac[PS * (LE - 1)] = g1 >= 0 ? r[g1] : 0.f;
          const float* rc = r + eb + i + LX * j;
          const float* mc = minv + eb + i + LX * j;
          float s0 = 0.f, s1 = 0.f;
#pragma unroll
          for (int c = 1; c < LE - 1; ++c) {
            const float val = rc[(c - 1) * LX2];
            Ac[PS * c] = val;
            if (corner) {
              const float wv = val * mc[(c - 1) * LX2];
              s0 = fmaf(sp[0][c - 1], wv, s0);
              s1 = fmaf(sp[1][c - 1], wv, s1);
            }
          }
          if (corner) {
#pragma unroll
            for (int v = 0; v < 8; ++v) part[v] = fmaf(sp[v & 1][i] * sp[(v >> 1) & 1][j], (v >> 2) ? s1 : s0, part[v]);
          }
        } else if (ia || ib) {
          // an r-face (a at the border) or s-face (b at the border) ghost column
          const int32_t* gf = ia ? gh + (vb == 0 ? 2 : 3) * LX2 + (u - 1) : gh + (u == 0 ? 0 : 1) * LX2 + (vb - 1);
          Ac[0] = 0.f;
          Ac[PS * (LE - 1)] = 0.f;
#pragma unroll
          for (int c = 1; c < LE - 1; ++c) {
            const int32_t gi = gf[LX * (c - 1)];
            Ac[PS * c] = gi >= 0 ? r[gi] : 0.f;
          }
        } else {
#pragma unroll
          for (int c = 0; c < LE; ++c) Ac[PS * c] = 0.f;
        }
      }
      if (corner) {
#pragma unroll
        for (int v = 0; v < 8; ++v) *crs_slot<LX>(A, red, el, tl, v) = part[v];
      }
    }
    if (!GEN && live) {
      const int exy = e / Ex, ex = e - exy * Ex, ez = exy / Ey, ey = exy - ez * Ey;
      int i = u - 1, dx = 0;
      if (i < 0) { dx = -1; i = N - 1; } else if (i > N) { dx = 1; i = 1; }
      const int nx = ex + dx;
      const int64_t zs = (int64_t)Ex * Ey * LX3;
      float part[8];
#pragma unroll
      for (int v = 0; v < 8; ++v) part[v] = 0.f;
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const int vb = q ? v2 : v1;
        int j = vb - 1, dy = 0;
        if (j < 0) { dy = -1; j = N - 1; } else if (j > N) { dy = 1; j = 1; }
        const int ny = ey + dy;
        const bool okxy = nx >= 0 && nx < Ex && ny >= 0 && ny < Ey;
        const float* rc = r + (int64_t)(nx + Ex * (ny + Ey * ez)) * LX3 + i + LX * j;
        float* Ac = A + u + RS * vb;
        Ac[0] = okxy && ez > 0 ? rc[(N - 1) * LX2 - zs] : 0.f;
        // own-element columns also feed the coarse restriction:
        // sum_k phi_vz(k) r / multiplicity, per column, then x / y weights
        float s0 = 0.f, s1 = 0.f;
#pragma unroll
        for (int c = 1; c < LE - 1; ++c) {
          const float val = okxy ? rc[(c - 1) * LX2] : 0.f;
          Ac[PS * c] = val;
          const int k = c - 1;
          const float wz = ((k == 0 && ez > 0) || (k == N && ez < Ez - 1)) ? 0.5f : 1.f;
          s0 = fmaf(sp[0][k] * wz, val, s0);
          s1 = fmaf(sp[1][k] * wz, val, s1);
        }
        Ac[PS * (LE - 1)] = okxy && ez < Ez - 1 ? rc[LX2 + zs] : 0.f;
        if (corner && dx == 0 && dy == 0) {
          const float wx = ((i == 0 && ex > 0) || (i == N && ex < Ex - 1)) ? 0.5f : 1.f;
          const float wy = ((j == 0 && ey > 0) || (j == N && ey < Ey - 1)) ? 0.5f : 1.f;
#pragma unroll
          for (int v = 0; v < 8; ++v)
            part[v] = fmaf(sp[v & 1][i] * wx * (sp[(v >> 1) & 1][j] * wy), (v >> 2) ? s1 : s0, part[v]);
        }
      }
      if (corner) {
#pragma unroll
        for (int v = 0; v < 8; ++v) *crs_slot<LX>(A, red, el, tl, v) = part[v];
      }
    }
    __syncthreads();
    // r forward: lines (b, c) = (u, v) along a
    {
      float* l1 = A + RS * u + PS * v1;
      float* l2 = A + RS * u + PS * v2;
#pragma unroll
      for (int p = 0; p < LE; ++p) in[p] = make_float2(l1[p], l2[p]);
      if constexpr (EO) fdm_fwd_eo<LE, 1>(sP, in, l1, l2);
      else fdm_pair<LE, 1>(sP, in, l1, l2);
    }
    __syncthreads();
    // s forward: lines (a, c) = (u, v) along b
    {
      float* l1 = A + u + PS * v1;
      float* l2 = A + u + PS * v2;
#pragma unroll
      for (int p = 0; p < LE; ++p) in[p] = make_float2(l1[RS * p], l2[RS * p]);
      if constexpr (EO) fdm_fwd_eo<LE, RS>(sP, in, l1, l2);
      else fdm_pair<LE, RS>(sP, in, l1, l2);
    }
    __syncthreads();
    // t forward, scale (c_e / D_e), t back: lines (a, b) = (u, v) along c
    {
      float* l1 = A + u + RS * v1;
      float* l2 = A + u + RS * v2;
      const float sx = es[0], sy = es[1], sz = es[2], ce = es[3], h1 = es[4], h2 = es[5];
      const float la1 = h1 * (sx * slam[u] + sy * slam[v1]) + h2, la2 = h1 * (sx * slam[u] + sy * slam[v2]) + h2;
#pragma unroll
      for (int p = 0; p < LE; ++p) in[p] = make_float2(l1[PS * p], l2[PS * p]);
      float2 t[LE];
      if constexpr (EO) fdm_fwd_eo_reg<LE>(sP, in, t);
      else fdm_pair_reg<LE>(sP, in, t);
#pragma unroll
      for (int f = 0; f < LE; ++f) {
        const float lf = h1 * sz * slam[f];
        in[f] = make_float2(__fdividef(ce * t[f].x, la1 + lf), __fdividef(ce * t[f].y, la2 + lf));
      }
      if constexpr (EO) fdm_bwd_eo<LE, PS>(sP, in, l1, l2);
      else fdm_pair<LE, PS>(sQ, in, l1, l2);
    }
    __syncthreads();
    // s back
    {
      float* l1 = A + u + PS * v1;
      float* l2 = A + u + PS * v2;
#pragma unroll
      for (int p = 0; p < LE; ++p) in[p] = make_float2(l1[RS * p], l2[RS * p]);
      if constexpr (EO) fdm_bwd_eo<LE, RS>(sP, in, l1, l2);
      else fdm_pair<LE, RS>(sQ, in, l1, l2);
    }
    __syncthreads();
    // r back
    {
      float* l1 = A + RS * u + PS * v1;
      float* l2 = A + RS * u + PS * v2;
#pragma unroll
      for (int p = 0; p < LE; ++p) in[p] = make_float2(l1[p], l2[p]);
      if constexpr (EO) fdm_bwd_eo<LE, 1>(sP, in, l1, l2);
      else fdm_pair<LE, 1>(sQ, in, l1, l2);
    }
    __syncthreads();
    // coarse restriction of the element: 8 threads sum the partials in order
    if (corner && live && tl < 8) {
      float acc = 0.f;
      for (int t = 0; t < TPE; ++t) acc += *crs_slot<LX>(A, red, el, t, tl);
      corner[(int64_t)e * 8 + tl] = acc;
    }
    // copy-out: columns (a, b) of ze[e][a + LE b + LE2 c] (consecutive lines -> consecutive addresses)
    if (live) {
#pragma unroll
      for (int c = 0; c < LE; ++c) {
        ze[(int64_t)e * LE3 + tl + LE2 * c] = A[u + RS * v1 + PS * c];
        ze[(int64_t)e * LE3 + tl + TPE + LE2 * c] = A[u + RS * v2 + PS * c];
      }
    }
    __syncthreads();
  }
}

// per-element scalars of the local model from the element lengths and the
// h1 / h2 means: (4/hx^2, 4/hy^2, 4/hz^2, 8/(hx hy hz), h1, h2)
__global__ void k_elem_scalars(const float* __restrict__ hl, const float* __restrict__ hc, float* __restrict__ esc,
                               int64_t nelv) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nelv; e += (int64_t)gridDim.x * blockDim.x) {
    const float hx = hl[3 * e], hy = hl[3 * e + 1], hz = hl[3 * e + 2];
    float* o = esc + 8 * e;
    o[0] = 4.f / (hx * hx);
    o[1] = 4.f / (hy * hy);
    o[2] = 4.f / (hz * hz);
    o[3] = 8.f / (hx * hy * hz);
    o[4] = hc[2 * e];
    o[5] = hc[2 * e + 1];
    o[6] = 0.f;
    o[7] = 0.f;
  }
}

// ---------------------------------------------------------------------------
// Coarse level: Q1 on the element vertices of the box.
//
//   z += P A_c^{-1} P^T r
//
// P interpolates vertex values trilinearly (in reference coordinates) to the
// GLL nodes; P^T r sums, per vertex, phi_v(node) r(node) / multiplicity over
// the local nodes of the adjacent elements (each global node once).  A_c is
// the separable Q1 operator on the vertex grid,
//   h1 (Mz x My x Kx + Mz x Ky x Mx + Kz x My x Mx) + h2 (Mz x My x Mx),
// with 1D linear-element stiffness K and consistent mass M assembled from the
// mean element length of each slab -- the Galerkin operator P^T A P itself on
// an undeformed box with constant h1, h2 -- and Dirichlet vertices removed on
// fully masked faces.  It is inverted by fast diagonalisation (three 1D
// generalised eigenproblems); a singular (all-Neumann) mode gets zero.
// ---------------------------------------------------------------------------
struct CoarseDims {
  int Ex, Ey, Ez;         // elements per direction (vertex grid (Ex+1) x (Ey+1) x (Ez+1))
  int lo[3], m[3];        // first active vertex and active count per direction
  float h1, h2, dmin;     // coefficients; eigenvalue sums below dmin are the null mode
};

// restricted residual on the active vertex grid (x fastest): per vertex the
// corner sums of its adjacent elements, in ascending element order
__global__ void k_crs_restrict(const float* __restrict__ corner, float* __restrict__ rc, CoarseDims d,
                               const Scalars* sc) {
  if (sc && sc->done) return;
  const int64_t total = (int64_t)d.m[0] * d.m[1] * d.m[2];
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int gx = d.lo[0] + (int)(q % d.m[0]), gy = d.lo[1] + (int)((q / d.m[0]) % d.m[1]);
    const int gz = d.lo[2] + (int)(q / ((int64_t)d.m[0] * d.m[1]));
    float acc = 0.f;
    for (int ez = gz - 1; ez <= gz; ++ez) {
      if (ez < 0 || ez >= d.Ez) continue;
      for (int ey = gy - 1; ey <= gy; ++ey) {
        if (ey < 0 || ey >= d.Ey) continue;
        for (int ex = gx - 1; ex <= gx; ++ex) {
          if (ex < 0 || ex >= d.Ex) continue;
          const int64_t e = ex + (int64_t)d.Ex * (ey + (int64_t)d.Ey * ez);
          acc += corner[e * 8 + (gx - ex) + 2 * (gy - ey) + 4 * (gz - ez)];
        }
      }
    }
    rc[q] = acc;
  }
}

// One direction of the coarse fast diagonalisation on the active vertex
// grid, one thread per output: forward t_f = sum_x S[x][f] in_x, back
// out_x = sum_f S[x][f] in_f (from the stored transpose), along direction
// DIR (0 = x, 1 = y, 2 = z).
// SCALE (z forward): divided by the eigenvalue sum, the null mode dropped;
// UC (x back): written into the full vertex grid.  The operands stay in L2
// (the grid is a few MB) and the lines of a warp share each S entry.
template <int DIR, bool BACK, bool SCALE, bool UC>
__global__ void __launch_bounds__(256)
    k_crs_mode(const float* __restrict__ in, float* __restrict__ out, const float* __restrict__ S,
               const float* __restrict__ lam, CoarseDims d, const Scalars* sc) {
  if (sc && sc->done) return;
  const int m0 = d.m[0], m1 = d.m[1], m = d.m[DIR];
  const int64_t stride = DIR == 0 ? 1 : DIR == 1 ? m0 : (int64_t)m0 * m1;
  const int64_t total = (int64_t)m0 * m1 * d.m[2];
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int t = (int)((q / stride) % m);
    const float* src = in + (q - (int64_t)t * stride);
    float acc = 0.f;
    // forward S[u][t], back S^T[u][t] = S[t][u]: consecutive t read consecutive entries
    const float* Mt = S + (BACK ? (int64_t)m * m : 0) + t;
    for (int u = 0; u < m; ++u) acc = fmaf(Mt[(int64_t)u * m], src[u * stride], acc);
    const int x = (int)(q % m0), y = (int)((q / m0) % m1), z = (int)(q / ((int64_t)m0 * m1));
    if (SCALE) {
      const float D = d.h1 * (lam[x] + lam[m0 + y] + lam[m0 + m1 + z]) + d.h2;
      acc = D > d.dmin ? acc / D : 0.f;
    }
    if (UC) {
      const int nx = d.Ex + 1, ny = d.Ey + 1;
      out[(d.lo[0] + x) + (int64_t)nx * ((d.lo[1] + y) + (int64_t)ny * (d.lo[2] + z))] = acc;
    } else {
      out[q] = acc;
    }
  }
}

// what the pull needs to add the prolongated coarse correction
struct CoarseView {
  const float* uc;  // full vertex grid, Dirichlet vertices zero; null: no coarse level
  CoarsePhi ph;
  const float* dw;  // additive diagonal term (mass fraction / diagonal); null: none
};

// dw = (h2 B)_assembled / diag(A)^2: the node's mass-dominance fraction
// w = (h2 B) / diag(A) in [0, 1] times the inverse diagonal (dinv = 1 on
// masked nodes, whose result the mask zeroes anyway)
__global__ void k_mass_term(const double* __restrict__ hBa, const double* __restrict__ dinv, float* __restrict__ dw,
                            int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double w = fmin(fmax(hBa[i] * dinv[i], 0.0), 1.0);
    dw[i] = (float)(w * dinv[i]);
  }
}

// Assembling prolongation: each local node sums the extended results of ALL
// elements whose extended box covers its global node, in ascending element
// order, so every copy of a shared node gets the bit-identical sum and no
// gather-scatter pass is needed.  Per direction a node has one covering
// element (its own) or two (own and the lower or upper neighbour); the
// 2x2x2 combinations are summed z-major, y, x (= ascending element index).
// A thread handles one row (j, k) of an element: per covering (y, z) choice
// it reads the covering element's extended row (LE values, float2 pairs) and
// the adjacent pair of each x neighbour.  DOT: also (r, z)_mult, summed over
// each node's owning copy (no multiplicity stream), reduced deterministically
// and finalised by FinRz (the mask applied afterwards does not change it: r
// vanishes on masked nodes); the mult argument only selects this variant.
// cv.uc: plus the trilinear prolongation of the coarse correction.
template <int LX, bool DOT>
__global__ void __launch_bounds__(256, 4)
    k_pull(const float* __restrict__ ze, float* __restrict__ z, int Ex, int Ey, int Ez,
           const float* __restrict__ r, const float* __restrict__ mult, int mode,
           double* __restrict__ part, Scalars* sc, CoarseView cv) {
  constexpr int N = LX - 1, LE = LX + 2, LE2 = LE * LE, LE3 = LE2 * LE, LX2 = LX * LX, LX3 = LX2 * LX;
  static_assert(N >= 3 && LE % 2 == 0, "one neighbour per direction; rows of float2 pairs");
  if (sc && sc->done) return;
  __shared__ float sp[2][LX];
  if (threadIdx.x == 0) {
#pragma unroll
    for (int t = 0; t < 2 * LX; ++t) sp[t / LX][t % LX] = cv.ph.p[t / LX][t % LX];  // constant indices
  }
  __syncthreads();
  const int64_t nrow = (int64_t)Ex * Ey * Ez * LX2;
  const int64_t sy = (int64_t)Ex * LE3, sz = (int64_t)Ex * Ey * LE3;
  float rz = 0.f;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nrow; t += (int64_t)gridDim.x * blockDim.x) {
    const int e = (int)(t / LX2);
    const int m = (int)(t - (int64_t)e * LX2), j = m % LX, k = m / LX;
    const int64_t o = (int64_t)e * LX3 + (int64_t)m * LX;  // first node of the row in z / r / mult
    float rv[LX];
    if (DOT || cv.dw) {
#pragma unroll
      for (int q = 0; q < LX; q += 2) {
        const float2 r2 = *reinterpret_cast<const float2*>(r + o + q);
        rv[q] = r2.x; rv[q + 1] = r2.y;
      }
    }
    const int exy = e / Ex, cx = e - exy * Ex, cz = exy / Ey, cy = exy - cz * Ey;
    const bool ly = j <= 1 && cy > 0, hy = j >= N - 1 && cy < Ey - 1;
    const bool lz = k <= 1 && cz > 0, hz = k >= N - 1 && cz < Ez - 1;
    const int64_t y0 = ly ? (cy - 1) * sy + LE * (N + 1 + j) : cy * sy + LE * (j + 1);
    const int64_t y1 = ly ? cy * sy + LE * (j + 1) : (cy + 1) * sy + LE * (j + 1 - N);
    const int64_t z0 = lz ? (cz - 1) * sz + LE2 * (N + 1 + k) : cz * sz + LE2 * (k + 1);
    const int64_t z1 = lz ? cz * sz + LE2 * (k + 1) : (cz + 1) * sz + LE2 * (k + 1 - N);
    const int ny = (ly || hy) ? 2 : 1, nz = (lz || hz) ? 2 : 1;
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
        // the covering row of element (cx, ., .) and its x neighbours' adjacent pairs
        const float* row = ze + (vz ? z1 : z0) + (vy ? y1 : y0) + (int64_t)cx * LE3;
        float w[LE];
#pragma unroll
        for (int a = 0; a < LE; a += 2) {
          const float2 p2 = *reinterpret_cast<const float2*>(row + a);
          w[a] = p2.x; w[a + 1] = p2.y;
        }
        const float2 lo = xl ? *reinterpret_cast<const float2*>(row - LE3 + (LE - 2)) : make_float2(0.f, 0.f);
        const float2 hi = xh ? *reinterpret_cast<const float2*>(row + LE3) : make_float2(0.f, 0.f);
        // per node: lower neighbour, own, upper neighbour (ascending element order)
        if (xl) { acc[0] += lo.x; acc[1] += lo.y; }
#pragma unroll
        for (int i = 0; i < LX; ++i) acc[i] += w[i + 1];
        if (xh) { acc[N - 1] += hi.x; acc[N] += hi.y; }
      }
    }
    if (cv.uc) {
      // + P u_c: trilinear in the element's eight vertices (z-, y-, x-major);
      // on a shared face the other element's vertices have weight exactly 0,
      // so every copy of a node sums the same terms in the same order
      const int nx = Ex + 1, nyv = Ey + 1;
      const float* u0 = cv.uc + cx + (int64_t)nx * (cy + (int64_t)nyv * cz);
      float cvz[2][2][2];
#pragma unroll
      for (int vz = 0; vz < 2; ++vz)
#pragma unroll
        for (int vy = 0; vy < 2; ++vy)
#pragma unroll
          for (int vx = 0; vx < 2; ++vx) cvz[vz][vy][vx] = u0[vx + (int64_t)nx * (vy + (int64_t)nyv * vz)];
      const float pj[2] = {sp[0][j], sp[1][j]}, pk[2] = {sp[0][k], sp[1][k]};
#pragma unroll
      for (int i = 0; i < LX; ++i) {
        float c = 0.f;
#pragma unroll
        for (int vz = 0; vz < 2; ++vz)
#pragma unroll
          for (int vy = 0; vy < 2; ++vy)
#pragma unroll
            for (int vx = 0; vx < 2; ++vx) c += (sp[vx][i] * pj[vy] * pk[vz]) * cvz[vz][vy][vx];
        acc[i] += c;
      }
    }
    if (cv.dw) {
#pragma unroll
      for (int q = 0; q < LX; q += 2) {
        const float2 d2 = *reinterpret_cast<const float2*>(cv.dw + o + q);
        acc[q] += d2.x * rv[q];
        acc[q + 1] += d2.y * rv[q + 1];
      }
    }
#pragma unroll
    for (int q = 0; q < LX; q += 2) *reinterpret_cast<float2*>(z + o + q) = make_float2(acc[q], acc[q + 1]);
    if constexpr (DOT) {
      // each global node once, from the element that owns it (the copy with
      // no lower neighbour in any direction): the sum over unique nodes that
      // the mult-weighted sum over local copies equals, without the mult stream
      if ((j > 0 || cy == 0) && (k > 0 || cz == 0)) {
#pragma unroll
        for (int i = 0; i < LX; ++i)
          if (i > 0 || cx == 0) rz += rv[i] * acc[i];
      }
    }
  }
  if constexpr (DOT) {
    double v[1] = {(double)rz};
    grid_reduce<1>(v, part, sc, FinRz{mode});
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
  float* hld = nullptr;  // E x 3 element lengths (device)
  float* esc = nullptr;  // E x 8 per-element scalars of the local model
  float* hc = nullptr;   // E x 2 (h1, h2 element means)
  std::vector<double> Sref, lamref;  // reference (h = 2) extended 1D eigenpairs
  float* ze = nullptr;   // E x LE^3 extended results
  int fdm_grid = 0;      // persistent grid of the FDM kernel (blocks resident on all SMs)
  std::vector<double> hl;  // element lengths (host)
  // coarse level (Q1 on the vertex grid); the FDM kernel writes its restriction
  int coarse = 0, coarse_ready = 0;
  ntg::sw::CoarseDims cd{};
  ntg::sw::CoarsePhi ph{};
  float* cS[3] = {nullptr, nullptr, nullptr};  // m_d x m_d eigenvectors S[x][f], then S^T[f][x]
  float* clam = nullptr;                       // m0 + m1 + m2 eigenvalues
  float* corner = nullptr;                     // E x 8 restricted corner sums
  float* cwork = nullptr;                      // 2 x m0 m1 m2: the coarse residual through its transforms
  float* uc = nullptr;                         // (Ex+1)(Ey+1)(Ez+1) coarse correction
  int mass_term = 0;
  float* dw = nullptr;  // additive diagonal term of the Brinkman mass part (n)
  // lx = 8: FDM local solves on the tensor cores (schwarz_tc.cu) when on
  ntg::sw::FdmTc ftc{};
  int fdm_tc = 0;
  int fdm_eo = 0;  // even-odd 1D transforms (chosen when the reference eigenvectors have parity)
  // general mesh: face-neighbour tables, global-node prolongation, Galerkin coarse level
  ntg::sw::GenTopo* gen = nullptr;
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
  dev_free(s->hld); dev_free(s->esc); dev_free(s->hc); dev_free(s->ze);
  for (int d = 0; d < 3; ++d) dev_free(s->cS[d]);
  dev_free(s->clam); dev_free(s->corner); dev_free(s->cwork); dev_free(s->uc); dev_free(s->dw);
  ntg::sw::fdm_tc_free(&s->ftc);
  ntg::sw::gen_free(s->gen);
  s->gen = nullptr;
}

// Generalised symmetric eigenproblem K s = lam M s (M SPD, n small): with
// M = L L^T, C = L^-1 K L^-T = V diag(lam) V^T and S = L^-T V, so that
// S^T M S = I and S^T K S = diag(lam).  S row-major (S[i * n + f]).
static void gen_eig(int n, const std::vector<double>& K, const std::vector<double>& M, std::vector<double>& S,
                    std::vector<double>& lam) {
  std::vector<double> L(n * n, 0.0);
  for (int j = 0; j < n; ++j) {
    double d = M[j * n + j];
    for (int k = 0; k < j; ++k) d -= L[j * n + k] * L[j * n + k];
    L[j * n + j] = std::sqrt(d);
    for (int i = j + 1; i < n; ++i) {
      double v = M[i * n + j];
      for (int k = 0; k < j; ++k) v -= L[i * n + k] * L[j * n + k];
      L[i * n + j] = v / L[j * n + j];
    }
  }
  // X = L^-1 K (forward substitution per column), C = X L^-T = (L^-1 X^T)^T
  std::vector<double> X(n * n), C(n * n), V(n * n), w(n);
  for (int c = 0; c < n; ++c)
    for (int i = 0; i < n; ++i) {
      double v = K[i * n + c];
      for (int k = 0; k < i; ++k) v -= L[i * n + k] * X[k * n + c];
      X[i * n + c] = v / L[i * n + i];
    }
  for (int r = 0; r < n; ++r)  // row r of C: solve L y = X[r, :]^T
    for (int i = 0; i < n; ++i) {
      double v = X[r * n + i];
      for (int k = 0; k < i; ++k) v -= L[i * n + k] * C[r * n + k];
      C[r * n + i] = v / L[i * n + i];
    }
  for (int i = 0; i < n; ++i)  // symmetrise against rounding
    for (int j = i + 1; j < n; ++j) C[i * n + j] = C[j * n + i] = 0.5 * (C[i * n + j] + C[j * n + i]);
  sw::jacobi_eig(n, C.data(), V.data(), w.data());
  // S = L^-T V: back substitution per column
  S.assign(n * n, 0.0);
  for (int f = 0; f < n; ++f)
    for (int i = n - 1; i >= 0; --i) {
      double v = V[i * n + f];
      for (int k = i + 1; k < n; ++k) v -= L[k * n + i] * S[k * n + f];
      S[i * n + f] = v / L[i * n + i];
    }
  lam = w;
}

// Order the reference eigenpairs by parity: the interval is symmetric about
// its centre, so each eigenvector (distinct eigenvalues) is symmetric or
// antisymmetric; put the symmetric ones at even positions and the
// antisymmetric ones at odd positions, each group by ascending eigenvalue,
// as the even-odd transforms expect.  A reordering of eigenpairs leaves the
// local solve unchanged.  Left as is when the split is not half and half.
static void parity_order(int LE, std::vector<double>& S, std::vector<double>& lam) {
  double smax = 0.0;
  for (double v : S) smax = std::max(smax, std::fabs(v));
  std::vector<int> sym, anti;
  for (int f = 0; f < LE; ++f) {
    double ds = 0.0, da = 0.0;
    for (int p = 0; p < LE; ++p) {
      ds = std::max(ds, std::fabs(S[(LE - 1 - p) * LE + f] - S[p * LE + f]));
      da = std::max(da, std::fabs(S[(LE - 1 - p) * LE + f] + S[p * LE + f]));
    }
    if (ds <= 1e-9 * smax) sym.push_back(f);
    else if (da <= 1e-9 * smax) anti.push_back(f);
    else return;
  }
  if ((int)sym.size() != LE / 2 || (int)anti.size() != LE / 2) return;
  auto by_lam = [&](int a, int b) { return lam[a] < lam[b]; };
  std::sort(sym.begin(), sym.end(), by_lam);
  std::sort(anti.begin(), anti.end(), by_lam);
  std::vector<double> S2(S.size()), l2(lam.size());
  for (int q = 0; q < LE; ++q) {
    const int f = (q & 1) ? anti[q / 2] : sym[q / 2];
    l2[q] = lam[f];
    for (int p = 0; p < LE; ++p) S2[p * LE + q] = S[p * LE + f];
  }
  S.swap(S2);
  lam.swap(l2);
}

// (Re)build the coarse level: Dirichlet faces from the plan's mask, slab
// lengths, 1D operators and their eigenvectors, h1/h2 means of the element means.
static int coarse_setup(ntg_schwarz* s) {
  ntg_plan* p = s->plan;
  const int lx = p->lx, N = lx - 1, lx3 = lx * lx * lx;
  const int E[3] = {s->Ex, s->Ey, s->Ez};
  const int64_t nelv = p->nelv;
  s->coarse_ready = 0;
  // Dirichlet faces: a face is Dirichlet when all its local nodes are masked
  int64_t cnt[6] = {0, 0, 0, 0, 0, 0};
  if (p->nmask > 0) {
    std::vector<int32_t> mk((size_t)p->nmask);
    NTG_CUDA_TRY(cudaMemcpyAsync(mk.data(), p->mask, sizeof(int32_t) * mk.size(), cudaMemcpyDeviceToHost, p->stream));
    NTG_CUDA_TRY(cudaStreamSynchronize(p->stream));
    for (int32_t l : mk) {
      const int64_t e = l / lx3;
      const int m = (int)(l - e * lx3), idx[3] = {m % lx, (m / lx) % lx, m / (lx * lx)};
      const int c[3] = {(int)(e % E[0]), (int)((e / E[0]) % E[1]), (int)(e / ((int64_t)E[0] * E[1]))};
      for (int d = 0; d < 3; ++d) {
        if (idx[d] == 0 && c[d] == 0) cnt[2 * d]++;
        if (idx[d] == N && c[d] == E[d] - 1) cnt[2 * d + 1]++;
      }
    }
  }
  bool dir[6];
  for (int d = 0; d < 3; ++d) {
    const int64_t face = (int64_t)E[(d + 1) % 3] * E[(d + 2) % 3] * lx * lx;
    dir[2 * d] = cnt[2 * d] == face;
    dir[2 * d + 1] = cnt[2 * d + 1] == face;
  }
  // h1, h2: means of the element means
  std::vector<float> hch((size_t)nelv * 2);
  NTG_CUDA_TRY(cudaMemcpyAsync(hch.data(), s->hc, sizeof(float) * hch.size(), cudaMemcpyDeviceToHost, p->stream));
  NTG_CUDA_TRY(cudaStreamSynchronize(p->stream));
  double h1 = 0, h2 = 0;
  for (int64_t e = 0; e < nelv; ++e) {
    h1 += hch[2 * e];
    h2 += hch[2 * e + 1];
  }
  h1 /= (double)nelv;
  h2 /= (double)nelv;
  // per direction: slab lengths, K and consistent M, active vertices, eigenpairs
  std::vector<float> lamall;
  double lmax = 0;
  for (int d = 0; d < 3; ++d) {
    std::vector<double> hs(E[d], 0.0);
    std::vector<int64_t> ns(E[d], 0);
    for (int64_t e = 0; e < nelv; ++e) {
      const int c = d == 0 ? (int)(e % E[0]) : d == 1 ? (int)((e / E[0]) % E[1]) : (int)(e / ((int64_t)E[0] * E[1]));
      hs[c] += s->hl[3 * e + d];
      ns[c]++;
    }
    const int nv = E[d] + 1, lo = dir[2 * d] ? 1 : 0, hi = nv - (dir[2 * d + 1] ? 1 : 0), m = hi - lo;
    s->cd.lo[d] = lo;
    s->cd.m[d] = m;
    if (m <= 0) return NTG_OK;  // no active vertex in this direction: the coarse space is empty
    std::vector<double> K(nv * nv, 0.0), M(nv * nv, 0.0);
    for (int c = 0; c < E[d]; ++c) {
      const double h = hs[c] / (double)ns[c];
      K[c * nv + c] += 1.0 / h;
      K[(c + 1) * nv + c + 1] += 1.0 / h;
      K[c * nv + c + 1] -= 1.0 / h;
      K[(c + 1) * nv + c] -= 1.0 / h;
      M[c * nv + c] += h / 3.0;
      M[(c + 1) * nv + c + 1] += h / 3.0;
      M[c * nv + c + 1] += h / 6.0;
      M[(c + 1) * nv + c] += h / 6.0;
    }
    std::vector<double> Ka(m * m), Ma(m * m), S, lam;
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) {
        Ka[i * m + j] = K[(lo + i) * nv + lo + j];
        Ma[i * m + j] = M[(lo + i) * nv + lo + j];
      }
    gen_eig(m, Ka, Ma, S, lam);
    std::vector<float> Sf(2 * (size_t)m * m);
    for (int x = 0; x < m; ++x)
      for (int f = 0; f < m; ++f) {
        Sf[(size_t)x * m + f] = (float)S[(size_t)x * m + f];
        Sf[(size_t)m * m + (size_t)f * m + x] = (float)S[(size_t)x * m + f];
      }
    dev_free(s->cS[d]);
    NTG_TRY(dev_alloc(&s->cS[d], 2 * (size_t)m * m));
    NTG_CUDA_TRY(cudaMemcpy(s->cS[d], Sf.data(), sizeof(float) * Sf.size(), cudaMemcpyHostToDevice));
    double lm = 0;
    for (double v : lam) {
      lamall.push_back((float)v);
      lm = std::max(lm, v);
    }
    lmax += lm;
  }
  const int m0 = s->cd.m[0], m1 = s->cd.m[1], m2 = s->cd.m[2];
  s->cd.Ex = E[0];
  s->cd.Ey = E[1];
  s->cd.Ez = E[2];
  s->cd.h1 = (float)h1;
  s->cd.h2 = (float)h2;
  s->cd.dmin = (float)(1e-6 * (h1 * lmax + h2));
  dev_free(s->clam);
  NTG_TRY(dev_alloc(&s->clam, lamall.size()));
  NTG_CUDA_TRY(cudaMemcpy(s->clam, lamall.data(), sizeof(float) * lamall.size(), cudaMemcpyHostToDevice));
  const size_t nv3 = (size_t)(E[0] + 1) * (E[1] + 1) * (E[2] + 1);
  if (!s->corner) NTG_TRY(dev_alloc(&s->corner, (size_t)nelv * 8));
  if (!s->uc) NTG_TRY(dev_alloc(&s->uc, nv3));
  dev_free(s->cwork);
  NTG_TRY(dev_alloc(&s->cwork, 2 * (size_t)m0 * m1 * m2));
  NTG_CUDA_TRY(cudaMemset(s->uc, 0, sizeof(float) * nv3));
  double xi[NTG_LXMAX], wq[NTG_LXMAX], Dm[NTG_LXMAX * NTG_LXMAX];
  gll_basis(lx, xi, wq, Dm);
  for (int i = 0; i < lx; ++i) {
    s->ph.p[0][i] = (float)(0.5 * (1.0 - xi[i]));
    s->ph.p[1][i] = (float)(0.5 * (1.0 + xi[i]));
  }
  s->ph.p[0][0] = 1.f;  // endpoints exact: shared faces then weigh the other element's vertices by 0
  s->ph.p[1][0] = 0.f;
  s->ph.p[0][N] = 0.f;
  s->ph.p[1][N] = 1.f;
  s->coarse_ready = 1;
  return NTG_OK;
}

namespace ntg {
namespace sw {

// 1 when the reference eigenvectors have the parity the even-odd
// transforms rely on: S[LE-1-p][f] = (-1)^f S[p][f]
inline int fdm_has_parity(const ntg_schwarz* w);

// persistent grid of the selected FP32-core variant: blocks resident on all SMs
template <int LX>
int fdm_prepare_grid(ntg_schwarz* w);

template <int LX>
using FdmFn = void (*)(const float*, float*, const float*, int, int, int, const Scalars*, float*, CoarsePhi,
                       const int32_t*, const float*, const FdmRef<LX + 2>);

// the FP32-core FDM kernel of the selected variant
template <int LX>
FdmFn<LX> fdm_kernel(const ntg_schwarz* w, bool eo) {
  const bool g = w->gen != nullptr;
  if (eo) return g ? k_fdm<LX, true, true> : k_fdm<LX, true, false>;
  return g ? k_fdm<LX, false, true> : k_fdm<LX, false, false>;
}

template <int LX>
int fdm_prepare(ntg_schwarz* w) {
  using C = FdmCfg<LX>;
  for (int v = 0; v < 2; ++v)
    NTG_CUDA_TRY(cudaFuncSetAttribute(fdm_kernel<LX>(w, v & 1), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)C::SMEM));
  return fdm_prepare_grid<LX>(w);
}

inline int fdm_has_parity(const ntg_schwarz* w) {
  const int LE = w->LE;
  double smax = 0.0, dev = 0.0;
  for (int q = 0; q < LE * LE; ++q) smax = std::max(smax, std::fabs(w->Sref[q]));
  for (int p = 0; p < LE; ++p)
    for (int f = 0; f < LE; ++f)
      dev = std::max(dev, std::fabs(w->Sref[(LE - 1 - p) * LE + f] - ((f & 1) ? -1.0 : 1.0) * w->Sref[p * LE + f]));
  return dev <= 1e-9 * smax ? 1 : 0;
}

template <int LX>
int fdm_prepare_grid(ntg_schwarz* w) {
  using C = FdmCfg<LX>;
  int per_sm = 0;
  NTG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fdm_kernel<LX>(w, w->fdm_eo),
                                                             C::THREADS, C::SMEM));
  const int64_t batches = (w->plan->nelv + C::EPB - 1) / C::EPB;
  const int64_t cap = (int64_t)num_sms() * (per_sm > 0 ? per_sm : 1);
  w->fdm_grid = (int)(batches < cap ? batches : cap);
  return NTG_OK;
}

template <int LX>
int fdm_launch(ntg_schwarz* w, const float* r, cudaStream_t s, const Scalars* sc) {
  using C = FdmCfg<LX>;
  constexpr int LE = LX + 2;
  FdmRef<LE> R;
  for (int a = 0; a < LE; ++a) {
    for (int f = 0; f < LE; ++f) {
      const float v = (float)w->Sref[a * LE + f];
      R.P[f >> 1][a][f & 1] = v;
      R.Q[a >> 1][f][a & 1] = v;
    }
    R.lam[a] = (float)w->lamref[a];
  }
  float* corner = w->coarse_ready ? w->corner : nullptr;
  const bool g = w->gen != nullptr;
  fdm_kernel<LX>(w, w->fdm_eo)<<<w->fdm_grid, C::THREADS, C::SMEM, s>>>(
      r, w->ze, w->esc, g ? (int)w->plan->nelv : w->Ex, g ? 1 : w->Ey, g ? 1 : w->Ez, sc, corner, w->ph,
      g ? w->gen->ghost : nullptr, g ? w->plan->multf : nullptr, R);
  NTG_COUNT_LAUNCH();
  return NTG_OK;
}

}  // namespace sw
}  // namespace ntg

namespace ntg {
namespace sw {

template <int LX>
int pull_launch(ntg_schwarz* w, float* z, const float* r, cudaStream_t s, Scalars* sc, const float* mult,
                double* part, int mode) {
  const int g = grid_for(w->plan->n / LX, 256);
  const CoarseView cv{w->coarse_ready ? w->uc : nullptr, w->ph, w->dw};
  if (mult)
    k_pull<LX, true><<<g, 256, 0, s>>>(w->ze, z, w->Ex, w->Ey, w->Ez, r, mult, mode, part, sc, cv);
  else
    k_pull<LX, false><<<g, 256, 0, s>>>(w->ze, z, w->Ex, w->Ey, w->Ez, r, nullptr, 0, nullptr, sc, cv);
  NTG_COUNT_LAUNCH();
  return NTG_OK;
}

// coarse solve (after the FDM kernel has written the corner sums): the
// restriction onto the vertex grid, then x, y, z forward (scaled), z, y, x back into uc
inline int coarse_launch(ntg_schwarz* w, cudaStream_t s, const Scalars* sc) {
  const CoarseDims& d = w->cd;
  const int64_t total = (int64_t)d.m[0] * d.m[1] * d.m[2];
  const int g = grid_for(total, 256);
  float* a = w->cwork;
  float* b = w->cwork + total;
  k_crs_restrict<<<g, 256, 0, s>>>(w->corner, a, d, sc);
  NTG_COUNT_LAUNCH();
  k_crs_mode<0, false, false, false><<<g, 256, 0, s>>>(a, b, w->cS[0], w->clam, d, sc);
  NTG_COUNT_LAUNCH();
  k_crs_mode<1, false, false, false><<<g, 256, 0, s>>>(b, a, w->cS[1], w->clam, d, sc);
  NTG_COUNT_LAUNCH();
  k_crs_mode<2, false, true, false><<<g, 256, 0, s>>>(a, b, w->cS[2], w->clam, d, sc);
  NTG_COUNT_LAUNCH();
  k_crs_mode<2, true, false, false><<<g, 256, 0, s>>>(b, a, w->cS[2], w->clam, d, sc);
  NTG_COUNT_LAUNCH();
  k_crs_mode<1, true, false, false><<<g, 256, 0, s>>>(a, b, w->cS[1], w->clam, d, sc);
  NTG_COUNT_LAUNCH();
  k_crs_mode<0, true, false, true><<<g, 256, 0, s>>>(b, w->uc, w->cS[0], w->clam, d, sc);
  NTG_COUNT_LAUNCH();
  return NTG_OK;
}

}  // namespace sw
}  // namespace ntg

namespace ntg {
namespace sw {

// the general-mesh application: FDM with the face-neighbour gather, the
// dense coarse level, the global-node prolongation
template <int LX>
int apply_gen(ntg_schwarz* w, float* z, const float* r, cudaStream_t s, Scalars* sc, bool dot, double* part,
              int rz_mode) {
  timer_start(TM_FDM, s);
  NTG_TRY(fdm_launch<LX>(w, r, s, sc));
  timer_stop(TM_FDM, s);
  if (w->coarse_ready) {
    timer_start(TM_CRS, s);
    NTG_TRY(gen_coarse_launch(w->gen, w->corner, s, sc));
    timer_stop(TM_CRS, s);
  }
  timer_start(TM_PULL, s);
  NTG_TRY(gen_pull_launch(w->gen, w->ze, z, r, w->dw, w->ph, dot, part, rz_mode, sc, s));
  timer_stop(TM_PULL, s);
  return NTG_OK;
}

}  // namespace sw
}  // namespace ntg

int ntg::schwarz_box(const ntg_schwarz* w, int* ex, int* ey, int* ez) {
  if (!w || w->gen) return 0;
  *ex = w->Ex;
  *ey = w->Ey;
  *ez = w->Ez;
  return 1;
}

int ntg::schwarz_apply(ntg_schwarz* w, float* z, const float* r, cudaStream_t s, Scalars* sc, const float* mult,
                       double* part, int rz_mode) {
  ntg_plan* p = w->plan;
  if (w->gen) {
    const bool dot = mult != nullptr;
    switch (p->lx) {
      case 4: NTG_TRY(sw::apply_gen<4>(w, z, r, s, sc, dot, part, rz_mode)); break;
      case 6: NTG_TRY(sw::apply_gen<6>(w, z, r, s, sc, dot, part, rz_mode)); break;
      case 8: NTG_TRY(sw::apply_gen<8>(w, z, r, s, sc, dot, part, rz_mode)); break;
      default:
        set_error("schwarz: lx=%d not compiled (4, 6, 8)", p->lx);
        return NTG_ERR_UNSUPPORTED;
    }
    NTG_CUDA_TRY(cudaGetLastError());
    return mask_guarded_f32(p, z, s, sc);
  }
  switch (p->lx) {
    case 4:
      timer_start(TM_FDM, s);
      NTG_TRY(sw::fdm_launch<4>(w, r, s, sc));
      timer_stop(TM_FDM, s);
      if (w->coarse_ready) {
        timer_start(TM_CRS, s);
        NTG_TRY(sw::coarse_launch(w, s, sc));
        timer_stop(TM_CRS, s);
      }
      timer_start(TM_PULL, s);
      NTG_TRY(sw::pull_launch<4>(w, z, r, s, sc, mult, part, rz_mode));
      timer_stop(TM_PULL, s);
      break;
    case 6:
      timer_start(TM_FDM, s);
      NTG_TRY(sw::fdm_launch<6>(w, r, s, sc));
      timer_stop(TM_FDM, s);
      if (w->coarse_ready) {
        timer_start(TM_CRS, s);
        NTG_TRY(sw::coarse_launch(w, s, sc));
        timer_stop(TM_CRS, s);
      }
      timer_start(TM_PULL, s);
      NTG_TRY(sw::pull_launch<6>(w, z, r, s, sc, mult, part, rz_mode));
      timer_stop(TM_PULL, s);
      break;
    case 8:
      timer_start(TM_FDM, s);
      if (w->fdm_tc)
        NTG_TRY(sw::fdm_tc_launch(w->ftc, r, w->ze, w->esc, w->Ex, w->Ey, w->Ez, sc,
                                  w->coarse_ready ? w->corner : nullptr, w->ph, p->dev_err, s));
      else
        NTG_TRY(sw::fdm_launch<8>(w, r, s, sc));
      timer_stop(TM_FDM, s);
      if (w->coarse_ready) {
        timer_start(TM_CRS, s);
        NTG_TRY(sw::coarse_launch(w, s, sc));
        timer_stop(TM_CRS, s);
      }
      timer_start(TM_PULL, s);
      NTG_TRY(sw::pull_launch<8>(w, z, r, s, sc, mult, part, rz_mode));
      timer_stop(TM_PULL, s);
      break;
    default:
      set_error("schwarz: lx=%d not compiled (4, 6, 8)", p->lx);
      return NTG_ERR_UNSUPPORTED;
  }
  NTG_CUDA_TRY(cudaGetLastError());
  // the pull assembles (identical sums on every copy): only the mask remains
  return mask_guarded_f32(p, z, s, sc);
}

extern "C" {

}  // extern "C"

// shared by the structured (box) and general-mesh constructors
static int schwarz_create_impl(ntg_plan* p, int ex, int ey, int ez, bool general, const double* x_d,
                               const double* y_d, const double* z_d, ntg_schwarz** out) {
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
    if (general && ((st = ensure_fp32(p)) || (st = sw::gen_create(p, &s->gen)))) break;
    if ((st = dev_alloc(&s->hld, (size_t)E * 3)) || (st = dev_alloc(&s->esc, (size_t)E * 8)) ||
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
    std::vector<float> hlf(s->hl.begin(), s->hl.end());
    if (cudaMemcpy(s->hld, hlf.data(), sizeof(float) * hlf.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
      st = NTG_ERR_CUDA;
      set_error("ntg_schwarz_create: upload");
      break;
    }
    // the reference interval's extended 1D eigenpairs (h = 2 on all three intervals)
    s->Sref.assign((size_t)LE2, 0.0);
    s->lamref.assign((size_t)LE, 0.0);
    fdm_1d(p, 2.0, 2.0, 2.0, s->Sref.data(), s->lamref.data());
    parity_order(LE, s->Sref, s->lamref);
    s->fdm_eo = sw::fdm_has_parity(s);
    st = p->lx == 4 ? sw::fdm_prepare<4>(s) : p->lx == 6 ? sw::fdm_prepare<6>(s) : sw::fdm_prepare<8>(s);
    if (st) break;
    if (!general && p->lx == 8 && p->dev_err) {
      // prepared, off by default: measured slower than the FP32-core kernel
      if ((st = sw::fdm_tc_prepare(s->Sref.data(), s->lamref.data(), &s->ftc))) break;
      s->fdm_tc = 0;
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

extern "C" {

int ntg_schwarz_create(ntg_plan* p, int ex, int ey, int ez, const double* x_d, const double* y_d, const double* z_d,
                       ntg_schwarz** out) {
  clear_error();
  NTG_CHECK_ARG(p && out && x_d && y_d && z_d, "ntg_schwarz_create: null argument");
  NTG_CHECK_ARG(ex > 0 && ey > 0 && ez > 0 && (int64_t)ex * ey * ez == p->nelv,
                "ntg_schwarz_create: ex*ey*ez must equal the plan's element count (structured box, x fastest)");
  NTG_CHECK_ARG(p->lx == 4 || p->lx == 6 || p->lx == 8, "ntg_schwarz_create: lx must be 4, 6 or 8");
  NTG_CHECK_ARG(p->nelv < (int64_t)1 << 30, "ntg_schwarz_create: element count must be below 2^30");
  return schwarz_create_impl(p, ex, ey, ez, false, x_d, y_d, z_d, out);
}

// any conforming hexahedral mesh: neighbours from the plan's global node ids
int ntg_schwarz_create_general(ntg_plan* p, const double* x_d, const double* y_d, const double* z_d,
                               ntg_schwarz** out) {
  clear_error();
  NTG_CHECK_ARG(p && out && x_d && y_d && z_d, "ntg_schwarz_create_general: null argument");
  NTG_CHECK_ARG(p->lx == 4 || p->lx == 6 || p->lx == 8, "ntg_schwarz_create_general: lx must be 4, 6 or 8");
  NTG_CHECK_ARG(p->nelv < (int64_t)1 << 30, "ntg_schwarz_create_general: element count must be below 2^30");
  return schwarz_create_impl(p, (int)p->nelv, 1, 1, true, x_d, y_d, z_d, out);
}

// refresh the element means of h1 / h2 after ntg_coef_set
int ntg_schwarz_update(ntg_schwarz* s) {
  clear_error();
  NTG_CHECK_ARG(s, "ntg_schwarz_update: null argument");
  ntg_plan* p = s->plan;
  const int lx3 = p->lx * p->lx * p->lx;
  { sw::k_coef_means<<<grid_for(p->nelv, 128), 128, 0, p->stream>>>(p->h1_const ? nullptr : p->h1, p->h1c, p->ifh2 ? p->hB : nullptr, p->B, p->nelv, lx3, s->hc); NTG_COUNT_LAUNCH(); }
  { sw::k_elem_scalars<<<grid_for(p->nelv, 128), 128, 0, p->stream>>>(s->hld, s->hc, s->esc, p->nelv); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  dev_free(s->dw);
  s->dw = nullptr;
  if (s->mass_term && p->ifh2) {
    NTG_TRY(jacobi_update(p));
    double* hBa = nullptr;
    NTG_TRY(dev_alloc(&hBa, (size_t)p->n));
    NTG_TRY(dev_alloc(&s->dw, (size_t)p->n));
    NTG_CUDA_TRY(cudaMemcpyAsync(hBa, p->hB, sizeof(double) * p->n, cudaMemcpyDeviceToDevice, p->stream));
    NTG_TRY(gs_launch(p, hBa, NTG_GS_ADD, p->stream));
    { sw::k_mass_term<<<grid_for(p->n, 256), 256, 0, p->stream>>>(hBa, p->dinv, s->dw, p->n); NTG_COUNT_LAUNCH(); }
    NTG_CUDA_TRY(cudaStreamSynchronize(p->stream));
    dev_free(hBa);
  }
  if (s->coarse && s->gen) {
    s->coarse_ready = 0;
    NTG_TRY(sw::gen_coarse_setup(p, s->gen));
    if (s->gen->coarse_ready) {
      if (!s->corner) NTG_TRY(dev_alloc(&s->corner, (size_t)p->nelv * 8));
      if (!s->ph.p[1][p->lx - 1]) {
        double xi[NTG_LXMAX], wq[NTG_LXMAX], Dm[NTG_LXMAX * NTG_LXMAX];
        gll_basis(p->lx, xi, wq, Dm);
        for (int i = 0; i < p->lx; ++i) {
          s->ph.p[0][i] = (float)(0.5 * (1.0 - xi[i]));
          s->ph.p[1][i] = (float)(0.5 * (1.0 + xi[i]));
        }
        s->ph.p[0][0] = 1.f; s->ph.p[1][0] = 0.f; s->ph.p[0][p->lx - 1] = 0.f; s->ph.p[1][p->lx - 1] = 1.f;
      }
      s->coarse_ready = 1;
    }
    return NTG_OK;
  }
  if (s->coarse) return coarse_setup(s);
  return NTG_OK;
}

// FDM local solves: 0 = FP32 cores, even-odd transforms when the reference
// eigenvectors have parity (default); 1 = tensor cores (lx = 8); 2 = FP32
// cores, full 1D products
int ntg_schwarz_set_fdm_path(ntg_schwarz* s, int path) {
  clear_error();
  NTG_CHECK_ARG(s && path >= 0 && path <= 2, "ntg_schwarz_set_fdm_path: bad argument");
  NTG_CHECK_ARG(path != 1 || s->ftc.img,
                "ntg_schwarz_set_fdm_path: the tensor-core path needs lx = 8 on a structured box");
  s->fdm_tc = path == 1 ? 1 : 0;
  if (path != 1) {
    s->fdm_eo = path == 0 ? sw::fdm_has_parity(s) : 0;
    const int lx = s->plan->lx;
    NTG_TRY(lx == 4 ? sw::fdm_prepare_grid<4>(s) : lx == 6 ? sw::fdm_prepare_grid<6>(s) : sw::fdm_prepare_grid<8>(s));
  }
  return NTG_OK;
}

int ntg_schwarz_set_mass_term(ntg_schwarz* s, int enable) {
  clear_error();
  NTG_CHECK_ARG(s, "ntg_schwarz_set_mass_term: null argument");
  s->mass_term = enable ? 1 : 0;
  return ntg_schwarz_update(s);
}

int ntg_schwarz_set_coarse(ntg_schwarz* s, int enable) {
  clear_error();
  NTG_CHECK_ARG(s, "ntg_schwarz_set_coarse: null argument");
  NTG_TRY(cudaStreamSynchronize(s->plan->stream) == cudaSuccess ? NTG_OK : NTG_ERR_CUDA);
  s->coarse = enable ? 1 : 0;
  s->coarse_ready = 0;
  if (s->gen) s->gen->coarse_ready = 0;
  return s->coarse ? ntg_schwarz_update(s) : NTG_OK;
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
