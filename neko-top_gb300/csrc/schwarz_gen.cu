// The Schwarz preconditioner on general (unstructured, conforming)
// hexahedral meshes: the tables that replace the structured box's index
// arithmetic, the assembling prolongation over global nodes and the coarse
// level on the element vertices.
//
// Subdomains.  Element e is extended by one node layer across each of its
// six faces: the ghost layer beyond face f holds the face neighbour's nodes
// one step inside it, matched through the shared face nodes' global ids, so
// neighbours in any relative orientation fit.  Edge and corner positions of
// the extended box are not part of the subdomain (zero in R_e r, dropped in
// R_e^T), as in the face-only overlap of Neko's Schwarz smoother on general
// meshes (Neko, src/krylov/schwarz.f90, which the reference configures as
// 'hsmg' for its pressure solves: examples/rugby_ball/rugby_ball.case:46-52).
// The local solves are the FDM kernel's, unchanged.
//
// Prolongation.  Every global node sums, in ascending order of their index
// in the extended-result array, the results of the subdomains covering it
// (its own element copies' interiors and the ghost layers that reach it),
// adds the coarse and mass-term corrections of its first copy, and writes
// the sum to every copy: bit-identical copies with no gather-scatter pass.
//
// Coarse level.  Q1 on the element vertices: P interpolates vertex values
// trilinearly (reference coordinates) to the GLL nodes, P^T r sums
// phi_v r / multiplicity (the FDM kernel's corner sums, then a fixed-order
// sum per vertex); A_c = P^T A P, the Galerkin operator of the fine
// operator A with its coefficients, assembled from element matrices that
// the fine Ax kernel computes (eight basis fields per element, masked nodes
// zeroed), Dirichlet vertices (any copy masked) removed.  A_c is inverted
// densely on the device (Gauss-Jordan in FP64, no pivoting: A_c is SPD)
// and applied as an FP32 matrix-vector product; an operator with a constant
// null mode (all-Neumann, no mass term: 1^T A_c 1 = 0) gets A_c + c 1 1^T
// (c = mean diagonal / nv), which equals the pseudo-inverse on residuals
// with zero vertex sum.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "reduce.cuh"
#include "schwarz.cuh"

namespace ntg {
namespace sw {

namespace {

// local index of the node of face f at tangential (s, t) with normal index nrm
inline int face_node(int lx, int f, int s, int t, int nrm) {
  const int d = f >> 1;
  const int i = d == 0 ? nrm : s, j = d == 0 ? s : d == 1 ? nrm : t, k = d == 2 ? nrm : t;
  return i + lx * (j + lx * k);
}

// extended-box index of the ghost node beyond face f at tangential (s, t)
inline int ext_ghost(int lx, int f, int s, int t) {
  const int LE = lx + 2, d = f >> 1, b0 = (f & 1) ? LE - 1 : 0;
  const int a = d == 0 ? b0 : s + 1, b = d == 0 ? s + 1 : d == 1 ? b0 : t + 1, c = d == 2 ? b0 : t + 1;
  return a + LE * (b + LE * c);
}

struct FaceRec {
  std::array<int64_t, 4> key;  // sorted global nodes of the face's corners
  int64_t ef;                  // e * 6 + f
  bool operator<(const FaceRec& o) const { return key != o.key ? key < o.key : ef < o.ef; }
};

struct PhiD {
  double p[2][NTG_LXMAX];
};

__global__ void k_q1_field(double* __restrict__ U, const uint8_t* __restrict__ flag, int v, int64_t n, int lx,
                           PhiD ph) {
  const int lx3 = lx * lx * lx;
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < n; l += (int64_t)gridDim.x * blockDim.x) {
    const int q = (int)(l % lx3), i = q % lx, j = (q / lx) % lx, k = q / (lx * lx);
    U[l] = flag[l] ? 0.0 : ph.p[v & 1][i] * ph.p[(v >> 1) & 1][j] * ph.p[v >> 2][k];
  }
}

// Ae[e][w][v] = sum_q phi_w(q) (1 - flag(q)) W(q), W = A_e phi_v; one thread per (e, w)
__global__ void k_q1_proj(const double* __restrict__ W, const uint8_t* __restrict__ flag, int v, int64_t nelv,
                          int lx, PhiD ph, double* __restrict__ Ae) {
  const int lx3 = lx * lx * lx;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nelv * 8;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = t >> 3;
    const int w = (int)(t & 7);
    double acc = 0.0;
    for (int q = 0; q < lx3; ++q) {
      const int64_t l = e * lx3 + q;
      if (flag[l]) continue;
      const int i = q % lx, j = (q / lx) % lx, k = q / (lx * lx);
      acc += ph.p[w & 1][i] * ph.p[(w >> 1) & 1][j] * ph.p[w >> 2][k] * W[l];
    }
    Ae[e * 64 + w * 8 + v] = acc;
  }
}

__global__ void k_flag_mask(const int32_t* __restrict__ mask, int64_t nmask, uint8_t* __restrict__ flag) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nmask; t += (int64_t)gridDim.x * blockDim.x)
    flag[mask[t]] = 1;
}

// in-place Gauss-Jordan inversion, step k: save row and column k ...
__global__ void k_gj_save(const double* __restrict__ A, int n, int k, double* __restrict__ rowk,
                          double* __restrict__ colk) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    rowk[t] = A[(int64_t)k * n + t];
    colk[t] = A[(int64_t)t * n + k];
  }
}
// ... then eliminate with pivot p = A[k][k]:
//   A[k][k] = 1/p, A[k][j] = a_kj / p, A[i][k] = -a_ik / p, A[i][j] -= a_ik a_kj / p
__global__ void k_gj_update(double* __restrict__ A, int n, int k, const double* __restrict__ rowk,
                            const double* __restrict__ colk) {
  const double pinv = 1.0 / rowk[k];
  const int64_t nn = (int64_t)n * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nn; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t / n), j = (int)(t - (int64_t)i * n);
    double v;
    if (i == k && j == k) v = pinv;
    else if (i == k) v = rowk[j] * pinv;
    else if (j == k) v = -colk[i] * pinv;
    else v = A[t] - colk[i] * rowk[j] * pinv;
    A[t] = v;
  }
}

__global__ void k_d2f_n(const double* __restrict__ a, float* __restrict__ b, int64_t n) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    b[t] = (float)a[t];
}

// rc[a] = sum of the corner sums of vertex a, in list order
__global__ void k_crs_gather(const float* __restrict__ corner, const int32_t* __restrict__ voff,
                             const int32_t* __restrict__ vsrc, int nv, float* __restrict__ rc, const Scalars* sc) {
  if (sc && sc->done) return;
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < nv; a += gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int t = voff[a]; t < voff[a + 1]; ++t) s += corner[vsrc[t]];
    rc[a] = s;
  }
}

// zc = Ainv rc: one warp per row, lanes over columns, fixed-order shuffle sum
__global__ void k_crs_gemv(const float* __restrict__ Ainv, const float* __restrict__ rc, int nv,
                           float* __restrict__ zc, const Scalars* sc) {
  if (sc && sc->done) return;
  const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
  for (int row = blockIdx.x * wpb + (threadIdx.x >> 5); row < nv; row += gridDim.x * wpb) {
    const float* a = Ainv + (int64_t)row * nv;
    float s = 0.f;
    for (int j = lane; j < nv; j += 32) s = fmaf(a[j], rc[j], s);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) zc[row] = s;
  }
}

// Assembling prolongation over global nodes (see the file comment).
template <int LX, bool DOT>
__global__ void __launch_bounds__(256)
    k_pull_gen(const float* __restrict__ ze, float* __restrict__ z, const int32_t* __restrict__ perm,
               const int64_t* __restrict__ offs, int64_t nu, const int64_t* __restrict__ soff,
               const int32_t* __restrict__ src, const int32_t* __restrict__ vid, const float* __restrict__ zc,
               CoarsePhi ph, const float* __restrict__ dw, const float* __restrict__ r, int mode,
               double* __restrict__ part, Scalars* sc) {
  constexpr int LX3 = LX * LX * LX;
  if (sc && sc->done) return;
  __shared__ float sp[2][LX];
  if (threadIdx.x < 2 * LX) sp[threadIdx.x / LX][threadIdx.x % LX] = ph.p[threadIdx.x / LX][threadIdx.x % LX];
  __syncthreads();
  float rz = 0.f;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < nu; g += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.f;
    const int64_t s1 = soff[g + 1];
    for (int64_t t = soff[g]; t < s1; ++t) s += ze[src[t]];
    const int64_t o0 = offs[g], o1 = offs[g + 1];
    const int l0 = perm[o0];
    if (zc) {
      const int e0 = l0 / LX3, q = l0 - e0 * LX3, i = q % LX, j = (q / LX) % LX, k = q / (LX * LX);
      const int32_t* ve = vid + (int64_t)e0 * 8;
      float c = 0.f;
#pragma unroll
      for (int v = 0; v < 8; ++v) {
        const int a = ve[v];
        if (a >= 0) c += (sp[v & 1][i] * sp[(v >> 1) & 1][j] * sp[v >> 2][k]) * zc[a];
      }
      s += c;
    }
    if (dw) s += dw[l0] * r[l0];
    for (int64_t t = o0; t < o1; ++t) z[perm[t]] = s;
    if constexpr (DOT) rz += r[l0] * s;
  }
  if constexpr (DOT) {
    double v[1] = {(double)rz};
    grid_reduce<1>(v, part, sc, FinRz{mode});
  }
}

}  // namespace

void gen_free(GenTopo* g) {
  if (!g) return;
  dev_free(g->ghost); dev_free(g->soff); dev_free(g->src);
  dev_free(g->vid); dev_free(g->voff); dev_free(g->vsrc);
  dev_free(g->ainv); dev_free(g->rc); dev_free(g->zc);
  delete g;
}

// The face-neighbour table of a conforming hexahedral mesh from the global
// node of every local node (gn: nelv * lx^3 entries, any integer ids):
// faces are keyed by their four corner nodes (sorted), pairs of equal keys
// are neighbours, and each face node is matched to the neighbour's node with
// the same id, so neighbours may meet in any relative orientation.
// ghost[(e * 6 + f) * lx^2 + p]: the local index one step inside the
// neighbour across face f from face node p, -1 on the boundary.
int ghost_table(int64_t E, int lx, const int64_t* gn, std::vector<int32_t>& ghost) {
  const int N = lx - 1, LX2 = lx * lx, LX3 = LX2 * lx;
  std::vector<FaceRec> faces((size_t)E * 6);
  for (int64_t e = 0; e < E; ++e)
    for (int f = 0; f < 6; ++f) {
      const int nrm = (f & 1) ? N : 0;
      FaceRec& fr = faces[e * 6 + f];
      for (int c = 0; c < 4; ++c) fr.key[c] = gn[e * LX3 + face_node(lx, f, (c & 1) ? N : 0, (c >> 1) ? N : 0, nrm)];
      std::sort(fr.key.begin(), fr.key.end());
      fr.ef = e * 6 + f;
    }
  std::sort(faces.begin(), faces.end());
  ghost.assign((size_t)E * 6 * LX2, -1);
  std::vector<std::pair<int64_t, int>> tb((size_t)LX2);
  auto match = [&](int64_t efA, int64_t efB) {
    const int64_t eA = efA / 6, eB = efB / 6;
    const int fA = (int)(efA % 6), fB = (int)(efB % 6);
    const int nA = (fA & 1) ? N : 0, nB = (fB & 1) ? N : 0, inB = (fB & 1) ? N - 1 : 1;
    for (int t = 0; t < lx; ++t)
      for (int s = 0; s < lx; ++s) tb[s + lx * t] = {gn[eB * LX3 + face_node(lx, fB, s, t, nB)], s + lx * t};
    std::sort(tb.begin(), tb.end());
    for (int t = 0; t < lx; ++t)
      for (int s = 0; s < lx; ++s) {
        const int64_t key = gn[eA * LX3 + face_node(lx, fA, s, t, nA)];
        auto it = std::lower_bound(tb.begin(), tb.end(), std::make_pair(key, -1));
        if (it == tb.end() || it->first != key) return false;
        const int sB = it->second % lx, tB = it->second / lx;
        ghost[efA * LX2 + s + lx * t] = (int32_t)(eB * LX3 + face_node(lx, fB, sB, tB, inB));
      }
    return true;
  };
  for (size_t a = 0; a < faces.size();) {
    size_t b = a + 1;
    while (b < faces.size() && faces[b].key == faces[a].key) ++b;
    if (b - a == 2) {
      if (!match(faces[a].ef, faces[a + 1].ef) || !match(faces[a + 1].ef, faces[a].ef)) {
        set_error("schwarz (general mesh): elements %lld and %lld share face corners but not the face's nodes",
                  (long long)(faces[a].ef / 6), (long long)(faces[a + 1].ef / 6));
        return NTG_ERR_INVALID;
      }
    } else if (b - a > 2) {
      set_error("schwarz (general mesh): a face is shared by %d elements (non-conforming mesh)", (int)(b - a));
      return NTG_ERR_INVALID;
    }
    a = b;
  }
  return NTG_OK;
}

int gen_create(ntg_plan* p, GenTopo** out) {
  *out = nullptr;
  const int lx = p->lx, LX2 = lx * lx, LX3 = LX2 * lx, LE = lx + 2, LE3 = LE * LE * LE;
  const int64_t n = p->n, E = p->nelv, nu = p->nu;
  if (E * (int64_t)LE3 >= ((int64_t)1 << 31)) {
    set_error("schwarz (general mesh): nelv * (lx+2)^3 must be below 2^31");
    return NTG_ERR_UNSUPPORTED;
  }
  std::vector<int32_t> perm((size_t)n);
  std::vector<int64_t> offs((size_t)nu + 1);
  NTG_CUDA_TRY(cudaMemcpyAsync(perm.data(), p->perm, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, p->stream));
  NTG_CUDA_TRY(cudaMemcpyAsync(offs.data(), p->offs, sizeof(int64_t) * (nu + 1), cudaMemcpyDeviceToHost, p->stream));
  NTG_CUDA_TRY(cudaStreamSynchronize(p->stream));
  GenTopo* g = new GenTopo();
  g->lx = lx;
  g->nelv = E;
  g->nu = nu;
  g->perm = p->perm;
  g->offs = p->offs;
  g->gnum.assign((size_t)n, -1);
  for (int64_t q = 0; q < nu; ++q)
    for (int64_t t = offs[q]; t < offs[q + 1]; ++t) g->gnum[perm[t]] = q;
  const std::vector<int64_t>& gn = g->gnum;
  std::vector<int32_t> ghost;
  int st = ghost_table(E, lx, gn.data(), ghost);
  // every global node's covering list: own copies' interiors, then the ghost layers reaching it
  std::vector<int64_t> soff;
  std::vector<int32_t> src;
  if (!st) {
    soff.assign((size_t)nu + 1, 0);
    for (int64_t l = 0; l < n; ++l) soff[gn[l] + 1]++;
    for (size_t t = 0; t < ghost.size(); ++t)
      if (ghost[t] >= 0) soff[gn[ghost[t]] + 1]++;
    for (int64_t q = 0; q < nu; ++q) soff[q + 1] += soff[q];
    src.resize((size_t)soff[nu]);
    std::vector<int64_t> fill(soff.begin(), soff.end() - 1);
    for (int64_t l = 0; l < n; ++l) {
      const int64_t e = l / LX3;
      const int q = (int)(l - e * LX3), i = q % lx, j = (q / lx) % lx, k = q / LX2;
      src[fill[gn[l]]++] = (int32_t)(e * LE3 + (i + 1) + LE * ((j + 1) + LE * (k + 1)));
    }
    for (int64_t e = 0; e < E; ++e)
      for (int f = 0; f < 6; ++f)
        for (int pp = 0; pp < LX2; ++pp) {
          const int32_t l = ghost[(e * 6 + f) * LX2 + pp];
          if (l >= 0) src[fill[gn[l]]++] = (int32_t)(e * LE3 + ext_ghost(lx, f, pp % lx, pp / lx));
        }
    for (int64_t q = 0; q < nu; ++q) std::sort(src.begin() + soff[q], src.begin() + soff[q + 1]);
  }
  do {
    if (st) break;
    if ((st = dev_alloc(&g->ghost, ghost.size())) || (st = dev_alloc(&g->soff, soff.size())) ||
        (st = dev_alloc(&g->src, std::max<size_t>(src.size(), 1))))
      break;
    if (cudaMemcpy(g->ghost, ghost.data(), sizeof(int32_t) * ghost.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(g->soff, soff.data(), sizeof(int64_t) * soff.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(g->src, src.data(), sizeof(int32_t) * src.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
      st = NTG_ERR_CUDA;
      set_error("schwarz (general mesh): table upload");
    }
  } while (0);
  if (st) {
    gen_free(g);
    return st;
  }
  *out = g;
  return NTG_OK;
}

int gen_coarse_setup(ntg_plan* p, GenTopo* g) {
  g->coarse_ready = 0;
  const int lx = p->lx, N = lx - 1, LX3 = lx * lx * lx;
  const int64_t E = p->nelv, n = p->n;
  cudaStream_t s = p->stream;
  // Dirichlet global nodes: any copy masked
  std::vector<uint8_t> gmask((size_t)g->nu, 0);
  std::vector<int32_t> mk((size_t)p->nmask);
  if (p->nmask > 0) {
    NTG_CUDA_TRY(cudaMemcpyAsync(mk.data(), p->mask, sizeof(int32_t) * mk.size(), cudaMemcpyDeviceToHost, s));
    NTG_CUDA_TRY(cudaStreamSynchronize(s));
    for (int32_t l : mk) gmask[g->gnum[l]] = 1;
  }
  // active vertices: the corners' global nodes, ascending, Dirichlet ones removed
  std::vector<int64_t> cg((size_t)E * 8);
  for (int64_t e = 0; e < E; ++e)
    for (int v = 0; v < 8; ++v)
      cg[e * 8 + v] = g->gnum[e * LX3 + ((v & 1) ? N : 0) + lx * (((v >> 1) & 1) ? N : 0) + lx * lx * ((v >> 2) ? N : 0)];
  std::vector<int64_t> verts;
  verts.reserve(cg.size());
  for (int64_t q : cg)
    if (!gmask[q]) verts.push_back(q);
  std::sort(verts.begin(), verts.end());
  verts.erase(std::unique(verts.begin(), verts.end()), verts.end());
  const int64_t nv = (int64_t)verts.size();
  if (nv == 0) return NTG_OK;  // every vertex Dirichlet: no coarse correction
  if (nv > kGenCoarseMax) {
    set_error("schwarz (general mesh): the dense coarse level takes at most %d active vertices (%lld here)",
              kGenCoarseMax, (long long)nv);
    return NTG_ERR_UNSUPPORTED;
  }
  std::vector<int32_t> vid((size_t)E * 8), voff((size_t)nv + 1, 0), vsrc;
  for (int64_t t = 0; t < E * 8; ++t) {
    auto it = std::lower_bound(verts.begin(), verts.end(), cg[t]);
    vid[t] = (it != verts.end() && *it == cg[t]) ? (int32_t)(it - verts.begin()) : -1;
    if (vid[t] >= 0) voff[vid[t] + 1]++;
  }
  for (int64_t a = 0; a < nv; ++a) voff[a + 1] += voff[a];
  vsrc.resize((size_t)voff[nv]);
  {
    std::vector<int32_t> fill(voff.begin(), voff.end() - 1);
    for (int64_t t = 0; t < E * 8; ++t)
      if (vid[t] >= 0) vsrc[fill[vid[t]]++] = (int32_t)t;
  }
  // element matrices of the Galerkin operator: A_e applied to the eight
  // (masked) trilinear basis fields by the fine FP64 Ax kernel
  double xi[NTG_LXMAX], wq[NTG_LXMAX], Dm[NTG_LXMAX * NTG_LXMAX];
  gll_basis(lx, xi, wq, Dm);
  PhiD ph{};
  for (int i = 0; i < lx; ++i) {
    ph.p[0][i] = 0.5 * (1.0 - xi[i]);
    ph.p[1][i] = 0.5 * (1.0 + xi[i]);
  }
  ph.p[0][0] = 1.0; ph.p[1][0] = 0.0; ph.p[0][N] = 0.0; ph.p[1][N] = 1.0;
  double *U = nullptr, *W = nullptr, *Ae = nullptr, *A = nullptr, *rowk = nullptr, *colk = nullptr;
  uint8_t* flag = nullptr;
  std::vector<double> Ah;
  int st = NTG_OK;
  do {
    if ((st = dev_alloc(&U, (size_t)n)) || (st = dev_alloc(&W, (size_t)n)) || (st = dev_alloc(&Ae, (size_t)E * 64)) ||
        (st = dev_alloc(&flag, (size_t)n)))
      break;
    if (cudaMemsetAsync(flag, 0, (size_t)n, s) != cudaSuccess) { st = NTG_ERR_CUDA; break; }
    if (p->nmask > 0) { k_flag_mask<<<grid_for(p->nmask, 256), 256, 0, s>>>(p->mask, p->nmask, flag); NTG_COUNT_LAUNCH(); }
    for (int v = 0; v < 8 && !st; ++v) {
      k_q1_field<<<grid_for(n, 256), 256, 0, s>>>(U, flag, v, n, lx, ph);
      NTG_COUNT_LAUNCH();
      if ((st = ax_launch(p, W, U, nullptr, 0, s))) break;
      k_q1_proj<<<grid_for(E * 8, 128), 128, 0, s>>>(W, flag, v, E, lx, ph, Ae);
      NTG_COUNT_LAUNCH();
    }
    if (st) break;
    std::vector<double> Aeh((size_t)E * 64);
    if (cudaMemcpyAsync(Aeh.data(), Ae, sizeof(double) * Aeh.size(), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
      st = NTG_ERR_CUDA;
      set_error("schwarz (general mesh): coarse element matrices");
      break;
    }
    Ah.assign((size_t)(nv * nv), 0.0);
    for (int64_t e = 0; e < E; ++e)
      for (int w = 0; w < 8; ++w) {
        const int32_t aw = vid[e * 8 + w];
        if (aw < 0) continue;
        for (int v = 0; v < 8; ++v) {
          const int32_t av = vid[e * 8 + v];
          if (av >= 0) Ah[(size_t)aw * nv + av] += Aeh[e * 64 + w * 8 + v];
        }
      }
    double tr = 0.0;
    for (int64_t a = 0; a < nv; ++a) {
      tr += Ah[(size_t)a * nv + a];
      for (int64_t b = a + 1; b < nv; ++b) {
        const double m = 0.5 * (Ah[(size_t)a * nv + b] + Ah[(size_t)b * nv + a]);
        Ah[(size_t)a * nv + b] = Ah[(size_t)b * nv + a] = m;
      }
    }
    if (!(tr > 0.0)) { st = NTG_ERR_INVALID; set_error("schwarz (general mesh): coarse operator has no positive diagonal"); break; }
    // a constant null mode (no Dirichlet vertex, no mass term): 1^T A_c 1
    // vanishes against the diagonal; shift it as A_c + c 1 1^T
    double sum = 0.0;
    for (double a : Ah) sum += a;
    if (std::fabs(sum) <= 1e-10 * tr) {
      const double c = tr / (double)nv / (double)nv;
      for (double& a : Ah) a += c;
    }
    // dense inverse on the device
    if ((st = dev_alloc(&A, (size_t)(nv * nv))) || (st = dev_alloc(&rowk, (size_t)nv)) ||
        (st = dev_alloc(&colk, (size_t)nv)))
      break;
    if (cudaMemcpyAsync(A, Ah.data(), sizeof(double) * Ah.size(), cudaMemcpyHostToDevice, s) != cudaSuccess) {
      st = NTG_ERR_CUDA;
      break;
    }
    const int gsv = grid_for(nv, 256), gup = grid_for(nv * nv, 256);
    for (int k = 0; k < (int)nv; ++k) {
      k_gj_save<<<gsv, 256, 0, s>>>(A, (int)nv, k, rowk, colk);
      NTG_COUNT_LAUNCH();
      k_gj_update<<<gup, 256, 0, s>>>(A, (int)nv, k, rowk, colk);
      NTG_COUNT_LAUNCH();
    }
    dev_free(g->ainv); dev_free(g->rc); dev_free(g->zc); dev_free(g->vid); dev_free(g->voff); dev_free(g->vsrc);
    if ((st = dev_alloc(&g->ainv, (size_t)(nv * nv))) || (st = dev_alloc(&g->rc, (size_t)nv)) ||
        (st = dev_alloc(&g->zc, (size_t)nv)) || (st = dev_alloc(&g->vid, vid.size())) ||
        (st = dev_alloc(&g->voff, voff.size())) || (st = dev_alloc(&g->vsrc, std::max<size_t>(vsrc.size(), 1))))
      break;
    k_d2f_n<<<gup, 256, 0, s>>>(A, g->ainv, nv * nv);
    NTG_COUNT_LAUNCH();
    if (cudaMemcpyAsync(g->vid, vid.data(), sizeof(int32_t) * vid.size(), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(g->voff, voff.data(), sizeof(int32_t) * voff.size(), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(g->vsrc, vsrc.data(), sizeof(int32_t) * vsrc.size(), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
      st = NTG_ERR_CUDA;
      set_error("schwarz (general mesh): coarse inverse");
      break;
    }
    g->nv = (int)nv;
    g->coarse_ready = 1;
  } while (0);
  cudaStreamSynchronize(s);
  dev_free(U); dev_free(W); dev_free(Ae); dev_free(flag); dev_free(A); dev_free(rowk); dev_free(colk);
  return st;
}

int gen_coarse_launch(GenTopo* g, const float* corner, cudaStream_t s, const Scalars* sc) {
  k_crs_gather<<<grid_for(g->nv, 256), 256, 0, s>>>(corner, g->voff, g->vsrc, g->nv, g->rc, sc);
  NTG_COUNT_LAUNCH();
  k_crs_gemv<<<std::max(1, std::min((g->nv + 7) / 8, 8 * num_sms())), 256, 0, s>>>(g->ainv, g->rc, g->nv, g->zc, sc);
  NTG_COUNT_LAUNCH();
  return NTG_OK;
}

template <int LX>
static int pull_gen(GenTopo* g, const float* ze, float* z, const float* r, const float* dw, const CoarsePhi& ph,
                    bool dot, double* part, int mode, Scalars* sc, cudaStream_t s) {
  const int grid = grid_for(g->nu, 256);
  const int32_t* vid = g->coarse_ready ? g->vid : nullptr;
  const float* zc = g->coarse_ready ? g->zc : nullptr;
  if (dot)
    k_pull_gen<LX, true><<<grid, 256, 0, s>>>(ze, z, g->perm, g->offs, g->nu, g->soff, g->src, vid, zc, ph, dw, r,
                                              mode, part, sc);
  else
    k_pull_gen<LX, false><<<grid, 256, 0, s>>>(ze, z, g->perm, g->offs, g->nu, g->soff, g->src, vid, zc, ph, dw, r,
                                               0, nullptr, sc);
  NTG_COUNT_LAUNCH();
  return NTG_OK;
}

int gen_pull_launch(GenTopo* g, const float* ze, float* z, const float* r, const float* dw, const CoarsePhi& ph,
                    bool dot, double* part, int mode, Scalars* sc, cudaStream_t s) {
  switch (g->lx) {
    case 4: return pull_gen<4>(g, ze, z, r, dw, ph, dot, part, mode, sc, s);
    case 6: return pull_gen<6>(g, ze, z, r, dw, ph, dot, part, mode, sc, s);
    case 8: return pull_gen<8>(g, ze, z, r, dw, ph, dot, part, mode, sc, s);
    default:
      set_error("schwarz (general mesh): lx=%d not compiled (4, 6, 8)", g->lx);
      return NTG_ERR_UNSUPPORTED;
  }
}

}  // namespace sw
}  // namespace ntg

extern "C" int ntg_schwarz_ghost_table(int64_t nelv, int lx, const int64_t* gid, int32_t* ghost) {
  ntg::clear_error();
  NTG_CHECK_ARG(nelv > 0 && lx >= 2 && lx <= NTG_LXMAX && gid && ghost, "ntg_schwarz_ghost_table: bad argument");
  NTG_CHECK_ARG(nelv * (int64_t)lx * lx * lx < ((int64_t)1 << 31), "ntg_schwarz_ghost_table: n must be < 2^31");
  std::vector<int32_t> tab;
  NTG_TRY(ntg::sw::ghost_table(nelv, lx, gid, tab));
  memcpy(ghost, tab.data(), sizeof(int32_t) * tab.size());
  return NTG_OK;
}
