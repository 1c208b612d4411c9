/*
 * CPU oracle for the spectral-element Helmholtz/Poisson hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA
 * library is compared against, and the timed CPU baseline.  Product code
 * never links, loads or calls it.
 *
 * What it restates, and from where:
 *   - GLL nodes/weights/derivative matrix, geometric factors G11..G33, mass
 *     matrix B, the matrix-free Helmholtz operator w = h1*(D^T G D)u + h2*B*u,
 *     gather-scatter (direct stiffness summation), the Jacobi diagonal and
 *     Jacobi-PCG: the textbook SEM formulation (Deville, Fischer & Mund,
 *     "High-Order Methods for Incompressible Fluid Flow", 2002, ch. 2 and 4).
 *     The reference obtains these from the external Neko library
 *     (imported at sources/mapping_functions/PDE_filter_mapping.f90:41-63 and
 *     sources/adjoint/adjoint_pnpn.f90:36-81); Neko's source is not part of
 *     the reference tree, so these are written from the mathematics.
 *   - Residual projection: Fischer, CMAME 163 (1998), A-conjugate basis of
 *     previous solutions; called by the reference at
 *     sources/adjoint/adjoint_pnpn.f90:729-741.
 *   - RAMP mapping: sources/mapping_functions/RAMP_mapping.f90:182-267.
 *   - PDE filter solve sequence: sources/mapping_functions/PDE_filter_mapping.f90:212-363.
 *   - Brinkman source term f -= chi*u:
 *     sources/source_terms/simple_brinkman_source_term.f90:139-153.
 *   - Masked vector ops and masked dot:
 *     sources/neko_ext/math/math_ext.f90:10-116 (1-based masks).
 *   - Permeability build kappa(phi): sources/topology_optimization/design.f90:316-348.
 *   - Minimum-dissipation sensitivity -u.u_adj + K|u|^2:
 *     sources/objectives/minimum_dissipation_objective_function.f90:260-301.
 *
 * Parity status: UNPINNED by the reference.  The reference tree holds no
 * test, golden vector or fixture for ax_helm, gs, CG, Jacobi or projection
 * (its only tests are the MMA toy programs tests/mma/mmatest1.f90 and
 * mmatest2.f90).  This oracle is
 * pinned instead by known-answer tests (A*1 = 0 for h2 = 0, exact weak
 * Laplacian of polynomials, gs(1) = multiplicity, symmetry, manufactured
 * solutions) and by an independent numpy/scipy assembly on small meshes.
 *
 * Layout: Neko's field layout x(lx,ly,lz,nelv), i fastest:
 *   idx(i,j,k,e) = i + lx*(j + lx*(k + lx*e)).
 * Derivative matrix: D[i*lx + j] = d(phi_j)/dr at node i.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_PI 3.14159265358979323846

/* ------------------------------------------------------------------ */
/* Counter-based RNG: SplitMix64 keyed by (seed, stream, index).        */
/* ------------------------------------------------------------------ */
static inline uint64_t orc_mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
uint64_t orc_rng_u64(uint64_t seed, uint64_t stream, uint64_t idx) {
  uint64_t key = orc_mix64(seed * 0x9E3779B97F4A7C15ULL + stream * 0xD1B54A32D192ED03ULL + 0x632BE59BD9B4E019ULL);
  return orc_mix64(key + (idx + 1) * 0x9E3779B97F4A7C15ULL);
}
double orc_rng_unif(uint64_t seed, uint64_t stream, uint64_t idx) {
  return (double)(orc_rng_u64(seed, stream, idx) >> 11) * (1.0 / 9007199254740992.0);
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void orc_set_threads(int t) {
#ifdef _OPENMP
  if (t > 0) omp_set_num_threads(t);
#else
  (void)t;
#endif
}

/* ------------------------------------------------------------------ */
/* GLL points, weights, derivative matrix.                              */
/* Newton iteration for the roots of (1-x^2) P_N'(x) from Chebyshev-     */
/* Gauss-Lobatto starting points; weights 2/(N(N+1) P_N(x)^2);          */
/* D_ij = P_N(x_i)/(P_N(x_j)(x_i-x_j)), D_00 = -N(N+1)/4, D_NN = -D_00.  */
/* ------------------------------------------------------------------ */
static void legendre_pair(int N, double x, double* pN, double* pNm1) {
  double p0 = 1.0, p1 = x;
  if (N == 0) { *pN = 1.0; *pNm1 = 0.0; return; }
  for (int k = 2; k <= N; ++k) {
    double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
    p0 = p1; p1 = p2;
  }
  *pN = p1; *pNm1 = p0;
}

void orc_gll(int lx, double* xi, double* w, double* D) {
  int N = lx - 1;
  for (int j = 0; j <= N; ++j) {
    double x = -cos(ORC_PI * j / N);
    for (int it = 0; it < 100; ++it) {
      double pN, pNm1;
      legendre_pair(N, x, &pN, &pNm1);
      double dx = (x * pN - pNm1) / ((N + 1) * pN);
      x -= dx;
      if (fabs(dx) < 1e-17) break;
    }
    xi[j] = x;
  }
  /* exact end points and exact antisymmetry */
  xi[0] = -1.0; xi[N] = 1.0;
  for (int j = 0; j < lx / 2; ++j) {
    double a = 0.5 * (xi[N - j] - xi[j]);
    xi[j] = -a; xi[N - j] = a;
  }
  if (lx % 2 == 1) xi[N / 2] = 0.0;
  double pn[64];
  for (int j = 0; j <= N; ++j) {
    double pNm1;
    legendre_pair(N, xi[j], &pn[j], &pNm1);
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

/* ------------------------------------------------------------------ */
/* Structured box mesh with an optional seeded sinusoidal deformation.  */
/* Element e = ex + Ex*(ey + Ey*ez); node (i,j,k) of e sits at global   */
/* structured index (ex*N+i, ey*N+j, ez*N+k); its global id is          */
/* gx + (Ex*N+1)*(gy + (Ey*N+1)*gz).                                    */
/* Displacement per axis d: amp*h_d*sin(2*pi*(a_d S + b_d T + c_d U)    */
/* + phi_d), with S,T,U the structured node positions in units of 16    */
/* elements ((ex + t_i)/16, ...), (a_d,b_d,c_d) in {1,2,3} and phi_d in  */
/* [0,2pi) drawn from the seed: a wavelength of 16/a elements whatever   */
/* the mesh size, so every element stays well shaped.                    */
/* ------------------------------------------------------------------ */
enum { ORC_STREAM_MESH = 1, ORC_STREAM_RHO = 2, ORC_STREAM_RHS = 3, ORC_STREAM_MODES = 4,
       ORC_STREAM_BLOBS = 5, ORC_STREAM_AR = 6, ORC_STREAM_PERT = 7 };

void orc_deform_params(uint64_t seed, int* abc /*9*/, double* phase /*3*/) {
  for (int d = 0; d < 3; ++d) {
    for (int q = 0; q < 3; ++q) abc[3 * d + q] = 1 + (int)(orc_rng_u64(seed, ORC_STREAM_MESH, 4 * d + q) % 3ULL);
    phase[d] = 2.0 * ORC_PI * orc_rng_unif(seed, ORC_STREAM_MESH, 4 * d + 3);
  }
}

void orc_mesh_box(int Ex, int Ey, int Ez, int lx, const double* lo, const double* hi, double amp, uint64_t seed,
                  double* x, double* y, double* z, int64_t* gid) {
  double xi[64], w[64], D[64 * 64];
  orc_gll(lx, xi, w, D);
  int N = lx - 1;
  double t[64];
  for (int i = 0; i < lx; ++i) t[i] = 0.5 * (xi[i] + 1.0);
  t[0] = 0.0; t[N] = 1.0;
  int abc[9]; double ph[3];
  orc_deform_params(seed, abc, ph);
  double h[3] = {(hi[0] - lo[0]) / Ex, (hi[1] - lo[1]) / Ey, (hi[2] - lo[2]) / Ez};
  int64_t nx = (int64_t)Ex * N + 1, ny = (int64_t)Ey * N + 1;
  int64_t nelv = (int64_t)Ex * Ey * Ez;
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < nelv; ++e) {
    int ex = (int)(e % Ex), ey = (int)((e / Ex) % Ey), ez = (int)(e / ((int64_t)Ex * Ey));
    for (int k = 0; k < lx; ++k)
      for (int j = 0; j < lx; ++j)
        for (int i = 0; i < lx; ++i) {
          int64_t l = i + lx * (j + lx * (k + (int64_t)lx * e));
          /* normalised coordinates, computed from integer structure so
             shared nodes agree bit for bit */
          double X = (ex + t[i]) / Ex, Y = (ey + t[j]) / Ey, Z = (ez + t[k]) / Ez;
          double px = lo[0] + X * (hi[0] - lo[0]);
          double py = lo[1] + Y * (hi[1] - lo[1]);
          double pz = lo[2] + Z * (hi[2] - lo[2]);
          if (amp != 0.0) {
            double S = (ex + t[i]) / 16.0, T = (ey + t[j]) / 16.0, U = (ez + t[k]) / 16.0;
            double s0 = sin(2.0 * ORC_PI * (abc[0] * S + abc[1] * T + abc[2] * U) + ph[0]);
            double s1 = sin(2.0 * ORC_PI * (abc[3] * S + abc[4] * T + abc[5] * U) + ph[1]);
            double s2 = sin(2.0 * ORC_PI * (abc[6] * S + abc[7] * T + abc[8] * U) + ph[2]);
            px += amp * h[0] * s0;
            py += amp * h[1] * s1;
            pz += amp * h[2] * s2;
          }
          x[l] = px; y[l] = py; z[l] = pz;
          int64_t gx = (int64_t)ex * N + i, gy = (int64_t)ey * N + j, gz = (int64_t)ez * N + k;
          gid[l] = gx + nx * (gy + ny * gz);
        }
  }
}

/* Local indices of the face x = hi (the element face i = N of the last
   element column), as a 1-based Neko-style mask, in increasing order.
   Pass mask = NULL to get the count only. */
int64_t orc_mask_face_xmax(int Ex, int Ey, int Ez, int lx, int32_t* mask) {
  int64_t cnt = 0;
  int64_t nelv = (int64_t)Ex * Ey * Ez;
  for (int64_t e = 0; e < nelv; ++e) {
    int ex = (int)(e % Ex);
    if (ex != Ex - 1) continue;
    for (int k = 0; k < lx; ++k)
      for (int j = 0; j < lx; ++j) {
        int64_t l = (lx - 1) + lx * (j + lx * (k + (int64_t)lx * e));
        if (mask) mask[cnt] = (int32_t)(l + 1);
        cnt++;
      }
  }
  return cnt; /* ascending: elements ascend, and within one element l ascends */
}

/* ------------------------------------------------------------------ */
/* Geometric factors.                                                    */
/* x_r = sum_l D[i][l] x(l,j,k) etc.; J = det(dx/dr);                    */
/* G_ab = w_i w_j w_k J (grad r_a . grad r_b); B = w_i w_j w_k J.        */
/* ------------------------------------------------------------------ */
void orc_geom(int64_t nelv, int lx, const double* x, const double* y, const double* z,
              double* g11, double* g12, double* g13, double* g22, double* g23, double* g33,
              double* B, double* jac) {
  double xi[64], w[64], D[64 * 64];
  orc_gll(lx, xi, w, D);
  int64_t lx3 = (int64_t)lx * lx * lx;
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < nelv; ++e) {
    const double* xe = x + e * lx3;
    const double* ye = y + e * lx3;
    const double* ze = z + e * lx3;
    for (int k = 0; k < lx; ++k)
      for (int j = 0; j < lx; ++j)
        for (int i = 0; i < lx; ++i) {
          double xr = 0, xs = 0, xt = 0, yr = 0, ys = 0, yt = 0, zr = 0, zs = 0, zt = 0;
          for (int l = 0; l < lx; ++l) {
            int ir = l + lx * (j + lx * k), is = i + lx * (l + lx * k), it = i + lx * (j + lx * l);
            double dr = D[i * lx + l], ds = D[j * lx + l], dt = D[k * lx + l];
            xr += dr * xe[ir]; yr += dr * ye[ir]; zr += dr * ze[ir];
            xs += ds * xe[is]; ys += ds * ye[is]; zs += ds * ze[is];
            xt += dt * xe[it]; yt += dt * ye[it]; zt += dt * ze[it];
          }
          double J = xr * (ys * zt - yt * zs) - xs * (yr * zt - yt * zr) + xt * (yr * zs - ys * zr);
          double iJ = 1.0 / J;
          double rx = (ys * zt - yt * zs) * iJ, ry = (xt * zs - xs * zt) * iJ, rz = (xs * yt - xt * ys) * iJ;
          double sx = (yt * zr - yr * zt) * iJ, sy = (xr * zt - xt * zr) * iJ, sz = (xt * yr - xr * yt) * iJ;
          double tx = (yr * zs - ys * zr) * iJ, ty = (xs * zr - xr * zs) * iJ, tz = (xr * ys - xs * yr) * iJ;
          double wJ = w[i] * w[j] * w[k] * J;
          int64_t m = e * lx3 + i + lx * (j + lx * k);
          g11[m] = wJ * (rx * rx + ry * ry + rz * rz);
          g12[m] = wJ * (rx * sx + ry * sy + rz * sz);
          g13[m] = wJ * (rx * tx + ry * ty + rz * tz);
          g22[m] = wJ * (sx * sx + sy * sy + sz * sz);
          g23[m] = wJ * (sx * tx + sy * ty + sz * tz);
          g33[m] = wJ * (tx * tx + ty * ty + tz * tz);
          B[m] = wJ;
          if (jac) jac[m] = J;
        }
  }
}

/* ------------------------------------------------------------------ */
/* Gather-scatter maps: local indices stably sorted by global id.       */
/* perm[n]: local index list; offs[nu+1]: segment offsets;               */
/* uid[n]: dense unique index of each local DOF.  Returns nu.           */
/* ------------------------------------------------------------------ */
static int cmp_pair(const void* a, const void* b) {
  const int64_t* pa = (const int64_t*)a;
  const int64_t* pb = (const int64_t*)b;
  if (pa[0] != pb[0]) return pa[0] < pb[0] ? -1 : 1;
  return pa[1] < pb[1] ? -1 : (pa[1] > pb[1]);
}

int64_t orc_gs_build(int64_t n, const int64_t* gid, int32_t* perm, int64_t* offs, int32_t* uid) {
  int64_t gmax = -1, gmin = INT64_MAX;
  for (int64_t l = 0; l < n; ++l) {
    if (gid[l] > gmax) gmax = gid[l];
    if (gid[l] < gmin) gmin = gid[l];
  }
  int64_t nu = 0;
  if (n == 0) { offs[0] = 0; return 0; }
  if (gmin >= 0 && gmax < 4 * n + 16) {
    /* counting sort: stable in the local index */
    int64_t range = gmax + 1;
    int64_t* cnt = (int64_t*)calloc((size_t)range + 1, sizeof(int64_t));
    for (int64_t l = 0; l < n; ++l) cnt[gid[l] + 1]++;
    for (int64_t g = 0; g < range; ++g) cnt[g + 1] += cnt[g];
    int64_t* pos = (int64_t*)malloc(sizeof(int64_t) * (size_t)(range + 1));
    memcpy(pos, cnt, sizeof(int64_t) * (size_t)(range + 1));
    for (int64_t l = 0; l < n; ++l) perm[pos[gid[l]]++] = (int32_t)l;
    for (int64_t g = 0; g < range; ++g)
      if (cnt[g + 1] > cnt[g]) offs[nu++] = cnt[g];
    offs[nu] = n;
    free(pos);
    free(cnt);
  } else {
    int64_t* pr = (int64_t*)malloc(sizeof(int64_t) * 2 * (size_t)n);
    for (int64_t l = 0; l < n; ++l) { pr[2 * l] = gid[l]; pr[2 * l + 1] = l; }
    qsort(pr, (size_t)n, 2 * sizeof(int64_t), cmp_pair);
    for (int64_t p = 0; p < n; ++p) {
      perm[p] = (int32_t)pr[2 * p + 1];
      if (p == 0 || pr[2 * p] != pr[2 * p - 2]) offs[nu++] = p;
    }
    offs[nu] = n;
    free(pr);
  }
  if (uid)
    for (int64_t s = 0; s < nu; ++s)
      for (int64_t p = offs[s]; p < offs[s + 1]; ++p) uid[perm[p]] = (int32_t)s;
  return nu;
}

/* op: 1 = add, 2 = mul, 3 = min, 4 = max (Neko GS_OP_ADD/MUL/MIN/MAX) */
void orc_gs_op(double* u, int64_t nu, const int32_t* perm, const int64_t* offs, int op) {
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < nu; ++s) {
    int64_t a = offs[s], b = offs[s + 1];
    if (b - a < 2) continue;
    double acc = u[perm[a]];
    for (int64_t p = a + 1; p < b; ++p) {
      double v = u[perm[p]];
      if (op == 1) acc += v;
      else if (op == 2) acc *= v;
      else if (op == 3) acc = v < acc ? v : acc;
      else acc = v > acc ? v : acc;
    }
    for (int64_t p = a; p < b; ++p) u[perm[p]] = acc;
  }
}

void orc_mult(int64_t n, int64_t nu, const int32_t* perm, const int64_t* offs, double* mult) {
  (void)n;
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < nu; ++s) {
    double c = (double)(offs[s + 1] - offs[s]);
    for (int64_t p = offs[s]; p < offs[s + 1]; ++p) mult[perm[p]] = 1.0 / c;
  }
}

/* ------------------------------------------------------------------ */
/* Helmholtz operator (element-local, unassembled):                     */
/*   w = h1 * (D^T G D) u + h2 * B * u                                   */
/* h1 == NULL -> constant h1c; h2 == NULL -> no mass term.              */
/* ------------------------------------------------------------------ */
/* Each contraction is written as a small matrix product whose innermost
   loop runs over contiguous memory (the mxm form of CPU SEM codes), so the
   compiler vectorises it; every sum over l still runs in ascending l. */
void orc_ax_helm(int64_t nelv, int lx, const double* D, double* w, const double* u,
                 const double* g11, const double* g12, const double* g13,
                 const double* g22, const double* g23, const double* g33,
                 const double* h1, double h1c, const double* h2, const double* B) {
  const int lx2 = lx * lx, lx3 = lx * lx * lx;
#pragma omp parallel
  {
    double ur[1000], us[1000], ut[1000], acc[1000];
#pragma omp for schedule(static)
    for (int64_t e = 0; e < nelv; ++e) {
      const double* ue = u + e * (int64_t)lx3;
      const int64_t base = e * (int64_t)lx3;
      for (int m = 0; m < lx3; ++m) ur[m] = us[m] = ut[m] = 0.0;
      /* ur[i + lx c] = sum_l D[i][l] u[l + lx c]   (c = j + lx k) */
      for (int c = 0; c < lx2; ++c)
        for (int l = 0; l < lx; ++l) {
          const double a = ue[l + lx * c];
          for (int i = 0; i < lx; ++i) ur[i + lx * c] += D[i * lx + l] * a;
        }
      /* us[i + lx (j + lx k)] = sum_l D[j][l] u[i + lx (l + lx k)] */
      for (int k = 0; k < lx; ++k)
        for (int j = 0; j < lx; ++j)
          for (int l = 0; l < lx; ++l) {
            const double d = D[j * lx + l];
            const double* src = ue + lx * (l + lx * k);
            double* dst = us + lx * (j + lx * k);
            for (int i = 0; i < lx; ++i) dst[i] += d * src[i];
          }
      /* ut[ij + lx2 k] = sum_l D[k][l] u[ij + lx2 l] */
      for (int k = 0; k < lx; ++k)
        for (int l = 0; l < lx; ++l) {
          const double d = D[k * lx + l];
          for (int ij = 0; ij < lx2; ++ij) ut[ij + lx2 * k] += d * ue[ij + lx2 * l];
        }
      /* metric mix: (wr, ws, wt) = h1 G (ur, us, ut), stored back in place */
      for (int m = 0; m < lx3; ++m) {
        const int64_t gm = base + m;
        const double hh = h1 ? h1[gm] : h1c;
        const double a = ur[m], b = us[m], c = ut[m];
        ur[m] = hh * (g11[gm] * a + g12[gm] * b + g13[gm] * c);
        us[m] = hh * (g12[gm] * a + g22[gm] * b + g23[gm] * c);
        ut[m] = hh * (g13[gm] * a + g23[gm] * b + g33[gm] * c);
        acc[m] = 0.0;
      }
      /* transposed contractions */
      for (int c = 0; c < lx2; ++c)
        for (int l = 0; l < lx; ++l) {
          const double a = ur[l + lx * c];
          for (int i = 0; i < lx; ++i) acc[i + lx * c] += D[l * lx + i] * a;
        }
      for (int k = 0; k < lx; ++k)
        for (int j = 0; j < lx; ++j)
          for (int l = 0; l < lx; ++l) {
            const double d = D[l * lx + j];
            const double* src = us + lx * (l + lx * k);
            double* dst = acc + lx * (j + lx * k);
            for (int i = 0; i < lx; ++i) dst[i] += d * src[i];
          }
      for (int k = 0; k < lx; ++k)
        for (int l = 0; l < lx; ++l) {
          const double d = D[l * lx + k];
          for (int ij = 0; ij < lx2; ++ij) acc[ij + lx2 * k] += d * ut[ij + lx2 * l];
        }
      for (int m = 0; m < lx3; ++m) {
        const int64_t gm = base + m;
        double v = acc[m];
        if (h2) v += h2[gm] * B[gm] * ue[m];
        w[gm] = v;
      }
    }
  }
}

/* Same operator evaluated in single precision throughout (inputs rounded
   to float, float accumulation), for the FP32 kernel's tolerance test. */
void orc_ax_helm_f32(int64_t nelv, int lx, const float* D, float* w, const float* u,
                     const float* g11, const float* g12, const float* g13,
                     const float* g22, const float* g23, const float* g33,
                     const float* h1, float h1c, const float* hB) {
  int64_t lx3 = (int64_t)lx * lx * lx;
#pragma omp parallel
  {
    float* wr = (float*)malloc(sizeof(float) * (size_t)lx3 * 3);
    float* ws = wr + lx3;
    float* wt = ws + lx3;
#pragma omp for schedule(static)
    for (int64_t e = 0; e < nelv; ++e) {
      const float* ue = u + e * lx3;
      int64_t base = e * lx3;
      for (int k = 0; k < lx; ++k)
        for (int j = 0; j < lx; ++j)
          for (int i = 0; i < lx; ++i) {
            float ur = 0, us = 0, ut = 0;
            for (int l = 0; l < lx; ++l) {
              ur += D[i * lx + l] * ue[l + lx * (j + lx * k)];
              us += D[j * lx + l] * ue[i + lx * (l + lx * k)];
              ut += D[k * lx + l] * ue[i + lx * (j + lx * l)];
            }
            int m = i + lx * (j + lx * k);
            int64_t gm = base + m;
            float hh = h1 ? h1[gm] : h1c;
            wr[m] = hh * (g11[gm] * ur + g12[gm] * us + g13[gm] * ut);
            ws[m] = hh * (g12[gm] * ur + g22[gm] * us + g23[gm] * ut);
            wt[m] = hh * (g13[gm] * ur + g23[gm] * us + g33[gm] * ut);
          }
      for (int k = 0; k < lx; ++k)
        for (int j = 0; j < lx; ++j)
          for (int i = 0; i < lx; ++i) {
            float acc = 0;
            for (int l = 0; l < lx; ++l) {
              acc += D[l * lx + i] * wr[l + lx * (j + lx * k)];
              acc += D[l * lx + j] * ws[i + lx * (l + lx * k)];
              acc += D[l * lx + k] * wt[i + lx * (j + lx * l)];
            }
            int m = i + lx * (j + lx * k);
            int64_t gm = base + m;
            if (hB) acc += hB[gm] * ue[m];
            w[gm] = acc;
          }
    }
    free(wr);
  }
}

/* Diagonal of the element-local operator (before assembly):
   h1-weighted sums of D^2 G_aa along each direction, the G12/G13/G23
   cross terms (non-zero only where D has a diagonal, i.e. element
   boundary nodes), plus h2*B. */
void orc_helm_diag(int64_t nelv, int lx, const double* D, double* d,
                   const double* g11, const double* g12, const double* g13,
                   const double* g22, const double* g23, const double* g33,
                   const double* h1, double h1c, const double* h2, const double* B) {
  int64_t lx3 = (int64_t)lx * lx * lx;
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < nelv; ++e) {
    int64_t base = e * lx3;
    for (int k = 0; k < lx; ++k)
      for (int j = 0; j < lx; ++j)
        for (int i = 0; i < lx; ++i) {
          double acc = 0;
          for (int l = 0; l < lx; ++l) {
            int64_t qr = base + l + lx * (j + lx * k);
            int64_t qs = base + i + lx * (l + lx * k);
            int64_t qt = base + i + lx * (j + lx * l);
            double hr = h1 ? h1[qr] : h1c, hs = h1 ? h1[qs] : h1c, ht = h1 ? h1[qt] : h1c;
            acc += D[l * lx + i] * D[l * lx + i] * g11[qr] * hr;
            acc += D[l * lx + j] * D[l * lx + j] * g22[qs] * hs;
            acc += D[l * lx + k] * D[l * lx + k] * g33[qt] * ht;
          }
          int64_t m = base + i + lx * (j + lx * k);
          double hm = h1 ? h1[m] : h1c;
          double di = D[i * lx + i], dj = D[j * lx + j], dk = D[k * lx + k];
          acc += 2.0 * hm * (di * dj * g12[m] + di * dk * g13[m] + dj * dk * g23[m]);
          if (h2) acc += h2[m] * B[m];
          d[m] = acc;
        }
  }
}

/* ------------------------------------------------------------------ */
/* Operator context used by the solvers.                                 */
/* ------------------------------------------------------------------ */
typedef struct {
  int64_t nelv; int lx; int64_t n; int64_t nu;
  const double* D;
  const double *g11, *g12, *g13, *g22, *g23, *g33, *B, *mult;
  const double* h1; double h1c; const double* h2;
  const int32_t* perm; const int64_t* offs;
  const int32_t* mask; int64_t nmask; /* 1-based Dirichlet mask */
  const double* dinv;
} orc_op_t;

/* assembled, masked operator: w = mask(gs(A u)) */
static void op_apply(const orc_op_t* o, double* w, const double* u) {
  orc_ax_helm(o->nelv, o->lx, o->D, w, u, o->g11, o->g12, o->g13, o->g22, o->g23, o->g33, o->h1, o->h1c, o->h2, o->B);
  orc_gs_op(w, o->nu, o->perm, o->offs, 1);
  for (int64_t q = 0; q < o->nmask; ++q) w[o->mask[q] - 1] = 0.0;
}

/* sum_l mult*a*b, accumulated in long double per thread chunk then summed
   in a fixed order */
static double wdot(int64_t n, const double* a, const double* b, const double* mult) {
  int nt = orc_num_threads();
  long double* part = (long double*)calloc((size_t)nt, sizeof(long double));
#pragma omp parallel
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    long double s = 0;
#pragma omp for schedule(static)
    for (int64_t l = 0; l < n; ++l) s += (long double)mult[l] * a[l] * b[l];
    part[tid] = s;
  }
  long double s = 0;
  for (int t = 0; t < nt; ++t) s += part[t];
  free(part);
  return (double)s;
}

double orc_glsc3(int64_t n, const double* a, const double* b, const double* c) { return wdot(n, a, b, c); }

/* Jacobi: dinv = 1 / gs(diag), 1 on masked nodes */
void orc_jacobi(int64_t nelv, int lx, const double* D,
                const double* g11, const double* g12, const double* g13,
                const double* g22, const double* g23, const double* g33,
                const double* h1, double h1c, const double* h2, const double* B,
                int64_t nu, const int32_t* perm, const int64_t* offs,
                const int32_t* mask, int64_t nmask, double* dinv) {
  int64_t n = nelv * (int64_t)lx * lx * lx;
  orc_helm_diag(nelv, lx, D, dinv, g11, g12, g13, g22, g23, g33, h1, h1c, h2, B);
  orc_gs_op(dinv, nu, perm, offs, 1);
  for (int64_t q = 0; q < nmask; ++q) dinv[mask[q] - 1] = 1.0;
#pragma omp parallel for schedule(static)
  for (int64_t l = 0; l < n; ++l) dinv[l] = 1.0 / dinv[l];
}

/* Jacobi-PCG.  x holds the initial guess on entry and the solution on
   exit.  f is the assembled RHS (gs applied, masked).  Stops when
   sqrt(sum mult r^2) <= max(abstol, rtol*sqrt(sum mult f^2)) or after
   max_iter iterations.  out[0] = iterations, out[1] = res_start,
   out[2] = res_final.  If max_iter < 0, exactly -max_iter iterations are
   run with no convergence test (fixed-iteration parity). */
void orc_cg(int64_t nelv, int lx, const double* D,
            const double* g11, const double* g12, const double* g13,
            const double* g22, const double* g23, const double* g33,
            const double* h1, double h1c, const double* h2, const double* B, const double* mult,
            int64_t nu, const int32_t* perm, const int64_t* offs,
            const int32_t* mask, int64_t nmask, const double* dinv,
            double* x, const double* f, double rtol, double abstol, int max_iter, double* out) {
  orc_op_t o = {nelv, lx, nelv * (int64_t)lx * lx * lx, nu, D, g11, g12, g13, g22, g23, g33, B, mult,
                h1, h1c, h2, perm, offs, mask, nmask, dinv};
  int64_t n = o.n;
  double* r = (double*)malloc(sizeof(double) * (size_t)n * 4);
  double* z = r + n;
  double* p = z + n;
  double* w = p + n;
  int fixed = max_iter < 0;
  int maxit = fixed ? -max_iter : max_iter;
  op_apply(&o, w, x);
#pragma omp parallel for schedule(static)
  for (int64_t l = 0; l < n; ++l) r[l] = f[l] - w[l];
  for (int64_t q = 0; q < nmask; ++q) r[mask[q] - 1] = 0.0;
  double fnorm = sqrt(wdot(n, f, f, mult));
  double rnorm = sqrt(wdot(n, r, r, mult));
  double tol = rtol * fnorm;
  if (abstol > tol) tol = abstol;
  out[1] = rnorm;
  int it = 0;
  if (!fixed && rnorm <= tol) { out[0] = 0; out[2] = rnorm; free(r); return; }
#pragma omp parallel for schedule(static)
  for (int64_t l = 0; l < n; ++l) { z[l] = dinv[l] * r[l]; p[l] = z[l]; }
  double rz = wdot(n, r, z, mult);
  for (it = 1; it <= maxit; ++it) {
    op_apply(&o, w, p);
    double pap = wdot(n, p, w, mult);
    double alpha = rz / pap;
#pragma omp parallel for schedule(static)
    for (int64_t l = 0; l < n; ++l) {
      x[l] += alpha * p[l];
      r[l] -= alpha * w[l];
      z[l] = dinv[l] * r[l];
    }
    double rz_new = wdot(n, r, z, mult);
    rnorm = sqrt(wdot(n, r, r, mult));
    if (!fixed && rnorm <= tol) break;
    double beta = rz_new / rz;
    rz = rz_new;
#pragma omp parallel for schedule(static)
    for (int64_t l = 0; l < n; ++l) p[l] = z[l] + beta * p[l];
  }
  if (it > maxit) it = maxit;
  out[0] = it;
  out[2] = rnorm;
  free(r);
}

/* Time a bounded number of CG iterations (CPU baseline sample).
   Returns seconds per iteration (wall clock, OpenMP threads). */
double orc_cg_time_per_iter(int64_t nelv, int lx, const double* D,
                            const double* g11, const double* g12, const double* g13,
                            const double* g22, const double* g23, const double* g33,
                            const double* h1, double h1c, const double* h2, const double* B, const double* mult,
                            int64_t nu, const int32_t* perm, const int64_t* offs,
                            const int32_t* mask, int64_t nmask, const double* dinv,
                            double* x, const double* f, int iters) {
  double out[3];
  double t0 = 0, t1 = 0;
#ifdef _OPENMP
  t0 = omp_get_wtime();
#endif
  orc_cg(nelv, lx, D, g11, g12, g13, g22, g23, g33, h1, h1c, h2, B, mult, nu, perm, offs, mask, nmask, dinv,
         x, f, 0.0, 0.0, -iters, out);
#ifdef _OPENMP
  t1 = omp_get_wtime();
#endif
  return (t1 - t0) / iters;
}

/* ------------------------------------------------------------------ */
/* Fischer residual projection (A-conjugate basis of earlier solves).   */
/* Basis xs[L][n], axs[L][n] (A applied, assembled), count *m.          */
/* pre:  alpha_k = (x_k, b); xbar = sum alpha_k x_k;                     */
/*       b <- b - sum alpha_k (A x_k)                                    */
/* post: dx (solution of the reduced system) is A-orthogonalised against */
/*       the basis (classical Gram-Schmidt, twice), normalised, appended; */
/*       x = xbar + dx.  When the basis is full it restarts from the     */
/*       normalised full solution.                                       */
/* ------------------------------------------------------------------ */
void orc_proj_pre(int64_t n, int m, const double* xs, const double* axs, const double* mult,
                  double* b, double* xbar, double* alpha) {
  for (int k = 0; k < m; ++k) alpha[k] = wdot(n, xs + (int64_t)k * n, b, mult);
  memset(xbar, 0, sizeof(double) * (size_t)n);
  for (int k = 0; k < m; ++k) {
    const double* xk = xs + (int64_t)k * n;
    const double* ak = axs + (int64_t)k * n;
    double a = alpha[k];
#pragma omp parallel for schedule(static)
    for (int64_t l = 0; l < n; ++l) { xbar[l] += a * xk[l]; b[l] -= a * ak[l]; }
  }
}

/* dx in/out (becomes the full solution x), adx = A dx (assembled),
   b_orig_minus_bres = A xbar = b - b_reduced.  Returns the new count. */
int orc_proj_post(int64_t n, int L, int m, double* xs, double* axs, const double* mult,
                  double* dx, double* adx, const double* xbar, const double* axbar) {
  if (m >= L) {
    /* restart from the full solution x = xbar + dx */
    double* x = xs; double* ax = axs;
#pragma omp parallel for schedule(static)
    for (int64_t l = 0; l < n; ++l) { x[l] = xbar[l] + dx[l]; ax[l] = axbar[l] + adx[l]; }
    double nrm = sqrt(wdot(n, x, ax, mult));
    if (nrm > 0) {
      double s = 1.0 / nrm;
#pragma omp parallel for schedule(static)
      for (int64_t l = 0; l < n; ++l) { x[l] *= s; ax[l] *= s; }
    }
#pragma omp parallel for schedule(static)
    for (int64_t l = 0; l < n; ++l) dx[l] = xbar[l] + dx[l];
    return nrm > 0 ? 1 : 0;
  }
  double* v = xs + (int64_t)m * n;
  double* av = axs + (int64_t)m * n;
  memcpy(v, dx, sizeof(double) * (size_t)n);
  memcpy(av, adx, sizeof(double) * (size_t)n);
  double c[64];
  for (int pass = 0; pass < 2; ++pass) {
    for (int k = 0; k < m; ++k) c[k] = wdot(n, axs + (int64_t)k * n, v, mult);
    for (int k = 0; k < m; ++k) {
      const double* xk = xs + (int64_t)k * n;
      const double* ak = axs + (int64_t)k * n;
      double a = c[k];
#pragma omp parallel for schedule(static)
      for (int64_t l = 0; l < n; ++l) { v[l] -= a * xk[l]; av[l] -= a * ak[l]; }
    }
  }
  double nrm = sqrt(wdot(n, v, av, mult));
  int mnew = m;
  if (nrm > 1e-300) {
    double s = 1.0 / nrm;
#pragma omp parallel for schedule(static)
    for (int64_t l = 0; l < n; ++l) { v[l] *= s; av[l] *= s; }
    mnew = m + 1;
  }
#pragma omp parallel for schedule(static)
  for (int64_t l = 0; l < n; ++l) dx[l] = xbar[l] + dx[l];
  return mnew;
}

/* ------------------------------------------------------------------ */
/* Coefficient path (neko-top in-tree code).                             */
/* ------------------------------------------------------------------ */
/* RAMP_mapping.f90:182-196 (convex down) and :227-245 (convex up) */
void orc_ramp_forward(int64_t n, const double* xin, double* xout, double fmin, double fmax, double q, int convex_up) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    double x = xin[i];
    if (convex_up) xout[i] = fmin + (fmax - fmin) * x * (1.0 + q) / (x + q);
    else xout[i] = fmin + (fmax - fmin) * x / (1.0 + q * (1.0 - x));
  }
}
/* RAMP_mapping.f90:203-222 and :250-267 */
void orc_ramp_backward(int64_t n, const double* xin, const double* dF_dout, double* dF_din, double fmin,
                       double fmax, double q, int convex_up) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    double x = xin[i];
    double d;
    if (convex_up) d = (fmax - fmin) * (q + 1.0) / ((x + q) * (x + q));
    else d = (fmax - fmin) * (q + 1.0) / ((1.0 - q * (x - 1.0)) * (1.0 - q * (x - 1.0)));
    dF_din[i] = d * dF_dout[i];
  }
}
/* simple_brinkman_source_term.f90:139-153: f_c -= u_c * chi */
void orc_brinkman(int64_t n, double* fx, double* fy, double* fz, const double* u, const double* v,
                  const double* w, const double* chi) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    fx[i] -= u[i] * chi[i];
    fy[i] -= v[i] * chi[i];
    fz[i] -= w[i] * chi[i];
  }
}
/* design.f90:316-348: kappa = -(perm_1 + (perm_0-perm_1)(pen+1) phi/(pen+phi)) */
void orc_permeability(int64_t n, const double* phi, double* kappa, double perm0, double perm1, double pen) {
  double c = (perm0 - perm1) * (pen + 1.0);
  for (int64_t i = 0; i < n; ++i) {
    double r = 1.0 / (pen + phi[i]);
    r = r * phi[i];
    r = r * c;
    r = r + perm1;
    kappa[i] = -1.0 * r;
  }
}
/* minimum_dissipation_objective_function.f90:272-296 */
void orc_sens_min_dissipation(int64_t n, double* s, const double* u, const double* v, const double* w,
                              const double* ua, const double* va, const double* wa, int if_lube, double K_scale) {
  for (int64_t i = 0; i < n; ++i) {
    double t = u[i] * ua[i];
    t += v[i] * va[i];
    t += w[i] * wa[i];
    t *= -1.0;
    if (if_lube) {
      double l = u[i] * u[i];
      l += v[i] * v[i];
      l += w[i] * w[i];
      t += K_scale * l;
    }
    s[i] = t;
  }
}

/* math_ext.f90:10-116 (1-based masks) */
void orc_cadd_mask(double* a, double c, const int32_t* mask, int64_t m) { for (int64_t i = 0; i < m; ++i) a[mask[i] - 1] += c; }
void orc_invcol1_mask(double* a, const int32_t* mask, int64_t m) { for (int64_t i = 0; i < m; ++i) a[mask[i] - 1] = 1.0 / a[mask[i] - 1]; }
void orc_cmult_mask(double* a, double c, const int32_t* mask, int64_t m) { for (int64_t i = 0; i < m; ++i) a[mask[i] - 1] = c * a[mask[i] - 1]; }
void orc_col2_mask(double* a, const double* b, const int32_t* mask, int64_t m) { for (int64_t i = 0; i < m; ++i) a[mask[i] - 1] *= b[mask[i] - 1]; }
void orc_col3_mask(double* a, const double* b, const double* c, const int32_t* mask, int64_t m) { for (int64_t i = 0; i < m; ++i) a[mask[i] - 1] = b[mask[i] - 1] * c[mask[i] - 1]; }
void orc_sub3_mask(double* a, const double* b, const double* c, const int32_t* mask, int64_t m) { for (int64_t i = 0; i < m; ++i) a[mask[i] - 1] = b[mask[i] - 1] - c[mask[i] - 1]; }
double orc_glsc2_mask(const double* a, const double* b, const int32_t* mask, int64_t m) {
  long double s = 0;
  for (int64_t i = 0; i < m; ++i) s += (long double)a[mask[i] - 1] * b[mask[i] - 1];
  return (double)s;
}

/* ------------------------------------------------------------------ */
/* Synthetic fields (seeded, per unique node so they are continuous).    */
/* ------------------------------------------------------------------ */
/* rho ~ U[0,1] per unique node */
void orc_field_uniform(int64_t n, const int64_t* gid, uint64_t seed, uint64_t stream, double lo, double hi, double* f) {
#pragma omp parallel for schedule(static)
  for (int64_t l = 0; l < n; ++l) f[l] = lo + (hi - lo) * orc_rng_unif(seed, stream, (uint64_t)gid[l]);
}

/* Fourier modes: f(x) = sum_m a_m cos(2 pi (k_m . X) + phi_m), X the
   coordinate normalised by the box (lo, hi); k_m integer in [1, kmax]^3,
   a_m = s_m / |k_m|^2 with s_m ~ U[-1,1]. Mode parameters depend only on
   (seed, m). */
void orc_fourier_params(uint64_t seed, int nmodes, int kmax, int* k, double* amp, double* ph) {
  for (int m = 0; m < nmodes; ++m) {
    double kk = 0;
    for (int d = 0; d < 3; ++d) {
      k[3 * m + d] = 1 + (int)(orc_rng_u64(seed, ORC_STREAM_MODES, 8 * m + d) % (uint64_t)kmax);
      kk += (double)k[3 * m + d] * k[3 * m + d];
    }
    amp[m] = (2.0 * orc_rng_unif(seed, ORC_STREAM_MODES, 8 * m + 3) - 1.0) / kk;
    ph[m] = 2.0 * ORC_PI * orc_rng_unif(seed, ORC_STREAM_MODES, 8 * m + 4);
  }
}
void orc_field_fourier(int64_t n, const double* x, const double* y, const double* z, const double* lo,
                       const double* hi, int nmodes, const int* k, const double* amp, const double* ph, double* f) {
#pragma omp parallel for schedule(static)
  for (int64_t l = 0; l < n; ++l) {
    double X = (x[l] - lo[0]) / (hi[0] - lo[0]);
    double Y = (y[l] - lo[1]) / (hi[1] - lo[1]);
    double Z = (z[l] - lo[2]) / (hi[2] - lo[2]);
    double s = 0;
    for (int m = 0; m < nmodes; ++m)
      s += amp[m] * cos(2.0 * ORC_PI * (k[3 * m] * X + k[3 * m + 1] * Y + k[3 * m + 2] * Z) + ph[m]);
    f[l] = s;
  }
}
/* Gaussian blobs: rho = clip(sum_b exp(-|x - c_b|^2 / (2 width^2)), 0, 1),
   centres c_b ~ U(box) from (seed, b). */
void orc_field_blobs(int64_t n, const double* x, const double* y, const double* z, const double* lo,
                     const double* hi, uint64_t seed, int nblobs, double width, double* f) {
  double c[3 * 64];
  for (int b = 0; b < nblobs; ++b)
    for (int d = 0; d < 3; ++d)
      c[3 * b + d] = lo[d] + (hi[d] - lo[d]) * orc_rng_unif(seed, ORC_STREAM_BLOBS, 4 * b + d);
#pragma omp parallel for schedule(static)
  for (int64_t l = 0; l < n; ++l) {
    double s = 0;
    for (int b = 0; b < nblobs; ++b) {
      double dx = x[l] - c[3 * b], dy = y[l] - c[3 * b + 1], dz = z[l] - c[3 * b + 2];
      s += exp(-(dx * dx + dy * dy + dz * dz) / (2.0 * width * width));
    }
    f[l] = s < 0 ? 0 : (s > 1 ? 1 : s);
  }
}
