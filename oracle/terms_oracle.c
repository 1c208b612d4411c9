/*
 * CPU oracle, part 2: the FP64 terms either side of the solves.
 *
 * TEST INFRASTRUCTURE ONLY: a compiled (OpenMP) restatement of
 * oracle/deriv_ref.py and oracle/dealias_ref.py, used as the timed CPU
 * baseline of those terms and checked against the numpy restatements.
 * Product code never links, loads or calls it.
 *
 * Conventions as in sem_oracle.c: layout idx = i + lx (j + lx (k + lx e));
 * D[a * lx + l] = l_l'(xi_a); the metric cofactors drdx..dtdz (of dx/dr)
 * and 1/jac stored as met[m * n + idx], m = 0..9 (drdx, drdy, drdz, dsdx,
 * dsdy, dsdz, dtdx, dtdy, dtdz, 1/jac).  Sources of the formulas:
 *   - derivative operators (opgrad, cdtp, curl): the SEM forms Neko's
 *     operators module implements (Deville, Fischer & Mund 2002, ch. 4), as
 *     the reference calls them in sources/adjoint/adv_adjoint_no_dealias.f90
 *     and sources/source_terms/adjoint_minimum_dissipation_source_term.f90;
 *   - adjoint / linearised advection, no dealiasing:
 *     sources/adjoint/adv_adjoint_no_dealias.f90:118-255 (device branch),
 *     :365-427;
 *   - dealiased: sources/adjoint/adv_adjoint_dealias.f90:235-600 (fields and
 *     cofactors interpolated to lxd Gauss-Legendre points, products there,
 *     J^T back).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* reference derivatives of one element tile s (nx^3) at every node */
static void rgrad(int nx, const double* D, const double* s, double* ur, double* us, double* ut) {
  const int n2 = nx * nx;
  for (int k = 0; k < nx; ++k)
    for (int j = 0; j < nx; ++j)
      for (int i = 0; i < nx; ++i) {
        double r = 0.0, q = 0.0, t = 0.0;
        for (int l = 0; l < nx; ++l) {
          r += D[i * nx + l] * s[k * n2 + j * nx + l];
          q += D[j * nx + l] * s[k * n2 + l * nx + i];
          t += D[k * nx + l] * s[l * n2 + j * nx + i];
        }
        const int q3 = k * n2 + j * nx + i;
        ur[q3] = r;
        us[q3] = q;
        ut[q3] = t;
      }
}

/* out[node] = sum_l D[l][i] fr(l,j,k) + D[l][j] fs(i,l,k) + D[l][k] ft(i,j,l) */
static void rgrad_t(int nx, const double* D, const double* fr, const double* fs, const double* ft, double* out) {
  const int n2 = nx * nx;
  for (int k = 0; k < nx; ++k)
    for (int j = 0; j < nx; ++j)
      for (int i = 0; i < nx; ++i) {
        double a = 0.0;
        for (int l = 0; l < nx; ++l) {
          a += D[l * nx + i] * fr[k * n2 + j * nx + l];
          a += D[l * nx + j] * fs[k * n2 + l * nx + i];
          a += D[l * nx + k] * ft[l * n2 + j * nx + i];
        }
        out[k * n2 + j * nx + i] = a;
      }
}

void orct_metrics(int64_t nelv, int lx, const double* D, const double* x, const double* y, const double* z,
                  double* met) {
  const int64_t l3 = (int64_t)lx * lx * lx, n = nelv * l3;
#pragma omp parallel
  {
    double* b = (double*)malloc(sizeof(double) * 9 * l3);
    double *xr = b, *xs = b + l3, *xt = b + 2 * l3, *yr = b + 3 * l3, *ys = b + 4 * l3, *yt = b + 5 * l3,
           *zr = b + 6 * l3, *zs = b + 7 * l3, *zt = b + 8 * l3;
#pragma omp for schedule(static)
    for (int64_t e = 0; e < nelv; ++e) {
      rgrad(lx, D, x + e * l3, xr, xs, xt);
      rgrad(lx, D, y + e * l3, yr, ys, yt);
      rgrad(lx, D, z + e * l3, zr, zs, zt);
      for (int64_t q = 0; q < l3; ++q) {
        const double c[9] = {ys[q] * zt[q] - yt[q] * zs[q], xt[q] * zs[q] - xs[q] * zt[q],
                             xs[q] * yt[q] - xt[q] * ys[q], yt[q] * zr[q] - yr[q] * zt[q],
                             xr[q] * zt[q] - xt[q] * zr[q], xt[q] * yr[q] - xr[q] * yt[q],
                             yr[q] * zs[q] - ys[q] * zr[q], xs[q] * zr[q] - xr[q] * zs[q],
                             xr[q] * ys[q] - xs[q] * yr[q]};
        const int64_t g = e * l3 + q;
        for (int m = 0; m < 9; ++m) met[m * n + g] = c[m];
        met[9 * n + g] = 1.0 / (xr[q] * c[0] + yr[q] * c[1] + zr[q] * c[2]);
      }
    }
    free(b);
  }
}

/* (o1, o2, o3) = B grad u = w3 (cofactor-weighted reference derivatives) */
void orct_opgrad(int64_t nelv, int lx, const double* D, const double* w, const double* met, const double* u,
                 double* o1, double* o2, double* o3) {
  const int64_t l3 = (int64_t)lx * lx * lx, n = nelv * l3;
  double* o[3] = {o1, o2, o3};
#pragma omp parallel
  {
    double* b = (double*)malloc(sizeof(double) * 3 * l3);
#pragma omp for schedule(static)
    for (int64_t e = 0; e < nelv; ++e) {
      rgrad(lx, D, u + e * l3, b, b + l3, b + 2 * l3);
      for (int64_t q = 0; q < l3; ++q) {
        const int i = q % lx, j = (q / lx) % lx, k = q / (lx * lx);
        const double w3 = w[i] * w[j] * w[k];
        const int64_t g = e * l3 + q;
        for (int d = 0; d < 3; ++d)
          o[d][g] = w3 * (met[d * n + g] * b[q] + met[(3 + d) * n + g] * b[l3 + q] +
                          met[(6 + d) * n + g] * b[2 * l3 + q]);
      }
    }
    free(b);
  }
}

/* out = sum_d cdtp_d(a_d) (a_d may be NULL) */
void orct_cdtp_sum(int64_t nelv, int lx, const double* D, const double* w, const double* met, const double* a0,
                   const double* a1, const double* a2, double* out) {
  const int64_t l3 = (int64_t)lx * lx * lx, n = nelv * l3;
  const double* a[3] = {a0, a1, a2};
#pragma omp parallel
  {
    double* b = (double*)malloc(sizeof(double) * 3 * l3);
#pragma omp for schedule(static)
    for (int64_t e = 0; e < nelv; ++e) {
      for (int64_t q = 0; q < l3; ++q) {
        const int i = q % lx, j = (q / lx) % lx, k = q / (lx * lx);
        const double w3 = w[i] * w[j] * w[k];
        const int64_t g = e * l3 + q;
        double r = 0.0, s = 0.0, t = 0.0;
        for (int d = 0; d < 3; ++d) {
          if (!a[d]) continue;
          r += met[d * n + g] * a[d][g];
          s += met[(3 + d) * n + g] * a[d][g];
          t += met[(6 + d) * n + g] * a[d][g];
        }
        b[q] = w3 * r;
        b[l3 + q] = w3 * s;
        b[2 * l3 + q] = w3 * t;
      }
      rgrad_t(lx, D, b, b + l3, b + 2 * l3, out + e * l3);
    }
    free(b);
  }
}

/* (o1, o2, o3) = B curl u, unassembled */
void orct_bcurl(int64_t nelv, int lx, const double* D, const double* w, const double* met, const double* u1,
                const double* u2, const double* u3, double* o1, double* o2, double* o3) {
  const int64_t l3 = (int64_t)lx * lx * lx, n = nelv * l3;
  const double* u[3] = {u1, u2, u3};
#pragma omp parallel
  {
    double* b = (double*)malloc(sizeof(double) * 9 * l3);
#pragma omp for schedule(static)
    for (int64_t e = 0; e < nelv; ++e) {
      for (int f = 0; f < 3; ++f) rgrad(lx, D, u[f] + e * l3, b + 3 * f * l3, b + (3 * f + 1) * l3, b + (3 * f + 2) * l3);
      for (int64_t q = 0; q < l3; ++q) {
        const int i = q % lx, j = (q / lx) % lx, k = q / (lx * lx);
        const double w3 = w[i] * w[j] * w[k];
        const int64_t g = e * l3 + q;
        double dd[3][3];  /* dd[f][dir] = d u_f / d x_dir (times jac) */
        for (int f = 0; f < 3; ++f)
          for (int d = 0; d < 3; ++d)
            dd[f][d] = met[d * n + g] * b[3 * f * l3 + q] + met[(3 + d) * n + g] * b[(3 * f + 1) * l3 + q] +
                       met[(6 + d) * n + g] * b[(3 * f + 2) * l3 + q];
        o1[g] = w3 * (dd[2][1] - dd[1][2]);
        o2[g] = w3 * (dd[0][2] - dd[2][0]);
        o3[g] = w3 * (dd[1][0] - dd[0][1]);
      }
    }
    free(b);
  }
}

/* The advection terms on one element, on an nx-point grid with weights w,
   differentiation matrix D and cofactors c[m * ng + q] (ng = nx^3 of this
   element): out_i = term_i (to be subtracted), mode 0 adjoint, 1 linear.
   U, V: the 3 + 3 fields on the grid; scratch: 12 nx^3 doubles. */
static void adv_tile(int mode, int nx, const double* D, const double* w, const double* c, const double* U,
                     const double* V, double* out, double* sc) {
  const int ng = nx * nx * nx;
  double* g = sc;            /* 9 ng: reference derivatives */
  double* W = sc + 9 * ng;   /* 3 ng: fluxes */
  for (int f = 0; f < 3; ++f) rgrad(nx, D, V + f * ng, g + 3 * f * ng, g + (3 * f + 1) * ng, g + (3 * f + 2) * ng);
  if (mode == 0) {
    for (int q = 0; q < ng; ++q) {
      const int i = q % nx, j = (q / nx) % nx, k = q / (nx * nx);
      const double w3 = w[i] * w[j] * w[k];
      for (int ii = 0; ii < 3; ++ii) {
        double a = 0.0;
        for (int jj = 0; jj < 3; ++jj)
          a += U[jj * ng + q] * (c[ii * ng + q] * g[3 * jj * ng + q] + c[(3 + ii) * ng + q] * g[(3 * jj + 1) * ng + q] +
                                 c[(6 + ii) * ng + q] * g[(3 * jj + 2) * ng + q]);
        out[ii * ng + q] = w3 * a;
      }
      for (int r = 0; r < 3; ++r)
        W[r * ng + q] = w3 * (c[3 * r * ng + q] * V[q] + c[(3 * r + 1) * ng + q] * V[ng + q] +
                              c[(3 * r + 2) * ng + q] * V[2 * ng + q]);
    }
    double* fl = g;  /* reuse: 3 ng fluxes u_i W, then the contraction */
    double* t = g + 3 * ng;
    for (int ii = 0; ii < 3; ++ii) {
      for (int q = 0; q < ng; ++q)
        for (int r = 0; r < 3; ++r) fl[r * ng + q] = U[ii * ng + q] * W[r * ng + q];
      rgrad_t(nx, D, fl, fl + ng, fl + 2 * ng, t);
      for (int q = 0; q < ng; ++q) out[ii * ng + q] += t[q];
    }
  } else {
    double* gu = sc + 9 * ng;  /* 3 ng at a time: derivatives of u_i */
    for (int ii = 0; ii < 3; ++ii) {
      rgrad(nx, D, U + ii * ng, gu, gu + ng, gu + 2 * ng);
      for (int q = 0; q < ng; ++q) {
        const int i = q % nx, j = (q / nx) % nx, k = q / (nx * nx);
        const double w3 = w[i] * w[j] * w[k];
        double ur[3], vr[3];
        for (int r = 0; r < 3; ++r) {
          ur[r] = c[3 * r * ng + q] * U[q] + c[(3 * r + 1) * ng + q] * U[ng + q] + c[(3 * r + 2) * ng + q] * U[2 * ng + q];
          vr[r] = c[3 * r * ng + q] * V[q] + c[(3 * r + 1) * ng + q] * V[ng + q] + c[(3 * r + 2) * ng + q] * V[2 * ng + q];
        }
        out[ii * ng + q] = w3 * (g[3 * ii * ng + q] * ur[0] + g[(3 * ii + 1) * ng + q] * ur[1] +
                                 g[(3 * ii + 2) * ng + q] * ur[2] + gu[q] * vr[0] + gu[ng + q] * vr[1] +
                                 gu[2 * ng + q] * vr[2]);
      }
    }
  }
}

/* tile transpose of the cofactor layout: c[m * ng + q] from met[m * n + e ng + q] */
static void gather_cof(const double* met, int64_t n, int64_t e, int ng, double* c) {
  for (int m = 0; m < 9; ++m) memcpy(c + m * ng, met + m * n + e * ng, sizeof(double) * ng);
}

/* f_i -= term_i without dealiasing; mode 0 adjoint, 1 linear */
void orct_adv_no_dealias(int mode, int64_t nelv, int lx, const double* D, const double* w, const double* met,
                         const double* u1, const double* u2, const double* u3, const double* b1, const double* b2,
                         const double* b3, double* f1, double* f2, double* f3) {
  const int ng = lx * lx * lx;
  const int64_t n = nelv * ng;
  const double* u[3] = {u1, u2, u3};
  const double* b[3] = {b1, b2, b3};
  double* f[3] = {f1, f2, f3};
#pragma omp parallel
  {
    double* s = (double*)malloc(sizeof(double) * 30 * ng);
    double *c = s, *U = s + 9 * ng, *V = s + 12 * ng, *out = s + 15 * ng, *sc = s + 18 * ng;
#pragma omp for schedule(static)
    for (int64_t e = 0; e < nelv; ++e) {
      gather_cof(met, n, e, ng, c);
      for (int d = 0; d < 3; ++d) {
        memcpy(U + d * ng, u[d] + e * ng, sizeof(double) * ng);
        memcpy(V + d * ng, b[d] + e * ng, sizeof(double) * ng);
      }
      adv_tile(mode, lx, D, w, c, U, V, out, sc);
      for (int d = 0; d < 3; ++d)
        for (int q = 0; q < ng; ++q) f[d][e * ng + q] -= out[d * ng + q];
    }
    free(s);
  }
}

/* tensor-product map of one tile: out (no^3) = J x J x J in (ni^3), J[A * ni + a] */
static void tmap(int ni, int no, const double* J, const double* in, double* out, double* t1, double* t2) {
  for (int c = 0; c < ni; ++c)
    for (int b = 0; b < ni; ++b)
      for (int A = 0; A < no; ++A) {
        double s = 0.0;
        for (int a = 0; a < ni; ++a) s += J[A * ni + a] * in[(c * ni + b) * ni + a];
        t1[(c * ni + b) * no + A] = s;
      }
  for (int c = 0; c < ni; ++c)
    for (int B = 0; B < no; ++B)
      for (int A = 0; A < no; ++A) {
        double s = 0.0;
        for (int b = 0; b < ni; ++b) s += J[B * ni + b] * t1[(c * ni + b) * no + A];
        t2[(c * no + B) * no + A] = s;
      }
  for (int C = 0; C < no; ++C)
    for (int B = 0; B < no; ++B)
      for (int A = 0; A < no; ++A) {
        double s = 0.0;
        for (int c = 0; c < ni; ++c) s += J[C * ni + c] * t2[(c * no + B) * no + A];
        out[(C * no + B) * no + A] = s;
      }
}

/* transpose map: out (ni^3) = J^T x J^T x J^T in (no^3) */
static void tmap_t(int ni, int no, const double* J, const double* in, double* out, double* t1, double* t2) {
  for (int c = 0; c < ni; ++c)
    for (int B = 0; B < no; ++B)
      for (int A = 0; A < no; ++A) {
        double s = 0.0;
        for (int C = 0; C < no; ++C) s += J[C * ni + c] * in[(C * no + B) * no + A];
        t2[(c * no + B) * no + A] = s;
      }
  for (int c = 0; c < ni; ++c)
    for (int b = 0; b < ni; ++b)
      for (int A = 0; A < no; ++A) {
        double s = 0.0;
        for (int B = 0; B < no; ++B) s += J[B * ni + b] * t2[(c * no + B) * no + A];
        t1[(c * ni + b) * no + A] = s;
      }
  for (int c = 0; c < ni; ++c)
    for (int b = 0; b < ni; ++b)
      for (int a = 0; a < ni; ++a) {
        double s = 0.0;
        for (int A = 0; A < no; ++A) s += J[A * ni + a] * t1[(c * ni + b) * no + A];
        out[(c * ni + b) * ni + a] = s;
      }
}

/* dealiased: fields and GLL cofactors mapped to the lxd GL points (J),
   products there with the GL weights wg and GL differentiation Dg, J^T back;
   f_i -= term_i.  mode 0 adjoint, 1 linear. */
void orct_adv_dealias(int mode, int64_t nelv, int lx, int lxd, const double* J, const double* Dg, const double* wg,
                      const double* met, const double* u1, const double* u2, const double* u3, const double* b1,
                      const double* b2, const double* b3, double* f1, double* f2, double* f3) {
  const int ng = lx * lx * lx, nd = lxd * lxd * lxd;
  const int64_t n = nelv * ng;
  const double* u[3] = {u1, u2, u3};
  const double* b[3] = {b1, b2, b3};
  double* f[3] = {f1, f2, f3};
#pragma omp parallel
  {
    double* s = (double*)malloc(sizeof(double) * (30 * nd + 2 * nd + ng));
    double *c = s, *U = s + 9 * nd, *V = s + 12 * nd, *out = s + 15 * nd, *sc = s + 18 * nd;
    double *t1 = s + 30 * nd, *t2 = t1 + nd, *back = t2 + nd;
#pragma omp for schedule(static)
    for (int64_t e = 0; e < nelv; ++e) {
      for (int m = 0; m < 9; ++m) tmap(lx, lxd, J, met + m * n + e * ng, c + m * nd, t1, t2);
      for (int d = 0; d < 3; ++d) {
        tmap(lx, lxd, J, u[d] + e * ng, U + d * nd, t1, t2);
        tmap(lx, lxd, J, b[d] + e * ng, V + d * nd, t1, t2);
      }
      adv_tile(mode, lxd, Dg, wg, c, U, V, out, sc);
      for (int d = 0; d < 3; ++d) {
        tmap_t(lx, lxd, J, out + d * nd, back, t1, t2);
        for (int q = 0; q < ng; ++q) f[d][e * ng + q] -= back[q];
      }
    }
    free(s);
  }
}
