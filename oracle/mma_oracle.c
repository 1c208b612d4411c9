/*
 * CPU oracle, part 3: the MMA design update, compiled with OpenMP.
 *
 * TEST INFRASTRUCTURE ONLY: the timed CPU baseline of the GPU MMA, a line-by-
 * line C form of oracle/mma_ref.py (which restates the reference's
 * sources/mma/bcknd/cpu/mma_cpu.f90: mma_gensub_cpu :8-184,
 * mma_subsolve_dpip_cpu :186-579) and checked against it by
 * tests/test_oracle_mma.py.  The n-sized loops are OpenMP loops, the
 * m-sized algebra is serial, as in the reference (one rank).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define MM 4
/* the reference's single-precision Fortran literals */
#define C001 ((double)0.01f)
#define C01 ((double)0.1f)
#define C09 ((double)0.9f)
#define C101 ((double)1.01f)

typedef struct {
  int64_t n;
  int m;
  const double *low, *upp, *alpha, *beta, *p0, *q0, *P, *Q;  /* P, Q: m rows of n */
  double a0;
  const double *a, *c, *d, *bi;
} sub_t;

/* residual pieces at (x, xsi, eta; lam): g_i sums, sum of squares and max of
   rex, rexsi, reeta (out[0..m), out[m], out[m+1]) */
static void resid_x(const sub_t* S, const double* x, const double* xsi, const double* eta, const double* lam,
                    double epsi, double* out) {
  const int m = S->m;
  double g[MM] = {0}, sq = 0.0, mx = 0.0;
#pragma omp parallel
  {
    double gl[MM] = {0}, sql = 0.0, mxl = 0.0;
#pragma omp for schedule(static)
    for (int64_t j = 0; j < S->n; ++j) {
      const double ux = S->upp[j] - x[j], xl = x[j] - S->low[j];
      double pl = S->p0[j], ql = S->q0[j];
      for (int i = 0; i < m; ++i) {
        const double p = S->P[i * S->n + j], q = S->Q[i * S->n + j];
        pl += p * lam[i];
        ql += q * lam[i];
        gl[i] += p / ux + q / xl;
      }
      const double rex = pl / (ux * ux) - ql / (xl * xl) - xsi[j] + eta[j];
      const double rexsi = xsi[j] * (x[j] - S->alpha[j]) - epsi;
      const double reeta = eta[j] * (S->beta[j] - x[j]) - epsi;
      sql += rex * rex + rexsi * rexsi + reeta * reeta;
      mxl = fmax(mxl, fmax(fabs(rex), fmax(fabs(rexsi), fabs(reeta))));
    }
#pragma omp critical
    {
      for (int i = 0; i < m; ++i) g[i] += gl[i];
      sq += sql;
      mx = fmax(mx, mxl);
    }
  }
  for (int i = 0; i < m; ++i) out[i] = g[i];
  out[m] = sq;
  out[m + 1] = mx;
}

static void full_resid(const sub_t* S, const double* o, const double* y, double z, const double* lam, const double* s,
                       const double* mu, double zeta, double epsi, double* norm, double* mx) {
  const int m = S->m;
  double sq = o[m], big = o[m + 1];
  double rez = S->a0 - zeta, rezeta = zeta * z - epsi;
  for (int i = 0; i < m; ++i) rez -= lam[i] * S->a[i];
  sq += rez * rez + rezeta * rezeta;
  big = fmax(big, fmax(fabs(rez), fabs(rezeta)));
  for (int i = 0; i < m; ++i) {
    const double rey = S->c[i] + S->d[i] * y[i] - lam[i] - mu[i];
    const double relam = o[i] - S->a[i] * z - y[i] + s[i] - S->bi[i];
    const double remu = mu[i] * y[i] - epsi, res = lam[i] * s[i] - epsi;
    sq += rey * rey + relam * relam + remu * remu + res * res;
    big = fmax(big, fmax(fmax(fabs(rey), fabs(relam)), fmax(fabs(remu), fabs(res))));
  }
  *norm = sqrt(sq);
  *mx = big;
}

static int solve_small(int k, double* A, double* b) {
  for (int c = 0; c < k; ++c) {
    int p = c;
    for (int r = c + 1; r < k; ++r)
      if (fabs(A[r * k + c]) > fabs(A[p * k + c])) p = r;
    if (A[p * k + c] == 0.0) return 1;
    if (p != c) {
      for (int q = 0; q < k; ++q) {
        const double t = A[c * k + q];
        A[c * k + q] = A[p * k + q];
        A[p * k + q] = t;
      }
      const double t = b[c];
      b[c] = b[p];
      b[p] = t;
    }
    for (int r = c + 1; r < k; ++r) {
      const double f = A[r * k + c] / A[c * k + c];
      for (int q = c; q < k; ++q) A[r * k + q] -= f * A[c * k + q];
      b[r] -= f * b[c];
    }
  }
  for (int c = k - 1; c >= 0; --c) {
    double s = b[c];
    for (int q = c + 1; q < k; ++q) s -= A[c * k + q] * b[q];
    b[c] = s / A[c * k + c];
  }
  return 0;
}

/* One MMA update.  State (n-sized, caller-owned): xold1, xold2, low, upp;
   design x in/out; xmin, xmax; df0dx; dfdx in the reference's (m, n)
   layout (i + m j); fval (m).  Scratch: 13 n + 2 m n doubles.  Dual state
   out: y, lam, s, mu (m) and z, zeta (dual[0], dual[1]).  Returns the
   number of Newton steps, or -1 on a singular Newton system. */
int orcm_update(int64_t n, int m, int iter, double* x, double* xold1, double* xold2, double* low, double* upp,
                const double* xmin, const double* xmax, const double* df0dx, const double* fval, const double* dfdx,
                double a0, const double* a, const double* c, const double* d, double epsimin, int max_iter,
                double asyinit, double asyincr, double asydecr, double* scratch, double* y, double* lam, double* s,
                double* mu, double* dual) {
  double *alpha = scratch, *beta = alpha + n, *p0 = beta + n, *q0 = p0 + n, *P = q0 + n, *Q = P + m * n;
  double *xs = Q + m * n, *xsi = xs + n, *eta = xsi + n, *dx = eta + n, *dxsi = dx + n, *deta = dxsi + n;
  double *x0 = deta + n, *xsi0 = x0 + n, *eta0 = xsi0 + n;
  double bi[MM] = {0};
  /* mma_gensub_cpu */
#pragma omp parallel
  {
    double bl[MM] = {0};
#pragma omp for schedule(static)
    for (int64_t j = 0; j < n; ++j) {
      const double xj = x[j], xr = xmax[j] - xmin[j];
      if (iter < 3) {
        low[j] = xj - asyinit * xr;
        upp[j] = xj + asyinit * xr;
      } else {
        const double sg = (xj - xold1[j]) * (xold1[j] - xold2[j]);
        const double fac = sg < 0 ? asydecr : (sg > 0 ? asyincr : 1.0);
        double lo = xj - fac * (xold1[j] - low[j]), up = xj + fac * (upp[j] - xold1[j]);
        lo = fmax(lo, xj - 10 * xr);
        lo = fmin(lo, xj - C001 * xr);
        up = fmin(up, xj + 10 * xr);
        up = fmax(up, xj + C001 * xr);
        low[j] = lo;
        upp[j] = up;
      }
      const double lo = low[j], up = upp[j];
      alpha[j] = fmax(fmax(xmin[j], lo + 0.1 * (xj - lo)), xj - 0.5 * xr);
      beta[j] = fmin(fmin(xmax[j], up - C01 * (up - xj)), xj + 0.5 * xr);
      const double r = 0.00001 / fmax(0.00001, xr), ux2 = (up - xj) * (up - xj), xl2 = (xj - lo) * (xj - lo);
      p0[j] = ux2 * (1.001 * fmax(df0dx[j], 0) + 0.001 * fmax(-df0dx[j], 0) + r);
      q0[j] = xl2 * (0.001 * fmax(df0dx[j], 0) + 1.001 * fmax(-df0dx[j], 0) + r);
      for (int i = 0; i < m; ++i) {
        const double g = dfdx[i + (int64_t)m * j];
        const double p = ux2 * (1.001 * fmax(g, 0) + 0.001 * fmax(-g, 0) + r);
        const double q = xl2 * (0.001 * fmax(g, 0) + 1.001 * fmax(-g, 0) + r);
        P[i * n + j] = p;
        Q[i * n + j] = q;
        bl[i] += p / (up - xj) + q / (xj - lo);
      }
    }
#pragma omp critical
    for (int i = 0; i < m; ++i) bi[i] += bl[i];
  }
  for (int i = 0; i < m; ++i) bi[i] -= fval[i];
  sub_t S = {n, m, low, upp, alpha, beta, p0, q0, P, Q, a0, a, c, d, bi};
  /* mma_subsolve_dpip_cpu */
  double epsi = 1.0, z = 1.0, zeta = 1.0, o[MM + 2];
  for (int i = 0; i < m; ++i) {
    y[i] = 1.0;
    lam[i] = 1.0;
    s[i] = 1.0;
    mu[i] = fmax(1.0, 0.5 * c[i]);
  }
#pragma omp parallel for schedule(static)
  for (int64_t j = 0; j < n; ++j) {
    xs[j] = 0.5 * (alpha[j] + beta[j]);
    xsi[j] = fmax(1.0, 1.0 / (xs[j] - alpha[j]));
    eta[j] = fmax(1.0, 1.0 / (beta[j] - xs[j]));
  }
  int steps = 0;
  while (epsi > C09 * epsimin) {
    double rnorm, rmax;
    resid_x(&S, xs, xsi, eta, lam, epsi, o);
    full_resid(&S, o, y, z, lam, s, mu, zeta, epsi, &rnorm, &rmax);
    for (int it = 0; it < max_iter; ++it) {
      if (rmax < epsi) break;
      ++steps;
      double gsum[MM] = {0}, bsum[MM] = {0}, asum[MM * MM] = {0};
#pragma omp parallel
      {
        double gl[MM] = {0}, bl[MM] = {0}, al[MM * MM] = {0};
#pragma omp for schedule(static)
        for (int64_t j = 0; j < n; ++j) {
          const double xj = xs[j], ux = upp[j] - xj, xl = xj - low[j], ux2 = ux * ux, xl2 = xl * xl;
          double pl = p0[j], ql = q0[j], gg[MM];
          for (int i = 0; i < m; ++i) {
            const double p = P[i * n + j], q = Q[i * n + j];
            pl += p * lam[i];
            ql += q * lam[i];
            gl[i] += p / ux + q / xl;
            gg[i] = p / ux2 - q / xl2;
          }
          const double delx = pl / ux2 - ql / xl2 - epsi / (xj - alpha[j]) + epsi / (beta[j] - xj);
          const double diagx = 2.0 * (pl / (ux2 * ux) + ql / (xl2 * xl)) + xsi[j] / (xj - alpha[j]) +
                               eta[j] / (beta[j] - xj);
          dx[j] = delx;      /* delx and diagx kept for the directions */
          dxsi[j] = diagx;
          for (int i = 0; i < m; ++i) {
            bl[i] += gg[i] * (delx / diagx);
            for (int k = 0; k < m; ++k) al[i * m + k] += gg[i] * (1.0 / diagx) * gg[k];
          }
        }
#pragma omp critical
        {
          for (int i = 0; i < m; ++i) {
            gsum[i] += gl[i];
            bsum[i] += bl[i];
          }
          for (int q = 0; q < m * m; ++q) asum[q] += al[q];
        }
      }
      double dely[MM], bb[MM + 1], AA[(MM + 1) * (MM + 1)];
      double delz = a0 - epsi / z;
      for (int i = 0; i < m; ++i) delz -= lam[i] * a[i];
      for (int i = 0; i < m; ++i) {
        dely[i] = c[i] + d[i] * y[i] - lam[i] - epsi / y[i];
        const double dellam = gsum[i] - a[i] * z - y[i] - bi[i] + epsi / lam[i];
        bb[i] = dellam + dely[i] / (d[i] + mu[i] / y[i]) - bsum[i];
      }
      bb[m] = delz;
      const int k1 = m + 1;
      for (int i = 0; i < m; ++i) {
        for (int k = 0; k < m; ++k) AA[i * k1 + k] = asum[i * m + k];
        AA[i * k1 + i] += s[i] / lam[i] + 1.0 / (d[i] + mu[i] / y[i]);
        AA[i * k1 + m] = a[i];
        AA[m * k1 + i] = a[i];
      }
      AA[m * k1 + m] = -zeta / z;
      if (solve_small(k1, AA, bb)) return -1;
      double dlam[MM], dy[MM], dmu[MM], ds[MM];
      for (int i = 0; i < m; ++i) dlam[i] = bb[i];
      const double dz = bb[m];
      for (int i = 0; i < m; ++i) {
        dy[i] = (-dely[i] + dlam[i]) / (d[i] + mu[i] / y[i]);
        dmu[i] = -mu[i] + (epsi - mu[i] * dy[i]) / y[i];
        ds[i] = -s[i] + (epsi - dlam[i] * s[i]) / lam[i];
      }
      const double dzeta = -zeta + (epsi - zeta * dz) / z;
      double steg = 1.0;
#pragma omp parallel
      {
        double sl = 1.0;
#pragma omp for schedule(static)
        for (int64_t j = 0; j < n; ++j) {
          const double xj = xs[j], ux = upp[j] - xj, xl = xj - low[j], ux2 = ux * ux, xl2 = xl * xl;
          double gl = 0.0;
          for (int i = 0; i < m; ++i) gl += (P[i * n + j] / ux2 - Q[i * n + j] / xl2) * dlam[i];
          const double delx = dx[j], diagx = dxsi[j];
          const double dxj = -delx / diagx - gl / diagx;
          const double dxs = -xsi[j] + (epsi - dxj * xsi[j]) / (xj - alpha[j]);
          const double det = -eta[j] + (epsi + dxj * eta[j]) / (beta[j] - xj);
          dx[j] = dxj;
          dxsi[j] = dxs;
          deta[j] = det;
          x0[j] = xj;
          xsi0[j] = xsi[j];
          eta0[j] = eta[j];
          sl = fmax(sl, fmax(fmax(-C101 * dxs / xsi[j], -C101 * det / eta[j]),
                             fmax(-C101 * dxj / (xj - alpha[j]), C101 * dxj / (beta[j] - xj))));
        }
#pragma omp critical
        steg = fmax(steg, sl);
      }
      for (int i = 0; i < m; ++i) {
        steg = fmax(steg, -C101 * dy[i] / y[i]);
        steg = fmax(steg, -C101 * dlam[i] / lam[i]);
        steg = fmax(steg, -C101 * dmu[i] / mu[i]);
        steg = fmax(steg, -C101 * ds[i] / s[i]);
      }
      steg = fmax(steg, -C101 * dz / z);
      steg = fmax(steg, -C101 * dzeta / zeta);
      steg = 1.0 / steg;
      double y0[MM], lam0[MM], mu0[MM], s0[MM];
      memcpy(y0, y, sizeof(double) * m);
      memcpy(lam0, lam, sizeof(double) * m);
      memcpy(mu0, mu, sizeof(double) * m);
      memcpy(s0, s, sizeof(double) * m);
      const double z0 = z, zeta0 = zeta;
      double newres = 2.0 * rnorm;
      int itto = 0;
      while (newres > rnorm && itto < 50) {
        ++itto;
#pragma omp parallel for schedule(static)
        for (int64_t j = 0; j < n; ++j) {
          xs[j] = x0[j] + steg * dx[j];
          xsi[j] = xsi0[j] + steg * dxsi[j];
          eta[j] = eta0[j] + steg * deta[j];
        }
        for (int i = 0; i < m; ++i) {
          y[i] = y0[i] + steg * dy[i];
          lam[i] = lam0[i] + steg * dlam[i];
          mu[i] = mu0[i] + steg * dmu[i];
          s[i] = s0[i] + steg * ds[i];
        }
        z = z0 + steg * dz;
        zeta = zeta0 + steg * dzeta;
        resid_x(&S, xs, xsi, eta, lam, epsi, o);
        full_resid(&S, o, y, z, lam, s, mu, zeta, epsi, &newres, &rmax);
        steg = steg / 2.0;
      }
      rnorm = newres;
    }
    epsi = 0.1 * epsi;
  }
  memcpy(xold2, xold1, sizeof(double) * n);
  memcpy(xold1, x, sizeof(double) * n);
  memcpy(x, xs, sizeof(double) * n);
  dual[0] = z;
  dual[1] = zeta;
  return steps;
}
