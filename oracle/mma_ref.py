"""numpy restatement of the reference's MMA optimiser (Svanberg's method of
moving asymptotes with the primal-dual interior-point subproblem solver).

TEST INFRASTRUCTURE ONLY: the checker for neko-top_gb300/csrc/mma.cu.

Follows sources/mma/mma.f90 (mma_init_attributes :186-295, defaults
:275-283) and sources/mma/bcknd/cpu/mma_cpu.f90 (mma_gensub_cpu :8-184,
mma_subsolve_dpip_cpu :186-579, mma_KKT_cpu :581-641), i.e. Svanberg,
"MMA and GCMMA - two methods for nonlinear optimization" (2007):

  minimise  f0(x) + a0 z + sum_i (c_i y_i + d_i y_i^2 / 2)
  s.t.      f_i(x) - a_i z - y_i <= 0,  xmin <= x <= xmax,  y, z >= 0.

The reference writes a few constants as default-kind (single precision)
Fortran literals (0.01 and 0.1 in the asymptote and move-limit bounds, 0.9
in the epsilon loop, 1.01 in the step length); they take those values here
too (F32 below), so the iterates follow the reference's.
dfdx is (m, n) as in the reference.
"""
from __future__ import annotations

import numpy as np

F32 = lambda v: float(np.float32(v))
C001, C01, C09, C101 = F32(0.01), F32(0.1), F32(0.9), F32(1.01)


class MMA:
    def __init__(self, x, m, a0, a, c, d, xmin, xmax, max_iter=100, epsimin=None, asyinit=0.5, asyincr=1.2,
                 asydecr=0.7):
        x = np.asarray(x, dtype=np.float64)
        n = x.size
        self.n, self.m = n, m
        self.xold1, self.xold2 = x.copy(), x.copy()
        self.a0 = float(a0)
        self.a, self.c, self.d = (np.broadcast_to(np.asarray(v, np.float64), (m,)).copy() for v in (a, c, d))
        self.xmin = np.broadcast_to(np.asarray(xmin, np.float64), (n,)).copy()
        self.xmax = np.broadcast_to(np.asarray(xmax, np.float64), (n,)).copy()
        self.low = np.full(n, x.min())
        self.upp = np.full(n, x.max())
        self.max_iter = max_iter
        self.epsimin = 1.0e-9 * np.sqrt(m + n) if epsimin is None else epsimin
        self.asyinit, self.asyincr, self.asydecr = asyinit, asyincr, asydecr
        self.residumax = self.residunorm = np.finfo(np.float64).max
        self.newton_steps = 0

    # mma_gensub_cpu
    def gensub(self, it, x, df0dx, fval, dfdx):
        xr = self.xmax - self.xmin
        if it < 3:
            self.low = x - self.asyinit * xr
            self.upp = x + self.asyinit * xr
        else:
            sg = (x - self.xold1) * (self.xold1 - self.xold2)
            fac = np.where(sg < 0, self.asydecr, np.where(sg > 0, self.asyincr, 1.0))
            low = x - fac * (self.xold1 - self.low)
            upp = x + fac * (self.upp - self.xold1)
            low = np.maximum(low, x - 10 * xr)
            low = np.minimum(low, x - C001 * xr)
            upp = np.minimum(upp, x + 10 * xr)
            upp = np.maximum(upp, x + C001 * xr)
            self.low, self.upp = low, upp
        low, upp = self.low, self.upp
        self.alpha = np.maximum(np.maximum(self.xmin, low + 0.1 * (x - low)), x - 0.5 * xr)
        self.beta = np.minimum(np.minimum(self.xmax, upp - C01 * (upp - x)), x + 0.5 * xr)
        r = 0.00001 / np.maximum(0.00001, xr)
        ux2, xl2 = (upp - x) ** 2, (x - low) ** 2
        self.p0 = ux2 * (1.001 * np.maximum(df0dx, 0) + 0.001 * np.maximum(-df0dx, 0) + r)
        self.q0 = xl2 * (0.001 * np.maximum(df0dx, 0) + 1.001 * np.maximum(-df0dx, 0) + r)
        self.P = ux2 * (1.001 * np.maximum(dfdx, 0) + 0.001 * np.maximum(-dfdx, 0) + r)
        self.Q = xl2 * (0.001 * np.maximum(dfdx, 0) + 1.001 * np.maximum(-dfdx, 0) + r)
        self.bi = (self.P / (upp - x) + self.Q / (x - low)).sum(axis=1) - fval

    def _resid(self, x, y, z, lam, xsi, eta, mu, zeta, s, epsi):
        ux, xl = self.upp - x, x - self.low
        rex = (self.p0 + self.P.T @ lam) / ux ** 2 - (self.q0 + self.Q.T @ lam) / xl ** 2 - xsi + eta
        rey = self.c + self.d * y - lam - mu
        rez = self.a0 - zeta - lam @ self.a
        relam = (self.P / ux + self.Q / xl).sum(axis=1) - self.a * z - y + s - self.bi
        rexsi = xsi * (x - self.alpha) - epsi
        reeta = eta * (self.beta - x) - epsi
        remu = mu * y - epsi
        rezeta = zeta * z - epsi
        res = lam * s - epsi
        small = np.concatenate([rey, [rez], relam, remu, [rezeta], res])
        norm = np.sqrt(np.sum(small ** 2) + np.sum(rex ** 2) + np.sum(rexsi ** 2) + np.sum(reeta ** 2))
        mx = max(np.abs(small).max(), np.abs(rex).max(), np.abs(rexsi).max(), np.abs(reeta).max())
        return norm, mx

    # mma_subsolve_dpip_cpu
    def subsolve(self, designx):
        m = self.m
        al, be, lo, up = self.alpha, self.beta, self.low, self.upp
        epsi = 1.0
        x = 0.5 * (al + be)
        y = np.ones(m)
        z = 1.0
        zeta = 1.0
        lam = np.ones(m)
        s = np.ones(m)
        xsi = np.maximum(1.0, 1.0 / (x - al))
        eta = np.maximum(1.0, 1.0 / (be - x))
        mu = np.maximum(1.0, 0.5 * self.c)
        while epsi > C09 * self.epsimin:
            residunorm, residumax = self._resid(x, y, z, lam, xsi, eta, mu, zeta, s, epsi)
            for _ in range(self.max_iter):
                if residumax < epsi:
                    break
                self.newton_steps += 1
                ux, xl = up - x, x - lo
                plam = self.p0 + self.P.T @ lam
                qlam = self.q0 + self.Q.T @ lam
                delx = plam / ux ** 2 - qlam / xl ** 2 - epsi / (x - al) + epsi / (be - x)
                dely = self.c + self.d * y - lam - epsi / y
                delz = self.a0 - lam @ self.a - epsi / z
                dellam = (self.P / ux + self.Q / xl).sum(axis=1) - self.a * z - y - self.bi + epsi / lam
                GG = self.P / ux ** 2 - self.Q / xl ** 2
                diagx = 2.0 * (plam / ux ** 3 + qlam / xl ** 3) + xsi / (x - al) + eta / (be - x)
                bb = np.empty(m + 1)
                bb[:m] = dellam + dely / (self.d + mu / y) - GG @ (delx / diagx)
                bb[m] = delz
                AA = np.empty((m + 1, m + 1))
                AA[:m, :m] = (GG / diagx) @ GG.T
                AA[np.arange(m), np.arange(m)] += s / lam + 1.0 / (self.d + mu / y)
                AA[:m, m] = self.a
                AA[m, :m] = self.a
                AA[m, m] = -zeta / z
                sol = np.linalg.solve(AA, bb)
                dlam, dz = sol[:m], sol[m]
                dx = -delx / diagx - (GG.T @ dlam) / diagx
                dy = (-dely + dlam) / (self.d + mu / y)
                dxsi = -xsi + (epsi - dx * xsi) / (x - al)
                deta = -eta + (epsi + dx * eta) / (be - x)
                dmu = -mu + (epsi - mu * dy) / y
                dzeta = -zeta + (epsi - zeta * dz) / z
                ds = -s + (epsi - dlam * s) / lam
                dxx = np.concatenate([dy, [dz], dlam, dxsi, deta, dmu, [dzeta], ds])
                xx = np.concatenate([y, [z], lam, xsi, eta, mu, [zeta], s])
                steg = max(1.0, (-C101 * dxx / xx).max(), (-C101 * dx / (x - al)).max(), (C101 * dx / (be - x)).max())
                steg = 1.0 / steg
                old = (x, y, z, lam, xsi, eta, mu, zeta, s)
                newres = 2.0 * residunorm
                itto = 0
                while newres > residunorm and itto < 50:
                    itto += 1
                    x = old[0] + steg * dx
                    y = old[1] + steg * dy
                    z = old[2] + steg * dz
                    lam = old[3] + steg * dlam
                    xsi = old[4] + steg * dxsi
                    eta = old[5] + steg * deta
                    mu = old[6] + steg * dmu
                    zeta = old[7] + steg * dzeta
                    s = old[8] + steg * ds
                    newres, residumax = self._resid(x, y, z, lam, xsi, eta, mu, zeta, s, epsi)
                    steg = steg / 2.0
                residunorm = newres
            epsi = 0.1 * epsi
        self.xold2 = self.xold1.copy()
        self.xold1 = designx.copy()
        self.y, self.z, self.lam, self.zeta = y, z, lam, zeta
        self.xsi, self.eta, self.mu, self.s = xsi, eta, mu, s
        return x

    def update(self, it, x, df0dx, fval, dfdx):
        """One MMA iteration (mma_update_cpu); returns the new design."""
        dfdx = np.asarray(dfdx, dtype=np.float64).reshape(self.m, self.n)
        self.gensub(it, x, np.asarray(df0dx, np.float64), np.asarray(fval, np.float64), dfdx)
        return self.subsolve(np.asarray(x, np.float64))

    def kkt(self, x, df0dx, fval, dfdx):
        """mma_KKT_cpu: (residumax, residunorm) at the design x."""
        dfdx = np.asarray(dfdx, dtype=np.float64).reshape(self.m, self.n)
        rex = df0dx + dfdx.T @ self.lam - self.xsi + self.eta
        rey = self.c + self.d * self.y - self.lam - self.mu
        rez = self.a0 - self.zeta - self.lam @ self.a
        relam = fval - self.a * self.z - self.y + self.s
        rexsi = self.xsi * (x - self.xmin)
        reeta = self.eta * (self.xmax - x)
        remu = self.mu * self.y
        rezeta = self.zeta * self.z
        res = self.lam * self.s
        allr = np.concatenate([rex, rey, [rez], relam, rexsi, reeta, remu, [rezeta], res])
        self.residumax = float(np.abs(allr).max())
        self.residunorm = float(np.sqrt(np.sum(allr ** 2)))
        return self.residumax, self.residunorm


def toy1(x):
    """Svanberg's toy problem 1 (tests/mma/mmatest1.f90:99-131)."""
    f0 = 0.0624 * x.sum()
    df0 = np.full(5, 0.0624)
    cf = np.array([61.0, 37.0, 19.0, 7.0, 1.0])
    f = np.array([np.sum(cf / x ** 3) - 1.0])
    df = (-3.0 * cf / x ** 4).reshape(1, 5)
    return f0, df0, f, df


def toy2(x):
    """Svanberg's toy problem 2 (tests/mma/mmatest2.f90:101-135)."""
    f0 = float(np.sum(x ** 2))
    df0 = 2 * x
    c1, c2 = np.array([5.0, 2.0, 1.0]), np.array([3.0, 4.0, 3.0])
    f = np.array([np.sum((x - c1) ** 2) - 9.0, np.sum((x - c2) ** 2) - 9.0])
    df = np.stack([2 * (x - c1), 2 * (x - c2)])
    return f0, df0, f, df
