"""numpy restatement of the dealiased (over-integrated) adjoint and
linearised advection terms.

TEST INFRASTRUCTURE ONLY: the checker for neko-top_gb300/csrc/dealias.cu.

Follows sources/adjoint/adv_adjoint_dealias.f90 (init_dealias :137-224,
compute_adjoint_advection_dealias :235-462, compute_linear_advection_dealias
:470-600): the fields are interpolated from the lx GLL points to lxd
Gauss-Legendre (GL) points (J, per direction), the products are formed there
with the GL quadrature weights and the metric cofactors interpolated to GL,
and the result is brought back with J^T (Neko's interp_t map to the GLL
space, the transpose of the GLL -> GL interpolation):

  adjoint:  f_i -= J^T [ sum_j u_j opgrad_i(Ub_j) + sum_d cdtp_d(u_i Ub_d) ]_GL
  linear:   f_i -= J^T [ u . opgrad(Ub_i) + Ub . opgrad(u_i) ]_GL

GL points and weights: numpy's Golub-Welsch leggauss; the interpolation and
GL differentiation matrices from the Lagrange basis written as products.
Default lxd = 3 lx / 2 (advection_adjoint_fctry.f90:66-90).
"""
from __future__ import annotations

import numpy as np

from . import deriv_ref as dr


def lagrange_matrix(src, dst):
    """L[A, a] = l_a(dst[A]) for the Lagrange basis on the nodes `src`."""
    L = np.ones((len(dst), len(src)))
    for a in range(len(src)):
        for k in range(len(src)):
            if k != a:
                L[:, a] *= (dst - src[k]) / (src[a] - src[k])
    return L


def lagrange_deriv(nodes):
    """Dm[A, l] = l_l'(nodes[A]) (sum over product-rule terms)."""
    n = len(nodes)
    Dm = np.zeros((n, n))
    for l in range(n):
        for A in range(n):
            s = 0.0
            for m in range(n):
                if m == l:
                    continue
                p = 1.0 / (nodes[l] - nodes[m])
                for k in range(n):
                    if k != l and k != m:
                        p *= (nodes[A] - nodes[k]) / (nodes[l] - nodes[k])
                s += p
            Dm[A, l] = s
    return Dm


class GL:
    def __init__(self, m, lxd=None):
        from . import oracle as orc
        self.lx = m.lx
        self.lxd = lxd or 3 * m.lx // 2
        xi, _, _ = orc.gll(m.lx)
        self.xg, self.wg = np.polynomial.legendre.leggauss(self.lxd)
        self.J = lagrange_matrix(xi, self.xg)
        self.D = lagrange_deriv(self.xg)
        self.nelv = m.nelv
        g, _, _ = dr.metrics(m)
        self.cof = {k: self.to_gl(v) for k, v in g.items()}
        w = self.wg
        self.w3 = np.tile(np.einsum("k,j,i->kji", w, w, w).ravel(), m.nelv)

    def to_gl(self, u):
        U = np.asarray(u).reshape(self.nelv, self.lx, self.lx, self.lx)
        J = self.J
        return np.einsum("Ck,Bj,Ai,ekji->eCBA", J, J, J, U).ravel()

    def to_gll(self, v):
        V = np.asarray(v).reshape(self.nelv, self.lxd, self.lxd, self.lxd)
        J = self.J
        return np.einsum("Ck,Bj,Ai,eCBA->ekji", J, J, J, V).ravel()

    def rgrad(self, u):
        U = u.reshape(self.nelv, self.lxd, self.lxd, self.lxd)
        D = self.D
        return (np.einsum("il,ekjl->ekji", D, U).ravel(), np.einsum("jl,ekli->ekji", D, U).ravel(),
                np.einsum("kl,elji->ekji", D, U).ravel())

    def opgrad(self, u):
        ur, us, ut = self.rgrad(u)
        c = self.cof
        return tuple(self.w3 * (c["drd" + d] * ur + c["dsd" + d] * us + c["dtd" + d] * ut) for d in "xyz")

    def cdtp(self, x, d):
        c, D = self.cof, self.D
        E = lambda a: a.reshape(self.nelv, self.lxd, self.lxd, self.lxd)
        a, b, cc = (E(self.w3 * c[k + d] * x) for k in ("drd", "dsd", "dtd"))
        return (np.einsum("li,ekjl->ekji", D, a) + np.einsum("lj,ekli->ekji", D, b)
                + np.einsum("lk,elji->ekji", D, cc)).ravel()


def adjoint_advection(m, f, u, ub, lxd=None):
    g = GL(m, lxd)
    U = [g.to_gl(a) for a in u]
    Ub = [g.to_gl(a) for a in ub]
    grads = [g.opgrad(Ub[j]) for j in range(3)]
    out = []
    for i in range(3):
        t1 = sum(U[j] * grads[j][i] for j in range(3))
        t2 = sum(g.cdtp(U[i] * Ub[d], "xyz"[d]) for d in range(3))
        out.append(f[i] - g.to_gll(t1) - g.to_gll(t2))
    return out


def linear_advection(m, f, u, ub, lxd=None):
    g = GL(m, lxd)
    U = [g.to_gl(a) for a in u]
    Ub = [g.to_gl(a) for a in ub]
    out = []
    for i in range(3):
        gb = g.opgrad(Ub[i])
        gu = g.opgrad(U[i])
        t1 = sum(U[d] * gb[d] for d in range(3))
        t2 = sum(Ub[d] * gu[d] for d in range(3))
        out.append(f[i] - g.to_gll(t1) - g.to_gll(t2))
    return out
