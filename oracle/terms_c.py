"""ctypes front end of oracle/terms_oracle.c: the compiled (OpenMP) CPU
restatement of the FP64 step terms, with the same call shapes as the numpy
restatements it is checked against (oracle/deriv_ref.py, pnpn_ref.py,
dealias_ref.py).

TEST INFRASTRUCTURE ONLY: the timed CPU baseline of those terms.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import oracle as orc

_d = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_I64, _vp = C.c_int64, C.c_void_p
_bound = False


def _lib():
    global _bound
    L = orc.lib()
    if not _bound:
        L.orct_metrics.argtypes = [_I64, C.c_int, _d, _d, _d, _d, _d]
        L.orct_opgrad.argtypes = [_I64, C.c_int, _d, _d, _d, _d, _d, _d, _d]
        L.orct_cdtp_sum.argtypes = [_I64, C.c_int, _d, _d, _d, _vp, _vp, _vp, _d]
        L.orct_bcurl.argtypes = [_I64, C.c_int, _d, _d, _d] + [_d] * 6
        L.orct_adv_no_dealias.argtypes = [C.c_int, _I64, C.c_int, _d, _d, _d] + [_d] * 9
        L.orct_adv_dealias.argtypes = [C.c_int, _I64, C.c_int, C.c_int, _d, _d, _d, _d] + [_d] * 9
        _bound = True
    return L


def _c(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Terms:
    """Per-mesh state: the metric cofactors and 1/gs(B)."""

    def __init__(self, m):
        self.m = m
        self.D, self.w = _c(m.D.ravel()), _c(m.w)
        self.met = np.empty(10 * m.n)
        _lib().orct_metrics(m.nelv, m.lx, self.D, _c(m.x), _c(m.y), _c(m.z), self.met)
        self.binv = 1.0 / orc.gs_op(m, m.B)

    def gs(self, a):
        return orc.gs_op(self.m, a)

    def opgrad(self, u):
        m = self.m
        o = [np.empty(m.n) for _ in range(3)]
        _lib().orct_opgrad(m.nelv, m.lx, self.D, self.w, self.met, _c(u), *o)
        return o

    def cdtp_sum(self, a0, a1, a2):
        m = self.m
        a = [None if v is None else _c(v) for v in (a0, a1, a2)]
        out = np.empty(m.n)
        _lib().orct_cdtp_sum(m.nelv, m.lx, self.D, self.w, self.met, *[_p(v) for v in a], out)
        return out

    def curl(self, u1, u2, u3):
        m = self.m
        o = [np.empty(m.n) for _ in range(3)]
        _lib().orct_bcurl(m.nelv, m.lx, self.D, self.w, self.met, _c(u1), _c(u2), _c(u3), *o)
        return [self.gs(a) * self.binv for a in o]

    def advection(self, f, u, ub, mode, gl=None):
        """f_i - term_i; mode "adjoint" or "linear"; gl: a dealias_ref.GL for
        the dealiased form."""
        m = self.m
        out = [_c(a).copy() for a in f]
        md = 0 if mode == "adjoint" else 1
        args = [_c(a) for a in u] + [_c(a) for a in ub] + out
        if gl is None:
            _lib().orct_adv_no_dealias(md, m.nelv, m.lx, self.D, self.w, self.met, *args)
        else:
            _lib().orct_adv_dealias(md, m.nelv, m.lx, gl.lxd, _c(gl.J.ravel()), _c(gl.D.ravel()), _c(gl.wg),
                                    self.met, *args)
        return out

    def vel_res(self, u, p, f, mu, rho, bd, dt):
        m = self.m
        mu_a = np.full(m.n, float(mu)) if np.isscalar(mu) else _c(mu)
        rho_a = np.full(m.n, float(rho)) if np.isscalar(rho) else _c(rho)
        g = self.opgrad(p)
        return [_c(f[c]) - orc.ax_helm(m, _c(u[c]), h1=mu_a, h2=rho_a * (bd / dt)) - g[c] for c in range(3)]

    def prs_res(self, p, u, ue, f, mu, rho, bd, dt, prs_surf=None, sym_surf=None):
        m = self.m
        mu_a = np.full(m.n, float(mu)) if np.isscalar(mu) else _c(mu)
        rho_a = np.full(m.n, float(rho)) if np.isscalar(rho) else _c(rho)
        wa = self.curl(*self.curl(*ue))
        ta = [self.gs(_c(f[d]) / rho_a - (mu_a / rho_a) * m.B * wa[d]) * self.binv for d in range(3)]
        out = -orc.ax_helm(m, _c(p), h1=1.0 / rho_a) + self.cdtp_sum(*ta)
        if prs_surf is not None:
            idx, s = prs_surf
            out[idx] -= (bd / dt) * sum(_c(u[c])[idx] * s[c] for c in range(3))
        if sym_surf is not None:
            idx, s = sym_surf
            out[idx] -= sum(ta[c][idx] * s[c] for c in range(3))
        return out

    def min_dissipation(self, f, u, scale, zone=None):
        c = self.curl(*self.curl(*u))
        if zone is not None:
            keep = np.zeros(self.m.n, dtype=bool)
            keep[np.asarray(zone) - 1] = True
            c = [np.where(keep, a, 0.0) for a in c]
        return [_c(f[i]) + scale * c[i] for i in range(3)]
