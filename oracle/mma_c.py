"""ctypes front end of oracle/mma_oracle.c: the compiled (OpenMP) MMA
update, same constructor and update() as oracle/mma_ref.MMA, which it is
checked against.

TEST INFRASTRUCTURE ONLY: the timed CPU baseline of the GPU MMA.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import oracle as orc

_d = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_bound = False


def _lib():
    global _bound
    L = orc.lib()
    if not _bound:
        L.orcm_update.restype = C.c_int
        L.orcm_update.argtypes = ([C.c_int64, C.c_int, C.c_int] + [_d] * 10 + [C.c_double, _d, _d, _d, C.c_double,
                                  C.c_int, C.c_double, C.c_double, C.c_double] + [_d] * 6)
        _bound = True
    return L


class MMAC:
    def __init__(self, x, m, a0, a, c, d, xmin, xmax, max_iter=100, epsimin=None, asyinit=0.5, asyincr=1.2,
                 asydecr=0.7):
        x = np.ascontiguousarray(x, dtype=np.float64)
        n = x.size
        self.n, self.m = n, m
        self.xold1, self.xold2 = x.copy(), x.copy()
        self.a0 = float(a0)
        self.a, self.c, self.d = (np.ascontiguousarray(np.broadcast_to(np.asarray(v, np.float64), (m,)))
                                  for v in (a, c, d))
        self.xmin = np.ascontiguousarray(np.broadcast_to(np.asarray(xmin, np.float64), (n,)))
        self.xmax = np.ascontiguousarray(np.broadcast_to(np.asarray(xmax, np.float64), (n,)))
        self.low = np.full(n, x.min())
        self.upp = np.full(n, x.max())
        self.max_iter = max_iter
        self.epsimin = 1.0e-9 * np.sqrt(m + n) if epsimin is None else epsimin
        self.asy = (asyinit, asyincr, asydecr)
        self.scratch = np.empty((13 + 2 * m) * n)
        self.y, self.lam, self.s, self.mu = (np.zeros(m) for _ in range(4))
        self.dual = np.zeros(2)
        self.newton_steps = 0

    def update(self, it, x, df0dx, fval, dfdx):
        """One MMA iteration; returns the new design (x is not modified)."""
        xd = np.ascontiguousarray(x, dtype=np.float64).copy()
        dfl = np.ascontiguousarray(np.asarray(dfdx, np.float64).reshape(self.m, self.n).T.ravel())
        k = _lib().orcm_update(self.n, self.m, int(it), xd, self.xold1, self.xold2, self.low, self.upp, self.xmin,
                               self.xmax, np.ascontiguousarray(df0dx, dtype=np.float64),
                               np.ascontiguousarray(fval, dtype=np.float64), dfl, self.a0, self.a, self.c, self.d,
                               float(self.epsimin), int(self.max_iter), *[float(v) for v in self.asy], self.scratch,
                               self.y, self.lam, self.s, self.mu, self.dual)
        if k < 0:
            raise RuntimeError("singular Newton system in the MMA subproblem")
        self.newton_steps += k
        return xd
