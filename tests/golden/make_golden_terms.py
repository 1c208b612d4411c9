"""Freeze small outputs of the step-term and MMA oracles as golden fixtures
(tests/golden/golden_terms.npz).

TEST INFRASTRUCTURE ONLY.  The Pn/Pn residuals and derivative operators are
restated from the published methods (Neko, which implements them, is not
part of the reference), the MMA from the reference's sources/mma/; these
fixtures freeze the restatements' outputs on small seeded cases so the CPU
suite notices any drift.  The MMA fixture also holds the reference's own
known answer (tests/mma/mmatest1.f90:53).  Regenerate only on a deliberate
oracle change:

    python tests/golden/make_golden_terms.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import dealias_ref, deriv_ref, oracle as orc, pnpn_ref  # noqa: E402
from oracle.mma_ref import MMA, toy1, toy2  # noqa: E402


def cases():
    out = {}
    rng = np.random.default_rng(20261204)
    m = orc.build_mesh(2, 2, 2, 6, amp=0.05, seed=9)
    x, y, z = m.x, m.y, m.z
    u = [rng.standard_normal(m.n) for _ in range(3)]
    ub = [np.sin(2 * x) + y * z, np.cos(y) * x, z * z - x]
    f = [rng.standard_normal(m.n) for _ in range(3)]
    p = np.cos(x + y) * z
    for k in range(3):
        out[f"u{k}"], out[f"ub{k}"], out[f"f{k}"] = u[k], ub[k], f[k]
    out["p"] = p
    gs = lambda a: orc.gs_op(m, a)
    for k, v in enumerate(pnpn_ref.vel_res(m, u, p, f, 0.02, 1.1, 1.5, 1e-3)):
        out[f"vel_res{k}"] = v
    face = np.nonzero(np.isclose(x, x.max()))[0]
    sym = np.nonzero(np.isclose(y, y.min()))[0]
    ps = np.stack([np.full(face.size, 0.25), rng.uniform(-0.1, 0.1, face.size), np.zeros(face.size)])
    ss = np.stack([np.zeros(sym.size), np.full(sym.size, -0.25), np.zeros(sym.size)])
    out["face"], out["ps"], out["sym"], out["ss"] = face, ps, sym, ss
    out["prs_res"] = pnpn_ref.prs_res(m, p, u, ub, f, 0.02, 1.1, 1.5, 1e-3, (face, ps), (sym, ss))
    for name, fn in (("adj", deriv_ref.adjoint_advection), ("lin", deriv_ref.linear_advection),
                     ("adj_d", dealias_ref.adjoint_advection), ("lin_d", dealias_ref.linear_advection)):
        for k, v in enumerate(fn(m, f, u, ub)):
            out[f"{name}{k}"] = v
    zone = (np.nonzero(x < 0.5)[0] + 1).astype(np.int32)
    out["zone"] = zone
    for k, v in enumerate(deriv_ref.min_dissipation_forcing(m, gs, f, ub, 0.7, zone=zone)):
        out[f"md{k}"] = v
    # MMA: the reference's toy problems, 12 iterations each
    for name, prob, x0, args in (("toy1", toy1, np.full(5, 5.0), (1, 1.0, 0.0, 1000.0, 0.0, 0.0, 10.0)),
                                 ("toy2", toy2, np.array([4.0, 3.0, 2.0]), (2, 1.0, 0.0, 1000.0, 1.0, 0.0, 5.0))):
        opt, xv, its = MMA(x0, *args), x0.copy(), []
        for it in range(1, 13):
            _, df0, fv, dfv = prob(xv)
            xv = opt.update(it, xv, df0, fv, dfv)
            its.append(xv.copy())
        out[f"mma_{name}"] = np.array(its)
    out["mma_toy1_stated_optimum"] = np.array([6.016, 5.309, 4.494, 3.502, 2.153])
    return out


if __name__ == "__main__":
    np.savez_compressed(os.path.join(HERE, "golden_terms.npz"), **cases())
    print("wrote", os.path.join(HERE, "golden_terms.npz"))
