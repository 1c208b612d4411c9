"""Freeze small oracle outputs as golden fixtures (tests/golden/golden.npz).

TEST INFRASTRUCTURE ONLY.  The reference (Fortran + the external Neko) cannot
be built here and its tests hold no vectors for this path, so these fixtures
are the oracle's own outputs on small seeded cases, frozen: the CPU suite
checks that the oracle still reproduces them and the GPU suite checks the CUDA
path against them.  Regenerate only on a deliberate oracle change:

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as orc  # noqa: E402
from oracle import schwarz_ref  # noqa: E402


def cases():
    out = {}
    rng = np.random.default_rng(20261204)
    # ax_helm (FP64) on a deformed 2x2x2, lx = 6 mesh with variable h1 and h2
    m = orc.build_mesh(2, 2, 2, 6, amp=0.05, seed=7)
    u = rng.standard_normal(m.n)
    h1 = rng.uniform(0.5, 2.0, m.n)
    h2 = rng.uniform(0.0, 3.0, m.n)
    out["ax_u"], out["ax_h1"], out["ax_h2"] = u, h1, h2
    out["ax_w"] = orc.ax_helm(m, u, h1=h1, h2=h2)
    out["ax_w_gs"] = orc.gs_op(m, out["ax_w"])
    out["gs_perm"], out["gs_offs"] = m.perm.copy(), m.offs.copy()
    out["mult"] = m.mult.copy()
    # Jacobi-PCG on a Poisson problem with a Dirichlet face (3x2x2, lx = 5)
    m2 = orc.build_mesh(3, 2, 2, 5, amp=0.05, seed=8)
    mask = orc.mask_face_xmax(3, 2, 2, 5)
    k, a, ph = orc.fourier_params(9, 8)
    f = orc.assemble_rhs(m2, orc.field_fourier(m2, k, a, ph), mask)
    dinv = orc.jacobi(m2, h1c=1.0, mask=mask)
    x, it, r0, r1 = orc.cg(m2, f, h1c=1.0, mask=mask, dinv=dinv, rtol=1e-10, max_iter=5000)
    out["cg_f"], out["cg_x"], out["cg_iters"] = f, x, np.array([it])
    # RAMP forward / backward (reference formulas, both convexities)
    xin = rng.uniform(0.0, 1.0, 257)
    dF = rng.standard_normal(257)
    out["ramp_x"], out["ramp_dF"] = xin, dF
    for cu in (0, 1):
        out[f"ramp_fwd_{cu}"] = orc.ramp_forward(xin, 0.0, 1e4, 8.0, cu)
        out[f"ramp_bwd_{cu}"] = orc.ramp_backward(xin, dF, 0.0, 1e4, 8.0, cu)
    # two-level Schwarz (numpy restatement) on 3x2x2, lx = 4
    m3 = orc.build_mesh(3, 2, 2, 4, amp=0.05, seed=9)
    mask3 = orc.mask_face_xmax(3, 2, 2, 4)
    r = orc.apply_mask_zero(orc.gs_op(m3, rng.standard_normal(m3.n)) * m3.mult, mask3)
    out["sw_r"] = r
    out["sw_z"] = schwarz_ref.apply(m3, r, (3, 2, 2), h1=1.0, h2=None, mask=mask3, coarse=True)
    return out


if __name__ == "__main__":
    data = cases()
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **data)
    print({k: v.shape for k, v in data.items()})
