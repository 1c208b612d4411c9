"""numpy restatement of the Pn/Pn splitting residuals that bracket the
pressure and velocity solves of each time step.

TEST INFRASTRUCTURE ONLY: the checker for neko-top_gb300/csrc/pnpn.cu.

The reference calls them as prs_res%compute and vel_res%compute
(sources/adjoint/adjoint_pnpn.f90:716-723 and :747-753); their code is in
the external Neko library (not vendored), so this follows the published
Pn/Pn splitting (Karniadakis, Israeli & Orszag 1991; Tomboulides, Lee &
Orszag 1997; Deville, Fischer & Mund 2002, sec. 6.5) in the form the
reference's arguments fix: fields mu, rho, the first BDF coefficient bd and
the step dt; the viscous term in the rotational (curl-curl) form.

  pressure residual
    wa   = curl(curl(u_e))                     (each curl: Binv gs(B curl))
    ta_d = Binv gs(f_d / rho - (mu / rho) B wa_d)
    p_res = -A(h1 = 1/rho) p + sum_d cdtp_d(ta_d)
            - (bd / dt) sum_c u_c s_c      on the velocity-surface nodes
            - sum_c ta_c s'_c              on the symmetry-surface nodes
    (s, s' = outward normal times facet area per surface node)

  velocity residual
    u_res_c = f_c - (mu K + rho (bd / dt) B) u_c - opgrad_c(p)

Neither is gs-assembled or masked here: the caller does that next
(adjoint_pnpn.f90:725-726 and :755-776).
"""
from __future__ import annotations

import numpy as np

from . import deriv_ref as dr
from . import oracle as orc


def _arr(m, v):
    return np.full(m.n, float(v)) if np.isscalar(v) else np.asarray(v, dtype=np.float64)


def prs_res(m, p, u, ue, f, mu, rho, bd, dt, prs_surf=None, sym_surf=None):
    """u, ue, f: 3-lists of fields; mu, rho: scalars or fields; *_surf:
    (idx 0-based, s [3 x ns]) or None."""
    gs = lambda a: orc.gs_op(m, a)
    mu, rho = _arr(m, mu), _arr(m, rho)
    binv = 1.0 / gs(m.B)
    wa = dr.curl(m, gs, *dr.curl(m, gs, *ue))
    ta = [gs(f[d] / rho - (mu / rho) * m.B * wa[d]) * binv for d in range(3)]
    out = -orc.ax_helm(m, p, h1=1.0 / rho)
    for d in range(3):
        out = out + dr.cdtp(m, ta[d], "xyz"[d])
    if prs_surf is not None:
        idx, s = prs_surf
        out[idx] -= (bd / dt) * sum(u[c][idx] * s[c] for c in range(3))
    if sym_surf is not None:
        idx, s = sym_surf
        out[idx] -= sum(ta[c][idx] * s[c] for c in range(3))
    return out


def vel_res(m, u, p, f, mu, rho, bd, dt):
    mu, rho = _arr(m, mu), _arr(m, rho)
    g = dr.opgrad(m, p)
    return [f[c] - orc.ax_helm(m, u[c], h1=mu, h2=rho * (bd / dt)) - g[c] for c in range(3)]
