"""numpy restatement of the spectral-element derivative operators used by
the adjoint advection and forcing terms.

TEST INFRASTRUCTURE ONLY: the checker for neko-top_gb300/csrc/deriv.cu.

Conventions (the Nek5000/Neko ones): per element, reference derivatives
u_r = D u along r (likewise s, t); the metric cofactors drdx = ys zt - yt zs
(and the other eight), jac = det dx/dr, so dr/dx = drdx / jac; w3 = the GLL
weight product, B = w3 jac.

  dudxyz(u, dr, ds, dt)  (dr u_r + ds u_s + dt u_t) / jac        strong derivative
  opgrad(u)              w3 (drdx u_r + dsdx u_s + dtdx u_t), ...   weak gradient (= B grad u)
  cdtp(x, dr, ds, dt)    D_r^T (w3 dr x) + D_s^T (w3 ds x) + D_t^T (w3 dt x)
                         (the transpose of opgrad's component: sum x * opgrad(u) = sum cdtp(x) * u)
  conv1(u, vx, vy, vz)   vx du/dx + vy du/dy + vz du/dz            strong, pointwise
  curl(u)                strong curl, then B-weighted average across element copies:
                         Binv gs(B curl)

Composite terms (sources/adjoint/adv_adjoint_no_dealias.f90:118-340 and
sources/source_terms/adjoint_minimum_dissipation_source_term.f90:175-249):

  adjoint advection:  f_i -= sum_j u_j opgrad_i(Ub_j) + sum_d cdtp_d(u_i Ub_d)
                      (the device branch of adjoint_weak_no_dealias; the CPU
                      branch there adds two of the three cdtp terms instead)
  linear advection:   f_i -= B conv1(u_i; Ub) + B conv1(Ub_i; u)
  min. dissipation:   f += scale curl(curl(u))   (optionally only inside a zone)
"""
from __future__ import annotations

import numpy as np


def _elem(m):
    lx = m.lx
    return lambda a: np.asarray(a).reshape(m.nelv, lx, lx, lx)  # (e, k, j, i)


def ref_derivs(m, u):
    """(u_r, u_s, u_t) per local node."""
    E = _elem(m)
    U = E(u)
    D = m.D
    ur = np.einsum("il,ekjl->ekji", D, U)
    us = np.einsum("jl,ekli->ekji", D, U)
    ut = np.einsum("kl,elji->ekji", D, U)
    return ur.ravel(), us.ravel(), ut.ravel()


def metrics(m):
    """drdx .. dtdz (cofactors), jac and w3 per local node."""
    xr, xs, xt = ref_derivs(m, m.x)
    yr, ys, yt = ref_derivs(m, m.y)
    zr, zs, zt = ref_derivs(m, m.z)
    jac = xr * (ys * zt - yt * zs) - xs * (yr * zt - yt * zr) + xt * (yr * zs - ys * zr)
    g = {
        "drdx": ys * zt - yt * zs, "drdy": xt * zs - xs * zt, "drdz": xs * yt - xt * ys,
        "dsdx": yt * zr - yr * zt, "dsdy": xr * zt - xt * zr, "dsdz": xt * yr - xr * yt,
        "dtdx": yr * zs - ys * zr, "dtdy": xs * zr - xr * zs, "dtdz": xr * ys - xs * yr,
    }
    w = m.w
    w3 = np.einsum("k,j,i->kji", w, w, w).ravel()
    w3 = np.tile(w3, m.nelv)
    return g, jac, w3


def dudxyz(m, u, d):
    g, jac, _ = metrics(m)
    ur, us, ut = ref_derivs(m, u)
    return (g["drd" + d] * ur + g["dsd" + d] * us + g["dtd" + d] * ut) / jac


def opgrad(m, u):
    g, _, w3 = metrics(m)
    ur, us, ut = ref_derivs(m, u)
    return tuple(w3 * (g["drd" + d] * ur + g["dsd" + d] * us + g["dtd" + d] * ut) for d in "xyz")


def cdtp(m, x, d):
    g, _, w3 = metrics(m)
    E = _elem(m)
    D = m.D
    a = E(w3 * g["drd" + d] * x)
    b = E(w3 * g["dsd" + d] * x)
    c = E(w3 * g["dtd" + d] * x)
    out = np.einsum("li,ekjl->ekji", D, a) + np.einsum("lj,ekli->ekji", D, b) + np.einsum("lk,elji->ekji", D, c)
    return out.ravel()


def conv1(m, u, vx, vy, vz):
    return vx * dudxyz(m, u, "x") + vy * dudxyz(m, u, "y") + vz * dudxyz(m, u, "z")


def curl(m, gs_op, ux, uy, uz):
    """Binv gs(B curl u); gs_op(v) is the assembled sum over copies."""
    w1 = dudxyz(m, uz, "y") - dudxyz(m, uy, "z")
    w2 = dudxyz(m, ux, "z") - dudxyz(m, uz, "x")
    w3_ = dudxyz(m, uy, "x") - dudxyz(m, ux, "y")
    Bg = gs_op(m.B)
    return tuple(gs_op(m.B * w) / Bg for w in (w1, w2, w3_))


def adjoint_advection(m, f, u, ub):
    """f (3 components) updated: f_i -= sum_j u_j opgrad_i(Ub_j) + sum_d cdtp_d(u_i Ub_d)."""
    grads = [opgrad(m, ub[j]) for j in range(3)]  # grads[j][i] = B d(Ub_j)/dx_i
    out = []
    for i in range(3):
        t1 = sum(u[j] * grads[j][i] for j in range(3))
        t2 = sum(cdtp(m, u[i] * ub[d], "xyz"[d]) for d in range(3))
        out.append(f[i] - t1 - t2)
    return out


def linear_advection(m, f, u, ub):
    """f_i -= B conv1(u_i; Ub) + B conv1(Ub_i; u)."""
    out = []
    for i in range(3):
        out.append(f[i] - m.B * conv1(m, u[i], *ub) - m.B * conv1(m, ub[i], *u))
    return out


def min_dissipation_forcing(m, gs_op, f, u, scale, zone=None):
    """f += scale curl(curl(u)); with `zone` (1-based local indices) the term
    is kept inside the zone and zero outside (mask_exterior_const,
    sources/neko_ext/mask_ops.f90:55-82)."""
    w = curl(m, gs_op, *u)
    c = list(curl(m, gs_op, *w))
    if zone is not None:
        keep = np.zeros(m.n, dtype=bool)
        keep[np.asarray(zone) - 1] = True
        c = [np.where(keep, a, 0.0) for a in c]
    return [f[i] + scale * c[i] for i in range(3)]
