"""One Pn/Pn step (pressure residual -> solve -> velocity residual ->
coupled solve) in the reference's order, against the same sequence composed
from the oracle's residuals and Jacobi-PCG."""
import numpy as np
import pytest
import torch

from oracle import pnpn_ref

pytestmark = pytest.mark.gpu


def T(a, dev, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device=dev, dtype=dtype)


def face_mask(c, m, which):
    """1-based local indices of a box face (x max for the pressure, x min for the velocity)."""
    x = m.x
    sel = np.isclose(x, x.max()) if which == "xmax" else np.isclose(x, x.min())
    return (np.nonzero(sel)[0] + 1).astype(np.int32)


def oracle_step(orc, m, u, p, ue, f, mu, rho, bd, dt, mp, mv):
    gs = lambda a: orc.gs_op(m, a)
    pr = orc.apply_mask_zero(gs(pnpn_ref.prs_res(m, p, u, ue, f, mu, rho, bd, dt)), mp)
    dp, itp, _, _ = orc.cg(m, pr, h1=np.full(m.n, 1.0 / rho), mask=mp, rtol=1e-10)
    p = p + dp
    res = pnpn_ref.vel_res(m, u, p, f, mu, rho, bd, dt)
    out = []
    for c in range(3):
        r = orc.apply_mask_zero(gs(res[c]), mv)
        du, _, _, _ = orc.cg(m, r, h1c=mu, h2=np.full(m.n, rho * bd / dt), mask=mv, rtol=1e-10)
        out.append(u[c] + du)
    return p, out, itp


def test_step_matches_oracle_sequence(pkg, orc, dev):
    ex, ey, ez, lx, amp = 3, 2, 2, 6, 0.04
    m = orc.build_mesh(ex, ey, ez, lx, amp=amp, seed=11)
    cp = pkg.coef_t.box(ex, ey, ez, lx, amp=amp, seed=11, device=dev)
    cv = pkg.coef_t.box(ex, ey, ez, lx, amp=amp, seed=11, device=dev)
    mp, mv = face_mask(cp, m, "xmax"), face_mask(cv, m, "xmin")
    cp.set_mask(T(mp, dev, torch.int32), base=1)
    cv.set_mask(T(mv, dev, torch.int32), base=1)
    rng = np.random.default_rng(3)
    x, y, z = m.x, m.y, m.z
    u = [np.sin(x) * y, np.cos(y) * z + x, x * z]
    ue = [a + 0.05 * np.sin(2 * x + z) for a in u]
    f = [rng.standard_normal(m.n) for _ in range(3)]
    p = np.cos(x + y) * z
    mu, rho, bd, dt = 0.05, 1.2, 1.5, 0.01
    st = pkg.pnpn_step_t(cp, cv, L=0)
    ud, pd = [T(a, dev) for a in u], T(p, dev)
    mon_p, mons_v = st.step(*ud, pd, *[T(a, dev) for a in ue], *[T(a, dev) for a in f], mu=mu, rho=rho, bd=bd,
                            dt=dt)
    p_ref, u_ref, itp = oracle_step(orc, m, u, p, ue, f, mu, rho, bd, dt, mp, mv)
    torch.cuda.synchronize()
    assert abs(mon_p.iter - itp) <= 2
    assert np.linalg.norm(pd.cpu().numpy() - p_ref) <= 1e-8 * np.linalg.norm(p_ref)
    for a, b in zip(ud, u_ref):
        assert np.linalg.norm(a.cpu().numpy() - b) <= 1e-8 * np.linalg.norm(b)
    assert all(mn.status == pkg.NTG_OK for mn in [mon_p] + mons_v)


def test_projection_reduces_pressure_iterations(pkg, orc, dev):
    """Over a few steps with slowly changing forcing the pressure projection
    lowers the iteration count and leaves the solution unchanged."""
    ex, ey, ez, lx = 3, 3, 2, 6
    m = orc.build_mesh(ex, ey, ez, lx, amp=0.03, seed=5)
    runs = {}
    for L in (0, 8):
        cp = pkg.coef_t.box(ex, ey, ez, lx, amp=0.03, seed=5, device=dev)
        cv = pkg.coef_t.box(ex, ey, ez, lx, amp=0.03, seed=5, device=dev)
        cp.set_mask(T(face_mask(cp, m, "xmax"), dev, torch.int32), base=1)
        cv.set_mask(T(face_mask(cv, m, "xmin"), dev, torch.int32), base=1)
        st = pkg.pnpn_step_t(cp, cv, L=L, activ_step=0)
        x, y, z = m.x, m.y, m.z
        u = [T(np.sin(x) * y, dev), T(np.cos(y) * z, dev), T(x * z, dev)]
        p = T(np.zeros(m.n), dev)
        its = []
        for t in range(1, 6):
            f = [T(np.sin(x + 0.05 * t + k) * np.cos(y), dev) for k in range(3)]
            mon_p, _ = st.step(*u, p, *[a.clone() for a in u], *f, mu=0.05, rho=1.0, bd=1.0, dt=0.01, tstep=t)
            its.append(mon_p.iter)
        runs[L] = (its, p.cpu().numpy())
    assert sum(runs[8][0][2:]) < sum(runs[0][0][2:])
    assert np.linalg.norm(runs[8][1] - runs[0][1]) <= 1e-7 * np.linalg.norm(runs[0][1])
