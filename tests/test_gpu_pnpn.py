"""Pn/Pn splitting residuals (pressure and velocity) against the numpy
restatement in oracle/pnpn_ref.py, with constant and field-valued mu/rho and
with velocity- and symmetry-surface terms."""
import numpy as np
import pytest
import torch

from oracle import pnpn_ref

pytestmark = pytest.mark.gpu


def T(a, dev, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device=dev, dtype=dtype)


def H(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def fields(m, seed):
    rng = np.random.default_rng(seed)
    x, y, z = m.x, m.y, m.z
    u = [np.sin(2 * x) * np.cos(y) + z, np.cos(1.5 * y) * x + np.sin(z), np.exp(0.3 * x) * np.sin(2 * z) - y * y]
    ue = [a + 0.1 * np.cos(3 * x + 2 * y - z) for a in u]
    f = [rng.standard_normal(m.n) for _ in range(3)]
    p = np.cos(x + 2 * y) * np.sin(z) + rng.uniform(-0.1, 0.1, m.n)
    return u, ue, f, p


def surfaces(m, rng):
    """velocity surface: the x = 1 face; symmetry surface: the y = 0 face
    (node lists, 1-based, and arbitrary normal-times-area vectors)."""
    xmax = np.nonzero(np.isclose(m.x, m.x.max()))[0]
    ymin = np.nonzero(np.isclose(m.y, m.y.min()))[0]
    sp = np.stack([rng.uniform(0.5, 1.0, xmax.size), rng.uniform(-0.1, 0.1, xmax.size), np.zeros(xmax.size)])
    ss = np.stack([np.zeros(ymin.size), -rng.uniform(0.5, 1.0, ymin.size), rng.uniform(-0.1, 0.1, ymin.size)])
    return (xmax, sp), (ymin, ss)


@pytest.mark.parametrize("shape,props", [((3, 2, 2, 8, 0.05), "const"), ((2, 2, 3, 6, 0.04), "field"),
                                         ((2, 3, 2, 5, 0.0), "field"), ((2, 1, 1, 10, 0.03), "const"),
                                         ((3, 2, 1, 3, 0.02), "field")])
def test_vel_res_matches_oracle(pkg, orc, dev, shape, props):
    ex, ey, ez, lx, amp = shape
    m = orc.build_mesh(ex, ey, ez, lx, amp=amp, seed=3)
    c = pkg.coef_t.box(ex, ey, ez, lx, amp=amp, seed=3, device=dev)
    u, _, f, p = fields(m, 1)
    rng = np.random.default_rng(2)
    mu, rho = (0.01, 1.3) if props == "const" else (rng.uniform(0.005, 0.02, m.n), rng.uniform(0.8, 1.2, m.n))
    bd, dt = 1.8333333333333333, 1e-3
    res = [torch.empty(m.n, dtype=torch.float64, device=dev) for _ in range(3)]
    pkg.pnpn_vel_res_t().compute(*[T(a, dev) for a in u], *res, T(p, dev), *[T(a, dev) for a in f], c,
                                 mu=mu if props == "const" else T(mu, dev),
                                 rho=rho if props == "const" else T(rho, dev), bd=bd, dt=dt)
    ref = pnpn_ref.vel_res(m, u, p, f, mu, rho, bd, dt)
    for a, b in zip(res, ref):
        assert rel(H(a), b) < 1e-12


@pytest.mark.parametrize("shape,props,surf", [((3, 2, 2, 8, 0.05), "const", True), ((2, 2, 3, 6, 0.04), "field", True),
                                              ((2, 3, 2, 5, 0.0), "const", False), ((2, 1, 2, 10, 0.03), "field", True)])
def test_prs_res_matches_oracle(pkg, orc, dev, shape, props, surf):
    ex, ey, ez, lx, amp = shape
    m = orc.build_mesh(ex, ey, ez, lx, amp=amp, seed=5)
    c = pkg.coef_t.box(ex, ey, ez, lx, amp=amp, seed=5, device=dev)
    u, ue, f, p = fields(m, 4)
    rng = np.random.default_rng(6)
    mu, rho = (0.02, 0.9) if props == "const" else (rng.uniform(0.005, 0.02, m.n), rng.uniform(0.8, 1.2, m.n))
    bd, dt = 1.5, 2e-3
    (pi, ps), (si, ss) = surfaces(m, rng)
    out = torch.empty(m.n, dtype=torch.float64, device=dev)
    prs = (T(pi + 1, dev, torch.int32), T(ps, dev)) if surf else None
    sym = (T(si + 1, dev, torch.int32), T(ss, dev)) if surf else None
    pkg.pnpn_prs_res_t().compute(T(p, dev), out, *[T(a, dev) for a in u], *[T(a, dev) for a in ue],
                                 *[T(a, dev) for a in f], c, prs, sym, bd=bd, dt=dt,
                                 mu=mu if props == "const" else T(mu, dev),
                                 rho=rho if props == "const" else T(rho, dev))
    ref = pnpn_ref.prs_res(m, p, u, ue, f, mu, rho, bd, dt, (pi, ps) if surf else None,
                           (si, ss) if surf else None)
    assert rel(H(out), ref) < 1e-11


def test_prs_res_reduces_to_minus_laplacian(pkg, orc, dev):
    """With no forcing, a curl-free extrapolated velocity and no surface
    terms, the pressure residual is -A(1/rho) p: the library's own Ax."""
    m = orc.build_mesh(2, 2, 2, 8, amp=0.03, seed=7)
    c = pkg.coef_t.box(2, 2, 2, 8, amp=0.03, seed=7, device=dev)
    rho = 1.25
    x, y, z = m.x, m.y, m.z
    ue = [2 * x + y, x - z, 3.0 - y]  # gradient of x^2 + xy - yz + 3z: curl 0
    zero = np.zeros(m.n)
    p = np.sin(x) * np.cos(2 * y) * z
    out = torch.empty(m.n, dtype=torch.float64, device=dev)
    pkg.pnpn_prs_res_t().compute(T(p, dev), out, *[T(zero, dev)] * 3, *[T(a, dev) for a in ue], *[T(zero, dev)] * 3,
                                 c, bd=1.0, dt=0.1, mu=0.01, rho=rho)
    c.set_coefs(h1c=1.0 / rho, ifh2=False)
    w = torch.empty(m.n, dtype=torch.float64, device=dev)
    pkg.ax_helm_t().compute(w, T(p, dev), c)
    assert rel(H(out), -H(w)) < 1e-10


def test_residual_arguments_are_checked(pkg, orc, dev):
    c = pkg.coef_t.box(2, 1, 1, 4, device=dev)
    z = torch.zeros(c.n, dtype=torch.float64, device=dev)
    with pytest.raises(pkg.NtgError):
        pkg.pnpn_vel_res_t().compute(z, z, z, z.clone(), z.clone(), z.clone(), z, z, z, z, c, dt=0.0)
    bad = (torch.ones(3, dtype=torch.int32, device=dev), torch.ones(2, 3, dtype=torch.float64, device=dev))
    with pytest.raises(ValueError):
        pkg.pnpn_prs_res_t().compute(z, z.clone(), z, z, z, z, z, z, z, z, z, c, bad)
