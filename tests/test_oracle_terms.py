"""The compiled CPU restatement of the step terms (oracle/terms_oracle.c,
the timed CPU baseline of those terms) against the numpy restatements the
GPU kernels are checked with."""
import numpy as np
import pytest

from oracle import dealias_ref, deriv_ref, oracle as orc, pnpn_ref
from oracle.terms_c import Terms


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.fixture(scope="module")
def case():
    m = orc.build_mesh(3, 2, 2, 6, amp=0.04, seed=2)
    rng = np.random.default_rng(1)
    x, y, z = m.x, m.y, m.z
    u = [rng.standard_normal(m.n) for _ in range(3)]
    ub = [np.sin(x) + y, np.cos(y) * z, x * z - y]
    f = [rng.standard_normal(m.n) for _ in range(3)]
    p = np.cos(x + y) * z
    return m, Terms(m), u, ub, f, p


def test_operators(case):
    m, t, u, ub, f, p = case
    for a, b in zip(t.opgrad(p), deriv_ref.opgrad(m, p)):
        assert rel(a, b) < 1e-13
    cs = t.cdtp_sum(u[0], u[1], u[2])
    ref = sum(deriv_ref.cdtp(m, u[d], "xyz"[d]) for d in range(3))
    assert rel(cs, ref) < 1e-13
    gs = lambda v: orc.gs_op(m, v)
    for a, b in zip(t.curl(*ub), deriv_ref.curl(m, gs, *ub)):
        assert rel(a, b) < 1e-12


@pytest.mark.parametrize("mode", ["adjoint", "linear"])
def test_advection(case, mode):
    m, t, u, ub, f, p = case
    ref_fn = deriv_ref.adjoint_advection if mode == "adjoint" else deriv_ref.linear_advection
    out, ref = t.advection(f, u, ub, mode), ref_fn(m, f, u, ub)
    for a, b, a0 in zip(out, ref, f):
        assert rel(a - a0, b - a0) < 1e-12
    gl = dealias_ref.GL(m)
    ref_fn = dealias_ref.adjoint_advection if mode == "adjoint" else dealias_ref.linear_advection
    out, ref = t.advection(f, u, ub, mode, gl), ref_fn(m, f, u, ub)
    for a, b, a0 in zip(out, ref, f):
        assert rel(a - a0, b - a0) < 1e-12


def test_residuals_and_forcing(case):
    m, t, u, ub, f, p = case
    mu, rho, bd, dt = 0.02, 1.1, 1.5, 1e-3
    for a, b in zip(t.vel_res(u, p, f, mu, rho, bd, dt), pnpn_ref.vel_res(m, u, p, f, mu, rho, bd, dt)):
        assert rel(a, b) < 1e-12
    face = np.nonzero(np.isclose(m.x, m.x.max()))[0]
    surf = (face, np.stack([np.full(face.size, 0.3), np.zeros(face.size), np.zeros(face.size)]))
    assert rel(t.prs_res(p, u, ub, f, mu, rho, bd, dt, surf, None),
               pnpn_ref.prs_res(m, p, u, ub, f, mu, rho, bd, dt, surf, None)) < 1e-11
    gs = lambda v: orc.gs_op(m, v)
    got = [a - a0 for a, a0 in zip(t.min_dissipation(f, ub, 0.5), f)]
    ref = [b - a0 for b, a0 in zip(deriv_ref.min_dissipation_forcing(m, gs, f, ub, 0.5), f)]
    # one component of curl(curl Ub) is 1e-5 of the others: compare against the term's scale
    scale = max(np.abs(b).max() for b in ref)
    assert max(np.abs(a - b).max() for a, b in zip(got, ref)) < 1e-11 * scale
