"""The derivative oracle (oracle/deriv_ref.py) on its own: exact on
polynomials of the element space, cdtp the transpose of opgrad, the curl of a
rigid rotation, and the minimum-dissipation forcing as minus the vector
Laplacian of a divergence-free polynomial field."""
import numpy as np

from oracle import deriv_ref as dr
from oracle import oracle as orc


def test_oracle_derivatives_exact_on_affine_mesh():
    m = orc.build_mesh(2, 2, 2, 6, amp=0.0, seed=1)
    x, y, z = m.x, m.y, m.z
    u = x * x * y + z ** 3 - x * z
    for d, ex in zip("xyz", (2 * x * y - z, x * x, 3 * z * z - x)):
        assert np.abs(dr.dudxyz(m, u, d) - ex).max() < 1e-11


def test_oracle_cdtp_transpose_and_rotation():
    m = orc.build_mesh(2, 2, 1, 5, amp=0.05, seed=2)
    rng = np.random.default_rng(0)
    u, a = rng.standard_normal(m.n), rng.standard_normal(m.n)
    g = dr.opgrad(m, u)
    for k, d in enumerate("xyz"):
        lhs, rhs = float(a @ g[k]), float(dr.cdtp(m, a, d) @ u)
        assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0)
    c = dr.curl(m, lambda v: orc.gs_op(m, v), -m.y, m.x, np.zeros(m.n))
    assert np.abs(c[0]).max() < 1e-12 and np.abs(c[1]).max() < 1e-12 and np.abs(c[2] - 2).max() < 1e-12


def test_oracle_min_dissipation_is_minus_laplacian():
    # u = (y^2, z^2, x^2) is divergence free with -lap u = (-2, -2, -2)
    m = orc.build_mesh(2, 2, 2, 6, amp=0.0, seed=3)
    u = [m.y ** 2, m.z ** 2, m.x ** 2]
    f = dr.min_dissipation_forcing(m, lambda v: orc.gs_op(m, v), [np.zeros(m.n)] * 3, u, 1.0)
    for c in f:
        assert np.abs(c + 2.0).max() < 1e-9


def test_oracle_adjoint_is_transpose_of_linearised():
    from oracle import dealias_ref as dl
    m = orc.build_mesh(2, 2, 1, 6, amp=0.04, seed=3)
    rng = np.random.default_rng(0)
    u = [rng.standard_normal(m.n) for _ in range(3)]
    a = [rng.standard_normal(m.n) for _ in range(3)]
    ub = [np.sin(m.x) + m.y, np.cos(m.y) * m.z, m.x * m.z]
    zero = [np.zeros(m.n)] * 3
    for mod in (dr, dl):
        L = [-t for t in mod.linear_advection(m, zero, u, ub)]
        A = [-t for t in mod.adjoint_advection(m, zero, a, ub)]
        lhs = sum(float(a[i] @ L[i]) for i in range(3))
        rhs = sum(float(A[i] @ u[i]) for i in range(3))
        assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


def test_oracle_gl_interpolation_exact_on_polynomials():
    from oracle import dealias_ref as dl
    m = orc.build_mesh(2, 1, 1, 8, amp=0.0, seed=1)
    g = dl.GL(m)
    p = m.x ** 3 * m.y - m.z ** 5
    xg, yg, zg = g.to_gl(m.x), g.to_gl(m.y), g.to_gl(m.z)
    assert np.abs(g.to_gl(p) - (xg ** 3 * yg - zg ** 5)).max() < 1e-12
    # GL weights integrate the mass exactly: sum over GL of w3 * jac = volume
    assert abs(g.wg.sum() - 2.0) < 1e-14
