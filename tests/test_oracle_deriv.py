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
