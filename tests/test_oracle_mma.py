"""The MMA oracle (oracle/mma_ref.py) on the reference's own test problems
(tests/mma/mmatest1.f90, mmatest2.f90: Svanberg's toy problems 1 and 2): it
reaches the optimum the reference's test states, and the one scipy's SLSQP
finds."""
import numpy as np
import pytest

from oracle.mma_ref import MMA, toy1, toy2


def run(prob, x, m, a0, a, c, d, xmin, xmax, iters=40):
    opt = MMA(x, m, a0, a, c, d, xmin, xmax)
    f0, df0, f, df = prob(x)
    for it in range(1, iters + 1):
        x = opt.update(it, x, df0, f, df)
        f0, df0, f, df = prob(x)
        opt.kkt(x, df0, f, df)
    return x, opt


def test_toy1_reaches_the_stated_optimum():
    x, opt = run(toy1, np.full(5, 5.0), 1, 1.0, 0.0, 1000.0, 0.0, 0.0, 10.0)
    # optimum written in tests/mma/mmatest1.f90:53 (3 decimals)
    assert np.allclose(x, [6.016, 5.309, 4.494, 3.502, 2.153], atol=6e-4)
    assert opt.residunorm < 1e-6


def test_toy2_matches_an_independent_solver():
    scipy_opt = pytest.importorskip("scipy.optimize")
    x, opt = run(toy2, np.array([4.0, 3.0, 2.0]), 2, 1.0, 0.0, 1000.0, 1.0, 0.0, 5.0)
    r = scipy_opt.minimize(lambda v: np.sum(v ** 2), [4.0, 3.0, 2.0], method="SLSQP", bounds=[(0, 5)] * 3,
                           constraints=[{"type": "ineq", "fun": lambda v: -toy2(v)[2]}], options={"ftol": 1e-14})
    assert np.allclose(x, r.x, atol=1e-6)
    assert opt.residunorm < 1e-6
