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


@pytest.mark.parametrize("case", ["toy1", "toy2", "large"])
def test_compiled_mma_follows_the_restatement(case):
    """oracle/mma_oracle.c (the timed CPU baseline of the GPU MMA) against
    the numpy restatement, iterate for iterate."""
    from oracle.mma_c import MMAC
    if case == "toy1":
        prob, x0, args = toy1, np.full(5, 5.0), (1, 1.0, 0.0, 1000.0, 0.0, 0.0, 10.0)
    elif case == "toy2":
        prob, x0, args = toy2, np.array([4.0, 3.0, 2.0]), (2, 1.0, 0.0, 1000.0, 1.0, 0.0, 5.0)
    else:
        n = 50_000
        rng = np.random.default_rng(3)
        w, v2 = rng.uniform(0.5, 2.0, n), rng.uniform(0.0, 1.0, n)

        def prob(x):
            return (None, -w / x ** 2 / n, np.array([x.mean() - 0.4, (v2 * x).mean() - 0.25]),
                    np.stack([np.full(n, 1.0 / n), v2 / n]))
        x0, args = np.full(n, 0.5), (2, 1.0, 0.0, 1000.0, 1.0, 1e-3, 1.0)
    ref, cc = MMA(x0, *args), MMAC(x0, *args)
    xr, xc = x0.copy(), x0.copy()
    for it in range(1, 11):
        _, df0, f, df = prob(xr)
        xr = ref.update(it, xr, df0, f, df)
        _, df0, f, df = prob(xc)
        xc = cc.update(it, xc, df0, f, df)
        assert np.abs(xc - xr).max() <= 1e-9 * np.abs(xr).max(), it
