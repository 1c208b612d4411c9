"""The MMA optimiser on the GPU against the numpy restatement of the
reference's algorithm (oracle/mma_ref.py): the reference's two test problems
iterate for iterate, and a large separable problem with two constraints."""
import numpy as np
import pytest
import torch

from oracle.mma_ref import MMA, toy1, toy2

pytestmark = pytest.mark.gpu


def T(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(dev)


def dfdx_dev(df, dev):
    # the reference's dfdx(m, n) layout: entry (i, j) at i + m j
    return T(np.asarray(df).T.ravel(), dev)


@pytest.mark.parametrize("case", ["toy1", "toy2"])
def test_reference_test_problems_iterate_like_the_oracle(pkg, dev, case):
    if case == "toy1":
        prob, x0, m, a0, a, c, d, lo, hi = toy1, np.full(5, 5.0), 1, 1.0, 0.0, 1000.0, 0.0, 0.0, 10.0
    else:
        prob, x0, m, a0, a, c, d, lo, hi = toy2, np.array([4.0, 3.0, 2.0]), 2, 1.0, 0.0, 1000.0, 1.0, 0.0, 5.0
    ref = MMA(x0, m, a0, a, c, d, lo, hi)
    xd = T(x0, dev)
    opt = pkg.mma_t(xd, x0.size, m, a0, a, c, d, lo, hi)
    xr = x0.copy()
    f0, df0, f, df = prob(xr)
    for it in range(1, 31):
        _, gd0, gf, gdf = prob(xd.cpu().numpy())
        opt.update(it, xd, T(gd0, dev), gf, dfdx_dev(gdf, dev))
        xr = ref.update(it, xr, df0, f, df)
        f0, df0, f, df = prob(xr)
        ref.kkt(xr, df0, f, df)
        xg = xd.cpu().numpy()
        assert np.allclose(xg, xr, rtol=1e-9, atol=1e-12), (it, xg, xr)
        g0, gd0, gf, gdf = prob(xg)
        mx, nr = opt.KKT(xd, T(gd0, dev), gf, dfdx_dev(gdf, dev))
        assert abs(nr - ref.residunorm) <= 1e-6 * max(ref.residunorm, 1e-12) + 1e-12
    assert opt.newton_steps > 0


def test_large_separable_problem_matches_oracle(pkg, dev):
    """Compliance-like objective sum w_j / x_j with a volume constraint and a
    weighted second constraint, n = 200,000."""
    n, m = 200_000, 2
    rng = np.random.default_rng(3)
    w = rng.uniform(0.5, 2.0, n)
    v2 = rng.uniform(0.0, 1.0, n)

    def prob(x):
        df0 = -w / x ** 2 / n
        f = np.array([x.mean() - 0.4, (v2 * x).mean() - 0.25])
        df = np.stack([np.full(n, 1.0 / n), v2 / n])
        return None, df0, f, df

    x0 = np.full(n, 0.5)
    ref = MMA(x0, m, 1.0, 0.0, 1000.0, 1.0, 1e-3, 1.0)
    xd = T(x0, dev)
    opt = pkg.mma_t(xd, n, m, 1.0, 0.0, 1000.0, 1.0, 1e-3, 1.0)
    xr = x0.copy()
    for it in range(1, 6):
        _, df0, f, df = prob(xr)
        xr = ref.update(it, xr, df0, f, df)
        _, gd0, gf, gdf = prob(xd.cpu().numpy())
        opt.update(it, xd, T(gd0, dev), gf, dfdx_dev(gdf, dev))
        xg = xd.cpu().numpy()
        assert np.abs(xg - xr).max() <= 1e-8 * np.abs(xr).max(), it
    _, df0, f, df = prob(xr)
    rm, rn = ref.kkt(xr, df0, f, df)
    mx, nr = opt.KKT(xd, T(df0, dev), f, dfdx_dev(df, dev))
    assert abs(nr - rn) <= 1e-6 * rn


def test_mma_rejects_bad_sizes(pkg, dev):
    x = torch.full((4,), 0.5, dtype=torch.float64, device=dev)
    with pytest.raises(pkg.NtgError):
        pkg.mma_t(x, 4, 5, 1.0, 0.0, 1000.0, 1.0, 0.0, 1.0)

