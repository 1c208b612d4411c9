"""CPU checks of the learned-guess network's oracle (oracle/mlp_ref.py):
analytic gradients against central finite differences, and the BF16
rounding helper against known bit patterns."""
import numpy as np

from oracle import mlp_ref


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.1415927, 0.0], dtype=np.float32)
    b = mlp_ref.bf16(x)
    assert b[0] == 1.0 and b[3] == -2.5 and b[5] == 0.0
    assert b[1] == 1.0          # exactly half an ulp: ties to even
    assert b[2] == 1.0078125    # above half: rounds up
    assert mlp_ref.bf16_bits(np.array([1.0], np.float32))[0] == 0x3F80
    assert abs(float(b[4]) - 3.140625) < 1e-7


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    F, H, O, E = 20, 8, 12, 5
    p = mlp_ref.init_params(F, H, O, rng)
    X = rng.standard_normal((E, F))
    T = rng.standard_normal((E, O))
    loss, g = mlp_ref.loss_and_grad(p, X, T, F, H, O, emulate_bf16=False)
    h = 1e-6
    idx = rng.choice(p.size, 60, replace=False)
    for i in idx:
        pp = p.copy(); pp[i] += h
        pm = p.copy(); pm[i] -= h
        lp, _ = mlp_ref.loss_and_grad(pp, X, T, F, H, O, emulate_bf16=False)
        lm, _ = mlp_ref.loss_and_grad(pm, X, T, F, H, O, emulate_bf16=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])
