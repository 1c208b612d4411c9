"""Dealiased (over-integrated) adjoint and linearised advection against the
numpy restatement in oracle/dealias_ref.py: the GLL <-> GL maps, both terms,
and the discrete transpose identity between them."""
import numpy as np
import pytest
import torch

from oracle import dealias_ref as dl

pytestmark = pytest.mark.gpu

SHAPES = [(2, 2, 2, 8, 0.05), (3, 2, 1, 6, 0.04), (2, 1, 2, 5, 0.0), (2, 2, 1, 7, 0.03), (3, 1, 1, 4, 0.05)]


def T(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device=dev, dtype=torch.float64)


def H(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def setup(pkg, orc, dev, shape, seed=3):
    ex, ey, ez, lx, amp = shape
    m = orc.build_mesh(ex, ey, ez, lx, amp=amp, seed=seed)
    c = pkg.coef_t.box(ex, ey, ez, lx, amp=amp, seed=seed, device=dev)
    return m, c


def base_flow(m):
    x, y, z = m.x, m.y, m.z
    return [np.sin(2 * x) * np.cos(y) + z, np.cos(1.5 * y) * x + np.sin(z), np.exp(0.3 * x) * np.sin(2 * z) - y * y]


@pytest.mark.parametrize("shape", SHAPES)
def test_maps_match_oracle(pkg, orc, dev, shape):
    m, c = setup(pkg, orc, dev, shape)
    adv = pkg.adv_lin_dealias_t(c)
    g = dl.GL(m)
    assert adv.lxd == g.lxd and adv.n_gl == m.nelv * g.lxd ** 3
    rng = np.random.default_rng(1)
    u = rng.standard_normal(m.n)
    v = rng.standard_normal(adv.n_gl)
    out_gl = torch.empty(adv.n_gl, dtype=torch.float64, device=dev)
    adv.map_to_gl(out_gl, T(u, dev))
    assert rel(H(out_gl), g.to_gl(u)) < 1e-13
    out = torch.empty(m.n, dtype=torch.float64, device=dev)
    adv.map_to_gll(out, T(v, dev))
    assert rel(H(out), g.to_gll(v)) < 1e-13


@pytest.mark.parametrize("shape", SHAPES)
def test_dealiased_terms_match_oracle(pkg, orc, dev, shape):
    m, c = setup(pkg, orc, dev, shape)
    rng = np.random.default_rng(2)
    u = [rng.standard_normal(m.n) for _ in range(3)]
    ub = base_flow(m)
    f0 = [rng.standard_normal(m.n) for _ in range(3)]
    adv = pkg.adv_lin_dealias_t(c)
    for kind, ref_fn, call in (("adjoint", dl.adjoint_advection, adv.compute_adjoint),
                               ("linear", dl.linear_advection, adv.compute_linear)):
        f = [T(a, dev) for a in f0]
        call(*[T(a, dev) for a in u], *[T(a, dev) for a in ub], *f)
        ref = ref_fn(m, f0, u, ub)
        for a, b, a0 in zip(f, ref, f0):
            assert rel(H(a) - a0, b - a0) < 1e-11, kind


@pytest.mark.parametrize("dealias", [False, True])
def test_adjoint_is_transpose_of_linearised(pkg, orc, dev, dealias):
    """sum_i <a_i, L_i(u)> = sum_i <A_i(a), u_i> for the added terms L
    (linearised) and A (adjoint) on the same base flow: the adjoint term is
    the exact discrete transpose, with or without over-integration."""
    m, c = setup(pkg, orc, dev, (2, 2, 2, 6, 0.04), seed=9)
    rng = np.random.default_rng(4)
    u = [rng.standard_normal(m.n) for _ in range(3)]
    a = [rng.standard_normal(m.n) for _ in range(3)]
    ub = [T(x, dev) for x in base_flow(m)]
    adv = pkg.adv_lin_dealias_t(c) if dealias else pkg.adv_lin_no_dealias_t(c)
    L = [torch.zeros(m.n, dtype=torch.float64, device=dev) for _ in range(3)]
    A = [torch.zeros(m.n, dtype=torch.float64, device=dev) for _ in range(3)]
    adv.compute_linear(*[T(x, dev) for x in u], *ub, *L)
    adv.compute_adjoint(*[T(x, dev) for x in a], *ub, *A)
    lhs = sum(float(np.dot(a[i], H(L[i]))) for i in range(3))
    rhs = sum(float(np.dot(H(A[i]), u[i])) for i in range(3))
    assert abs(lhs - rhs) <= 1e-11 * max(abs(lhs), 1.0)


def test_unsupported_order_is_refused(pkg, orc, dev):
    m, c = setup(pkg, orc, dev, (2, 1, 1, 8, 0.0))
    with pytest.raises(pkg.NtgError):
        pkg.adv_lin_dealias_t(c, lxd=11)
