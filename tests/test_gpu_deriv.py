"""Derivative operators (dudxyz, opgrad, cdtp, conv1, curl) and the adjoint
terms built on them (adjoint and linearised advection without dealiasing,
minimum-dissipation forcing) against the numpy restatement in
oracle/deriv_ref.py, plus the identities they obey on the GPU."""
import numpy as np
import pytest
import torch

from oracle import deriv_ref as dr

pytestmark = pytest.mark.gpu

SHAPES = [(3, 2, 2, 8, 0.05), (2, 2, 3, 5, 0.04), (2, 3, 1, 4, 0.0), (2, 1, 2, 10, 0.03), (3, 3, 2, 2, 0.0),
          (5, 3, 1, 3, 0.04)]


def T(a, dev, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device=dev, dtype=dtype)


def H(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def setup(pkg, orc, dev, shape, seed=4):
    ex, ey, ez, lx, amp = shape
    m = orc.build_mesh(ex, ey, ez, lx, amp=amp, seed=seed)
    c = pkg.coef_t.box(ex, ey, ez, lx, amp=amp, seed=seed, device=dev)
    return m, c


def smooth_fields(m, k=3):
    """Continuous fields (functions of the coordinates), so copies of a node agree."""
    x, y, z = m.x, m.y, m.z
    u = np.sin(2 * x + 0.3) * np.cos(y - 0.2 * z) + 0.5 * z * z
    v = np.cos(1.5 * y) * x + np.sin(z + x)
    w = np.exp(0.3 * x) * np.sin(2 * z) - y * y
    return u, v, w


@pytest.mark.parametrize("shape", SHAPES)
def test_derivatives_match_oracle(pkg, orc, dev, shape):
    m, c = setup(pkg, orc, dev, shape)
    rng = np.random.default_rng(5)
    u = rng.standard_normal(m.n)
    vx, vy, vz = (rng.standard_normal(m.n) for _ in range(3))
    ud = T(u, dev)
    out = torch.empty(m.n, dtype=torch.float64, device=dev)
    for d, name in enumerate("xyz"):
        pkg.dudxyz(out, ud, name, c)
        assert rel(H(out), dr.dudxyz(m, u, name)) < 1e-12, ("dudxyz", name)
        pkg.cdtp(out, ud, d, c)
        assert rel(H(out), dr.cdtp(m, u, name)) < 1e-12, ("cdtp", name)
    g = [torch.empty(m.n, dtype=torch.float64, device=dev) for _ in range(3)]
    pkg.opgrad(*g, ud, c)
    for a, b in zip(g, dr.opgrad(m, u)):
        assert rel(H(a), b) < 1e-12
    pkg.conv1(out, ud, T(vx, dev), T(vy, dev), T(vz, dev), c)
    assert rel(H(out), dr.conv1(m, u, vx, vy, vz)) < 1e-12


def test_cdtp_is_transpose_of_opgrad(pkg, orc, dev):
    m, c = setup(pkg, orc, dev, (3, 2, 2, 8, 0.05))
    rng = np.random.default_rng(6)
    u, a = rng.standard_normal(m.n), rng.standard_normal(m.n)
    g = [torch.empty(m.n, dtype=torch.float64, device=dev) for _ in range(3)]
    pkg.opgrad(*g, T(u, dev), c)
    t = torch.empty(m.n, dtype=torch.float64, device=dev)
    for d in range(3):
        pkg.cdtp(t, T(a, dev), d, c)
        lhs = float(np.dot(a, H(g[d])))
        rhs = float(np.dot(H(t), u))
        assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0)


def test_derivatives_exact_on_affine_mesh(pkg, orc, dev):
    # polynomials of degree <= 7 are in the space of lx = 8 on an undeformed box
    m, c = setup(pkg, orc, dev, (2, 3, 2, 8, 0.0))
    x, y, z = m.x, m.y, m.z
    u = x ** 3 * y - 2 * z ** 4 + x * y * z
    exact = (3 * x ** 2 * y + y * z, x ** 3 + x * z, -8 * z ** 3 + x * y)
    out = torch.empty(m.n, dtype=torch.float64, device=dev)
    for d, name in enumerate("xyz"):
        pkg.dudxyz(out, T(u, dev), name, c)
        assert np.abs(H(out) - exact[d]).max() < 1e-10
    # B grad u with the assembled mass matrix
    g = [torch.empty(m.n, dtype=torch.float64, device=dev) for _ in range(3)]
    pkg.opgrad(*g, T(u, dev), c)
    for d in range(3):
        assert np.abs(H(g[d]) - m.B * exact[d]).max() < 1e-12


@pytest.mark.parametrize("shape", SHAPES[:3])
def test_curl_matches_oracle(pkg, orc, dev, shape):
    m, c = setup(pkg, orc, dev, shape)
    u, v, w = smooth_fields(m)
    out = [torch.empty(m.n, dtype=torch.float64, device=dev) for _ in range(3)]
    pkg.curl(*out, T(u, dev), T(v, dev), T(w, dev), c)
    ref = dr.curl(m, lambda a: orc.gs_op(m, a), u, v, w)
    for a, b in zip(out, ref):
        assert rel(H(a), b) < 1e-12
    # a rigid rotation (-y, x, 0) has curl (0, 0, 2) on any mesh
    pkg.curl(*out, T(-m.y, dev), T(m.x, dev), T(np.zeros(m.n), dev), c)
    assert np.abs(H(out[0])).max() < 1e-11 and np.abs(H(out[1])).max() < 1e-11
    assert np.abs(H(out[2]) - 2.0).max() < 1e-11


@pytest.mark.parametrize("shape", SHAPES[:3])
def test_adjoint_and_linear_advection_match_oracle(pkg, orc, dev, shape):
    m, c = setup(pkg, orc, dev, shape)
    rng = np.random.default_rng(8)
    u = [rng.standard_normal(m.n) for _ in range(3)]
    ub = list(smooth_fields(m))
    f0 = [rng.standard_normal(m.n) for _ in range(3)]
    adv = pkg.adv_lin_no_dealias_t(c)
    for kind, ref_fn, call in (("adjoint", dr.adjoint_advection, adv.compute_adjoint),
                               ("linear", dr.linear_advection, adv.compute_linear)):
        f = [T(a, dev) for a in f0]
        call(*[T(a, dev) for a in u], *[T(a, dev) for a in ub], *f)
        ref = ref_fn(m, f0, u, ub)
        for a, b, a0 in zip(f, ref, f0):
            # compare the added term, relative to its own size
            assert rel(H(a) - a0, b - a0) < 1e-11, kind


def test_adjoint_advection_weak_identity(pkg, orc, dev):
    """Tested against a field a, the adjoint term is
    -sum_i <a_i, f_i> = sum_ij <a_i u_j, opgrad_i(Ub_j)> + sum_id <opgrad_d(a_i), u_i Ub_d>,
    since cdtp is the transpose of opgrad."""
    m, c = setup(pkg, orc, dev, (2, 2, 2, 6, 0.04))
    rng = np.random.default_rng(9)
    u = [rng.standard_normal(m.n) for _ in range(3)]
    a = [rng.standard_normal(m.n) for _ in range(3)]
    ub = list(smooth_fields(m))
    zero = [np.zeros(m.n) for _ in range(3)]
    f = [T(z, dev) for z in zero]
    pkg.adv_lin_no_dealias_t(c).compute_adjoint(*[T(x, dev) for x in u], *[T(x, dev) for x in ub], *f)
    # -<a, f> = sum_ij <a_i u_j, opgrad_i(Ub_j)> + sum_id <a_i, cdtp_d(u_i Ub_d)>
    #         = sum_ij <a_i u_j, opgrad_i(Ub_j)> + sum_id <opgrad_d(a_i), u_i Ub_d>
    lhs = -sum(float(np.dot(a[i], H(f[i]))) for i in range(3))
    g_ub = [dr.opgrad(m, ub[j]) for j in range(3)]
    g_a = [dr.opgrad(m, a[i]) for i in range(3)]
    rhs = sum(float(np.dot(a[i] * u[j], g_ub[j][i])) for i in range(3) for j in range(3))
    rhs += sum(float(np.dot(g_a[i][d], u[i] * ub[d])) for i in range(3) for d in range(3))
    assert abs(lhs - rhs) <= 1e-11 * max(abs(rhs), 1.0)


@pytest.mark.parametrize("zone", [False, True])
def test_min_dissipation_forcing_matches_oracle(pkg, orc, dev, zone):
    shape = (3, 2, 2, 6, 0.04)
    m, c = setup(pkg, orc, dev, shape)
    u = list(smooth_fields(m))
    rng = np.random.default_rng(10)
    f0 = [rng.standard_normal(m.n) for _ in range(3)]
    zidx = None
    if zone:
        # nodes with x < 0.5 (1-based, unique)
        zidx = (np.nonzero(m.x < 0.5)[0] + 1).astype(np.int32)
    f = [T(a, dev) for a in f0]
    st = pkg.adjoint_minimum_dissipation_source_term_t(f, *[T(a, dev) for a in u], c, obj_scale=0.7,
                                                       mask=None if zidx is None else T(zidx, dev, torch.int32))
    st.compute()
    ref = dr.min_dissipation_forcing(m, lambda a: orc.gs_op(m, a), f0, u, 0.7, zone=zidx)
    for a, b, a0 in zip(f, ref, f0):
        assert rel(H(a) - a0, b - a0) < 1e-11
    if zone:
        out = np.ones(m.n, dtype=bool)
        out[zidx - 1] = False
        for a, a0 in zip(f, f0):
            assert np.array_equal(H(a)[out], a0[out])


def test_metrics_required_and_bad_direction(pkg, orc, dev):
    import ctypes as C
    m, c = setup(pkg, orc, dev, (2, 1, 1, 4, 0.0))
    out = torch.empty(m.n, dtype=torch.float64, device=dev)
    u = torch.zeros(m.n, dtype=torch.float64, device=dev)
    lib = pkg.lib()
    po, pu = C.c_void_p(out.data_ptr()), C.c_void_p(u.data_ptr())
    assert lib.ntg_dudxyz(c.handle, po, pu, 0) == 1  # before ntg_metrics_set
    c.metrics()
    assert lib.ntg_dudxyz(c.handle, po, pu, 3) == 1  # no fourth direction
    assert lib.ntg_dudxyz(c.handle, po, pu, 2) == 0
