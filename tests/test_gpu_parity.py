"""GPU parity of the sm_103a library against the oracle, through the C ABI.

Bars: index maps and integer outputs bit-exact; FP64 Ax / Jacobi / geometry
within 1e-12 relative (max-abs error over max-abs value); fixed-iteration
CG within 1e-11; converged solves to the same 1e-10 relative residual
with iteration counts within 2 and solutions within 1e-8 relative (the
residual tolerance bounds how far two correct solutions may differ).
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TOL64 = 1e-12


def relerr(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else a
    b = b.detach().cpu().numpy() if isinstance(b, torch.Tensor) else b
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def T(a, dev, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device=dev, dtype=dtype)


def make(pkg, orc, dev, ex, ey, ez, lx, amp=0.0, seed=0, lo=(0, 0, 0), hi=(1, 1, 1)):
    m = orc.build_mesh(ex, ey, ez, lx, lo=lo, hi=hi, amp=amp, seed=seed)
    c = pkg.coef_t.box(ex, ey, ez, lx, lo=lo, hi=hi, amp=amp, seed=seed, device=dev)
    return m, c


@pytest.mark.parametrize("shape", [(2, 2, 2, 8, 0.05), (3, 2, 4, 5, 0.05), (4, 4, 4, 8, 0.0), (2, 3, 2, 3, 0.05)])
def test_mesh_maps_geometry(pkg, orc, dev, shape):
    ex, ey, ez, lx, amp = shape
    m, c = make(pkg, orc, dev, ex, ey, ez, lx, amp, seed=5)
    # global ids bit-exact, coordinates to rounding (sin on the device)
    assert np.array_equal(c.gid.cpu().numpy(), m.gid)
    for a, b in ((c.x, m.x), (c.y, m.y), (c.z, m.z)):
        assert relerr(a, b) < 1e-15
    assert c.nu == m.nu
    perm, offs = c.gs_maps()
    assert np.array_equal(perm.cpu().numpy(), m.perm)
    assert np.array_equal(offs.cpu().numpy(), m.offs)
    g = c.geometry()
    assert np.array_equal(g["mult"].cpu().numpy(), m.mult)
    for k in ("g11", "g12", "g13", "g22", "g23", "g33"):
        scale = np.abs(m.G["g11"]).max()
        assert np.abs(g[k].cpu().numpy() - m.G[k]).max() / scale < TOL64, k
    assert relerr(g["B"], m.B) < TOL64


def test_geometry_from_identical_coordinates(pkg, orc, dev):
    m = orc.build_mesh(3, 3, 2, 8, amp=0.05, seed=17)
    c = pkg.coef_t(m.nelv, 8, T(m.x, dev), T(m.y, dev), T(m.z, dev), T(m.gid, dev, torch.int64))
    g = c.geometry()
    for k in ("g11", "g12", "g13", "g22", "g23", "g33"):
        assert np.abs(g[k].cpu().numpy() - m.G[k]).max() / np.abs(m.G["g11"]).max() < 1e-13, k


@pytest.mark.parametrize("case", ["poisson_deformed", "helm_chi", "h1_array", "lx5", "lx3"])
def test_ax_helm_fp64(pkg, orc, dev, case):
    lx = {"lx5": 5, "lx3": 3}.get(case, 8)
    m, c = make(pkg, orc, dev, 3, 2, 2, lx, amp=0.05, seed=3)
    rng = np.random.default_rng(11)
    u = rng.standard_normal(m.n)
    h1 = h2 = None
    h1c = 1.0
    if case == "helm_chi":
        rho = orc.field_uniform(m, 1, orc.STREAM_RHO, 0.0, 1.0)
        h2 = orc.ramp_forward(1.0 - rho, 0.0, 1e4, 8.0, 0)
    if case == "h1_array":
        h1 = rng.uniform(0.5, 2.0, m.n)
        h2 = rng.uniform(0.0, 3.0, m.n)
    c.set_coefs(h1=None if h1 is None else T(h1, dev), h1c=h1c, h2=None if h2 is None else T(h2, dev),
                ifh2=h2 is not None)
    w_ref = orc.ax_helm(m, u, h1=h1, h1c=h1c, h2=h2)
    w = torch.empty(m.n, dtype=torch.float64, device=dev)
    pkg.ax_helm_t().compute(w, T(u, dev), c)
    torch.cuda.synchronize()
    assert relerr(w, w_ref) < TOL64


def test_ax_helm_fp32(pkg, orc, dev):
    m, c = make(pkg, orc, dev, 4, 3, 2, 8, amp=0.05, seed=3)
    rng = np.random.default_rng(12)
    u = rng.standard_normal(m.n)
    rho = orc.field_uniform(m, 2, orc.STREAM_RHO, 0.0, 1.0)
    h2 = orc.ramp_forward(1.0 - rho, 0.0, 1e4, 8.0, 0)
    c.set_coefs(h1c=0.01, h2=T(h2, dev), ifh2=True)
    w_ref = orc.ax_helm(m, u, h1c=0.01, h2=h2)
    w32_ref = orc.ax_helm_f32(m, u, h1c=0.01, hB=h2 * m.B)
    w = torch.empty(m.n, dtype=torch.float32, device=dev)
    pkg.ax_helm_t().compute(w, T(u, dev, torch.float32), c)
    torch.cuda.synchronize()
    # FP32 tolerance: a few units of float epsilon times the operator scale
    assert relerr(w.double(), w_ref) < 2e-5
    assert relerr(w.double(), w32_ref.astype(np.float64)) < 2e-5


@pytest.mark.parametrize("op", [1, 2, 3, 4])
@pytest.mark.parametrize("shape", [(3, 3, 2, 6), (5, 1, 3, 3), (9, 7, 5, 8)])
@pytest.mark.parametrize("path", [1, 0])
def test_gs_ops_bitexact(pkg, orc, dev, op, shape, path):
    ex, ey, ez, lx = shape
    m, c = make(pkg, orc, dev, ex, ey, ez, lx, amp=0.05, seed=8)
    c.set_gs_path(path)
    rng = np.random.default_rng(op)
    u = rng.uniform(0.5, 1.5, m.n)
    ref = orc.gs_op(m, u, op)
    for dt in (torch.float64, torch.float32):
        v = T(u, dev, dt)
        pkg.gs_t(c).op(v, op)
        torch.cuda.synchronize()
        if dt == torch.float64:
            assert np.array_equal(v.cpu().numpy(), ref)
        else:
            ref32 = orc.gs_op(m, u.astype(np.float32).astype(np.float64), op)
            assert np.allclose(v.cpu().numpy(), ref32, rtol=1e-6)


def test_jacobi_and_mask(pkg, orc, dev):
    m, c = make(pkg, orc, dev, 3, 2, 3, 8, amp=0.05, seed=4)
    mask = orc.mask_face_xmax(3, 2, 3, 8)
    gmask = pkg.mask_face_xmax(3, 2, 3, 8, device=dev)
    assert np.array_equal(gmask.cpu().numpy(), mask)
    c.set_mask(gmask, base=1)
    rng = np.random.default_rng(5)
    h1 = rng.uniform(0.5, 2.0, m.n)
    h2 = rng.uniform(0.0, 3.0, m.n)
    c.set_coefs(h1=T(h1, dev), h2=T(h2, dev), ifh2=True)
    ref = orc.jacobi(m, h1=h1, h2=h2, mask=mask)
    pc = pkg.jacobi_t(c)
    pc.update()
    assert relerr(pc.dinv(), ref) < TOL64


def c1_like(pkg, orc, dev, E=4, lx=8):
    """The plain-method case at reduced size: affine unit cube, h1 = 1,
    h2 = chi(rho), rho ~ U[0,1] per node, zero-mean uniform RHS."""
    m, c = make(pkg, orc, dev, E, E, E, lx)
    rho = orc.field_uniform(m, 1, orc.STREAM_RHO, 0.0, 1.0)
    chi = orc.ramp_forward(1.0 - rho, 0.0, 1e4, 8.0, 0)
    b = orc.field_uniform(m, 1, orc.STREAM_RHS, -1.0, 1.0)
    b = b - np.sum(b * m.mult) / m.nu
    c.set_coefs(h1c=1.0, h2=T(chi, dev), ifh2=True)
    return m, c, chi, b


def test_cg_fixed_iterations(pkg, orc, dev):
    m, c, chi, b = c1_like(pkg, orc, dev, E=3)
    x_ref, it, _, _ = orc.cg(m, b, h2=chi, fixed_iters=20)
    ksp = pkg.krylov_solver_factory(c, "cg", 20, 0.0)
    x = torch.zeros(m.n, dtype=torch.float64, device=dev)
    mon = ksp.solve(x, T(b, dev))
    torch.cuda.synchronize()
    assert mon.iter == 20 and mon.status == pkg.NTG_MAXITER
    assert relerr(x, x_ref) < 1e-11


def test_cg_converged_c1_like(pkg, orc, dev):
    m, c, chi, b = c1_like(pkg, orc, dev, E=4)
    x_ref, it_ref, r0, r1 = orc.cg(m, b, h2=chi, rtol=1e-10)
    ksp = pkg.krylov_solver_factory(c, "cg", 800, 1e-10)
    x = torch.zeros(m.n, dtype=torch.float64, device=dev)
    mon = ksp.solve(x, T(b, dev))
    torch.cuda.synchronize()
    assert mon.status == pkg.NTG_OK
    assert abs(mon.iter - it_ref) <= 2
    assert abs(mon.res_start - r0) <= 1e-12 * r0
    assert mon.res_final <= 1e-10 * mon.rhs_norm
    xn = x.cpu().numpy()
    assert np.linalg.norm(xn - x_ref) <= 1e-8 * np.linalg.norm(x_ref)
    # the true residual, evaluated by the oracle
    r = b - orc.op_apply(m, xn, h2=chi)
    assert np.sqrt(orc.glsc3(r, r, m.mult)) <= 1.5e-10 * np.sqrt(orc.glsc3(b, b, m.mult))


def poisson_deformed(pkg, orc, dev, E=(4, 3, 3), lx=8, nmodes=16):
    ex, ey, ez = E
    m, c = make(pkg, orc, dev, ex, ey, ez, lx, amp=0.05, seed=21)
    mask = orc.mask_face_xmax(ex, ey, ez, lx)
    c.set_mask(T(mask, dev, torch.int32), base=1)
    c.set_coefs(h1c=1.0, ifh2=False)
    k, a, ph = orc.fourier_params(21, nmodes)
    f = orc.assemble_rhs(m, orc.field_fourier(m, k, a, ph), mask)
    return m, c, mask, f


def test_cg_converged_poisson_dirichlet(pkg, orc, dev):
    m, c, mask, f = poisson_deformed(pkg, orc, dev)
    x_ref, it_ref, r0, r1 = orc.cg(m, f, mask=mask, rtol=1e-10)
    ksp = pkg.krylov_solver_factory(c, "cg", 1000, 1e-10)
    x = torch.zeros(m.n, dtype=torch.float64, device=dev)
    mon = ksp.solve(x, T(f, dev))
    torch.cuda.synchronize()
    assert mon.status == pkg.NTG_OK and abs(mon.iter - it_ref) <= 2
    xn = x.cpu().numpy()
    assert np.all(xn[mask - 1] == 0.0)
    assert np.linalg.norm(xn - x_ref) <= 1e-8 * np.linalg.norm(x_ref)


def test_mixed_precision_solver(pkg, orc, dev):
    m, c, mask, f = poisson_deformed(pkg, orc, dev)
    # Brinkman Helmholtz: h1 = 1/Re, h2 = chi(blobs)
    rho = orc.field_blobs(m, 5, 12, 0.1)
    chi = orc.ramp_forward(1.0 - rho, 0.0, 1e4, 8.0, 0)
    c.set_coefs(h1c=0.01, h2=T(chi, dev), ifh2=True)
    x_ref, it_ref, _, _ = orc.cg(m, f, h1c=0.01, h2=chi, mask=mask, rtol=1e-12)
    ksp = pkg.krylov_solver_factory(c, "fcg_mixed", 100, 1e-10)
    ksp.set_inner(1e-4, 500)
    x = torch.zeros(m.n, dtype=torch.float64, device=dev)
    mon = ksp.solve(x, T(f, dev))
    torch.cuda.synchronize()
    assert mon.status == pkg.NTG_OK, mon
    xn = x.cpu().numpy()
    r = f - orc.op_apply(m, xn, h1c=0.01, h2=chi, mask=mask)
    assert np.sqrt(orc.glsc3(r, r, m.mult)) <= 1.5e-10 * np.sqrt(orc.glsc3(f, f, m.mult))
    # error against the FP64 oracle solution (solved to 1e-12)
    assert np.linalg.norm(xn - x_ref) <= 1e-7 * np.linalg.norm(x_ref)
    assert mon.inner_iter > 0 and mon.iter <= 10


def test_projection_sequence(pkg, orc, dev):
    m, c, mask, f0 = poisson_deformed(pkg, orc, dev, E=(3, 3, 2))
    rng = np.random.default_rng(7)
    proj = pkg.projection_t(c, 4)
    P = orc.Projection(m.n, 4)
    fp = orc.assemble_rhs(m, rng.uniform(-1, 1, m.n), mask)
    iters = []
    for k in range(7):
        f = f0 + 0.02 * k * fp
        # GPU: pre -> solve (zero guess) -> post
        b = T(f, dev)
        # absolute tolerance: 1e-10 of the original right-hand side
        fn = np.sqrt(orc.glsc3(f, f, m.mult))
        ksp = pkg.krylov_solver_factory(c, "cg", 1000, 0.0, 1e-10 * fn)
        proj.pre_solving(b)
        x = torch.zeros(m.n, dtype=torch.float64, device=dev)
        mon = ksp.solve(x, b)
        proj.post_solving(x)
        torch.cuda.synchronize()
        iters.append(mon.iter)
        # oracle
        bo = f.copy()
        P.pre(bo, m.mult)
        dx, _, _, _ = orc.cg(m, bo, mask=mask, rtol=0.0, abstol=1e-10 * fn)
        xo = P.post(dx, orc.op_apply(m, dx, mask=mask), m.mult)
        assert np.linalg.norm(x.cpu().numpy() - xo) <= 1e-7 * np.linalg.norm(xo)
        assert proj.size == P.m
    assert iters[-1] < iters[0]


def test_projection_activ_step(pkg, orc, dev):
    """projection_t(L, activ_step): steps up to activ_step run from a zero
    guess and leave the basis empty; later steps project."""
    m, c, mask, f0 = poisson_deformed(pkg, orc, dev, E=(3, 3, 2))
    rng = np.random.default_rng(9)
    fp = orc.assemble_rhs(m, rng.uniform(-1, 1, m.n), mask)
    proj = pkg.projection_t(c, 4, activ_step=2)
    plain = []
    for tstep in range(1, 6):
        f = f0 + 0.02 * tstep * fp
        fn = np.sqrt(orc.glsc3(f, f, m.mult))
        b = T(f, dev)
        proj.pre_solving(b, tstep)
        ksp = pkg.krylov_solver_factory(c, "cg", 1000, 0.0, 1e-10 * fn)
        x = torch.zeros(m.n, dtype=torch.float64, device=dev)
        mon = ksp.solve(x, b)
        proj.post_solving(x, tstep)
        torch.cuda.synchronize()
        ref = pkg.krylov_solver_factory(c, "cg", 1000, 0.0, 1e-10 * fn)
        x0 = torch.zeros_like(x)
        mon0 = ref.solve(x0, T(f, dev))
        if tstep <= 2:
            assert proj.size == 0 and mon.iter == mon0.iter
        else:
            # the first active step still starts from an empty basis
            assert proj.size == tstep - 2
            assert mon.iter == mon0.iter if tstep == 3 else mon.iter < mon0.iter
        xn = x.cpu().numpy()
        r = f - orc.op_apply(m, xn, mask=mask)
        assert np.sqrt(orc.glsc3(r, r, m.mult)) <= 1.5e-10 * fn


def test_masked_kernels_bitexact(pkg, orc, dev):
    rng = np.random.default_rng(9)
    n = 5000
    a, b, cc = (rng.uniform(1, 2, n) for _ in range(3))
    mask = np.sort(rng.choice(n, 700, replace=False)).astype(np.int32) + 1
    gm = T(mask, dev, torch.int32)
    for name, args, gargs in (
            ("cadd_mask", (2.5,), (2.5,)), ("invcol1_mask", (), ()), ("cmult_mask", (3.0,), (3.0,)),
            ("col2_mask", (b,), (T(b, dev),)), ("col3_mask", (b, cc), (T(b, dev), T(cc, dev))),
            ("sub3_mask", (b, cc), (T(b, dev), T(cc, dev)))):
        ref = orc.masked(name, a, *args, mask, len(mask))
        ga = T(a, dev)
        getattr(pkg, name)(ga, *gargs, gm)
        torch.cuda.synchronize()
        assert np.array_equal(ga.cpu().numpy(), ref), name
    d = pkg.glsc2_mask(T(a, dev), T(b, dev), gm)
    assert abs(d - orc.glsc2_mask(a, b, mask)) <= 1e-13 * abs(d)


def test_coefficient_kernels(pkg, orc, dev):
    rng = np.random.default_rng(10)
    n = 10007
    x = rng.uniform(0, 1, n)
    for up in (0, 1):
        r = pkg.RAMP_mapping_t(0.0, 1e4, 8.0, bool(up))
        out = torch.empty(n, dtype=torch.float64, device=dev)
        r.apply_forward(out, T(x, dev))
        assert relerr(out, orc.ramp_forward(x, 0.0, 1e4, 8.0, up)) < 1e-15
        g = rng.standard_normal(n)
        din = torch.empty_like(out)
        r.apply_backward(din, T(g, dev), T(x, dev))
        assert relerr(din, orc.ramp_backward(x, g, 0.0, 1e4, 8.0, up)) < 1e-15
    f = [rng.standard_normal(n) for _ in range(7)]
    gf = [T(a, dev) for a in f]
    pkg.simple_brinkman_source_term_t(*gf).compute()
    ref = orc.brinkman(*f)
    for a, b in zip(gf[:3], ref):
        # f - u*chi: the device fuses it into one FMA, so allow one rounding
        assert np.abs(a.cpu().numpy() - b).max() <= 2.3e-16 * np.abs(b).max() * 4
    k = torch.empty(n, dtype=torch.float64, device=dev)
    pkg.permeability(k, T(x, dev), 1e5, 0.0, 1.0)
    assert relerr(k, orc.permeability(x, 1e5, 0.0, 1.0)) < 1e-15
    s = torch.empty(n, dtype=torch.float64, device=dev)
    pkg.sens_min_dissipation(s, *[T(a, dev) for a in f[:6]], True, 0.5)
    assert relerr(s, orc.sens_min_dissipation(*f[:6], True, 0.5)) < 1e-14


def test_pde_filter(pkg, orc, dev):
    m, c = make(pkg, orc, dev, 3, 3, 3, 8, amp=0.05, seed=2)
    rho = orc.field_uniform(m, 3, orc.STREAM_RHO, 0.0, 1.0)
    filt = pkg.PDE_filter_t(c, r=0.05, abstol=1e-12, max_iter=500)
    out = torch.empty(m.n, dtype=torch.float64, device=dev)
    mon = filt.apply_forward(out, T(rho, dev))
    torch.cuda.synchronize()
    assert mon.status == pkg.NTG_OK
    rhs = orc.gs_op(m, rho * m.B)
    ref, _, _, _ = orc.cg(m, rhs, x0=rho, h1c=0.05 ** 2, h2=np.ones(m.n), rtol=0.0, abstol=1e-12, max_iter=500)
    assert relerr(out, ref) < 1e-9
    # a filtered constant stays constant
    filt.apply_forward(out, torch.full((m.n,), 0.3, dtype=torch.float64, device=dev))
    torch.cuda.synchronize()
    assert np.abs(out.cpu().numpy() - 0.3).max() < 1e-9


def test_determinism(pkg, orc, dev):
    m, c, chi, b = c1_like(pkg, orc, dev, E=3)
    ksp = pkg.krylov_solver_factory(c, "cg", 800, 1e-10)
    xs = []
    for _ in range(2):
        x = torch.zeros(m.n, dtype=torch.float64, device=dev)
        ksp.solve(x, T(b, dev))
        torch.cuda.synchronize()
        xs.append(x.cpu().numpy())
    assert np.array_equal(xs[0], xs[1])


def test_fault_statuses_on_host_inputs(pkg, orc, dev):
    """Failure detection without a GPU fault: a NaN right-hand side and an
    indefinite operator end the solve with a status, never a hang."""
    m, c, chi, b = c1_like(pkg, orc, dev, E=2)
    ksp = pkg.krylov_solver_factory(c, "cg", 50, 1e-10)
    bad = b.copy()
    bad[7] = np.nan
    x = torch.zeros(m.n, dtype=torch.float64, device=dev)
    mon = ksp.solve(x, T(bad, dev))
    assert mon.status == pkg.NTG_NONFINITE
    c.set_coefs(h1c=-1.0, h2=T(chi, dev), ifh2=True)  # indefinite: negative h1
    x.zero_()
    mon = ksp.solve(x, T(b, dev))
    assert mon.status in (pkg.NTG_BREAKDOWN, pkg.NTG_MAXITER, pkg.NTG_NONFINITE)
    assert mon.iter <= 50


def test_synthetic_generators_match_oracle(pkg, orc, dev):
    m, c = make(pkg, orc, dev, 3, 2, 2, 8, amp=0.05, seed=1)
    assert relerr(c.field_uniform(4, 2, -1.0, 1.0), orc.field_uniform(m, 4, 2, -1.0, 1.0)) < 1e-15
    k, a, ph = orc.fourier_params(2, 16)
    assert relerr(c.field_fourier(16, 2), orc.field_fourier(m, k, a, ph)) < 1e-13
    assert relerr(c.field_blobs(3, 12, 0.1), orc.field_blobs(m, 3, 12, 0.1)) < 1e-13
    mask = orc.mask_face_xmax(3, 2, 2, 8)
    c.set_mask(T(mask, dev, torch.int32), base=1)
    f = orc.field_fourier(m, k, a, ph)
    assert relerr(c.rhs_assemble(T(f, dev)), orc.assemble_rhs(m, f, mask)) < 1e-14


@pytest.mark.parametrize("coefs", ["poisson", "h2", "h1_h2"])
def test_ax_fp32_bulk_copy_pipeline(pkg, orc, dev, coefs):
    """The bulk-copy (TMA) FP32 kernel against the generic FP32 kernel and the
    oracle, on 27 elements (six full groups of four and a partial one)."""
    m, c = make(pkg, orc, dev, 3, 3, 3, 8, amp=0.05, seed=6)
    rng = np.random.default_rng(13)
    u = rng.standard_normal(m.n)
    h1 = rng.uniform(0.5, 2.0, m.n) if coefs == "h1_h2" else None
    h2 = rng.uniform(0.0, 3.0, m.n) if coefs != "poisson" else None
    c.set_coefs(h1=None if h1 is None else T(h1, dev), h1c=1.0, h2=None if h2 is None else T(h2, dev),
                ifh2=h2 is not None)
    ref = orc.ax_helm(m, u, h1=h1, h2=h2)
    out = {}
    for path in (1, 0):
        c.set_ax_path(path)
        w = torch.full((m.n,), float("nan"), dtype=torch.float32, device=dev)
        pkg.ax_helm_t().compute(w, T(u, dev, torch.float32), c)
        torch.cuda.synchronize()
        out[path] = w.double()
    assert not c.check_error()
    assert relerr(out[1], ref) < 2e-5
    assert relerr(out[1], out[0]) < 1e-5


def test_cg_mixed_reliable_updates(pkg, orc, dev):
    m, c, mask, f = poisson_deformed(pkg, orc, dev)
    x_ref, it_ref, _, _ = orc.cg(m, f, mask=mask, rtol=1e-12)
    _, it64, _, _ = orc.cg(m, f, mask=mask, rtol=1e-10)
    ksp = pkg.krylov_solver_factory(c, "cg_mixed", 5000, 1e-10)
    x = torch.zeros(m.n, dtype=torch.float64, device=dev)
    mon = ksp.solve(x, T(f, dev))
    torch.cuda.synchronize()
    assert mon.status == pkg.NTG_OK, mon
    xn = x.cpu().numpy()
    r = f - orc.op_apply(m, xn, mask=mask)
    assert np.sqrt(orc.glsc3(r, r, m.mult)) <= 1.5e-10 * np.sqrt(orc.glsc3(f, f, m.mult))
    assert np.linalg.norm(xn - x_ref) <= 1e-7 * np.linalg.norm(x_ref)
    # one Krylov space: close to the FP64 iteration count
    assert mon.iter <= 1.3 * it64 + 10, (mon.iter, it64)
    assert mon.fp64_ax >= 1
    # with a non-zero initial guess (the solution itself): converges at once
    mon2 = ksp.solve(x, T(f, dev))
    assert mon2.status == pkg.NTG_OK and mon2.iter <= 2
