"""Parity at the benchmark configurations' own sizes, against the oracle,
through the C ABI.

C1: 8^3 affine unit cube, N = 7 (262,144 local DOFs), h1 = 1, h2 = chi(rho)
    with rho ~ U[0,1] per node, RAMP q = 8, chimax = 1e4, zero-mean uniform
    RHS; FP64 Jacobi-PCG to 1e-10.
C2: 32^3 box deformed by the seeded 0.05 h sinusoid, N = 7 (16.8M local
    DOFs), pressure-Poisson with a Dirichlet face at x = 1, 16 Fourier modes.
C3: the C2 mesh with h1 = 1/Re = 0.01 and h2 = chi(12 Gaussian blobs).

Bars (written in each test): global ids, gather-scatter permutation and
offsets, multiplicity and Dirichlet mask bit-exact; gather-scatter ADD
bit-exact in FP64; FP64 Ax and geometry within 1e-12 relative (max-abs
error over max-abs value); a fixed 20-iteration FP64 CG within 1e-11;
converged FP64 solves with the same iteration count (within 2) and x within
1e-10 relative (2-norm) of the oracle's x, residuals re-evaluated by the
oracle; the FP32-inner solve's error against the oracle's FP64 solution
(solved to 1e-12) printed and held to 1e-8.  The measured errors are
printed (pytest -s shows them).
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

LX = 8
MESH_SEED, RHS_SEED, RHO_SEED = 1, 2, 3


def relerr(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else a
    b = b.detach().cpu().numpy() if isinstance(b, torch.Tensor) else b
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def rel2(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else a
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def T(a, dev, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device=dev, dtype=dtype)


def wnorm(orc, m, v):
    return float(np.sqrt(orc.glsc3(v, v, m.mult)))


# ---------------------------------------------------------------------------
# C1
# ---------------------------------------------------------------------------
def test_c1_full_size(pkg, orc, dev):
    m = orc.build_mesh(8, 8, 8, LX)
    c = pkg.coef_t.box(8, 8, 8, LX, device=dev)
    assert np.array_equal(c.gid.cpu().numpy(), m.gid)
    rho = orc.field_uniform(m, RHO_SEED, 2, 0.0, 1.0)
    chi = orc.ramp_forward(1.0 - rho, 0.0, 1e4, 8.0, 0)
    b = orc.field_uniform(m, RHS_SEED, 3, -1.0, 1.0)
    b = b - np.sum(b * m.mult) / m.nu
    # the library's own generators give the same fields
    rho_d = c.field_uniform(RHO_SEED, 2, 0.0, 1.0)
    assert np.array_equal(rho_d.cpu().numpy(), rho)
    chi_d = torch.empty_like(rho_d)
    pkg.RAMP_mapping_t(0.0, 1e4, 8.0, False).apply_forward(chi_d, 1.0 - rho_d)
    assert relerr(chi_d, chi) < 1e-15
    c.set_coefs(h1c=1.0, h2=T(chi, dev), ifh2=True)
    x_ref, it_ref, r0, r1 = orc.cg(m, b, h2=chi, rtol=1e-10, max_iter=20000)
    ksp = pkg.krylov_solver_factory(c, "cg", 20000, 1e-10)
    x = torch.zeros(m.n, dtype=torch.float64, device=dev)
    mon = ksp.solve(x, T(b, dev))
    torch.cuda.synchronize()
    xn = x.cpu().numpy()
    err = rel2(xn, x_ref)
    r = b - orc.op_apply(m, xn, h2=chi)
    res = wnorm(orc, m, r) / wnorm(orc, m, b)
    print(f"\nC1: iterations gpu {mon.iter} oracle {it_ref}; x rel err {err:.3e}; ||Ax-b||/||b|| {res:.3e}")
    assert mon.status == pkg.NTG_OK
    assert abs(mon.iter - it_ref) <= 2
    assert abs(mon.res_start - r0) <= 1e-12 * r0
    assert err <= 1e-10
    assert res <= 1.5e-10


# ---------------------------------------------------------------------------
# C2 / C3 (one 32^3 mesh shared by the tests of this module)
# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def c2(pkg, orc, dev):
    m = orc.build_mesh(32, 32, 32, LX, amp=0.05, seed=MESH_SEED)
    mask = orc.mask_face_xmax(32, 32, 32, LX)
    c = pkg.coef_t.box(32, 32, 32, LX, amp=0.05, seed=MESH_SEED, device=dev)
    gmask = pkg.mask_face_xmax(32, 32, 32, LX, device=dev)
    c.set_mask(gmask, base=1)
    k, a, ph = orc.fourier_params(RHS_SEED, 16)
    f = orc.assemble_rhs(m, orc.field_fourier(m, k, a, ph), mask)
    yield m, c, mask, gmask, f
    c.free()


def test_c2_maps_bitexact(orc, c2):
    m, c, mask, gmask, f = c2
    assert m.n == 16_777_216 and m.nu == 11_390_625 == c.nu
    assert np.array_equal(c.gid.cpu().numpy(), m.gid)
    perm, offs = c.gs_maps()
    assert np.array_equal(perm.cpu().numpy(), m.perm)
    assert np.array_equal(offs.cpu().numpy(), m.offs)
    g = c.geometry()
    assert np.array_equal(g["mult"].cpu().numpy(), m.mult)
    assert np.array_equal(gmask.cpu().numpy(), mask)
    for key in ("g11", "g12", "g13", "g22", "g23", "g33"):
        e = np.abs(g[key].cpu().numpy() - m.G[key]).max() / np.abs(m.G["g11"]).max()
        assert e < 1e-12, (key, e)
    assert relerr(g["B"], m.B) < 1e-12


def test_c2_rhs_generator(pkg, orc, dev, c2):
    m, c, mask, gmask, f = c2
    c.set_coefs(h1c=1.0, ifh2=False)
    f_d = c.rhs_assemble(c.field_fourier(16, RHS_SEED))
    torch.cuda.synchronize()
    e = relerr(f_d, f)
    print(f"\nC2 RHS generator: rel err {e:.3e}")
    assert e < 1e-12


def test_c2_ax_and_gs(pkg, orc, dev, c2):
    m, c, mask, gmask, f = c2
    c.set_coefs(h1c=1.0, ifh2=False)
    rng = np.random.default_rng(3)
    u = rng.standard_normal(m.n)
    w_ref = orc.ax_helm(m, u)
    w = torch.empty(m.n, dtype=torch.float64, device=dev)
    pkg.ax_helm_t().compute(w, T(u, dev), c)
    torch.cuda.synchronize()
    e64 = relerr(w, w_ref)
    w32 = torch.empty(m.n, dtype=torch.float32, device=dev)
    pkg.ax_helm_t().compute(w32, T(u, dev, torch.float32), c)
    torch.cuda.synchronize()
    e32 = relerr(w32.double(), w_ref)
    print(f"\nC2 Ax: FP64 rel err {e64:.3e}, FP32 rel err {e32:.3e}")
    assert e64 < 1e-12
    assert e32 < 2e-5
    # gather-scatter ADD, bit-exact in FP64
    v = T(w_ref, dev)
    pkg.gs_t(c).op(v)
    torch.cuda.synchronize()
    assert np.array_equal(v.cpu().numpy(), orc.gs_op(m, w_ref, 1))


def test_c2_cg_fixed_iterations(pkg, orc, dev, c2):
    m, c, mask, gmask, f = c2
    c.set_coefs(h1c=1.0, ifh2=False)
    x_ref, it, _, _ = orc.cg(m, f, mask=mask, fixed_iters=20)
    ksp = pkg.krylov_solver_factory(c, "cg", 20, 0.0)
    x = torch.zeros(m.n, dtype=torch.float64, device=dev)
    mon = ksp.solve(x, T(f, dev))
    torch.cuda.synchronize()
    e = relerr(x, x_ref)
    print(f"\nC2 20-iteration FP64 CG: rel err {e:.3e}")
    assert mon.iter == 20 and mon.status == pkg.NTG_MAXITER
    assert e < 1e-11


@pytest.fixture(scope="module")
def c3_ref(orc, c2):
    """The oracle's FP64 Jacobi-PCG solution of C3, solved to 1e-12."""
    m, c, mask, gmask, f = c2
    rho = orc.field_blobs(m, RHO_SEED, 12, 0.1)
    chi = orc.ramp_forward(1.0 - rho, 0.0, 1e4, 8.0, 0)
    x_ref, it_ref, r0, r1 = orc.cg(m, f, h1c=0.01, h2=chi, mask=mask, rtol=1e-12, max_iter=20000)
    return chi, x_ref, it_ref


def test_c3_ax_and_fixed_cg(pkg, orc, dev, c2, c3_ref):
    m, c, mask, gmask, f = c2
    chi, _, _ = c3_ref
    c.set_coefs(h1c=0.01, h2=T(chi, dev), ifh2=True)
    rng = np.random.default_rng(4)
    u = rng.standard_normal(m.n)
    w_ref = orc.ax_helm(m, u, h1c=0.01, h2=chi)
    w = torch.empty(m.n, dtype=torch.float64, device=dev)
    pkg.ax_helm_t().compute(w, T(u, dev), c)
    torch.cuda.synchronize()
    e64 = relerr(w, w_ref)
    x_ref, _, _, _ = orc.cg(m, f, h1c=0.01, h2=chi, mask=mask, fixed_iters=20)
    ksp = pkg.krylov_solver_factory(c, "cg", 20, 0.0)
    x = torch.zeros(m.n, dtype=torch.float64, device=dev)
    ksp.solve(x, T(f, dev))
    torch.cuda.synchronize()
    ecg = relerr(x, x_ref)
    print(f"\nC3 FP64 Ax rel err {e64:.3e}; 20-iteration CG rel err {ecg:.3e}")
    assert e64 < 1e-12
    assert ecg < 1e-11


def test_c3_converged_fp64_and_mixed(pkg, orc, dev, c2, c3_ref):
    m, c, mask, gmask, f = c2
    chi, x_ref, it_ref = c3_ref
    c.set_coefs(h1c=0.01, h2=T(chi, dev), ifh2=True)
    fd = T(f, dev)
    # the FP64 drop-in to the oracle's tolerance: same iterations, same x
    ksp = pkg.krylov_solver_factory(c, "cg", 20000, 1e-12)
    x = torch.zeros(m.n, dtype=torch.float64, device=dev)
    mon = ksp.solve(x, fd)
    torch.cuda.synchronize()
    e64 = rel2(x, x_ref)
    # the FP32-inner / FP64-refined solve to 1e-10 (Jacobi, as under Brinkman)
    mx = pkg.krylov_solver_factory(c, "cg_mixed", 50000, 1e-10)
    mx.set_inner(0.1, 1)
    y = torch.zeros(m.n, dtype=torch.float64, device=dev)
    mon_mx = mx.solve(y, fd)
    torch.cuda.synchronize()
    yn = y.cpu().numpy()
    emx = rel2(yn, x_ref)
    r = f - orc.op_apply(m, yn, h1c=0.01, h2=chi, mask=mask)
    res = wnorm(orc, m, r) / wnorm(orc, m, f)
    print(f"\nC3 FP64 CG to 1e-12: iterations gpu {mon.iter} oracle {it_ref}, x rel err {e64:.3e}; "
          f"cg_mixed to 1e-10: {mon_mx.iter} iterations, {mon_mx.fp64_ax} FP64 Ax, error vs the oracle's FP64 "
          f"solution {emx:.3e}, ||Ax-b||/||b|| {res:.3e}")
    assert mon.status == pkg.NTG_OK and abs(mon.iter - it_ref) <= 2
    assert e64 <= 1e-10
    assert mon_mx.status == pkg.NTG_OK
    assert res <= 1.5e-10
    assert emx <= 1e-8
