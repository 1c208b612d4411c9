"""Overlapping Schwarz preconditioner (FP32) against its numpy restatement,
its symmetry, and the reliable-update mixed CG preconditioned by it.  For
lx = 8 both FDM paths are checked: the FP32-core kernel against the exact
restatement (2e-5), the tensor-core kernel against the restatement with the
same BF16-rounded plane operator (1e-4: the data's two-term BF16 split
carries 16 bits) and against the FP32-core kernel (the rounding of the
plane operator, 3e-3)."""
import numpy as np
import pytest
import torch

from oracle import schwarz_ref

pytestmark = pytest.mark.gpu


def T(a, dev, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device=dev, dtype=dtype)


@pytest.mark.parametrize("shape", [(3, 2, 2, 8, 0.05, 1), (3, 2, 2, 8, 0.05, 0), (3, 2, 2, 8, 0.05, 2),
                                   (2, 3, 2, 4, 0.0, 0), (2, 3, 2, 4, 0.0, 2), (4, 1, 2, 6, 0.05, 0),
                                   (5, 3, 2, 8, 0.05, 1)])
def test_schwarz_apply_matches_oracle(pkg, orc, dev, shape):
    """path 0: FP32 cores, even-odd transforms; 2: FP32 cores, full products;
    1: tensor cores (lx = 8)."""
    ex, ey, ez, lx, amp, path = shape
    tensor_cores = path == 1
    m = orc.build_mesh(ex, ey, ez, lx, amp=amp, seed=2)
    c = pkg.coef_t.box(ex, ey, ez, lx, amp=amp, seed=2, device=dev)
    mask = orc.mask_face_xmax(ex, ey, ez, lx)
    c.set_mask(T(mask, dev, torch.int32), base=1)
    rng = np.random.default_rng(1)
    h2 = rng.uniform(0.0, 2.0, m.n)
    c.set_coefs(h1c=0.5, h2=T(h2, dev), ifh2=True)
    sw = pkg.schwarz_t(c)
    sw.set_fdm_path(path)
    r = orc.apply_mask_zero(orc.gs_op(m, rng.standard_normal(m.n)) * m.mult, mask).astype(np.float32)
    z = torch.empty(m.n, dtype=torch.float32, device=dev)
    sw.apply(z, T(r, dev, torch.float32))
    torch.cuda.synchronize()
    ref = schwarz_ref.apply(m, r.astype(np.float64), (ex, ey, ez), h1=0.5, h2=h2, mask=mask,
                            plane_bf16=bool(tensor_cores))
    zz = z.cpu().numpy().astype(np.float64)
    err = np.linalg.norm(zz - ref) / np.linalg.norm(ref)
    assert err <= (1e-4 if tensor_cores else 2e-5), err
    if tensor_cores:
        # against the FP32-core path: the plane operator's BF16 rounding
        sw.set_fdm_path(0)
        z32 = torch.empty_like(z)
        sw.apply(z32, T(r, dev, torch.float32))
        torch.cuda.synchronize()
        d = np.linalg.norm(zz - z32.cpu().numpy()) / np.linalg.norm(zz)
        print("tensor-core vs FP32-core FDM", d, "vs oracle", err)
        assert d <= 3e-3


@pytest.mark.parametrize("tensor_cores", [1, 0])
def test_schwarz_is_symmetric(pkg, orc, dev, tensor_cores):
    ex, ey, ez, lx = 4, 3, 2, 8
    m = orc.build_mesh(ex, ey, ez, lx, amp=0.05, seed=3)
    c = pkg.coef_t.box(ex, ey, ez, lx, amp=0.05, seed=3, device=dev)
    c.set_coefs(h1c=1.0, ifh2=False)
    sw = pkg.schwarz_t(c)
    sw.set_fdm_path(int(tensor_cores))
    rng = np.random.default_rng(4)
    u = (orc.gs_op(m, rng.standard_normal(m.n)) * m.mult).astype(np.float32)
    v = (orc.gs_op(m, rng.standard_normal(m.n)) * m.mult).astype(np.float32)
    Mu = torch.empty(m.n, dtype=torch.float32, device=dev)
    Mv = torch.empty_like(Mu)
    sw.apply(Mu, T(u, dev, torch.float32))
    sw.apply(Mv, T(v, dev, torch.float32))
    torch.cuda.synchronize()
    a = float(np.sum(m.mult * v * Mu.cpu().numpy()))
    b = float(np.sum(m.mult * u * Mv.cpu().numpy()))
    assert abs(a - b) <= (1e-4 if tensor_cores else 1e-5) * max(abs(a), abs(b))
    assert float(np.sum(m.mult * u * Mu.cpu().numpy())) > 0


@pytest.mark.parametrize("case", ["poisson", "brinkman"])
def test_cg_mixed_with_schwarz(pkg, orc, dev, case):
    ex, ey, ez, lx = 6, 4, 4, 8
    m = orc.build_mesh(ex, ey, ez, lx, amp=0.05, seed=21)
    c = pkg.coef_t.box(ex, ey, ez, lx, amp=0.05, seed=21, device=dev)
    mask = orc.mask_face_xmax(ex, ey, ez, lx)
    c.set_mask(T(mask, dev, torch.int32), base=1)
    h1c, h2 = 1.0, None
    if case == "brinkman":
        rho = orc.field_blobs(m, 5, 12, 0.1)
        h2 = orc.ramp_forward(1.0 - rho, 0.0, 1e4, 8.0, 0)
        h1c = 0.01
        c.set_coefs(h1c=h1c, h2=T(h2, dev), ifh2=True)
    else:
        c.set_coefs(h1c=1.0, ifh2=False)
    k, a, ph = orc.fourier_params(21, 16)
    f = orc.assemble_rhs(m, orc.field_fourier(m, k, a, ph), mask)
    ksp_j = pkg.krylov_solver_factory(c, "cg_mixed", 20000, 1e-10)
    xj = torch.zeros(m.n, dtype=torch.float64, device=dev)
    mon_j = ksp_j.solve(xj, T(f, dev))
    sw = pkg.schwarz_t(c)
    ksp = pkg.krylov_solver_factory(c, "cg_mixed", 20000, 1e-10)
    ksp.set_schwarz(sw)
    x = torch.zeros(m.n, dtype=torch.float64, device=dev)
    mon = ksp.solve(x, T(f, dev))
    torch.cuda.synchronize()
    assert mon.status == pkg.NTG_OK, mon
    xn = x.cpu().numpy()
    r = f - orc.op_apply(m, xn, h1c=h1c, h2=h2, mask=mask)
    assert np.sqrt(orc.glsc3(r, r, m.mult)) <= 1.5e-10 * np.sqrt(orc.glsc3(f, f, m.mult))
    assert np.linalg.norm(xn - xj.cpu().numpy()) <= 1e-7 * np.linalg.norm(xn)
    print(case, "jacobi", mon_j.iter, "schwarz", mon.iter)
    if case == "poisson":
        # the pressure-Poisson operator: Schwarz cuts the iterations (measured 475 -> 198)
        assert mon.iter < 0.6 * mon_j.iter
    # Brinkman (h2 = chi(rho) varying by 1e4 inside elements): the FDM local
    # solves see only element means of h2, so pointwise Jacobi is the better
    # preconditioner there (measured 73 vs 562); the solve still converges.


@pytest.mark.parametrize("shape", [(3, 2, 2, 8, 0.05, True), (2, 3, 2, 4, 0.0, False), (4, 1, 2, 6, 0.05, True)])
def test_schwarz_coarse_apply_matches_oracle(pkg, orc, dev, shape):
    ex, ey, ez, lx, amp, dirichlet = shape
    m = orc.build_mesh(ex, ey, ez, lx, amp=amp, seed=2)
    c = pkg.coef_t.box(ex, ey, ez, lx, amp=amp, seed=2, device=dev)
    mask = orc.mask_face_xmax(ex, ey, ez, lx) if dirichlet else None
    if dirichlet:
        c.set_mask(T(mask, dev, torch.int32), base=1)
    rng = np.random.default_rng(5)
    h2 = rng.uniform(0.0, 2.0, m.n)
    c.set_coefs(h1c=0.5, h2=T(h2, dev), ifh2=True)
    sw = pkg.schwarz_t(c, coarse=True)
    g = orc.gs_op(m, rng.standard_normal(m.n)) * m.mult
    r = (orc.apply_mask_zero(g, mask) if dirichlet else g).astype(np.float32)
    z = torch.empty(m.n, dtype=torch.float32, device=dev)
    sw.apply(z, T(r, dev, torch.float32))
    torch.cuda.synchronize()
    ref = schwarz_ref.apply(m, r.astype(np.float64), (ex, ey, ez), h1=0.5, h2=h2, mask=mask, coarse=True)
    zz = z.cpu().numpy().astype(np.float64)
    assert np.linalg.norm(zz - ref) <= 2e-5 * np.linalg.norm(ref)
    # every copy of a shared node holds the bit-identical value
    order = np.argsort(m.gid, kind="stable")
    gid, v = m.gid[order], zz[order]
    starts = np.r_[0, np.nonzero(np.diff(gid))[0] + 1]
    assert np.array_equal(np.maximum.reduceat(v, starts), np.minimum.reduceat(v, starts))


def test_schwarz_coarse_is_symmetric(pkg, orc, dev):
    ex, ey, ez, lx = 4, 3, 2, 8
    m = orc.build_mesh(ex, ey, ez, lx, amp=0.05, seed=3)
    c = pkg.coef_t.box(ex, ey, ez, lx, amp=0.05, seed=3, device=dev)
    c.set_coefs(h1c=1.0, ifh2=False)
    sw = pkg.schwarz_t(c, coarse=True)
    rng = np.random.default_rng(4)
    u = (orc.gs_op(m, rng.standard_normal(m.n)) * m.mult).astype(np.float32)
    v = (orc.gs_op(m, rng.standard_normal(m.n)) * m.mult).astype(np.float32)
    Mu = torch.empty(m.n, dtype=torch.float32, device=dev)
    Mv = torch.empty_like(Mu)
    sw.apply(Mu, T(u, dev, torch.float32))
    sw.apply(Mv, T(v, dev, torch.float32))
    torch.cuda.synchronize()
    a = float(np.sum(m.mult * v * Mu.cpu().numpy()))
    b = float(np.sum(m.mult * u * Mv.cpu().numpy()))
    assert abs(a - b) <= 1e-5 * max(abs(a), abs(b))
    # all-Neumann: the constant null mode is dropped, the rest stays positive
    assert float(np.sum(m.mult * u * Mu.cpu().numpy())) > 0


def test_cg_mixed_with_two_level_schwarz(pkg, orc, dev):
    """The coarse level cuts the pressure-Poisson iterations further and the
    solution is the same."""
    ex, ey, ez, lx = 8, 8, 8, 8
    m = orc.build_mesh(ex, ey, ez, lx, amp=0.05, seed=21)
    c = pkg.coef_t.box(ex, ey, ez, lx, amp=0.05, seed=21, device=dev)
    mask = orc.mask_face_xmax(ex, ey, ez, lx)
    c.set_mask(T(mask, dev, torch.int32), base=1)
    c.set_coefs(h1c=1.0, ifh2=False)
    k, a, ph = orc.fourier_params(21, 16)
    f = orc.assemble_rhs(m, orc.field_fourier(m, k, a, ph), mask)
    its = {}
    xs = {}
    for name, coarse in (("one_level", False), ("two_level", True)):
        sw = pkg.schwarz_t(c, coarse=coarse)
        ksp = pkg.krylov_solver_factory(c, "cg_mixed", 20000, 1e-10)
        ksp.set_schwarz(sw)
        x = torch.zeros(m.n, dtype=torch.float64, device=dev)
        mon = ksp.solve(x, T(f, dev))
        torch.cuda.synchronize()
        assert mon.status == pkg.NTG_OK, mon
        its[name] = mon.iter
        xs[name] = x.cpu().numpy()
    xn = xs["two_level"]
    r = f - orc.op_apply(m, xn, h1c=1.0, mask=mask)
    assert np.sqrt(orc.glsc3(r, r, m.mult)) <= 1.5e-10 * np.sqrt(orc.glsc3(f, f, m.mult))
    assert np.linalg.norm(xn - xs["one_level"]) <= 1e-7 * np.linalg.norm(xn)
    print("iterations", its)
    assert its["two_level"] < 0.7 * its["one_level"]


def test_mass_term_keeps_symmetry_and_converges(pkg, orc, dev):
    """The optional additive diagonal term for a Brinkman mass part: the
    preconditioner stays symmetric and the mixed CG reaches the tolerance
    with the same solution."""
    ex, ey, ez, lx = 6, 4, 4, 8
    m = orc.build_mesh(ex, ey, ez, lx, amp=0.05, seed=23)
    c = pkg.coef_t.box(ex, ey, ez, lx, amp=0.05, seed=23, device=dev)
    mask = orc.mask_face_xmax(ex, ey, ez, lx)
    c.set_mask(T(mask, dev, torch.int32), base=1)
    rho = orc.field_blobs(m, 5, 12, 0.1)
    h2 = orc.ramp_forward(1.0 - rho, 0.0, 1e4, 8.0, 0)
    c.set_coefs(h1c=1.0, h2=T(h2, dev), ifh2=True)
    sw = pkg.schwarz_t(c, coarse=True)
    sw.set_mass_term(True)
    rng = np.random.default_rng(8)
    u = orc.apply_mask_zero(orc.gs_op(m, rng.standard_normal(m.n)) * m.mult, mask).astype(np.float32)
    v = orc.apply_mask_zero(orc.gs_op(m, rng.standard_normal(m.n)) * m.mult, mask).astype(np.float32)
    Mu = torch.empty(m.n, dtype=torch.float32, device=dev)
    Mv = torch.empty_like(Mu)
    sw.apply(Mu, T(u, dev, torch.float32))
    sw.apply(Mv, T(v, dev, torch.float32))
    torch.cuda.synchronize()
    a = float(np.sum(m.mult * v * Mu.cpu().numpy()))
    b = float(np.sum(m.mult * u * Mv.cpu().numpy()))
    assert abs(a - b) <= 1e-5 * max(abs(a), abs(b))
    k, am, ph = orc.fourier_params(23, 16)
    f = orc.assemble_rhs(m, orc.field_fourier(m, k, am, ph), mask)
    ksp = pkg.krylov_solver_factory(c, "cg_mixed", 20000, 1e-10)
    ksp.set_inner(1e-3, 1)
    ksp.set_schwarz(sw)
    x = torch.zeros(m.n, dtype=torch.float64, device=dev)
    mon = ksp.solve(x, T(f, dev))
    torch.cuda.synchronize()
    assert mon.status == pkg.NTG_OK, mon
    xn = x.cpu().numpy()
    r = f - orc.op_apply(m, xn, h1c=1.0, h2=h2, mask=mask)
    assert np.sqrt(orc.glsc3(r, r, m.mult)) <= 1.5e-10 * np.sqrt(orc.glsc3(f, f, m.mult))


def test_tensor_core_fdm_keeps_the_iteration_count(pkg, orc, dev):
    """The mixed CG with the two-level Schwarz takes the same number of
    iterations (within 2) with either FDM path, and the solutions agree."""
    ex, ey, ez, lx = 8, 6, 5, 8
    m = orc.build_mesh(ex, ey, ez, lx, amp=0.05, seed=31)
    c = pkg.coef_t.box(ex, ey, ez, lx, amp=0.05, seed=31, device=dev)
    mask = orc.mask_face_xmax(ex, ey, ez, lx)
    c.set_mask(T(mask, dev, torch.int32), base=1)
    c.set_coefs(h1c=1.0, ifh2=False)
    k, a, ph = orc.fourier_params(31, 16)
    f = orc.assemble_rhs(m, orc.field_fourier(m, k, a, ph), mask)
    its, xs = {}, {}
    for tcore in (1, 0):
        sw = pkg.schwarz_t(c, coarse=True)
        sw.set_fdm_path(int(tcore))
        ksp = pkg.krylov_solver_factory(c, "cg_mixed", 20000, 1e-10)
        ksp.set_inner(2.2e-4, 1)
        ksp.set_schwarz(sw)
        x = torch.zeros(m.n, dtype=torch.float64, device=dev)
        mon = ksp.solve(x, T(f, dev))
        torch.cuda.synchronize()
        assert mon.status == pkg.NTG_OK, mon
        its[tcore], xs[tcore] = mon.iter, x.cpu().numpy()
    print("iterations tensor-core", its[1], "FP32-core", its[0])
    assert abs(its[1] - its[0]) <= 2
    assert np.linalg.norm(xs[1] - xs[0]) <= 1e-8 * np.linalg.norm(xs[0])
    r = f - orc.op_apply(m, xs[1], h1c=1.0, mask=mask)
    assert np.sqrt(orc.glsc3(r, r, m.mult)) <= 1.5e-10 * np.sqrt(orc.glsc3(f, f, m.mult))


def test_fused_update_equals_separate_kernels(pkg, orc, dev):
    """On a box, the cg_mixed update that does the gather-scatter and mask of
    A p itself sums the same terms in the same order as gs + mask + update:
    the same iterations and the same solution to the last bits."""
    ex, ey, ez, lx = 6, 5, 4, 8
    m = orc.build_mesh(ex, ey, ez, lx, amp=0.05, seed=21)
    c = pkg.coef_t.box(ex, ey, ez, lx, amp=0.05, seed=21, device=dev)
    mask = orc.mask_face_xmax(ex, ey, ez, lx)
    c.set_mask(T(mask, dev, torch.int32), base=1)
    rho = orc.field_blobs(m, 5, 12, 0.1)
    h2 = orc.ramp_forward(1.0 - rho, 0.0, 1e4, 8.0, 0)
    c.set_coefs(h1c=1.0, h2=T(h2, dev), ifh2=True)
    k, a, ph = orc.fourier_params(21, 16)
    f = orc.assemble_rhs(m, orc.field_fourier(m, k, a, ph), mask)
    out = {}
    for fused in (True, False):
        sw = pkg.schwarz_t(c, coarse=True)
        ksp = pkg.krylov_solver_factory(c, "cg_mixed", 20000, 1e-10)
        ksp.set_schwarz(sw)
        ksp.set_fused_update(fused)
        x = torch.zeros(m.n, dtype=torch.float64, device=dev)
        mon = ksp.solve(x, T(f, dev))
        torch.cuda.synchronize()
        assert mon.status == pkg.NTG_OK, mon
        out[fused] = (mon.iter, x.cpu().numpy())
    assert out[True][0] == out[False][0], (out[True][0], out[False][0])
    xa, xb = out[True][1], out[False][1]
    assert np.linalg.norm(xa - xb) <= 1e-12 * np.linalg.norm(xb)
    r = f - orc.op_apply(m, xa, h1c=1.0, h2=h2, mask=mask)
    assert np.sqrt(orc.glsc3(r, r, m.mult)) <= 1.5e-10 * np.sqrt(orc.glsc3(f, f, m.mult))
