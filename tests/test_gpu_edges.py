"""Edge cases through every solver: a single element, a one-element-thick
box, a zero right-hand side, and an all-Neumann (singular, compatible)
problem; each with the plain FP64 CG, the mixed CG with Jacobi and with the
two-level Schwarz, and GMRES."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

SOLVERS = [("cg", None), ("cg_mixed", None), ("cg_mixed", "schwarz2"), ("gmres", None), ("gmres_mixed", "schwarz2")]


def T(a, dev, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device=dev, dtype=dtype)


def make_solver(pkg, c, kind, pc):
    ksp = pkg.krylov_solver_factory(c, kind, 20000, 1e-10)
    if kind == "cg_mixed":
        ksp.set_inner(1e-3 if pc else 0.1, 1)
    if pc == "schwarz2":
        ksp.set_schwarz(pkg.schwarz_t(c, coarse=True))
    return ksp


@pytest.mark.parametrize("kind,pc", SOLVERS)
@pytest.mark.parametrize("shape", [(1, 1, 1, 8), (2, 1, 1, 6), (3, 2, 1, 4)])
def test_tiny_meshes_with_dirichlet(pkg, orc, dev, kind, pc, shape):
    ex, ey, ez, lx = shape
    m = orc.build_mesh(ex, ey, ez, lx, amp=0.05, seed=5)
    c = pkg.coef_t.box(ex, ey, ez, lx, amp=0.05, seed=5, device=dev)
    mask = orc.mask_face_xmax(ex, ey, ez, lx)
    c.set_mask(T(mask, dev, torch.int32), base=1)
    c.set_coefs(h1c=1.0, ifh2=False)
    k, a, ph = orc.fourier_params(5, 8)
    f = orc.assemble_rhs(m, orc.field_fourier(m, k, a, ph), mask)
    ksp = make_solver(pkg, c, kind, pc)
    x = torch.zeros(m.n, dtype=torch.float64, device=dev)
    mon = ksp.solve(x, T(f, dev))
    torch.cuda.synchronize()
    assert mon.status == pkg.NTG_OK, (kind, pc, mon)
    xn = x.cpu().numpy()
    r = f - orc.op_apply(m, xn, h1c=1.0, mask=mask)
    assert np.sqrt(orc.glsc3(r, r, m.mult)) <= 1.5e-10 * np.sqrt(orc.glsc3(f, f, m.mult))


@pytest.mark.parametrize("kind,pc", SOLVERS)
def test_zero_right_hand_side(pkg, orc, dev, kind, pc):
    ex, ey, ez, lx = 3, 2, 2, 8
    c = pkg.coef_t.box(ex, ey, ez, lx, amp=0.05, seed=6, device=dev)
    c.set_mask(pkg.mask_face_xmax(ex, ey, ez, lx, device=dev), base=1)
    c.set_coefs(h1c=1.0, ifh2=False)
    ksp = make_solver(pkg, c, kind, pc)
    x = torch.zeros(c.n, dtype=torch.float64, device=dev)
    mon = ksp.solve(x, torch.zeros(c.n, dtype=torch.float64, device=dev))
    torch.cuda.synchronize()
    assert mon.status == pkg.NTG_OK and mon.iter == 0, (kind, pc, mon)
    assert float(x.abs().max()) == 0.0


@pytest.mark.parametrize("kind,pc", SOLVERS)
def test_all_neumann_compatible(pkg, orc, dev, kind, pc):
    """Pure Neumann Poisson with a zero-mean right-hand side: singular but
    consistent; every solver reaches the tolerance."""
    ex, ey, ez, lx = 4, 3, 2, 8
    m = orc.build_mesh(ex, ey, ez, lx, amp=0.05, seed=7)
    c = pkg.coef_t.box(ex, ey, ez, lx, amp=0.05, seed=7, device=dev)
    c.set_coefs(h1c=1.0, ifh2=False)
    k, a, ph = orc.fourier_params(7, 8)
    f = orc.assemble_rhs(m, orc.field_fourier(m, k, a, ph), None)
    f = f - np.sum(f * m.mult) / np.sum(m.mult) * (orc.gs_op(m, m.B) != 0)  # remove the mean (unique-node sum)
    f = f - orc.gs_op(m, m.B) * (np.sum(f * m.mult) / np.sum(orc.gs_op(m, m.B) * m.mult))
    ksp = make_solver(pkg, c, kind, pc)
    x = torch.zeros(m.n, dtype=torch.float64, device=dev)
    mon = ksp.solve(x, T(f, dev))
    torch.cuda.synchronize()
    assert mon.status == pkg.NTG_OK, (kind, pc, mon)
    xn = x.cpu().numpy()
    r = f - orc.op_apply(m, xn, h1c=1.0)
    assert np.sqrt(orc.glsc3(r, r, m.mult)) <= 1.5e-10 * np.sqrt(orc.glsc3(f, f, m.mult))
