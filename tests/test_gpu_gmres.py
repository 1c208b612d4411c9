"""Restarted flexible GMRES (FP64, and FP32 cycles inside FP64 iterative
refinement) against the oracle's solution of the same problem, with Jacobi
and with the two-level Schwarz preconditioner, and across restarts."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def T(a, dev, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device=dev, dtype=dtype)


@pytest.fixture(scope="module")
def problem(pkg, orc, dev):
    ex, ey, ez, lx = 4, 3, 3, 8
    m = orc.build_mesh(ex, ey, ez, lx, amp=0.05, seed=31)
    c = pkg.coef_t.box(ex, ey, ez, lx, amp=0.05, seed=31, device=dev)
    mask = orc.mask_face_xmax(ex, ey, ez, lx)
    c.set_mask(T(mask, dev, torch.int32), base=1)
    c.set_coefs(h1c=1.0, ifh2=False)
    k, a, ph = orc.fourier_params(31, 16)
    f = orc.assemble_rhs(m, orc.field_fourier(m, k, a, ph), mask)
    x_ref, it_ref, _, _ = orc.cg(m, f, mask=mask, rtol=1e-12, max_iter=20000)
    return m, c, mask, f, x_ref


@pytest.mark.parametrize("kind,pc,restart", [("gmres", "jacobi", 30), ("gmres", "schwarz2", 30),
                                             ("gmres_mixed", "jacobi", 30), ("gmres_mixed", "schwarz2", 30),
                                             ("gmres", "jacobi", 5)])
def test_gmres_solves_to_tolerance(pkg, orc, dev, problem, kind, pc, restart):
    m, c, mask, f, x_ref = problem
    ksp = pkg.krylov_solver_factory(c, kind, 20000, 1e-10)
    ksp.set_restart(restart)
    if pc == "schwarz2":
        ksp.set_schwarz(pkg.schwarz_t(c, coarse=True))
    x = torch.zeros(m.n, dtype=torch.float64, device=dev)
    mon = ksp.solve(x, T(f, dev))
    torch.cuda.synchronize()
    assert mon.status == pkg.NTG_OK, mon
    xn = x.cpu().numpy()
    r = f - orc.op_apply(m, xn, h1c=1.0, mask=mask)
    assert np.sqrt(orc.glsc3(r, r, m.mult)) <= 1.5e-10 * np.sqrt(orc.glsc3(f, f, m.mult))
    assert np.linalg.norm(xn - x_ref) <= 1e-7 * np.linalg.norm(x_ref)
    assert np.all(xn[mask - 1] == 0.0)
    print(kind, pc, restart, "iterations", mon.iter, "cycles", mon.inner_iter, "fp64 Ax", mon.fp64_ax)
    # the FP64 operator runs once per cycle (the restart residual), never per step
    assert mon.fp64_ax <= mon.inner_iter + 1
    if pc == "schwarz2":
        assert mon.inner_iter <= 3  # the two-level Schwarz converges within a few cycles


def test_gmres_nonzero_guess_and_already_converged(pkg, orc, dev, problem):
    m, c, mask, f, x_ref = problem
    ksp = pkg.krylov_solver_factory(c, "gmres_mixed", 20000, 1e-10)
    x = T(x_ref, dev)
    mon = ksp.solve(x, T(f, dev))
    torch.cuda.synchronize()
    assert mon.status == pkg.NTG_OK and mon.iter == 0, mon
