"""The CUDA path against the frozen golden fixtures (tests/golden/golden.npz):
the same seeded meshes rebuilt on the device, FP64 Ax and gather-scatter,
the index maps bit-exact, the FP64 Jacobi-PCG solution, RAMP, and the
two-level Schwarz preconditioner (FP32)."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden.npz")


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLDEN))


def T(a, dev, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device=dev, dtype=dtype)


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def test_golden_ax_gs_maps(pkg, dev, gold):
    c = pkg.coef_t.box(2, 2, 2, 6, amp=0.05, seed=7, device=dev)
    perm, offs = c.gs_maps()
    assert np.array_equal(perm.cpu().numpy(), gold["gs_perm"])
    assert np.array_equal(offs.cpu().numpy(), gold["gs_offs"])
    assert np.array_equal(c.geometry()["mult"].cpu().numpy(), gold["mult"])
    c.set_coefs(h1=T(gold["ax_h1"], dev), h2=T(gold["ax_h2"], dev), ifh2=True)
    w = torch.empty(c.n, dtype=torch.float64, device=dev)
    pkg.ax_helm_t().compute(w, T(gold["ax_u"], dev), c)
    torch.cuda.synchronize()
    assert rel(w.cpu().numpy(), gold["ax_w"]) < 1e-12
    pkg.gs_t(c).op(w, pkg.GS_OP_ADD)
    torch.cuda.synchronize()
    assert rel(w.cpu().numpy(), gold["ax_w_gs"]) < 1e-12


def test_golden_cg(pkg, dev, gold):
    c = pkg.coef_t.box(3, 2, 2, 5, amp=0.05, seed=8, device=dev)
    c.set_mask(pkg.mask_face_xmax(3, 2, 2, 5), base=1)
    c.set_coefs(h1c=1.0, ifh2=False)
    ksp = pkg.krylov_solver_factory(c, "cg", 5000, 1e-10)
    x = torch.zeros(c.n, dtype=torch.float64, device=dev)
    mon = ksp.solve(x, T(gold["cg_f"], dev))
    torch.cuda.synchronize()
    assert mon.status == pkg.NTG_OK and abs(mon.iter - int(gold["cg_iters"][0])) <= 2
    assert np.linalg.norm(x.cpu().numpy() - gold["cg_x"]) <= 1e-8 * np.linalg.norm(gold["cg_x"])


def test_golden_ramp(pkg, dev, gold):
    x = T(gold["ramp_x"], dev)
    for up in (0, 1):
        r = pkg.RAMP_mapping_t(0.0, 1e4, 8.0, bool(up))
        out = torch.empty_like(x)
        r.apply_forward(out, x)
        din = torch.empty_like(x)
        r.apply_backward(din, T(gold["ramp_dF"], dev), x)
        torch.cuda.synchronize()
        assert rel(out.cpu().numpy(), gold[f"ramp_fwd_{up}"]) < 1e-15
        assert rel(din.cpu().numpy(), gold[f"ramp_bwd_{up}"]) < 1e-15


def test_golden_two_level_schwarz(pkg, dev, gold):
    c = pkg.coef_t.box(3, 2, 2, 4, amp=0.05, seed=9, device=dev)
    c.set_mask(pkg.mask_face_xmax(3, 2, 2, 4), base=1)
    c.set_coefs(h1c=1.0, ifh2=False)
    sw = pkg.schwarz_t(c, coarse=True)
    z = torch.empty(c.n, dtype=torch.float32, device=dev)
    sw.apply(z, T(gold["sw_r"], dev, torch.float32))
    torch.cuda.synchronize()
    zz = z.cpu().numpy().astype(np.float64)
    assert np.linalg.norm(zz - gold["sw_z"]) <= 2e-5 * np.linalg.norm(gold["sw_z"])
