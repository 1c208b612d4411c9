"""The Schwarz preconditioner on general meshes (ntg_schwarz_create_general:
face-neighbour tables, global-node prolongation, Galerkin coarse level)
against its numpy restatement (oracle/schwarz_ref.apply_general), and the
reliable-update mixed CG preconditioned by it on an O-grid pipe read back
from a .nmsh file."""
import numpy as np
import pytest
import torch

import meshgen
from oracle import schwarz_ref

pytestmark = pytest.mark.gpu


def T(a, dev, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device=dev, dtype=dtype)


def corner_ids(m):
    lx, N = m.lx, m.lx - 1
    g = m.gid.reshape(m.nelv, lx ** 3)
    return np.stack([g[:, (v & 1) * N + lx * ((v >> 1) & 1) * N + lx * lx * (v >> 2) * N] for v in range(8)], 1)


def ogrid(orc, pkg, lx, dims=(2, 2, 3)):
    ev, xyz, zones = meshgen.ogrid_pipe(*dims)
    gid = pkg.dofmap.dofmap_from_vertices(ev, lx)
    m = orc.mesh_general(*meshgen.nodes_from_vertices(xyz, lx), gid, lx)
    return m, ev, xyz, zones


def outlet_mask(m, zones, label=2):
    lx, N = m.lx, m.lx - 1
    sel = []
    for e, f, _, lab, *_ in zones:
        if lab != label:
            continue
        e, f = e - 1, f - 1
        d, nrm = f // 2, (N if f % 2 else 0)
        for t in range(lx):
            for s in range(lx):
                i, j, k = [(nrm, s, t), (s, nrm, t), (s, t, nrm)][d]
                sel.append(e * lx ** 3 + i + lx * (j + lx * k))
    return (np.nonzero(np.isin(m.gid, np.unique(m.gid[sel])))[0] + 1).astype(np.int32)


def general_coef(pkg, m, dev):
    return pkg.coef_t(m.nelv, m.lx, T(m.x, dev), T(m.y, dev), T(m.z, dev), T(m.gid, dev, torch.int64))


CASES = [("box", 8, True, 0), ("box", 4, False, 2), ("box_reoriented", 8, True, 0), ("ogrid", 6, True, 0),
         ("ogrid", 8, False, 0), ("ogrid", 8, True, 2), ("box_neumann", 6, True, 0), ("box_pure_neumann", 6, True, 0)]


@pytest.mark.parametrize("case", CASES)
def test_general_apply_matches_oracle(pkg, orc, dev, case):
    """path 0: even-odd transforms, 2: full products; every copy of a node
    holds the bit-identical value."""
    kind, lx, coarse, path = case
    rng = np.random.default_rng(5)
    if kind.startswith("box"):
        m = orc.build_mesh(3, 2, 2, lx, amp=0.05, seed=2)
        mask = None if kind in ("box_neumann", "box_pure_neumann") else orc.mask_face_xmax(3, 2, 2, lx)
        if kind == "box_reoriented":
            flag = np.zeros(m.n)
            flag[mask - 1] = 1
            _, (x2, y2, z2, g2, f2) = meshgen.reorient(lx, corner_ids(m), [m.x, m.y, m.z, m.gid, flag], rng)
            m = orc.mesh_general(x2, y2, z2, g2.astype(np.int64), lx)
            mask = (np.nonzero(f2)[0] + 1).astype(np.int32)
    else:
        m, _, _, zones = ogrid(orc, pkg, lx)
        mask = outlet_mask(m, zones)
    c = general_coef(pkg, m, dev)
    if mask is not None:
        c.set_mask(T(mask, dev, torch.int32), base=1)
    h2 = rng.uniform(0.0, 2.0, m.n)
    if kind == "box_pure_neumann":
        # no Dirichlet vertex and no mass term: the coarse operator's constant
        # null mode is shifted (A_c + c 1 1^T) on both sides
        h2 = None
        c.set_coefs(h1c=0.5, ifh2=False)
    else:
        c.set_coefs(h1c=0.5, h2=T(h2, dev), ifh2=True)
    sw = pkg.schwarz_t(c, coarse=coarse)
    assert sw.general
    sw.set_fdm_path(path)
    g = orc.gs_op(m, rng.standard_normal(m.n)) * m.mult
    r = (orc.apply_mask_zero(g, mask) if mask is not None else g).astype(np.float32)
    z = torch.empty(m.n, dtype=torch.float32, device=dev)
    sw.apply(z, T(r, dev, torch.float32))
    torch.cuda.synchronize()
    ref = schwarz_ref.apply_general(m, r.astype(np.float64), h1=0.5, h2=h2, mask=mask, coarse=coarse)
    zz = z.cpu().numpy().astype(np.float64)
    err = np.linalg.norm(zz - ref) / np.linalg.norm(ref)
    print(case, "rel err", err)
    assert err <= 2e-5, err
    order = np.argsort(m.gid, kind="stable")
    gid, v = m.gid[order], zz[order]
    starts = np.r_[0, np.nonzero(np.diff(gid))[0] + 1]
    assert np.array_equal(np.maximum.reduceat(v, starts), np.minimum.reduceat(v, starts))


def test_general_is_symmetric(pkg, orc, dev):
    m, _, _, zones = ogrid(orc, pkg, 8)
    mask = outlet_mask(m, zones)
    c = general_coef(pkg, m, dev)
    c.set_mask(T(mask, dev, torch.int32), base=1)
    c.set_coefs(h1c=1.0, ifh2=False)
    sw = pkg.schwarz_t(c, coarse=True)
    rng = np.random.default_rng(4)
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
    assert float(np.sum(m.mult * u * Mu.cpu().numpy())) > 0


def test_general_equals_box_form_reoriented(pkg, orc, dev):
    """The general form on a box whose elements are re-oriented gives the
    general form's result on the original box, permuted (FP32 rounding)."""
    lx = 8
    m = orc.build_mesh(3, 3, 2, lx, amp=0.05, seed=6)
    mask = orc.mask_face_xmax(3, 3, 2, lx)
    rng = np.random.default_rng(9)
    r = orc.apply_mask_zero(orc.gs_op(m, rng.standard_normal(m.n)) * m.mult, mask)
    flag = np.zeros(m.n)
    flag[mask - 1] = 1
    idx = np.arange(m.n, dtype=np.float64)
    _, (x2, y2, z2, g2, f2, r2, i2) = meshgen.reorient(lx, corner_ids(m), [m.x, m.y, m.z, m.gid, flag, r, idx], rng)
    m2 = orc.mesh_general(x2, y2, z2, g2.astype(np.int64), lx)
    mask2 = (np.nonzero(f2)[0] + 1).astype(np.int32)
    out = []
    for mm, mk, rr in ((m, mask, r), (m2, mask2, r2)):
        c = general_coef(pkg, mm, dev)
        c.set_mask(T(mk, dev, torch.int32), base=1)
        c.set_coefs(h1c=1.0, ifh2=False)
        sw = pkg.schwarz_t(c, coarse=True, general=True)
        z = torch.empty(mm.n, dtype=torch.float32, device=dev)
        sw.apply(z, T(rr, dev, torch.float32))
        torch.cuda.synchronize()
        out.append(z.cpu().numpy().astype(np.float64))
    ref = out[0][i2.astype(np.int64)]
    assert np.linalg.norm(out[1] - ref) <= 1e-6 * np.linalg.norm(ref)


@pytest.mark.parametrize("coarse", [True, False])
def test_cg_mixed_on_nmsh_ogrid(pkg, orc, dev, tmp_path, coarse):
    """O-grid pipe written to .nmsh and read back, lx = 8, outlet Dirichlet:
    cg_mixed with the general Schwarz converges to the oracle's FP64
    solution in far fewer iterations than Jacobi."""
    lx = 8
    ev, xyz, zones = meshgen.ogrid_pipe(3, 2, 4)
    path = tmp_path / "ogrid.nmsh"
    pkg.nmsh.write(path, pkg.nmsh.nmsh_t(3, np.arange(1, len(ev) + 1, dtype=np.int32), ev.astype(np.int32), xyz,
                                         zones))
    mesh = pkg.nmsh.read(path)
    c = pkg.nmsh.coef_from_nmsh(mesh, lx, device=dev)
    mask_t = pkg.nmsh.face_mask(c, mesh.zone_faces(labels=[2]))
    c.set_mask(mask_t, base=1)
    c.set_coefs(h1c=1.0, ifh2=False)
    m = orc.mesh_general(c.x.cpu().numpy(), c.y.cpu().numpy(), c.z.cpu().numpy(), c.gid.cpu().numpy(), lx)
    mx, my, mz = meshgen.nodes_from_vertices(xyz, lx)
    assert np.allclose(m.x, mx, atol=1e-14) and np.allclose(m.z, mz, atol=1e-14)
    mask = mask_t.cpu().numpy()
    assert np.array_equal(np.sort(mask), outlet_mask(m, zones))
    k, a, ph = orc.fourier_params(21, 16)
    f = orc.assemble_rhs(m, orc.field_fourier(m, k, a, ph), mask)
    x_ref, it_ref, _, _ = orc.cg(m, f, mask=mask, rtol=1e-13, max_iter=20000)
    ksp = pkg.krylov_solver_factory(c, "cg_mixed", 20000, 1e-10)
    sw = pkg.schwarz_t(c, coarse=coarse)
    ksp.set_schwarz(sw)
    x = torch.zeros(m.n, dtype=torch.float64, device=dev)
    mon = ksp.solve(x, T(f, dev))
    torch.cuda.synchronize()
    assert mon.status == pkg.NTG_OK, mon
    xn = x.cpu().numpy()
    r = f - orc.op_apply(m, xn, mask=mask)
    assert np.sqrt(orc.glsc3(r, r, m.mult)) <= 1.5e-10 * np.sqrt(orc.glsc3(f, f, m.mult))
    err = np.linalg.norm(xn - x_ref) / np.linalg.norm(x_ref)
    print("O-grid", m.nelv, "elements, coarse", coarse, ": jacobi (FP64 oracle)", it_ref, "schwarz", mon.iter,
          "error", err)
    assert err <= 1e-8
    assert mon.iter < (0.35 if coarse else 0.6) * it_ref


@pytest.mark.parametrize("kind", ["gmres", "gmres_mixed"])
def test_gmres_with_general_schwarz(pkg, orc, dev, kind):
    """The reference's pressure solver pairing (GMRES + the Schwarz part of
    'hsmg') on the O-grid pipe: converges to the oracle's solution."""
    m, _, _, zones = ogrid(orc, pkg, 6)
    mask = outlet_mask(m, zones)
    c = general_coef(pkg, m, dev)
    c.set_mask(T(mask, dev, torch.int32), base=1)
    c.set_coefs(h1c=1.0, ifh2=False)
    k, a, ph = orc.fourier_params(7, 8)
    f = orc.assemble_rhs(m, orc.field_fourier(m, k, a, ph), mask)
    x_ref, it_ref, _, _ = orc.cg(m, f, mask=mask, rtol=1e-13, max_iter=20000)
    ksp = pkg.krylov_solver_factory(c, kind, 5000, 1e-10)
    ksp.set_schwarz(pkg.schwarz_t(c, coarse=True))
    x = torch.zeros(m.n, dtype=torch.float64, device=dev)
    mon = ksp.solve(x, T(f, dev))
    torch.cuda.synchronize()
    assert mon.status == pkg.NTG_OK, mon
    xn = x.cpu().numpy()
    r = f - orc.op_apply(m, xn, mask=mask)
    assert np.sqrt(orc.glsc3(r, r, m.mult)) <= 1.5e-10 * np.sqrt(orc.glsc3(f, f, m.mult))
    assert np.linalg.norm(xn - x_ref) <= 1e-8 * np.linalg.norm(x_ref)
    print(kind, "iterations", mon.iter, "(Jacobi-PCG oracle", it_ref, ")")
    assert mon.iter < 0.5 * it_ref


def test_dense_coarse_limit(pkg, orc, dev):
    """The general form's dense coarse level takes at most 8192 active
    vertices: above that the coarse level is refused with a clear error and
    the one-level form still works."""
    ex = ey = ez = 21  # 22^3 = 10,648 vertices
    lx = 4
    c = pkg.coef_t.box(ex, ey, ez, lx, amp=0.0, seed=1, device=dev)
    c.set_coefs(h1c=1.0, ifh2=False)
    with pytest.raises(pkg.NtgError, match="at most 8192"):
        pkg.schwarz_t(c, coarse=True, general=True)
    sw = pkg.schwarz_t(c, coarse=False, general=True)
    r = torch.randn(c.n, dtype=torch.float32, device=dev)
    pkg.gs_t(c).op(r)
    z = torch.empty_like(r)
    sw.apply(z, r)
    torch.cuda.synchronize()
    assert torch.isfinite(z).all()
