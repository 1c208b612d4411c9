"""The oracle's Schwarz preconditioner on general meshes (face-only overlap,
Galerkin coarse level; oracle/schwarz_ref.apply_general), on the CPU:
independent of the elements' local orientation, symmetric, and a good
preconditioner for the pressure-Poisson operator on an O-grid pipe and on
the reference's own pipe mesh (data/debugging_pipe.nmsh, when present)."""
import importlib.util
import os

import numpy as np
import pytest

import meshgen
from oracle import schwarz_ref

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("NTG_REFERENCE_DIR", "/root/reference")
PIPE = os.path.join(REF, "data", "debugging_pipe.nmsh")


@pytest.fixture(scope="module")
def dofmap():
    spec = importlib.util.spec_from_file_location("ntg_dofmap", os.path.join(ROOT, "neko-top_gb300", "dofmap.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def pcg(orc, m, f, M, mask, tol=1e-10, maxit=3000):
    x = np.zeros(m.n)
    r = f.copy()
    z = M(r)
    p = z.copy()
    rz = np.sum(m.mult * r * z)
    fn = np.sqrt(np.sum(m.mult * f * f))
    for it in range(1, maxit):
        w = orc.op_apply(m, p, mask=mask)
        a = rz / np.sum(m.mult * p * w)
        x += a * p
        r -= a * w
        if np.sqrt(np.sum(m.mult * r * r)) < tol * fn:
            return x, it
        z = M(r)
        rz2 = np.sum(m.mult * r * z)
        p = z + rz2 / rz * p
        rz = rz2
    return x, maxit


def zone_mask(lx, gid, faces):
    N = lx - 1
    sel = []
    for e, f in faces:
        d, nrm = f // 2, (N if f % 2 else 0)
        for t in range(lx):
            for s in range(lx):
                i, j, k = [(nrm, s, t), (s, nrm, t), (s, t, nrm)][d]
                sel.append(e * lx ** 3 + i + lx * (j + lx * k))
    return (np.nonzero(np.isin(gid, np.unique(gid[sel])))[0] + 1).astype(np.int32)


def test_orientation_independent(orc, dofmap):
    """Re-orienting every element by a random rotation of the cube permutes
    the result and changes nothing else."""
    ex, ey, ez, lx = 3, 2, 2, 4
    m = orc.build_mesh(ex, ey, ez, lx, amp=0.05, seed=1)
    mask = orc.mask_face_xmax(ex, ey, ez, lx)
    rng = np.random.default_rng(3)
    r = orc.apply_mask_zero(orc.gs_op(m, rng.standard_normal(m.n)) * m.mult, mask)
    ref = schwarz_ref.apply_general(m, r, h1=0.7, mask=mask, coarse=True)
    ev = np.zeros((m.nelv, 8), dtype=np.int64)  # vertex ids: the corner nodes' global ids
    l3, N = lx ** 3, lx - 1
    for v in range(8):
        ev[:, v] = m.gid.reshape(m.nelv, l3)[:, (v & 1) * N + lx * ((v >> 1) & 1) * N + lx * lx * (v >> 2) * N]
    flag = np.zeros(m.n)
    flag[mask - 1] = 1.0
    idx = np.arange(m.n, dtype=np.float64)
    _, (x2, y2, z2, g2, r2, f2, i2) = meshgen.reorient(lx, ev, [m.x, m.y, m.z, m.gid, r, flag, idx], rng)
    m2 = orc.mesh_general(x2, y2, z2, g2.astype(np.int64), lx)
    mask2 = (np.nonzero(f2)[0] + 1).astype(np.int32)
    z = schwarz_ref.apply_general(m2, r2, h1=0.7, mask=mask2, coarse=True)
    assert np.allclose(z, ref[i2.astype(np.int64)], rtol=1e-11, atol=1e-12 * np.abs(ref).max())


def test_ogrid_symmetric_and_preconditions(orc, dofmap):
    ev, xyz, zones = meshgen.ogrid_pipe(2, 1, 2)
    lx = 4
    gid = dofmap.dofmap_from_vertices(ev, lx)
    m = orc.mesh_general(*meshgen.nodes_from_vertices(xyz, lx), gid, lx)
    mask = zone_mask(lx, gid, [(e - 1, f - 1) for e, f, _, lab, *_ in zones if lab == 2])
    rng = np.random.default_rng(7)
    u = orc.apply_mask_zero(orc.gs_op(m, rng.standard_normal(m.n)) * m.mult, mask)
    v = orc.apply_mask_zero(orc.gs_op(m, rng.standard_normal(m.n)) * m.mult, mask)
    Mu = schwarz_ref.apply_general(m, u, mask=mask, coarse=True)
    Mv = schwarz_ref.apply_general(m, v, mask=mask, coarse=True)
    a, b = np.sum(m.mult * v * Mu), np.sum(m.mult * u * Mv)
    assert abs(a - b) <= 1e-12 * abs(a) and np.sum(m.mult * u * Mu) > 0
    k, amp, ph = orc.fourier_params(11, 8)
    f = orc.assemble_rhs(m, orc.field_fourier(m, k, amp, ph), mask)
    dinv = orc.jacobi(m, mask=mask)
    xj, itj = pcg(orc, m, f, lambda r: dinv * r, mask)
    xs, its = pcg(orc, m, f, lambda r: schwarz_ref.apply_general(m, r, mask=mask, coarse=True), mask)
    print("O-grid pipe: jacobi", itj, "two-level Schwarz", its)
    assert its < 0.5 * itj
    assert np.linalg.norm(xs - xj) <= 1e-8 * np.linalg.norm(xj)


@pytest.mark.skipif(not os.path.exists(PIPE), reason="reference mesh files not present")
def test_reference_pipe(orc, dofmap, pkg):
    """The reference's debugging pipe (160 elements), outlet Dirichlet."""
    mesh = pkg.nmsh.read(PIPE)
    lx = 4
    gid = dofmap.dofmap_from_vertices(mesh.v_idx.astype(np.int64), lx)
    m = orc.mesh_general(*meshgen.nodes_from_vertices(mesh.xyz, lx), gid, lx)
    assert m.B.min() > 0 and abs(m.B.sum() - 10.0) < 1e-9  # the 10 x 1 x 1 channel
    mask = zone_mask(lx, gid, mesh.zone_faces(labels=[3]))
    k, amp, ph = orc.fourier_params(5, 8)
    f = orc.assemble_rhs(m, orc.field_fourier(m, k, amp, ph), mask)
    dinv = orc.jacobi(m, mask=mask)
    xj, itj = pcg(orc, m, f, lambda r: dinv * r, mask)
    xs, its = pcg(orc, m, f, lambda r: schwarz_ref.apply_general(m, r, mask=mask, coarse=True), mask)
    print("reference pipe: jacobi", itj, "two-level Schwarz", its)
    assert its < 0.5 * itj
    assert np.linalg.norm(xs - xj) <= 1e-8 * np.linalg.norm(xj)


def test_ogrid_orientation_independent(orc, dofmap):
    """On the O-grid pipe (edges shared by three elements), re-orienting
    every element by a random rotation permutes the result, nothing else."""
    ev, xyz, zones = meshgen.ogrid_pipe(2, 1, 2)
    lx = 4
    gid = dofmap.dofmap_from_vertices(ev, lx)
    x, y, z = meshgen.nodes_from_vertices(xyz, lx)
    m = orc.mesh_general(x, y, z, gid, lx)
    mask = zone_mask(lx, gid, [(e - 1, f - 1) for e, f, _, lab, *_ in zones if lab == 2])
    rng = np.random.default_rng(11)
    r = orc.apply_mask_zero(orc.gs_op(m, rng.standard_normal(m.n)) * m.mult, mask)
    ref = schwarz_ref.apply_general(m, r, h1=1.0, mask=mask, coarse=True)
    flag = np.zeros(m.n)
    flag[mask - 1] = 1.0
    idx = np.arange(m.n, dtype=np.float64)
    _, (x2, y2, z2, g2, r2, f2, i2) = meshgen.reorient(lx, ev, [x, y, z, gid, r, flag, idx], rng)
    m2 = orc.mesh_general(x2, y2, z2, g2.astype(np.int64), lx)
    assert m2.B.min() > 0
    mask2 = (np.nonzero(f2)[0] + 1).astype(np.int32)
    z2v = schwarz_ref.apply_general(m2, r2, h1=1.0, mask=mask2, coarse=True)
    assert np.allclose(z2v, ref[i2.astype(np.int64)], rtol=1e-11, atol=1e-12 * np.abs(ref).max())
