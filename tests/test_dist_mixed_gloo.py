"""The fast solver sharded (neko-top_gb300/dist.py: DistMixedCG with the
two-level DistSchwarz) on CPU ranks over gloo, with the oracle as each
rank's local operator and the numpy Schwarz restatement as each rank's
one-level part on its ghosted slab.  One rank and two ranks take the same
iterations (within 2) and both match the single-rank oracle FP64 solution
to 1e-10; the FP64 residual, re-evaluated by the oracle, meets the
tolerance."""
import importlib.util
import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHAPE = (3, 2, 6, 4)  # ex, ey, ez, lx: two ranks own three element planes each
RTOL = 1e-12


def _dist_module():
    spec = importlib.util.spec_from_file_location("ntg_dist", os.path.join(ROOT, "neko-top_gb300", "dist.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


class OracleOps:
    """Rank-local operator of the oracle: FP64 and FP32 Ax, gs, mask."""

    def __init__(self, orc, m, mask_local):
        self.orc, self.m, self.mask_local = orc, m, mask_local
        self.n = m.n
        self.gid = torch.from_numpy(m.gid.astype(np.int64))

    def ax(self, w, u):
        w.copy_(torch.from_numpy(self.orc.ax_helm(self.m, u.numpy(), h1c=1.0)))

    def ax32(self, w, u):
        w.copy_(torch.from_numpy(self.orc.ax_helm_f32(self.m, u.numpy(), h1c=1.0)))

    def gs(self, u):
        u.copy_(torch.from_numpy(self.orc.gs_op(self.m, u.double().numpy())).to(u.dtype))

    def mask(self, u):
        if len(self.mask_local):
            u[torch.from_numpy(self.mask_local - 1)] = 0.0


class OracleGhostOps:
    """The one-level Schwarz (numpy restatement) on a rank's ghosted slab."""

    def __init__(self, m_g, box, mask_g):
        from oracle import schwarz_ref
        self.ref, self.m, self.box, self.mask = schwarz_ref, m_g, box, mask_g

    def schwarz(self, z, r):
        out = self.ref.apply(self.m, r.double().numpy(), self.box, h1=1.0, h2=None,
                             mask=self.mask if len(self.mask) else None)
        z.copy_(torch.from_numpy(out).to(z.dtype))


def _local_mask(mask, lo, hi):
    return (mask[(mask - 1 >= lo) & (mask - 1 < hi)] - lo).astype(np.int32)


def _worker(rank, world, port, outdir):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import sys
    sys.path.insert(0, ROOT)
    from oracle import oracle as orc
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    try:
        D = _dist_module()
        ex, ey, ez, lx = SHAPE
        l3 = lx ** 3
        m = orc.build_mesh(ex, ey, ez, lx, amp=0.05, seed=13)
        mask = orc.mask_face_xmax(ex, ey, ez, lx)
        part = D.SlabPartition(ex, ey, ez, world, rank)
        ms = orc.mesh_slice(m, part.e0, part.e1)
        lo, hi = part.e0 * l3, part.e1 * l3
        ops = OracleOps(orc, ms, _local_mask(mask, lo, hi))
        iface = D.Interface(part, ops.gid, lx)
        ones = torch.ones(ops.n, dtype=torch.float64)
        ops.gs(ones)
        iface.exchange_add(ones)
        mult = 1.0 / ones
        ghost = D.GhostSlab(part, lx)
        m_g = orc.mesh_slice(m, ghost.gz0 * ex * ey, ghost.gz1 * ex * ey)
        gops = OracleGhostOps(m_g, (ex, ey, ghost.gz1 - ghost.gz0),
                              _local_mask(mask, ghost.gz0 * ex * ey * l3, ghost.gz1 * ex * ey * l3))
        hl = D.element_lengths(torch.from_numpy(ms.x), torch.from_numpy(ms.y), torch.from_numpy(ms.z), lx)
        coarse = D.CoarseQ1((ex, ey, ez), D.slab_mean_lengths(part, hl), 1.0, 0.0,
                            D.dirichlet_faces_dist(part, ops.mask_local, lx), lx)
        pc = D.DistSchwarz(part, ghost, gops, ops, mult, coarse)
        k, a, ph = orc.fourier_params(13, 8)
        f = orc.assemble_rhs(m, orc.field_fourier(m, k, a, ph), mask)
        x = torch.zeros(ms.n, dtype=torch.float64)
        cg = D.DistMixedCG(ops, iface, pc, mult, rtol=RTOL, delta=1e-3)
        it, r0, r1, fn, nrep = cg.solve(x, torch.from_numpy(f[lo:hi].copy()))
        np.savez(os.path.join(outdir, f"w{world}r{rank}.npz"), x=x.numpy(), it=it, r1=r1, fn=fn, nrep=nrep)
    finally:
        torch.distributed.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_sharded_mixed_schwarz_matches_single_rank(orc, tmp_path):
    ex, ey, ez, lx = SHAPE
    m = orc.build_mesh(ex, ey, ez, lx, amp=0.05, seed=13)
    mask = orc.mask_face_xmax(ex, ey, ez, lx)
    k, a, ph = orc.fourier_params(13, 8)
    f = orc.assemble_rhs(m, orc.field_fourier(m, k, a, ph), mask)
    x_ref, it_ref, _, _ = orc.cg(m, f, mask=mask, rtol=1e-14, max_iter=20000)
    res = {}
    for world in (1, 2):
        mp.spawn(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
        parts = [dict(np.load(os.path.join(tmp_path, f"w{world}r{r}.npz"))) for r in range(world)]
        x = np.concatenate([p["x"] for p in parts])
        its = {int(p["it"]) for p in parts}
        assert len(its) == 1, its  # every rank took the same iterations
        res[world] = (its.pop(), x)
        err = np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref)
        r = f - orc.op_apply(m, x, mask=mask)
        rel = np.sqrt(orc.glsc3(r, r, m.mult)) / np.sqrt(orc.glsc3(f, f, m.mult))
        print(f"world {world}: {res[world][0]} iterations, {int(parts[0]['nrep'])} FP64 residuals, "
              f"error vs the oracle {err:.2e}, residual {rel:.2e} (oracle Jacobi-PCG: {it_ref} iterations)")
        assert err <= 1e-10
        assert rel <= 1.5 * RTOL
    assert abs(res[1][0] - res[2][0]) <= 2
    assert np.linalg.norm(res[1][1] - res[2][1]) <= 1e-10 * np.linalg.norm(res[1][1])
