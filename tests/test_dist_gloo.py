"""The element-partitioned solve (neko-top_gb300/dist.py) on two CPU ranks
over gloo, with the oracle as each rank's local operator: the distributed
gather-scatter and multiplicity equal the single-rank ones, and the
distributed Jacobi-PCG reproduces the single-rank oracle solution."""
import importlib.util
import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHAPE = (3, 2, 5, 5)  # ex, ey, ez, lx


def _dist_module():
    spec = importlib.util.spec_from_file_location("ntg_dist", os.path.join(ROOT, "neko-top_gb300", "dist.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


class OracleOps:
    """The rank-local operations of the oracle (CPU, FP64)."""

    def __init__(self, orc, m, mask_local):
        self.orc, self.m, self.mask_local = orc, m, mask_local
        self.n = m.n
        self.gid = torch.from_numpy(m.gid.astype(np.int64))

    def ax(self, w, u):
        w.copy_(torch.from_numpy(self.orc.ax_helm(self.m, u.numpy(), h1c=1.0)))

    def gs(self, u):
        u.copy_(torch.from_numpy(self.orc.gs_op(self.m, u.numpy())))

    def mask(self, u):
        if len(self.mask_local):
            u[torch.from_numpy(self.mask_local - 1)] = 0.0

    def dinv_local(self):
        return torch.from_numpy(self.orc.jacobi(self.m, h1c=1.0, mask=self.mask_local if len(self.mask_local) else None))


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
        m = orc.build_mesh(ex, ey, ez, lx, amp=0.05, seed=11)
        mask = orc.mask_face_xmax(ex, ey, ez, lx)
        part = D.SlabPartition(ex, ey, ez, world, rank)
        ms = orc.mesh_slice(m, part.e0, part.e1)
        lo, hi = part.e0 * lx ** 3, part.e1 * lx ** 3
        mloc = mask[(mask - 1 >= lo) & (mask - 1 < hi)] - lo
        ops = OracleOps(orc, ms, mloc)
        iface = D.Interface(part, ops.gid, lx)
        # distributed gather-scatter and multiplicity
        rng = np.random.default_rng(5)
        u = rng.standard_normal(m.n)
        v = torch.from_numpy(u[lo:hi].copy())
        ops.gs(v)
        iface.exchange_add(v)
        pcg = D.DistPCG(ops, iface, rtol=1e-10, max_iter=5000)
        # the right-hand side: the global one, sliced
        k, a, ph = orc.fourier_params(11, 8)
        f = orc.assemble_rhs(m, orc.field_fourier(m, k, a, ph), mask)
        x = torch.zeros(ms.n, dtype=torch.float64)
        it, r0, r1, fn = pcg.solve(x, torch.from_numpy(f[lo:hi].copy()))
        np.savez(os.path.join(outdir, f"rank{rank}.npz"), gs=v.numpy(), mult=pcg.mult.numpy(), x=x.numpy(),
                 it=it, r1=r1, fn=fn, lo=lo, hi=hi)
    finally:
        torch.distributed.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("world", [2, 3])
def test_distributed_pcg_matches_single_rank(orc, tmp_path, world):
    mp.spawn(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    ex, ey, ez, lx = SHAPE
    m = orc.build_mesh(ex, ey, ez, lx, amp=0.05, seed=11)
    mask = orc.mask_face_xmax(ex, ey, ez, lx)
    rng = np.random.default_rng(5)
    u = rng.standard_normal(m.n)
    gs_ref = orc.gs_op(m, u)
    k, a, ph = orc.fourier_params(11, 8)
    f = orc.assemble_rhs(m, orc.field_fourier(m, k, a, ph), mask)
    x_ref, it_ref, _, _ = orc.cg(m, f, mask=mask, rtol=1e-10, max_iter=5000)
    parts = [dict(np.load(os.path.join(tmp_path, f"rank{r}.npz"))) for r in range(world)]
    gs = np.concatenate([p["gs"] for p in parts])
    mult = np.concatenate([p["mult"] for p in parts])
    x = np.concatenate([p["x"] for p in parts])
    # the sharded gather-scatter: the same sums (order of two partial sums aside)
    assert np.allclose(gs, gs_ref, rtol=1e-13, atol=1e-13 * np.abs(gs_ref).max())
    assert np.array_equal(mult, m.mult)
    # every rank agrees on the iteration count; the solution matches the single-rank one
    its = {int(p["it"]) for p in parts}
    assert len(its) == 1 and abs(its.pop() - it_ref) <= 2
    assert np.linalg.norm(x - x_ref) <= 1e-8 * np.linalg.norm(x_ref)
    assert all(float(p["r1"]) <= 1e-10 * float(p["fn"]) * (1 + 1e-9) for p in parts)


def _worker_general(rank, world, port, outdir):
    """A random (non-contiguous) element partition with the GeneralInterface."""
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import sys
    sys.path.insert(0, ROOT)
    from oracle import oracle as orc
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    try:
        D = _dist_module()
        ex, ey, ez, lx = SHAPE
        m = orc.build_mesh(ex, ey, ez, lx, amp=0.05, seed=11)
        mask = orc.mask_face_xmax(ex, ey, ez, lx)
        owner = np.random.default_rng(99).integers(0, world, m.nelv)
        elems = np.nonzero(owner == rank)[0]
        ms = orc.mesh_subset(m, elems)
        nl = lx ** 3
        sel = (elems[:, None] * nl + np.arange(nl)[None, :]).ravel()
        pos = np.full(m.n, -1)
        pos[sel] = np.arange(sel.size)
        mloc = (pos[mask - 1][pos[mask - 1] >= 0] + 1).astype(np.int32)
        ops = OracleOps(orc, ms, mloc)
        iface = D.GeneralInterface(ops.gid)
        rng = np.random.default_rng(5)
        u = rng.standard_normal(m.n)
        v = torch.from_numpy(u[sel].copy())
        ops.gs(v)
        iface.exchange_add(v)
        pcg = D.DistPCG(ops, iface, rtol=1e-10, max_iter=5000)
        k, a, ph = orc.fourier_params(11, 8)
        f = orc.assemble_rhs(m, orc.field_fourier(m, k, a, ph), mask)
        x = torch.zeros(ms.n, dtype=torch.float64)
        it, r0, r1, fn = pcg.solve(x, torch.from_numpy(f[sel].copy()))
        np.savez(os.path.join(outdir, f"grank{rank}.npz"), gs=v.numpy(), mult=pcg.mult.numpy(), x=x.numpy(),
                 it=it, sel=sel, gid=ms.gid)
    finally:
        torch.distributed.destroy_process_group()


def test_general_partition_matches_single_rank(orc, tmp_path):
    world = 3
    mp.spawn(_worker_general, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    ex, ey, ez, lx = SHAPE
    m = orc.build_mesh(ex, ey, ez, lx, amp=0.05, seed=11)
    mask = orc.mask_face_xmax(ex, ey, ez, lx)
    u = np.random.default_rng(5).standard_normal(m.n)
    gs_ref = orc.gs_op(m, u)
    k, a, ph = orc.fourier_params(11, 8)
    f = orc.assemble_rhs(m, orc.field_fourier(m, k, a, ph), mask)
    x_ref, it_ref, _, _ = orc.cg(m, f, mask=mask, rtol=1e-10, max_iter=5000)
    parts = [dict(np.load(os.path.join(tmp_path, f"grank{r}.npz"))) for r in range(world)]
    gs, mult, x = np.zeros(m.n), np.zeros(m.n), np.zeros(m.n)
    for p in parts:
        gs[p["sel"]], mult[p["sel"]], x[p["sel"]] = p["gs"], p["mult"], p["x"]
    assert np.allclose(gs, gs_ref, rtol=1e-13, atol=1e-13 * np.abs(gs_ref).max())
    assert np.array_equal(mult, m.mult)
    # every copy of a node, on every rank, holds the same bits
    for g in np.unique(m.gid)[:: max(1, len(np.unique(m.gid)) // 2000)]:
        vals = np.concatenate([p["gs"][p["gid"] == g] for p in parts])
        assert vals.min() == vals.max()
    its = {int(p["it"]) for p in parts}
    assert len(its) == 1 and abs(its.pop() - it_ref) <= 2
    assert np.linalg.norm(x - x_ref) <= 1e-8 * np.linalg.norm(x_ref)


def test_rcb_partition_is_balanced_and_compact(orc):
    D = _dist_module()
    m = orc.build_mesh(6, 5, 4, 3, amp=0.05, seed=1)
    cen = np.stack([a.reshape(m.nelv, -1).mean(1) for a in (m.x, m.y, m.z)], 1)
    for world in (1, 2, 3, 5, 8):
        owner = D.rcb_partition(cen, world)
        counts = np.bincount(owner, minlength=world)
        assert counts.sum() == m.nelv and counts.max() - counts.min() <= 1
    # two parts of a 6x5x4 box: a cut across x (the longest extent)
    owner = D.rcb_partition(cen, 2)
    assert set(np.unique(owner[cen[:, 0] < 0.45])) == {0} and set(np.unique(owner[cen[:, 0] > 0.55])) == {1}
