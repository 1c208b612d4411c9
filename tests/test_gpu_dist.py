"""The element-partitioned solve with the CUDA library as each rank's
backend (neko-top_gb300/dist.py, LibraryOps): two slabs of one box held in
one process with the interface exchange done by plain copies (no collective:
one GPU), and a one-rank NCCL process group driving DistPCG."""
import os
import socket

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

SHAPE = (3, 2, 4, 8)


def slab_coef(pkg, full, part, lx):
    lo, hi = part.e0 * lx ** 3, part.e1 * lx ** 3
    x, y, z, gid = (a[lo:hi].contiguous() for a in full)
    c = pkg.coef_t(part.nelv, lx, x, y, z, gid)
    return c, gid, lo, hi


def test_two_slabs_exchange_matches_full_mesh(pkg, dev):
    import importlib
    D = importlib.import_module(pkg.__name__ + ".dist")
    ex, ey, ez, lx = SHAPE
    full = pkg.build_box(ex, ey, ez, lx, amp=0.05, seed=3, device=dev)
    cf = pkg.coef_t(ex * ey * ez, lx, *full)
    n = cf.n
    u = torch.randn(n, dtype=torch.float64, device=dev)
    w_full = torch.empty_like(u)
    pkg.ax_helm_t().compute(w_full, u, cf)
    pkg.gs_t(cf).op(w_full)
    ranks = []
    for r in range(2):
        part = D.SlabPartition(ex, ey, ez, 2, r)
        c, gid, lo, hi = slab_coef(pkg, full, part, lx)
        ops = D.LibraryOps(c, gid)
        w = torch.empty(c.n, dtype=torch.float64, device=dev)
        ops.ax(w, u[lo:hi].contiguous())
        ops.gs(w)
        ranks.append((part, ops, D.Interface(part, gid, lx), w, lo, hi))
    outs = []
    for r, (part, ops, iface, w, lo, hi) in enumerate(ranks):
        v = w.clone()
        for nb, idx, slot, rep, uniq in iface.faces:
            pf = [f for f in ranks[nb][2].faces if f[0] == r][0]
            assert torch.equal(pf[4], uniq)
            v[idx] = v[idx] + ranks[nb][3][pf[3]][slot]
        outs.append(v)
    w_dist = torch.cat(outs)
    torch.cuda.synchronize()
    err = (w_dist - w_full).abs().max().item() / w_full.abs().max().item()
    assert err < 1e-14


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_one_rank_distributed_pcg(pkg, orc, dev):
    import importlib
    import torch.distributed as dist
    D = importlib.import_module(pkg.__name__ + ".dist")
    ex, ey, ez, lx = SHAPE
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(_port())
    dist.init_process_group("nccl", rank=0, world_size=1, device_id=dev)
    try:
        m = orc.build_mesh(ex, ey, ez, lx, amp=0.05, seed=3)
        mask = orc.mask_face_xmax(ex, ey, ez, lx)
        full = pkg.build_box(ex, ey, ez, lx, amp=0.05, seed=3, device=dev)
        part = D.SlabPartition(ex, ey, ez, 1, 0)
        c, gid, lo, hi = slab_coef(pkg, full, part, lx)
        c.set_mask(torch.from_numpy(mask).to(dev), base=1)
        c.set_coefs(h1c=1.0, ifh2=False)
        k, a, ph = orc.fourier_params(3, 8)
        f = orc.assemble_rhs(m, orc.field_fourier(m, k, a, ph), mask)
        pcg = D.DistPCG(D.LibraryOps(c, gid), D.Interface(part, gid, lx), rtol=1e-10, max_iter=5000)
        x = torch.zeros(m.n, dtype=torch.float64, device=dev)
        it, r0, r1, fn = pcg.solve(x, torch.from_numpy(f).to(dev))
        x_ref, it_ref, _, _ = orc.cg(m, f, mask=mask, rtol=1e-10, max_iter=5000)
        assert abs(it - it_ref) <= 2 and r1 <= 1e-10 * fn * (1 + 1e-9)
        xn = x.cpu().numpy()
        assert np.linalg.norm(xn - x_ref) <= 1e-8 * np.linalg.norm(x_ref)
    finally:
        dist.destroy_process_group()


def test_one_rank_sharded_mixed_schwarz(pkg, orc, dev):
    """The sharded fast solver (DistMixedCG + DistSchwarz) with the CUDA
    library as the rank's backend, one NCCL rank: the one-level Schwarz on
    the ghosted slab (here the whole box), the coarse level in the host
    logic; the solution matches the oracle's FP64 solution."""
    import importlib
    import torch.distributed as dist
    D = importlib.import_module(pkg.__name__ + ".dist")
    ex, ey, ez, lx = SHAPE
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(_port())
    dist.init_process_group("nccl", rank=0, world_size=1, device_id=dev)
    try:
        m = orc.build_mesh(ex, ey, ez, lx, amp=0.05, seed=3)
        mask = orc.mask_face_xmax(ex, ey, ez, lx)
        full = pkg.build_box(ex, ey, ez, lx, amp=0.05, seed=3, device=dev)
        part = D.SlabPartition(ex, ey, ez, 1, 0)
        c, gid, lo, hi = slab_coef(pkg, full, part, lx)
        mt = torch.from_numpy(mask).to(dev)
        c.set_mask(mt, base=1)
        c.set_coefs(h1c=1.0, ifh2=False)
        ops = D.LibraryOps(c, gid)
        iface = D.Interface(part, gid, lx)
        ones = torch.ones(c.n, dtype=torch.float64, device=dev)
        ops.gs(ones)
        iface.exchange_add(ones)
        mult = 1.0 / ones
        ghost = D.GhostSlab(part, lx)
        cg_, gid_g, _, _ = slab_coef(pkg, full, part, lx)  # one rank: the ghosted slab is the box
        cg_.set_mask(mt, base=1)
        cg_.set_coefs(h1c=1.0, ifh2=False)
        gops = D.LibraryGhostOps(cg_, (ex, ey, ghost.gz1 - ghost.gz0))
        hl = D.element_lengths(c.x, c.y, c.z, lx)
        coarse = D.CoarseQ1((ex, ey, ez), D.slab_mean_lengths(part, hl), 1.0, 0.0,
                            D.dirichlet_faces_dist(part, mask, lx, dev), lx, device=dev)
        pc = D.DistSchwarz(part, ghost, gops, ops, mult, coarse)
        k, a, ph = orc.fourier_params(3, 8)
        f = orc.assemble_rhs(m, orc.field_fourier(m, k, a, ph), mask)
        x = torch.zeros(m.n, dtype=torch.float64, device=dev)
        solver = D.DistMixedCG(ops, iface, pc, mult, rtol=1e-12, delta=1e-3)
        it, r0, r1, fn, nrep = solver.solve(x, torch.from_numpy(f).to(dev))
        x_ref, it_ref, _, _ = orc.cg(m, f, mask=mask, rtol=1e-14, max_iter=20000)
        xn = x.cpu().numpy()
        err = np.linalg.norm(xn - x_ref) / np.linalg.norm(x_ref)
        print("sharded mixed Schwarz, one rank:", it, "iterations,", nrep, "FP64 residuals, error", err)
        assert r1 <= 1e-12 * fn * (1 + 1e-9)
        assert err <= 1e-10
    finally:
        dist.destroy_process_group()
