"""Element-partitioned (sharded) solves across ranks.

The spectral-element path shards by element partition: each rank owns a
contiguous range of elements and runs the operator, its rank-local
gather-scatter and the preconditioner on them; the only exchanges are the
partial sums of the global nodes on the partition interface (after each
rank-local gather-scatter) and the scalar sums of the dot products.  This
is Neko's own decomposition (gs_t's shared-node exchange between MPI ranks
and the MPI_Allreduce of glsc3) without MPI: torch.distributed (NCCL for
CUDA tensors, gloo for CPU tensors).

  SlabPartition   structured boxes cut into slabs of whole element planes
                  along z, so each rank's elements are contiguous
  Interface       the exchange plan: per neighbour slab, the global ids of the
                  shared face sorted on both sides (the buffers line up
                  without sending index lists), one representative local
                  copy per global node to send, every local copy to update
  GeneralInterface  the same for any element partition (shared ids found by
                  one all-gather of the ranks' sorted unique ids)
  rcb_partition   balanced recursive coordinate bisection of the elements
  DistPCG         Jacobi-PCG in FP64 on the distributed operator, every dot
                  weighted by the global multiplicity

Determinism: a shared face node has exactly two owning slabs, and the
exchange adds the partner's partial to the rank's own, a + b on one side and
b + a on the other, so both copies stay bit-identical; dot products gather
the per-rank partial sums and add them in rank order on every rank.

The rank-local operations come from a backend object with

    n              local node count
    gid            int64 tensor of the local nodes' global ids
    ax(w, u)       w = A u on the rank's elements (unassembled)
    gs(u)          rank-local direct stiffness summation, in place
    mask(u)        zero the rank's Dirichlet nodes, in place
    dinv_local()   inverse of the rank-locally assembled diagonal (1 on masked nodes)

`LibraryOps` is the backend over this package's CUDA library (one coef_t per
rank); tests drive the same host logic with the oracle on CPU ranks.
"""
from __future__ import annotations

import math

import torch
import torch.distributed as dist


class SlabPartition:
    """Rank `rank` of `world` owns the element planes [z0, z1) of an
    ex x ey x ez box numbered x fastest (elements [e0, e1))."""

    def __init__(self, ex, ey, ez, world, rank):
        if not 0 <= rank < world or world > ez:
            raise ValueError("need 0 <= rank < world <= ez (at least one element plane per rank)")
        base, extra = divmod(ez, world)
        self.z0 = rank * base + min(rank, extra)
        self.z1 = self.z0 + base + (1 if rank < extra else 0)
        self.ex, self.ey, self.ez, self.world, self.rank = ex, ey, ez, world, rank
        self.e0, self.e1 = ex * ey * self.z0, ex * ey * self.z1

    @property
    def nelv(self):
        return self.e1 - self.e0


class Interface:
    """Exchange plan of a slab with its neighbours (see the module docstring)."""

    def __init__(self, part: SlabPartition, gid: torch.Tensor, lx: int):
        N, lx2, lx3 = lx - 1, lx * lx, lx ** 3
        planes = part.z1 - part.z0
        per_plane = part.ex * part.ey * lx3
        self.faces = []  # (neighbour rank, all local indices on the face, slot of each, one index per slot)
        dev = gid.device
        for nb, plane, k in ((part.rank - 1, 0, 0), (part.rank + 1, planes - 1, N)):
            if nb < 0 or nb >= part.world:
                continue
            # local nodes with k fixed in every element of the boundary plane
            el = torch.arange(part.ex * part.ey, device=dev)
            q = torch.arange(lx2, device=dev)
            idx = (plane * per_plane + el[:, None] * lx3 + k * lx2 + q[None, :]).reshape(-1)
            g = gid[idx]
            uniq, slot = torch.unique(g, sorted=True, return_inverse=True)
            rep = torch.full((uniq.numel(),), torch.iinfo(torch.int64).max, dtype=torch.int64, device=dev)
            rep = rep.scatter_reduce(0, slot, idx, reduce="amin")
            self.faces.append((nb, idx, slot, rep, uniq))

    def exchange_add(self, u: torch.Tensor):
        """u holds rank-locally assembled values; add each shared node's
        partial from the neighbouring slab (in place)."""
        if not self.faces:
            return u
        sends, recvs, reqs = [], [], []
        for nb, idx, slot, rep, _ in self.faces:
            s = u[rep].contiguous()
            r = torch.empty_like(s)
            reqs.append(dist.isend(s, nb))
            reqs.append(dist.irecv(r, nb))
            sends.append(s)
            recvs.append(r)
        for q in reqs:
            q.wait()
        for (nb, idx, slot, rep, _), r in zip(self.faces, recvs):
            u[idx] = u[idx] + r[slot]
        return u


def rcb_partition(centroids, world):
    """Recursive coordinate bisection of elements (centroids: E x 3 numpy)
    into `world` parts of sizes differing by at most one: split along the
    longest extent at the weighted median, recursing with the rank counts
    floor(w/2) and ceil(w/2).  Returns the owner rank of each element."""
    import numpy as np
    c = np.asarray(centroids, dtype=np.float64)
    owner = np.empty(c.shape[0], dtype=np.int64)

    def split(ids, r0, w):
        if w == 1:
            owner[ids] = r0
            return
        wl = w // 2
        pts = c[ids]
        d = int(np.argmax(pts.max(0) - pts.min(0))) if len(ids) else 0
        order = ids[np.argsort(pts[:, d], kind="stable")]
        cut = (len(ids) * wl) // w
        split(order[:cut], r0, wl)
        split(order[cut:], r0 + wl, w - wl)

    split(np.arange(c.shape[0]), 0, int(world))
    return owner


class GeneralInterface:
    """Exchange plan for any element partition (the elements a rank owns need
    not be contiguous or slab-shaped; meshes numbered by dofmap.py).  The
    ranks all-gather their sorted unique global ids once; the ids a rank
    shares with rank q are the sorted intersection, the same list on both
    sides, so the exchange buffers line up without index lists.
    exchange_add sums the partials of a node's owners in ascending rank
    order on every owner, so all copies stay bit-identical whatever the
    number of owners.  Same interface as Interface."""

    def __init__(self, gid: torch.Tensor):
        world, rank = dist.get_world_size(), dist.get_rank()
        dev = gid.device
        uniq, inv = torch.unique(gid, sorted=True, return_inverse=True)
        size = torch.tensor([uniq.numel()], dtype=torch.int64, device=dev)
        sizes = [torch.zeros_like(size) for _ in range(world)]
        dist.all_gather(sizes, size)
        cap = int(max(int(s.item()) for s in sizes))
        pad = torch.full((cap,), -1, dtype=torch.int64, device=dev)
        pad[: uniq.numel()] = uniq
        allg = [torch.empty_like(pad) for _ in range(world)]
        dist.all_gather(allg, pad)
        self.rank, self.faces = rank, []
        for q in range(world):
            if q == rank:
                continue
            other = allg[q][: int(sizes[q].item())]
            shared = uniq[torch.isin(uniq, other)]  # sorted, identical on both sides
            if shared.numel() == 0:
                continue
            on = torch.isin(gid, shared)
            idx = torch.nonzero(on).squeeze(1)
            slot = torch.searchsorted(shared, gid[idx])
            rep = torch.full((shared.numel(),), torch.iinfo(torch.int64).max, dtype=torch.int64, device=dev)
            rep = rep.scatter_reduce(0, slot, idx, reduce="amin")
            self.faces.append((q, idx, slot, rep, shared))

    def exchange_add(self, u: torch.Tensor):
        if not self.faces:
            return u
        recvs, reqs = [], []
        for q, idx, slot, rep, _ in self.faces:
            s = u[rep].contiguous()
            r = torch.empty_like(s)
            reqs.append(dist.isend(s, q))
            reqs.append(dist.irecv(r, q))
            recvs.append((s, r))
        for rq in reqs:
            rq.wait()
        tot = torch.zeros_like(u)
        own = False
        for (q, idx, slot, rep, _), (_, r) in sorted(zip(self.faces, recvs), key=lambda t: t[0][0]):
            if not own and q > self.rank:
                tot += u
                own = True
            tot[idx] += r[slot]
        if not own:
            tot += u
        u.copy_(tot)
        return u


def dist_dot(a: torch.Tensor, b: torch.Tensor, w: torch.Tensor) -> float:
    """sum(a * b * w) over all ranks, per-rank partials added in rank order."""
    local = torch.sum(a * b * w).reshape(1).to(torch.float64)
    world = dist.get_world_size()
    parts = [torch.zeros_like(local) for _ in range(world)]
    dist.all_gather(parts, local)
    total = 0.0
    for p in parts:
        total += float(p.item())
    return total


class DistPCG:
    """FP64 Jacobi-PCG on the element-partitioned operator (the plain
    drop-in, sharded).  solve(x, f) mirrors ksp_t%solve: f is the assembled,
    masked right-hand side (rank slices), x the initial guess, updated in
    place; returns (iterations, ||r0||, ||r||, ||f||) in the unique-node norm."""

    def __init__(self, ops, iface: Interface, rtol=1e-10, abstol=0.0, max_iter=10000):
        self.ops, self.iface = ops, iface
        self.rtol, self.abstol, self.max_iter = rtol, abstol, max_iter
        ones = torch.ones(ops.n, dtype=torch.float64, device=ops.gid.device)
        ops.gs(ones)
        iface.exchange_add(ones)
        self.mult = 1.0 / ones  # 1 / global multiplicity
        d = 1.0 / ops.dinv_local()
        iface.exchange_add(d)
        dinv = 1.0 / d
        mk = torch.zeros_like(dinv)
        ops.mask(mk.fill_(1.0))  # masked nodes become 0
        self.dinv = torch.where(mk == 0.0, torch.ones_like(dinv), dinv)

    def apply(self, w, u):
        """w = mask(gs(A u)) across ranks."""
        self.ops.ax(w, u)
        self.ops.gs(w)
        self.iface.exchange_add(w)
        self.ops.mask(w)
        return w

    def solve(self, x, f):
        dot = lambda a, b: dist_dot(a, b, self.mult)
        w = torch.empty_like(x)
        ff = dot(f, f)
        if float(dot(x, x)) != 0.0:
            r = f - self.apply(w, x)
        else:
            r = f.clone()
        rr = dot(r, r)
        r0 = math.sqrt(rr)
        tol = max(self.abstol, self.rtol * math.sqrt(ff))
        z = self.dinv * r
        p = z.clone()
        rz = dot(r, z)
        it = 0
        while math.sqrt(rr) > tol and it < self.max_iter:
            self.apply(w, p)
            alpha = rz / dot(p, w)
            x.add_(p, alpha=alpha)
            r.sub_(w, alpha=alpha)
            rr = dot(r, r)
            it += 1
            if math.sqrt(rr) <= tol:
                break
            z = self.dinv * r
            rz_new = dot(r, z)
            p.mul_(rz_new / rz).add_(z)
            rz = rz_new
        return it, r0, math.sqrt(rr), math.sqrt(ff)


class LibraryOps:
    """Backend over the CUDA library for one rank: a coef_t of the rank's
    elements (built from its slice of the coordinates and global ids) with
    its Dirichlet mask and coefficients set."""

    def __init__(self, coef, gid):
        from . import api
        self.coef, self.gid, self.n = coef, gid, coef.n
        self._ax = api.ax_helm_t()
        self._gs = api.gs_t(coef)
        self._jac = api.jacobi_t(coef)
        self._api = api

    def ax(self, w, u):
        self._ax.compute(w, u, self.coef)

    def gs(self, u):
        self._gs.op(u)

    def mask(self, u):
        self._api.bc_list_apply_scalar(self.coef, u)

    def dinv_local(self):
        self._jac.update()
        return self._jac.dinv()
