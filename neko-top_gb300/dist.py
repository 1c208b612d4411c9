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
  GhostSlab, CoarseQ1, DistSchwarz, DistMixedCG
                  the fast solver sharded: FP32 PCG with FP64 reliable updates
                  and the two-level Schwarz on slab ranks (ghost planes for
                  the overlap, a global coarse level; see below)

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

import numpy as np
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

    def ax32(self, w, u):  # FP32 operator (the library picks it from the dtype)
        self._ax.compute(w, u, self.coef)

    def gs(self, u):
        self._gs.op(u)

    def mask(self, u):
        self._api.bc_list_apply_scalar(self.coef, u)

    def dinv_local(self):
        self._jac.update()
        return self._jac.dinv()


class LibraryGhostOps:
    """The one-level Schwarz of the CUDA library on a rank's ghosted slab:
    a coef_t of the slab's element planes plus the ghost planes (a box of
    ex x ey x planes elements, x fastest), its mask and coefficients set by
    the caller, and a schwarz_t without the coarse level."""

    def __init__(self, coef, box):
        from . import api
        coef.box_dims = tuple(box)
        self.coef = coef
        self.sw = api.schwarz_t(coef, coarse=False)

    def update(self):
        self.sw.update()

    def schwarz(self, z, r):
        self.sw.apply(z, r)


# ---------------------------------------------------------------------------
# The fast solver sharded: FP32-inner / FP64-refined CG with the two-level
# overlapping Schwarz preconditioner on slab ranks.
#
# Halo.  The Schwarz local solve of an element reads its box extended by one
# node layer into every neighbour, and its result reaches one node layer
# into every neighbour.  A slab rank therefore runs the one-level part on its
# own element planes plus up to two ghost planes on each side, filled from
# the neighbouring slabs: the first ghost plane's elements contribute to the
# rank's boundary nodes, and their extended inputs reach into the second
# ghost plane.  The results on the rank's own nodes then equal the
# single-rank ones (the second ghost plane's results, which miss their outer
# inputs, only land on ghost nodes and are dropped).  Every rank must own at
# least two planes.  The coarse level (Q1 on the element vertices) is global
# and small: each rank restricts its own elements' residual, the vertex-grid
# partials are summed over ranks, every rank solves the same separable
# coarse problem, and each prolongs onto its own elements.
# ---------------------------------------------------------------------------


class GhostSlab:
    """A slab rank's element planes plus `g` ghost planes on each side
    (clipped to the box).  fill(u) returns the ghosted array with the ghost
    planes received from the neighbouring slabs; own is the slice of the
    rank's elements in it."""

    def __init__(self, part: SlabPartition, lx: int, g: int = 2):
        if part.world > 1 and part.z1 - part.z0 < g:
            raise ValueError(f"every slab rank must own at least {g} element planes")
        self.part, self.g = part, g
        self.per = part.ex * part.ey * lx ** 3
        self.gz0, self.gz1 = max(0, part.z0 - g), min(part.ez, part.z1 + g)
        self.lo, self.hi = part.z0 - self.gz0, self.gz1 - part.z1
        own_planes = part.z1 - part.z0
        self.own = slice(self.lo * self.per, (self.lo + own_planes) * self.per)
        self.n = (self.gz1 - self.gz0) * self.per

    def fill(self, u: torch.Tensor) -> torch.Tensor:
        p, per, g = self.part, self.per, self.g
        ug = torch.zeros(self.n, dtype=u.dtype, device=u.device)
        ug[self.own] = u
        reqs, bufs = [], []
        if self.lo:  # my first g planes go down, the lower neighbour's last planes come up
            s = u[: g * per].contiguous()
            r = torch.empty(self.lo * per, dtype=u.dtype, device=u.device)
            reqs += [dist.isend(s, p.rank - 1), dist.irecv(r, p.rank - 1)]
            bufs.append((slice(0, self.lo * per), r, s))
        if self.hi:
            s = u[u.numel() - g * per:].contiguous()
            r = torch.empty(self.hi * per, dtype=u.dtype, device=u.device)
            reqs += [dist.isend(s, p.rank + 1), dist.irecv(r, p.rank + 1)]
            bufs.append((slice(self.n - self.hi * per, self.n), r, s))
        for q in reqs:
            q.wait()
        for sl, r, _ in bufs:
            ug[sl] = r
        return ug


def element_lengths(x, y, z, lx):
    """Mean distance between opposite faces of each element along r, s, t
    (E x 3, float64), from the node coordinates (Neko layout)."""
    E = x.numel() // lx ** 3
    X = torch.stack([x, y, z]).to(torch.float64).reshape(3, E, lx, lx, lx)  # (d, e, k, j, i)
    out = []
    for a0, a1 in ((np.s_[..., 0], np.s_[..., -1]),
                   (np.s_[:, :, :, 0, :], np.s_[:, :, :, -1, :]),
                   (np.s_[:, :, 0, :, :], np.s_[:, :, -1, :, :])):
        d = X[a1] - X[a0]
        out.append(torch.sqrt((d * d).sum(0)).reshape(E, -1).mean(1))
    return torch.stack(out, 1)


def _gll_nodes(lx):
    """GLL points on [-1, 1] (Newton on (1 - x^2) P_N'(x) from Chebyshev points)."""
    N = lx - 1
    x = -np.cos(np.pi * np.arange(lx) / N)
    for _ in range(100):
        p0, p1 = np.ones(lx), x.copy()
        for k in range(2, N + 1):
            p0, p1 = p1, ((2 * k - 1) * x * p1 - (k - 1) * p0) / k
        dx = (x * p1 - p0) / (lx * p1)
        x = x - dx
        if np.abs(dx).max() < 1e-15:
            break
    return x


class CoarseQ1:
    """The coarse level of the two-level Schwarz on the global vertex grid of
    an ex x ey x ez box (the library's coarse part, restated in torch for the
    sharded solver): restriction P^T (r mult) by the trilinear vertex basis
    at the GLL nodes, the separable Q1 operator
      A_c = h1 (Mz x My x Kx + Mz x Ky x Mx + Kz x My x Mx) + h2 Mz x My x Mx
    from the slab-mean element lengths with Dirichlet vertices removed on
    fully masked faces, solved by fast diagonalisation (the constant null
    mode of an all-Neumann box dropped), and prolongation P."""

    def __init__(self, E, slab_lengths, h1, h2, dirichlet, lx, device="cpu", dtype=torch.float32):
        self.E, self.lx = tuple(E), lx
        xi = _gll_nodes(lx)
        phi = np.stack([0.5 * (1 - xi), 0.5 * (1 + xi)])
        self.phi = torch.tensor(phi, dtype=dtype, device=device)
        self.S, self.act, lams = [], [], []
        for d in range(3):
            hs = np.asarray(slab_lengths[d], dtype=np.float64)
            nv = E[d] + 1
            K, M = np.zeros((nv, nv)), np.zeros((nv, nv))
            for s, h in enumerate(hs):
                K[s:s + 2, s:s + 2] += np.array([[1.0, -1.0], [-1.0, 1.0]]) / h
                M[s:s + 2, s:s + 2] += np.array([[2.0, 1.0], [1.0, 2.0]]) * h / 6.0
            a = np.arange(1 if dirichlet[2 * d] else 0, nv - (1 if dirichlet[2 * d + 1] else 0))
            Ka, Ma = K[np.ix_(a, a)], M[np.ix_(a, a)]
            L = np.linalg.cholesky(Ma)
            Li = np.linalg.inv(L)
            lam, V = np.linalg.eigh(Li @ Ka @ Li.T)
            self.S.append(torch.tensor(Li.T @ V, dtype=torch.float64, device=device))
            self.act.append(torch.tensor(a, device=device))
            lams.append(lam)
        D = h1 * (lams[0][None, None, :] + lams[1][None, :, None] + lams[2][:, None, None]) + h2  # (z, y, x)
        dmin = 1e-6 * (h1 * sum(l.max() for l in lams) + h2)
        Dinv = np.where(np.abs(D) > dmin, 1.0 / np.where(np.abs(D) > dmin, D, 1.0), 0.0)
        self.Dinv = torch.tensor(Dinv, dtype=torch.float64, device=device)
        self.dtype = dtype

    def restrict(self, rw, ecoord):
        """Vertex-grid partials (ez+1, ey+1, ex+1) of the elements with
        weighted residual rw (E_own x lx^3, r times mult) at box positions
        ecoord (E_own x 3: ex, ey, ez)."""
        lx, ph = self.lx, self.phi
        r4 = rw.reshape(-1, lx, lx, lx).to(ph.dtype)
        c = torch.einsum("ekji,ck,bj,ai->ecba", r4, ph, ph, ph).to(torch.float64)  # corners (vz, vy, vx)
        Ex, Ey, Ez = self.E
        g = torch.zeros(Ez + 1, Ey + 1, Ex + 1, dtype=torch.float64, device=rw.device)
        for vz in (0, 1):
            for vy in (0, 1):
                for vx in (0, 1):
                    iz, iy, ix = ecoord[:, 2] + vz, ecoord[:, 1] + vy, ecoord[:, 0] + vx
                    flat = (iz * (Ey + 1) + iy) * (Ex + 1) + ix
                    g.view(-1).index_add_(0, flat, c[:, vz, vy, vx])
        return g

    def solve(self, g):
        """A_c^+ g on the active vertices (zero on Dirichlet vertices)."""
        ax, ay, az = self.act
        Sx, Sy, Sz = self.S
        r = g[az][:, ay][:, :, ax]
        t = torch.einsum("zyx,xa,yb,zc->cba", r, Sx, Sy, Sz) * self.Dinv
        u = torch.einsum("cba,xa,yb,zc->zyx", t, Sx, Sy, Sz)
        out = torch.zeros_like(g)
        out[az[:, None, None], ay[None, :, None], ax[None, None, :]] = u
        return out

    def prolong(self, uc, ecoord):
        """P uc on the elements at ecoord: (E_own x lx^3)."""
        lx, ph = self.lx, self.phi.to(torch.float64)
        corners = torch.stack([torch.stack([torch.stack([uc[ecoord[:, 2] + vz, ecoord[:, 1] + vy, ecoord[:, 0] + vx]
                                                         for vx in (0, 1)], 1) for vy in (0, 1)], 1)
                               for vz in (0, 1)], 1)  # (e, vz, vy, vx)
        z = torch.einsum("ecba,ck,bj,ai->ekji", corners, ph, ph, ph)
        return z.reshape(-1, lx ** 3).reshape(-1).to(self.dtype)


def slab_element_coords(part: SlabPartition, device="cpu"):
    """Box positions (ex, ey, ez) of a slab rank's elements (x fastest)."""
    e = torch.arange(part.e0, part.e1, device=device)
    return torch.stack([e % part.ex, (e // part.ex) % part.ey, e // (part.ex * part.ey)], 1)


def slab_mean_lengths(part: SlabPartition, hl: torch.Tensor):
    """Mean element length of every x-, y- and z-slab of the box, over all
    ranks (sums and counts all-reduced): the coarse operator's 1D lengths."""
    coords = slab_element_coords(part, hl.device)
    out = []
    for d, nd in enumerate((part.ex, part.ey, part.ez)):
        s = torch.zeros(2 * nd, dtype=torch.float64, device=hl.device)
        s[:nd].index_add_(0, coords[:, d], hl[:, d].to(torch.float64))
        s[nd:].index_add_(0, coords[:, d], torch.ones_like(hl[:, d], dtype=torch.float64))
        dist.all_reduce(s)
        out.append((s[:nd] / s[nd:]).cpu().numpy())
    return out


class DistSchwarz:
    """Two-level overlapping Schwarz across slab ranks (FP32): z = mask(
    one-level part on the ghosted slab + P A_c^+ P^T (r mult)).  ghost_ops
    provides schwarz(z_g, r_g): the one-level Schwarz (masked) on the
    rank's ghosted slab as one box."""

    def __init__(self, part: SlabPartition, ghost: GhostSlab, ghost_ops, ops, mult, coarse: CoarseQ1 = None):
        self.part, self.ghost, self.gops, self.ops = part, ghost, ghost_ops, ops
        self.mult32 = mult.to(torch.float32)
        self.coarse = coarse
        self.ecoord = slab_element_coords(part, mult.device)

    def apply(self, z, r):
        rg = self.ghost.fill(r)
        zg = torch.empty_like(rg)
        self.gops.schwarz(zg, rg)
        z.copy_(zg[self.ghost.own])
        if self.coarse is not None:
            g = self.coarse.restrict(r * self.mult32, self.ecoord)
            dist.all_reduce(g)
            z.add_(self.coarse.prolong(self.coarse.solve(g), self.ecoord))
            self.ops.mask(z)
        return z


class DistMixedCG:
    """The fast solver sharded: PCG iterated in FP32 (operator, Schwarz
    preconditioner, vectors) with FP64 reliable updates -- when the FP32
    residual has dropped by delta since the last replacement (or reached the
    tolerance) the FP32 correction is folded into the FP64 solution and the
    residual recomputed in FP64 -- on the element-partitioned operator.  Dots
    in FP64, per-rank partials added in rank order.  solve(x, f) as
    DistPCG.solve; returns (iterations, ||r0||, ||r||, ||f||, FP64
    residual evaluations)."""

    def __init__(self, ops, iface, precond, mult, rtol=1e-10, abstol=0.0, delta=1e-3, max_iter=20000):
        self.ops, self.iface, self.pc = ops, iface, precond
        self.mult = mult
        self.mult32 = mult.to(torch.float32)
        self.rtol, self.abstol, self.delta, self.max_iter = rtol, abstol, delta, max_iter

    def apply64(self, w, u):
        self.ops.ax(w, u)
        self.ops.gs(w)
        self.iface.exchange_add(w)
        self.ops.mask(w)
        return w

    def apply32(self, w, u):
        self.ops.ax32(w, u)
        self.ops.gs(w)
        self.iface.exchange_add(w)
        self.ops.mask(w)
        return w

    def solve(self, x, f):
        d64 = lambda a, b: dist_dot(a.to(torch.float64), b.to(torch.float64), self.mult)
        fn = math.sqrt(d64(f, f))
        tol = max(self.abstol, self.rtol * fn)
        w64 = torch.empty_like(x)
        r64 = f - self.apply64(w64, x) if d64(x, x) != 0.0 else f.clone()
        nrep = 1
        rn = math.sqrt(d64(r64, r64))
        r0 = rn
        it = 0
        if rn <= tol:
            return it, r0, rn, fn, nrep
        r = r64.to(torch.float32)
        xc = torch.zeros_like(r)
        z = torch.empty_like(r)
        w = torch.empty_like(r)
        self.pc.apply(z, r)
        p = z.clone()
        rz = d64(r, z)
        ref = rn
        while it < self.max_iter:
            self.apply32(w, p)
            alpha = rz / d64(p, w)
            xc.add_(p, alpha=alpha)
            r.sub_(w, alpha=alpha)
            it += 1
            rr = math.sqrt(d64(r, r))
            if rr <= self.delta * ref or rr <= tol:
                # reliable update: fold the correction into x, FP64 residual
                x.add_(xc.to(torch.float64))
                xc.zero_()
                r64 = f - self.apply64(w64, x)
                nrep += 1
                rn = math.sqrt(d64(r64, r64))
                if rn <= tol:
                    break
                r = r64.to(torch.float32)
                ref = rn
            self.pc.apply(z, r)
            rz_new = d64(r, z)
            p.mul_(rz_new / rz).add_(z)
            rz = rz_new
        return it, r0, rn, fn, nrep


def dirichlet_faces_dist(part: SlabPartition, mask_local, lx: int, device="cpu"):
    """(x-, x+, y-, y+, z-, z+): a box face is Dirichlet for the coarse level
    when all its local nodes are masked, counted over every rank's own
    elements (mask_local: the rank's 1-based Dirichlet indices; device: where
    the process group's collectives run)."""
    N, l3 = lx - 1, lx ** 3
    cnt = torch.zeros(6, dtype=torch.float64)
    if mask_local is not None and len(mask_local):
        l = torch.as_tensor(np.asarray(mask_local, dtype=np.int64) - 1)
        e = l // l3 + part.e0
        q = l % l3
        idx = (q % lx, (q // lx) % lx, q // (lx * lx))
        c = (e % part.ex, (e // part.ex) % part.ey, e // (part.ex * part.ey))
        E = (part.ex, part.ey, part.ez)
        for d in range(3):
            cnt[2 * d] = float(((idx[d] == 0) & (c[d] == 0)).sum())
            cnt[2 * d + 1] = float(((idx[d] == N) & (c[d] == E[d] - 1)).sum())
    cnt = cnt.to(device)
    dist.all_reduce(cnt)
    cnt = cnt.cpu()
    E = (part.ex, part.ey, part.ez)
    out = []
    for d in range(3):
        face = E[(d + 1) % 3] * E[(d + 2) % 3] * lx * lx
        out += [bool(cnt[2 * d] == face), bool(cnt[2 * d + 1] == face)]
    return out
