"""numpy restatement of the overlapping additive Schwarz preconditioner.

TEST INFRASTRUCTURE ONLY: the checker for neko-top_gb300/csrc/schwarz.cu.

    z = sum_e R_e^T  A~_e^{-1}  R_e r

on structured boxes (elements numbered x fastest).  R_e gathers the
assembled residual on element e extended by one node layer into each
neighbour; A~_e = h1 (Bz x By x Kx + Bz x Ky x Bx + Kz x By x Bx) + h2 Bz x By x Bx
with 1D operators assembled from the element's GLL interval and one
interval of the element's own length on each side (Dirichlet one node
beyond the extension), inverted through the
generalised eigenvectors (numpy.linalg.eigh); R_e^T adds the extended result
into a global structured grid (a different prolongation than the kernel's
assembling pull).  Element lengths: mean distance between opposite faces.
With coarse=True it adds the vertex-grid coarse correction (coarse_apply).
"""
from __future__ import annotations

import numpy as np

from oracle import numpy_ref


def element_lengths(m):
    lx = m.lx
    X = np.stack([m.x, m.y, m.z]).reshape(3, m.nelv, lx, lx, lx)  # (d, e, k, j, i)
    out = np.zeros((m.nelv, 3))
    for d, (a0, a1) in enumerate(((np.s_[:, :, :, :, 0], np.s_[:, :, :, :, -1]),
                                  (np.s_[:, :, :, 0, :], np.s_[:, :, :, -1, :]),
                                  (np.s_[:, :, 0, :, :], np.s_[:, :, -1, :, :]))):
        diff = X[a1] - X[a0]
        out[:, d] = np.sqrt((diff ** 2).sum(0)).mean(axis=(1, 2))
    return out


def ext_1d(lx, hl, hc, hr):
    N = lx - 1
    _, w, D = numpy_ref.gll(lx)
    Kh = D.T @ np.diag(w) @ D
    ng = 3 * N + 1
    K = np.zeros((ng, ng))
    B = np.zeros(ng)
    for el, h in enumerate((hl, hc, hr)):
        s = slice(el * N, el * N + lx)
        K[s, s] += (2.0 / h) * Kh
        B[s] += 0.5 * h * w
    sl = slice(N - 1, 2 * N + 2)
    Ke, Be = K[sl, sl], B[sl]
    bi = 1.0 / np.sqrt(Be)
    lam, Q = np.linalg.eigh(bi[:, None] * Ke * bi[None, :])
    return bi[:, None] * Q, lam


def dirichlet_faces(m, box, mask):
    """(x-, x+, y-, y+, z-, z+): a face is Dirichlet when all its local nodes are masked."""
    Ex, Ey, Ez = box
    lx, N = m.lx, m.lx - 1
    E = (Ex, Ey, Ez)
    cnt = [0] * 6
    if mask is not None and len(mask):
        l = np.asarray(mask, dtype=np.int64) - 1
        e, q = l // lx ** 3, l % lx ** 3
        idx = (q % lx, (q // lx) % lx, q // lx ** 2)
        c = (e % Ex, (e // Ex) % Ey, e // (Ex * Ey))
        for d in range(3):
            cnt[2 * d] = int(np.sum((idx[d] == 0) & (c[d] == 0)))
            cnt[2 * d + 1] = int(np.sum((idx[d] == N) & (c[d] == E[d] - 1)))
    out = []
    for d in range(3):
        face = E[(d + 1) % 3] * E[(d + 2) % 3] * lx * lx
        out += [cnt[2 * d] == face, cnt[2 * d + 1] == face]
    return out


def coarse_apply(m, r, box, h1, h2, mask):
    """P A_c^+ P^T r: the coarse level on the element vertices.

    P: trilinear interpolation (reference coordinates) of vertex values to
    the GLL nodes; P^T r = sum over local nodes of phi * r * mult (mult =
    1/multiplicity); A_c = h1 (Mz x My x Kx + Mz x Ky x Mx + Kz x My x Mx)
    + h2 Mz x My x Mx assembled densely from 1D linear elements with the mean
    element length of each slab, Dirichlet vertices removed; pseudo-inverse
    (an all-Neumann box has the constant null mode)."""
    Ex, Ey, Ez = box
    E = (Ex, Ey, Ez)
    lx = m.lx
    xi, _, _ = numpy_ref.gll(lx)
    phi = np.stack([0.5 * (1 - xi), 0.5 * (1 + xi)])  # (2, lx)
    hl = element_lengths(m)
    dirf = dirichlet_faces(m, box, mask)
    Ks, Ms, act = [], [], []
    for d in range(3):
        c = (np.arange(m.nelv) // (1, Ex, Ex * Ey)[d]) % E[d]
        hs = np.array([hl[c == s, d].mean() for s in range(E[d])])
        nv = E[d] + 1
        K, M = np.zeros((nv, nv)), np.zeros((nv, nv))
        for s, h in enumerate(hs):
            K[s:s + 2, s:s + 2] += np.array([[1, -1], [-1, 1]]) / h
            M[s:s + 2, s:s + 2] += np.array([[2, 1], [1, 2]]) * h / 6
        a = np.arange(1 if dirf[2 * d] else 0, nv - (1 if dirf[2 * d + 1] else 0))
        Ks.append(K[np.ix_(a, a)])
        Ms.append(M[np.ix_(a, a)])
        act.append(a)
    if any(len(a) == 0 for a in act):
        return np.zeros(m.n)
    Kx, Ky, Kz = Ks
    Mx, My, Mz = Ms
    A = h1 * (np.kron(Mz, np.kron(My, Kx)) + np.kron(Mz, np.kron(Ky, Mx)) + np.kron(Kz, np.kron(My, Mx))) \
        + h2 * np.kron(Mz, np.kron(My, Mx))
    # P as a dense (n_local x n_active) matrix
    nvx, nvy = Ex + 1, Ey + 1
    col = -np.ones((Ex + 1) * (Ey + 1) * (Ez + 1), dtype=np.int64)
    gx, gy, gz = np.meshgrid(act[0], act[1], act[2], indexing="ij")
    flat = (gx + nvx * (gy + nvy * gz)).transpose(2, 1, 0).ravel()  # x fastest
    col[flat] = np.arange(flat.size)
    P = np.zeros((m.n, flat.size))
    for e in range(m.nelv):
        c = (e % Ex, (e // Ex) % Ey, e // (Ex * Ey))
        for k in range(lx):
            for j in range(lx):
                for i in range(lx):
                    l = e * lx ** 3 + i + lx * j + lx * lx * k
                    for v in range(8):
                        vx, vy, vz = v & 1, (v >> 1) & 1, v >> 2
                        g = (c[0] + vx) + nvx * ((c[1] + vy) + nvy * (c[2] + vz))
                        if col[g] >= 0:
                            P[l, col[g]] += phi[vx, i] * phi[vy, j] * phi[vz, k]
    rc = P.T @ (np.asarray(r) * m.mult)
    return P @ (np.linalg.pinv(A) @ rc)


def plane_operator_bf16(lx):
    """The in-plane operator of the tensor-core FDM path: K~[(a,b),(f,g)] =
    bf16(S^[a][f] S^[b][g]) with S^ the reference (h = 2) extended
    eigenvectors, the product rounded to float32 first (as the kernel's
    table is built).  Returns (K~ as float64 [LE^2 x LE^2], S^, lam^)."""
    from oracle import mlp_ref
    S, lam = ext_1d(lx, 2.0, 2.0, 2.0)
    LE = lx + 2
    # index (a, b) -> a + LE b and (f, g) -> f + LE g (a and f fastest)
    K = np.einsum("af,bg->bagf", S, S).reshape(LE * LE, LE * LE)
    Kb = mlp_ref.bf16(K.astype(np.float32)).astype(np.float64)
    return Kb, S, lam


def apply(m, r, box, h1=1.0, h2=None, mask=None, coarse=False, plane_bf16=False):
    """z = M r for an oracle Mesh `m` built as a box of `box` = (Ex, Ey, Ez).

    plane_bf16: the local solves as the tensor-core path computes them: the
    reference pair scaled by the element lengths, with the in-plane
    operator S^ x S^ rounded to BF16 (plane_operator_bf16); the data stay in
    FP64 here (the kernel's two-term BF16 split carries 16 bits)."""
    Ex, Ey, Ez = box
    lx = m.lx
    N, LE = lx - 1, lx + 2
    hl = element_lengths(m)
    r4 = np.asarray(r).reshape(m.nelv, lx, lx, lx)  # (e, k, j, i)
    G = np.zeros((Ex * N + 1, Ey * N + 1, Ez * N + 1))  # indexed (gx, gy, gz)
    h2e = np.zeros(m.nelv) if h2 is None else np.asarray(h2).reshape(m.nelv, -1).mean(1)
    dims = (Ex, Ey, Ez)
    if plane_bf16:
        Kb, Sr, lamr = plane_operator_bf16(lx)
    for e in range(m.nelv):
        c = (e % Ex, (e // Ex) % Ey, e // (Ex * Ey))
        strides = (1, Ex, Ex * Ey)
        Ss, Ls = [], []
        for d in range(3):
            # the local model extends the element with intervals of its own
            # length (the kernel's shared-reference form)
            hc = hl[e, d]
            S, lam = ext_1d(lx, hc, hc, hc)
            Ss.append(S)
            Ls.append(lam)
        # gather R_e r on the extended box (index order a=x, b=y, c=z)
        rext = np.zeros((LE, LE, LE))
        for a in range(LE):
            for b in range(LE):
                for cc in range(LE):
                    g = (c[0] * N + a - 1, c[1] * N + b - 1, c[2] * N + cc - 1)
                    if not all(0 <= g[q] <= dims[q] * N for q in range(3)):
                        continue
                    # any element holding the global node: pick by clamping
                    ec = [min(g[q] // N, dims[q] - 1) for q in range(3)]
                    loc = [g[q] - ec[q] * N for q in range(3)]
                    en = ec[0] + Ex * (ec[1] + Ey * ec[2])
                    rext[a, b, cc] = r4[en, loc[2], loc[1], loc[0]]
        Sx, Sy, Sz = Ss
        if plane_bf16:
            hx, hy, hz = hl[e]
            # rext[a, b, c] -> X[(a + LE b), c]
            X = rext.transpose(1, 0, 2).reshape(LE * LE, LE)
            Y1 = Kb.T @ X                                   # [(f + LE g), c]
            y = Y1 @ Sr                                     # [(f g), h]
            fgl = (4.0 / hx ** 2) * lamr[None, :] + (4.0 / hy ** 2) * lamr[:, None]  # [g, f]
            den = h1 * (fgl.reshape(-1)[:, None] + (4.0 / hz ** 2) * lamr[None, :]) + h2e[e]
            z = (8.0 / (hx * hy * hz)) * y / den
            W1 = z @ Sr.T                                   # [(f g), c']
            W = Kb @ W1                                     # [(a + LE b), c']
            zext = W.reshape(LE, LE, LE).transpose(1, 0, 2)
        else:
            t = np.einsum("pa,qb,sc,pqs->abc", Sx, Sy, Sz, rext)
            t /= h1 * (Ls[0][:, None, None] + Ls[1][None, :, None] + Ls[2][None, None, :]) + h2e[e]
            zext = np.einsum("ap,bq,cs,pqs->abc", Sx, Sy, Sz, t)
        for a in range(LE):
            for b in range(LE):
                for cc in range(LE):
                    g = (c[0] * N + a - 1, c[1] * N + b - 1, c[2] * N + cc - 1)
                    if all(0 <= g[q] <= dims[q] * N for q in range(3)):
                        G[g] += zext[a, b, cc]
    # back to the local layout
    z = np.zeros_like(r4)
    for e in range(m.nelv):
        c = (e % Ex, (e // Ex) % Ey, e // (Ex * Ey))
        z[e] = G[c[0] * N:c[0] * N + lx, c[1] * N:c[1] * N + lx, c[2] * N:c[2] * N + lx].transpose(2, 1, 0)
    z = z.ravel()
    if coarse:
        h2m = 0.0 if h2 is None else float(np.asarray(h2).reshape(m.nelv, -1).mean(1).mean())
        z = z + coarse_apply(m, r, box, h1, h2m, mask)
    if mask is not None and len(mask):
        z[np.asarray(mask) - 1] = 0.0
    return z


# ---------------------------------------------------------------------------
# General (unstructured, conforming) hexahedral meshes
# ---------------------------------------------------------------------------

def _face_nodes(lx, f, normal):
    """Local indices of face f's nodes (r-, r+, s-, s+, t-, t+ = 0..5) in
    tangential order (lower axis fastest), at normal index `normal`."""
    d = f // 2
    out = []
    for t in range(lx):
        for s in range(lx):
            ijk = [s, t] if d == 0 else [s, t]
            if d == 0:
                i, j, k = normal, s, t
            elif d == 1:
                i, j, k = s, normal, t
            else:
                i, j, k = s, t, normal
            out.append(i + lx * (j + lx * k))
    return np.array(out)


def face_ghosts(m):
    """ghost[e, f, p]: the local index (into the whole field) of the node one
    step inside the face neighbour of element e across face f, matching face
    node p of e through the global ids; -1 on boundary faces.  Neighbours are
    the elements holding all four corner ids of the face."""
    lx, N, l3 = m.lx, m.lx - 1, m.lx ** 3
    E = m.nelv
    gid = m.gid.reshape(E, l3)
    corner_sets = {}
    for e in range(E):
        for f in range(6):
            fn = _face_nodes(lx, f, N if f % 2 else 0)
            key = tuple(sorted(gid[e, fn[[0, N, N * lx, N * lx + N]]]))
            corner_sets.setdefault(key, []).append((e, f))
    ghost = -np.ones((E, 6, lx * lx), dtype=np.int64)
    for key, lst in corner_sets.items():
        if len(lst) == 1:
            continue
        assert len(lst) == 2, "non-conforming mesh"
        for (ea, fa), (eb, fb) in (lst, lst[::-1]):
            own = gid[ea, _face_nodes(lx, fa, N if fa % 2 else 0)]
            other_face = _face_nodes(lx, fb, N if fb % 2 else 0)
            other_in = _face_nodes(lx, fb, N - 1 if fb % 2 else 1)
            pos = {g: q for q, g in enumerate(gid[eb, other_face])}
            ghost[ea, fa] = [eb * l3 + other_in[pos[g]] for g in own]
    return ghost


def _ghost_ext_index(lx, f):
    """(a, b, c) index arrays of the ghost layer beyond face f in the
    extended box, in face-node order."""
    LE = lx + 2
    d, b0 = f // 2, (LE - 1 if f % 2 else 0)
    s, t = np.meshgrid(np.arange(lx), np.arange(lx), indexing="xy")
    s, t = s.ravel() + 1, t.ravel() + 1
    b0v = np.full(s.shape, b0)
    return [(b0v, s, t), (s, b0v, t), (s, t, b0v)][d]


def coarse_galerkin(m, h1=1.0, h2=None, mask=None):
    """The Galerkin Q1 coarse operator P^T A P on the element vertices
    (active = not masked), with P the trilinear interpolation zeroed on
    masked nodes.  Returns (A_c, vid) with vid[e, v] the active vertex of
    corner v (i + 2j + 4k) of element e or -1."""
    lx, N, l3, E = m.lx, m.lx - 1, m.lx ** 3, m.nelv
    xi, _, _ = numpy_ref.gll(lx)
    phi = np.stack([0.5 * (1 - xi), 0.5 * (1 + xi)])
    phi[:, 0], phi[:, N] = (1.0, 0.0), (0.0, 1.0)
    flag = np.zeros(m.n, dtype=bool)
    if mask is not None and len(mask):
        flag[np.asarray(mask) - 1] = True
    masked_g = set(m.gid[flag].tolist())
    corners = np.array([((v & 1) * N) + lx * (((v >> 1) & 1) * N) + lx * lx * ((v >> 2) * N) for v in range(8)])
    cg = m.gid.reshape(E, l3)[:, corners]
    verts = sorted({int(g) for g in cg.ravel() if int(g) not in masked_g})
    index = {g: a for a, g in enumerate(verts)}
    vid = np.array([[index.get(int(g), -1) for g in row] for row in cg])
    q = np.arange(l3)
    i, j, k = q % lx, (q // lx) % lx, q // (lx * lx)
    basis = np.stack([phi[v & 1][i] * phi[(v >> 1) & 1][j] * phi[v >> 2][k] for v in range(8)])  # (8, l3)
    keep = ~flag.reshape(E, l3)
    h1f = h1 if np.ndim(h1) else None
    h1c = 1.0 if h1f is not None else float(h1)
    W = []
    for v in range(8):
        U = (basis[v][None, :] * keep).ravel()
        W.append(numpy_ref_ax(m, U, h1f, h1c, h2).reshape(E, l3))
    nv = len(verts)
    A = np.zeros((nv, nv))
    for e in range(E):
        Ue = basis * keep[e][None, :]
        Ae = Ue @ np.stack([W[v][e] for v in range(8)]).T  # [w, v]
        for w in range(8):
            if vid[e, w] < 0:
                continue
            for v in range(8):
                if vid[e, v] >= 0:
                    A[vid[e, w], vid[e, v]] += Ae[w, v]
    A = 0.5 * (A + A.T)
    if abs(A.sum()) <= 1e-10 * np.trace(A):  # constant null mode: A + c 1 1^T
        A = A + np.trace(A) / nv / nv
    return A, vid


def numpy_ref_ax(m, u, h1, h1c, h2):
    from oracle import oracle as orc
    return orc.ax_helm(m, u, h1=h1, h1c=h1c, h2=h2)


def apply_general(m, r, h1=1.0, h2=None, mask=None, coarse=False):
    """z = M r on a general mesh: each element extended by one node layer
    across its six faces only (the face neighbour's nodes one step inside,
    edge and corner positions excluded), the local solves of `apply`
    (element lengths, shared reference pair), the results summed per
    global node; with coarse=True plus P A_c^-1 P^T r with the Galerkin
    operator of coarse_galerkin; masked nodes zeroed."""
    lx, N, LE, l3, E = m.lx, m.lx - 1, m.lx + 2, m.lx ** 3, m.nelv
    hl = element_lengths(m)
    ghost = face_ghosts(m)
    r = np.asarray(r, dtype=np.float64)
    r4 = r.reshape(E, lx, lx, lx)  # (e, k, j, i)
    h1e = np.full(E, float(h1)) if not np.ndim(h1) else np.asarray(h1).reshape(E, -1).mean(1)
    h2e = np.zeros(E) if h2 is None else np.asarray(h2).reshape(E, -1).mean(1)
    acc = {}
    gid = m.gid
    for e in range(E):
        Ss, Ls = [], []
        for d in range(3):
            S, lam = ext_1d(lx, hl[e, d], hl[e, d], hl[e, d])
            Ss.append(S)
            Ls.append(lam)
        rext = np.zeros((LE, LE, LE))  # [a, b, c]
        rext[1:-1, 1:-1, 1:-1] = r4[e].transpose(2, 1, 0)
        for f in range(6):
            a, b, c = _ghost_ext_index(lx, f)
            src = ghost[e, f]
            ok = src >= 0
            rext[a[ok], b[ok], c[ok]] = r[src[ok]]
        Sx, Sy, Sz = Ss
        t = np.einsum("pa,qb,sc,pqs->abc", Sx, Sy, Sz, rext)
        t /= h1e[e] * (Ls[0][:, None, None] + Ls[1][None, :, None] + Ls[2][None, None, :]) + h2e[e]
        zext = np.einsum("ap,bq,cs,pqs->abc", Sx, Sy, Sz, t)
        own = zext[1:-1, 1:-1, 1:-1].transpose(2, 1, 0).ravel()
        for q in range(l3):
            g = int(gid[e * l3 + q])
            acc[g] = acc.get(g, 0.0) + own[q]
        for f in range(6):
            a, b, c = _ghost_ext_index(lx, f)
            for p in range(lx * lx):
                src = ghost[e, f, p]
                if src >= 0:
                    g = int(gid[src])
                    acc[g] = acc.get(g, 0.0) + zext[a[p], b[p], c[p]]
    z = np.array([acc[int(g)] for g in gid])
    if coarse:
        A, vid = coarse_galerkin(m, h1, h2, mask)
        if A.shape[0]:
            xi, _, _ = numpy_ref.gll(lx)
            phi = np.stack([0.5 * (1 - xi), 0.5 * (1 + xi)])
            q = np.arange(l3)
            i, j, k = q % lx, (q // lx) % lx, q // (lx * lx)
            basis = np.stack([phi[v & 1][i] * phi[(v >> 1) & 1][j] * phi[v >> 2][k] for v in range(8)])
            rm = (r * m.mult).reshape(E, l3)
            rc = np.zeros(A.shape[0])
            for e in range(E):
                cs = basis @ rm[e]
                for v in range(8):
                    if vid[e, v] >= 0:
                        rc[vid[e, v]] += cs[v]
            zc = np.linalg.solve(A, rc)
            zcv = np.where(vid >= 0, zc[np.maximum(vid, 0)], 0.0)  # (E, 8)
            z = z + (zcv @ basis).ravel()
    if mask is not None and len(mask):
        z[np.asarray(mask) - 1] = 0.0
    return z
