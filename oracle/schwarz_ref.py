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
