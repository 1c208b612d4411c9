"""Independent numpy/scipy restatement for small meshes.

TEST INFRASTRUCTURE ONLY.  It cross-checks the C oracle with a different
algorithm: GLL nodes from numpy's Legendre roots, the derivative matrix from
barycentric weights, element stiffness matrices assembled as explicit
Kronecker products and the global operator as a scipy sparse matrix built
from the global ids (Deville, Fischer & Mund 2002, ch. 4).
"""
from __future__ import annotations

import numpy as np
from numpy.polynomial import legendre as L
import scipy.sparse as sp


def gll(lx):
    N = lx - 1
    cN = np.zeros(N + 1)
    cN[N] = 1.0
    inner = np.sort(np.real(L.legroots(L.legder(cN)))) if N > 1 else np.array([])
    xi = np.concatenate([[-1.0], inner, [1.0]])
    PN = L.legval(xi, cN)
    w = 2.0 / (N * (N + 1) * PN ** 2)
    # barycentric derivative matrix
    lam = np.array([1.0 / np.prod([xi[j] - xi[k] for k in range(lx) if k != j]) for j in range(lx)])
    D = np.zeros((lx, lx))
    for i in range(lx):
        for j in range(lx):
            if i != j:
                D[i, j] = lam[j] / lam[i] / (xi[i] - xi[j])
        D[i, i] = -D[i].sum()
    return xi, w, D


def element_ops(lx, xe, ye, ze):
    """Dense element stiffness K (lx^3 x lx^3, Laplacian) and diagonal mass
    from the element's node coordinates (i fastest)."""
    _, w, D = gll(lx)
    I = np.eye(lx)
    Dr = np.kron(I, np.kron(I, D))  # i fastest -> r acts on the last kron factor
    Ds = np.kron(I, np.kron(D, I))
    Dt = np.kron(D, np.kron(I, I))
    X = np.stack([xe, ye, ze])  # 3 x lx^3
    J = np.zeros((lx ** 3, 3, 3))
    for a, Dm in enumerate((Dr, Ds, Dt)):
        J[:, :, a] = (Dm @ X.T)  # dx_c / dr_a
    det = np.linalg.det(J)
    Jinv = np.linalg.inv(J)  # dr_a / dx_c
    W = np.einsum("k,j,i->kji", w, w, w).ravel()  # w_i w_j w_k at local index i + lx*(j + lx*k)
    wJ = W * det
    grads = [Dr, Ds, Dt]
    K = np.zeros((lx ** 3, lx ** 3))
    for a in range(3):
        for b in range(3):
            Gab = wJ * np.einsum("qc,qc->q", Jinv[:, a, :], Jinv[:, b, :])
            K += grads[a].T @ (Gab[:, None] * grads[b])
    return K, wJ


def assembled_operator(x, y, z, gid, lx, h2=None):
    """Sparse global matrix over unique ids (sorted) and the restriction
    map local -> unique index."""
    lx3 = lx ** 3
    nelv = len(x) // lx3
    uniq, uidx = np.unique(gid, return_inverse=True)
    rows, cols, vals = [], [], []
    for e in range(nelv):
        s = slice(e * lx3, (e + 1) * lx3)
        K, wJ = element_ops(lx, x[s], y[s], z[s])
        if h2 is not None:
            K = K + np.diag(h2[s] * wJ)
        g = uidx[s]
        rows.append(np.repeat(g, lx3))
        cols.append(np.tile(g, lx3))
        vals.append(K.ravel())
    A = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(len(uniq), len(uniq)))
    return A, uidx
