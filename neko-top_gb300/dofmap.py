"""Global node numbering of a hexahedral spectral-element mesh from its
element-vertex connectivity (what Neko's dofmap_t builds from the mesh),
so meshes other than the generated boxes can make a plan: coef_t(nelv, lx,
x, y, z, dofmap_from_vertices(ev, lx)).

ev[e, v] is the global vertex id of element e's corner v = a + 2 b + 4 c at
reference position (a, b, c) in {0, 1}^3 (tensor order; Neko's hex vertex
order).  Neighbouring elements may be oriented differently: shared nodes
are matched through canonical keys,

  corner  the vertex id;
  edge    the sorted end-vertex pair and the position counted from the end
          with the smaller id;
  face    the sorted four corner ids and the position in the face frame
          whose origin is the face's smallest corner and whose first axis
          points to that corner's smaller neighbour;
  interior  the element and the local index,

and every distinct key gets one global id (0-based, int64).  Host code,
vectorised with numpy; it runs once per mesh.
"""
from __future__ import annotations

import numpy as np


def _keys_edge(ev, lx, d, fixed):
    """Local indices and keys of the edge nodes along direction d with the
    other two reference coordinates at `fixed` (each 0 or 1)."""
    N = lx - 1
    t = np.arange(1, N)
    idx3 = []
    for s in t:
        ijk = [0, 0, 0]
        ijk[d] = s
        o = [q for q in range(3) if q != d]
        ijk[o[0]] = fixed[0] * N
        ijk[o[1]] = fixed[1] * N
        idx3.append(ijk[0] + lx * (ijk[1] + lx * ijk[2]))
    c0 = [0, 0, 0]
    c1 = [0, 0, 0]
    c1[d] = 1
    o = [q for q in range(3) if q != d]
    for c in (c0, c1):
        c[o[0]], c[o[1]] = fixed
    v0 = ev[:, c0[0] + 2 * c0[1] + 4 * c0[2]]
    v1 = ev[:, c1[0] + 2 * c1[1] + 4 * c1[2]]
    lo, hi = np.minimum(v0, v1), np.maximum(v0, v1)
    pos = np.where((v0 < v1)[:, None], t[None, :], (N - t)[None, :])
    return np.array(idx3), lo, hi, pos


def _keys_face(ev, lx, d, side):
    """Local indices and keys of the interior nodes of the face normal to d
    at reference coordinate `side` (0 or 1)."""
    N = lx - 1
    o = [q for q in range(3) if q != d]  # face axes (s along o[0], t along o[1])
    corners = []
    for tb in (0, 1):
        for sb in (0, 1):
            c = [0, 0, 0]
            c[d] = side
            c[o[0]], c[o[1]] = sb, tb
            corners.append(c[0] + 2 * c[1] + 4 * c[2])
    cv = ev[:, corners]  # (E, 4) at face positions (0,0), (1,0), (0,1), (1,1)
    E = ev.shape[0]
    # the eight symmetries of the square: (origin corner, swap axes)
    st = np.array([(s, t) for t in range(1, N) for s in range(1, N)])  # local face positions
    idx3 = []
    for s, t in st:
        ijk = [0, 0, 0]
        ijk[d] = side * N
        ijk[o[0]], ijk[o[1]] = s, t
        idx3.append(ijk[0] + lx * (ijk[1] + lx * ijk[2]))
    pos_c = np.array([(0, 0), (1, 0), (0, 1), (1, 1)])
    m = np.argmin(cv, axis=1)  # the smallest corner
    mc = pos_c[m]  # its (s, t) corner bits
    # neighbours of the smallest corner along s and along t
    ns = cv[np.arange(E), (1 - mc[:, 0]) + 2 * mc[:, 1]]
    nt = cv[np.arange(E), mc[:, 0] + 2 * (1 - mc[:, 1])]
    swap = nt < ns  # the first canonical axis follows the smaller neighbour
    s = st[None, :, 0].repeat(E, 0)
    t = st[None, :, 1].repeat(E, 0)
    s = np.where(mc[:, 0:1] == 1, N - s, s)  # origin at the smallest corner
    t = np.where(mc[:, 1:2] == 1, N - t, t)
    a = np.where(swap[:, None], t, s)
    b = np.where(swap[:, None], s, t)
    key = np.sort(cv, axis=1)
    return np.array(idx3), key, a, b


def dofmap_from_vertices(ev, lx):
    """int64 global node ids (Neko layout, i fastest) from the element-vertex
    connectivity ev (E x 8, tensor corner order; vertex ids in [0, 2^31)).

    Host memory: the key table holds 6 int64 per local node and np.unique
    sorts a copy of it, so the peak is about 100 bytes per local node (5 GB
    for 2^21 elements of lx = 8, 13 GB for the 64^3-element lx = 8 box).
    Number such meshes in parts, or generate box ids directly
    (coef_t.box), when that is too much."""
    ev = np.ascontiguousarray(ev, dtype=np.int64)
    E = ev.shape[0]
    if ev.ndim != 2 or ev.shape[1] != 8:
        raise ValueError("ev must be E x 8")
    if lx < 2:
        raise ValueError("lx must be >= 2")
    if E and (int(ev.min()) < 0 or int(ev.max()) >= 2 ** 31):
        # face keys pack two sorted corner ids into one int64
        raise ValueError("vertex ids must lie in [0, 2^31)")
    N, l3 = lx - 1, lx ** 3
    records = []  # (local index array, key columns)
    vmax = int(ev.max()) + 1
    # corners: kind 0, key (vid, 0, 0, 0, 0)
    for v in range(8):
        a, b, c = v & 1, (v >> 1) & 1, (v >> 2) & 1
        li = a * N + lx * (b * N + lx * c * N)
        k = np.zeros((E, 6), dtype=np.int64)
        k[:, 1] = ev[:, v]
        records.append((np.full(E, li), k))
    if N > 1:
        for d in range(3):
            for f0 in (0, 1):
                for f1 in (0, 1):
                    idx3, lo, hi, pos = _keys_edge(ev, lx, d, (f0, f1))
                    for q, li in enumerate(idx3):
                        k = np.zeros((E, 6), dtype=np.int64)
                        k[:, 0] = 1
                        k[:, 1], k[:, 2], k[:, 3] = lo, hi, pos[:, q]
                        records.append((np.full(E, li), k))
        for d in range(3):
            for side in (0, 1):
                idx3, key, a, b = _keys_face(ev, lx, d, side)
                for q, li in enumerate(idx3):
                    k = np.zeros((E, 6), dtype=np.int64)
                    k[:, 0] = 2
                    # the sorted corner ids packed in pairs (ids < 2^31 each)
                    k[:, 1] = key[:, 0] * vmax + key[:, 1]
                    k[:, 2] = key[:, 2] * vmax + key[:, 3]
                    k[:, 3], k[:, 4] = a[:, q], b[:, q]
                    records.append((np.full(E, li), k))
        inner = [i + lx * (j + lx * k) for k in range(1, N) for j in range(1, N) for i in range(1, N)]
        for li in inner:
            k = np.zeros((E, 6), dtype=np.int64)
            k[:, 0] = 3
            k[:, 1] = np.arange(E)
            k[:, 2] = li
            records.append((np.full(E, li), k))
    loc = np.concatenate([e_off + r[0] for r, e_off in zip(records, [np.arange(E) * l3] * len(records))])
    keys = np.concatenate([r[1] for r in records])
    _, gid_of_row = np.unique(keys, axis=0, return_inverse=True)
    gid = np.empty(E * l3, dtype=np.int64)
    gid[loc] = gid_of_row.ravel()
    if len(loc) != E * l3 or len(np.unique(loc)) != E * l3:
        raise AssertionError("every local node must get exactly one key")
    return gid
