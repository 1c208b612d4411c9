"""Synthetic unstructured hexahedral meshes for the tests.

ogrid_pipe: a circular pipe whose cross-section is an O-grid (a central
square block of n x n elements and four curved-side blocks of n x m
elements between the square and the circle), extruded along z in nz
layers.  The square's corners are edges shared by three elements, and the
blocks' local frames differ, so face neighbours meet in several relative
orientations.  Sides are straight between vertices.  Elements are given by
global vertex ids in tensor corner order (v = i + 2j + 4k), and zones mark
the inlet (z = 0, label 1), outlet (z = L, label 2) and wall (label 3) as
labeled zones (type 7) with the 1-based faces r-, r+, s-, s+, t-, t+.

reorient: applies a symmetry of the cube to every element (node and corner
order permuted), which changes no geometry or global id.
"""
import itertools

import numpy as np


def ogrid_pipe(n=2, m=2, nz=3, radius=0.5, length=1.5, seed=None):
    a = radius * 0.45
    quads = []  # four (x, y) corners in tensor order, per 2D element
    t = np.linspace(-1.0, 1.0, n + 1)
    # central square
    for j in range(n):
        for i in range(n):
            c = [(a * t[i + di], a * t[j + dj]) for dj in (0, 1) for di in (0, 1)]
            quads.append((c[0], c[1], c[2], c[3]))
    # four outer blocks: side of the square (u in [-1, 1]) to the arc, radial v in [0, 1]
    r01 = np.linspace(0.0, 1.0, m + 1)
    for k in range(4):
        ang = k * np.pi / 2
        rot = np.array([[np.cos(ang), -np.sin(ang)], [np.sin(ang), np.cos(ang)]])

        def point(u, v):
            sq = np.array([a, a * u])
            th = u * np.pi / 4
            ci = np.array([radius * np.cos(th), radius * np.sin(th)])
            return tuple(rot @ ((1 - v) * sq + v * ci))

        for j in range(m):
            for i in range(n):
                # tensor order with xi along the radial direction, eta along the side
                c = [point(t[i + di], r01[j + dj]) for di in (0, 1) for dj in (0, 1)]
                quads.append((c[0], c[1], c[2], c[3]))
    # orient every quad counter-clockwise in (xi, eta)
    oq = []
    for c in quads:
        c = [np.array(p) for p in c]
        d1, d2 = c[1] - c[0], c[2] - c[0]
        cr = d1[0] * d2[1] - d1[1] * d2[0]
        oq.append(c if cr > 0 else [c[1], c[0], c[3], c[2]])
    # shared 2D vertex ids by coordinates
    key = {}
    ids2 = []
    for c in oq:
        row = []
        for p in c:
            kk = (round(float(p[0]), 9), round(float(p[1]), 9))
            if kk not in key:
                key[kk] = len(key)
            row.append(key[kk])
        ids2.append(row)
    pts2 = np.zeros((len(key), 2))
    for kk, v in key.items():
        pts2[v] = kk
    nv2 = len(key)
    zs = np.linspace(0.0, length, nz + 1)
    ev, xyz = [], []
    for lz in range(nz):
        for q, row in enumerate(ids2):
            ids = [row[v & 3] + nv2 * (lz + (v >> 2)) for v in range(8)]
            ev.append(ids)
            xyz.append([(pts2[row[v & 3], 0], pts2[row[v & 3], 1], zs[lz + (v >> 2)]) for v in range(8)])
    ev = np.array(ev, dtype=np.int64) + 1
    xyz = np.array(xyz)
    # zones: faces that no other element shares
    faces = {0: [0, 2, 4, 6], 1: [1, 3, 5, 7], 2: [0, 1, 4, 5], 3: [2, 3, 6, 7], 4: [0, 1, 2, 3], 5: [4, 5, 6, 7]}
    cnt = {}
    for e in range(len(ev)):
        for f, vs in faces.items():
            k = tuple(sorted(ev[e, vs]))
            cnt[k] = cnt.get(k, 0) + 1
    zones = []
    for e in range(len(ev)):
        for f, vs in faces.items():
            if cnt[tuple(sorted(ev[e, vs]))] == 1:
                zc = xyz[e, vs, 2]
                label = 1 if np.all(zc == 0.0) else 2 if np.all(zc == length) else 3
                zones.append([e + 1, f + 1, 0, label, 0, 0, 0, 0, 7])
    return ev, xyz, np.array(zones, dtype=np.int32)


SYMS = [(p, f) for p in itertools.permutations(range(3)) for f in itertools.product((0, 1), repeat=3)]


def _parity(p):
    return sum(1 for a in range(3) for b in range(a + 1, 3) if p[a] > p[b]) % 2


# the 24 rotations of the cube (the symmetries that keep elements right-handed)
ROTATIONS = [(p, f) for p, f in SYMS if (_parity(p) + sum(f)) % 2 == 0]


def reorient(lx, ev, fields, rng, rotations_only=True):
    """Apply a random symmetry of the cube to each element (by default a
    rotation, so the geometry stays right-handed): new local node q takes
    old node sigma(q); corners follow.  `fields` are per-node arrays
    (E * lx^3, x fastest) permuted the same way.  Returns (ev2, fields2)."""
    N, l3 = lx - 1, lx ** 3
    E = ev.shape[0]
    ev2 = ev.copy()
    out = [np.asarray(a).reshape(E, l3).copy() for a in fields]
    idx = np.arange(l3)
    new = np.stack([idx % lx, (idx // lx) % lx, idx // (lx * lx)], 1)
    syms = ROTATIONS if rotations_only else SYMS
    for e in range(E):
        p, f = syms[rng.integers(len(syms))]
        old = np.empty_like(new)
        for q in range(3):
            old[:, p[q]] = np.where(f[q], N - new[:, q], new[:, q])
        src = old[:, 0] + lx * (old[:, 1] + lx * old[:, 2])
        for a, o in zip(fields, out):
            o[e] = np.asarray(a).reshape(E, l3)[e, src]
        for v in range(8):
            nb = np.array([v & 1, (v >> 1) & 1, (v >> 2) & 1]) * N
            ob = np.empty(3, dtype=int)
            for q in range(3):
                ob[p[q]] = N - nb[q] if f[q] else nb[q]
            ov = int(ob[0] // N + 2 * (ob[1] // N) + 4 * (ob[2] // N))
            ev2[e, v] = ev[e, ov]
    return ev2, [o.ravel() for o in out]


def nodes_from_vertices(xyz, lx):
    """GLL node coordinates (E * lx^3 each, x fastest), trilinear in the
    tensor-ordered vertices (numpy, for the oracle side of a test)."""
    from oracle import numpy_ref
    xi, _, _ = numpy_ref.gll(lx)
    xi = xi.copy()
    xi[0], xi[-1] = -1.0, 1.0
    q = np.arange(lx ** 3)
    i, j, k = q % lx, (q // lx) % lx, q // (lx * lx)
    w = np.stack([0.125 * np.where(v & 1, 1 + xi[i], 1 - xi[i]) * np.where((v >> 1) & 1, 1 + xi[j], 1 - xi[j])
                  * np.where(v >> 2, 1 + xi[k], 1 - xi[k]) for v in range(8)])  # (8, l3)
    X = np.einsum("vq,evd->edq", w, xyz)  # (E, 3, l3)
    return X[:, 0].ravel(), X[:, 1].ravel(), X[:, 2].ravel()
