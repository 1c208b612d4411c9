"""Global node numbering from element-vertex connectivity (dofmap.py):
on boxes it yields the same node partition as the box generator's global
ids, also after every element is re-oriented by a random symmetry of the
cube (so shared edges and faces are seen in different local frames)."""
import importlib.util
import itertools
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def dofmap():
    spec = importlib.util.spec_from_file_location("ntg_dofmap", os.path.join(ROOT, "neko-top_gb300", "dofmap.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def box_vertices(ex, ey, ez):
    ev = np.empty((ex * ey * ez, 8), dtype=np.int64)
    for e in range(ex * ey * ez):
        cx, cy, cz = e % ex, (e // ex) % ey, e // (ex * ey)
        for v in range(8):
            a, b, c = v & 1, (v >> 1) & 1, (v >> 2) & 1
            ev[e, v] = (cx + a) + (ex + 1) * ((cy + b) + (ey + 1) * (cz + c))
    return ev


def same_partition(g1, g2):
    pairs = np.unique(np.stack([g1, g2], 1), axis=0)
    return len(pairs) == len(np.unique(g1)) == len(np.unique(g2))


SYMS = [(p, f) for p in itertools.permutations(range(3)) for f in itertools.product((0, 1), repeat=3)]


def reorient(lx, ev, gid, rng):
    """Apply a random cube symmetry to each element: new local node q takes
    old node sigma(q); corners follow."""
    N, l3 = lx - 1, lx ** 3
    E = ev.shape[0]
    g = gid.reshape(E, l3).copy()
    ev2 = ev.copy()
    idx = np.arange(l3)
    new = np.stack([idx % lx, (idx // lx) % lx, idx // (lx * lx)], 1)
    for e in range(E):
        p, f = SYMS[rng.integers(len(SYMS))]
        old = np.empty_like(new)
        for q in range(3):
            old[:, p[q]] = np.where(f[q], N - new[:, q], new[:, q])
        src = old[:, 0] + lx * (old[:, 1] + lx * old[:, 2])
        g[e] = gid.reshape(E, l3)[e, src]
        for v in range(8):
            nb = np.array([v & 1, (v >> 1) & 1, (v >> 2) & 1]) * N
            ob = np.empty(3, dtype=int)
            for q in range(3):
                ob[p[q]] = N - nb[q] if f[q] else nb[q]
            ov = int(ob[0] // N + 2 * (ob[1] // N) + 4 * (ob[2] // N))
            ev2[e, v] = ev[e, ov]
    return ev2, g.ravel()


@pytest.mark.parametrize("shape", [(3, 2, 2, 4), (2, 2, 2, 5), (2, 3, 1, 2), (1, 1, 1, 6)])
def test_box_partition(orc, dofmap, shape):
    ex, ey, ez, lx = shape
    m = orc.build_mesh(ex, ey, ez, lx, amp=0.0, seed=0)
    gid = dofmap.dofmap_from_vertices(box_vertices(ex, ey, ez), lx)
    assert same_partition(gid, m.gid)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_reoriented_elements(orc, dofmap, seed):
    ex, ey, ez, lx = 3, 3, 2, 5
    m = orc.build_mesh(ex, ey, ez, lx, amp=0.0, seed=0)
    ev2, g2 = reorient(lx, box_vertices(ex, ey, ez), m.gid, np.random.default_rng(seed))
    gid = dofmap.dofmap_from_vertices(ev2, lx)
    assert same_partition(gid, g2)


def test_bad_input(dofmap):
    with pytest.raises(ValueError):
        dofmap.dofmap_from_vertices(np.zeros((2, 7), dtype=np.int64), 4)
    ev = np.arange(16, dtype=np.int64).reshape(2, 8)
    ev[1, 7] = 2 ** 31  # face keys pack two ids into one int64
    with pytest.raises(ValueError):
        dofmap.dofmap_from_vertices(ev, 4)
