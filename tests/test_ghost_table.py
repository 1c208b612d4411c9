"""The general-mesh Schwarz preconditioner's face-neighbour table as the
library builds it (ntg_schwarz_ghost_table, host code, no GPU) against the
oracle's independent construction (oracle/schwarz_ref.face_ghosts): equal
entry for entry on the O-grid pipe, on boxes with re-oriented elements and
on the reference's own pipe mesh (data/debugging_pipe.nmsh, when present);
a non-conforming mesh is refused."""
import ctypes as C
import os

import numpy as np
import pytest

import meshgen
from oracle import schwarz_ref

REF = os.environ.get("NTG_REFERENCE_DIR", "/root/reference")
PIPE = os.path.join(REF, "data", "debugging_pipe.nmsh")


def lib_table(pkg, gid, nelv, lx):
    gid = np.ascontiguousarray(gid, dtype=np.int64)
    out = np.empty(nelv * 6 * lx * lx, dtype=np.int32)
    st = pkg.lib().ntg_schwarz_ghost_table(nelv, lx, C.c_void_p(gid.ctypes.data), C.c_void_p(out.ctypes.data))
    return st, out.reshape(nelv, 6, lx * lx)


class _Mesh:
    def __init__(self, gid, nelv, lx):
        self.gid, self.nelv, self.lx = gid, nelv, lx


@pytest.mark.parametrize("lx", [4, 6])
def test_ogrid(pkg, lx):
    ev, xyz, zones = meshgen.ogrid_pipe(2, 2, 3)
    gid = pkg.dofmap.dofmap_from_vertices(ev, lx)
    st, tab = lib_table(pkg, gid, len(ev), lx)
    assert st == 0
    ref = schwarz_ref.face_ghosts(_Mesh(gid, len(ev), lx))
    assert np.array_equal(tab, ref)
    # boundary faces are exactly the zones
    bnd = {(e, f) for e in range(len(ev)) for f in range(6) if tab[e, f, 0] < 0}
    assert bnd == {(int(e) - 1, int(f) - 1) for e, f in zones[:, :2]}


def test_reoriented_box(pkg, orc):
    lx = 5
    m = orc.build_mesh(3, 3, 2, lx, amp=0.0, seed=0)
    N, l3 = lx - 1, lx ** 3
    ev = np.stack([m.gid.reshape(m.nelv, l3)[:, (v & 1) * N + lx * ((v >> 1) & 1) * N + lx * lx * (v >> 2) * N]
                   for v in range(8)], 1)
    _, (g2,) = meshgen.reorient(lx, ev, [m.gid], np.random.default_rng(4), rotations_only=False)
    g2 = g2.astype(np.int64)
    st, tab = lib_table(pkg, g2, m.nelv, lx)
    assert st == 0
    assert np.array_equal(tab, schwarz_ref.face_ghosts(_Mesh(g2, m.nelv, lx)))
    # every interior face of the 3 x 3 x 2 box has a neighbour: 2*(2*3*2 + 3*2*2 + 3*3*1) faces x 2 sides
    assert int((tab[:, :, 0] >= 0).sum()) == 2 * (2 * 3 * 2 + 3 * 2 * 2 + 3 * 3 * 1)


@pytest.mark.skipif(not os.path.exists(PIPE), reason="reference mesh files not present")
def test_reference_pipe(pkg):
    mesh = pkg.nmsh.read(PIPE)
    lx = 4
    gid = pkg.dofmap.dofmap_from_vertices(mesh.v_idx.astype(np.int64), lx)
    st, tab = lib_table(pkg, gid, mesh.nelv, lx)
    assert st == 0
    assert np.array_equal(tab, schwarz_ref.face_ghosts(_Mesh(gid, mesh.nelv, lx)))
    bnd = {(e, f) for e in range(mesh.nelv) for f in range(6) if tab[e, f, 0] < 0}
    assert bnd == {(int(e) - 1, int(f) - 1) for e, f in mesh.zones[:, :2]}


def test_non_conforming_refused(pkg):
    # three elements claiming the same face: element 2 duplicates element 1
    lx = 3
    ev, _, _ = meshgen.ogrid_pipe(1, 1, 1)
    ev = np.concatenate([ev[:2], ev[1:2]])
    gid = pkg.dofmap.dofmap_from_vertices(ev, lx)
    st, _ = lib_table(pkg, gid, len(ev), lx)
    assert st != 0
    assert b"non-conforming" in pkg.lib().ntg_last_error()
