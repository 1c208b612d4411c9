"""Neko's binary mesh files (.nmsh) and solver meshes built from them.

The reference's cases load their meshes from .nmsh files ("mesh_file":
"*.nmsh", e.g. examples/brinkman_term/brinkman_term.case:4,
examples/mma/default.case:4).  The record layout (header, element records
of 8 (3D) or 4 (2D) vertex ids with coordinates, zones, curves) is read and
written by the C ABI (ntg_nmsh_info / ntg_nmsh_read / ntg_nmsh_write); this
module holds the records in numpy arrays, builds a coef_t from them
(global node ids from the vertex ids, GLL node coordinates by the
trilinear map of the vertices) and turns zones into Dirichlet masks.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np
import torch

from ._native import check, lib

# zone types as stored; labeled zones carry their label in p_f (column 3)
ZONE_LABELED = 7


@dataclass
class nmsh_t:
    """The records of one .nmsh file.  v_idx / xyz hold each element's
    vertices in tensor corner order (v = i + 2j + 4k); zones are the stored
    int32[9] records (e, f, p_e, p_f, pt_ids[4], type; e and f 1-based,
    faces r-, r+, s-, s+, t-, t+); curves the stored element, 12 x 5 data
    and 12 types."""
    gdim: int
    el_idx: np.ndarray
    v_idx: np.ndarray
    xyz: np.ndarray
    zones: np.ndarray = field(default_factory=lambda: np.zeros((0, 9), dtype=np.int32))
    curve_el: np.ndarray = field(default_factory=lambda: np.zeros(0, dtype=np.int32))
    curve_data: np.ndarray = field(default_factory=lambda: np.zeros((0, 12, 5)))
    curve_type: np.ndarray = field(default_factory=lambda: np.zeros((0, 12), dtype=np.int32))

    @property
    def nelv(self) -> int:
        return int(self.el_idx.shape[0])

    @property
    def nv(self) -> int:
        return 8 if self.gdim == 3 else 4

    def zone_faces(self, types=None, labels=None):
        """(element, face) pairs, 0-based, of the zones with a type in
        `types` and, for labeled zones, a label in `labels` (None: any)."""
        z = self.zones
        sel = np.ones(len(z), dtype=bool)
        if types is not None:
            sel &= np.isin(z[:, 8], list(types))
        if labels is not None:
            sel &= (z[:, 8] == ZONE_LABELED) & np.isin(z[:, 3], list(labels))
        return [(int(e) - 1, int(f) - 1) for e, f in z[sel, :2]]


def _vp(a):
    return None if a is None or a.size == 0 else C.c_void_p(a.ctypes.data)


def read(path) -> nmsh_t:
    """Read a .nmsh file (ntg_nmsh_read)."""
    p = os.fsencode(path)
    ne, gd, nz, nc = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
    check(lib().ntg_nmsh_info(p, C.byref(ne), C.byref(gd), C.byref(nz), C.byref(nc)))
    nv = 8 if gd.value == 3 else 4
    m = nmsh_t(int(gd.value), np.zeros(ne.value, dtype=np.int32), np.zeros((ne.value, nv), dtype=np.int32),
               np.zeros((ne.value, nv, 3)), np.zeros((nz.value, 9), dtype=np.int32),
               np.zeros(nc.value, dtype=np.int32), np.zeros((nc.value, 12, 5)), np.zeros((nc.value, 12), dtype=np.int32))
    check(lib().ntg_nmsh_read(p, _vp(m.el_idx), _vp(m.v_idx), _vp(m.xyz), _vp(m.zones), _vp(m.curve_el),
                              _vp(m.curve_data), _vp(m.curve_type)))
    return m


def write(path, m: nmsh_t) -> None:
    """Write a .nmsh file (ntg_nmsh_write)."""
    arrs = [np.ascontiguousarray(a, dtype=t) for a, t in
            ((m.el_idx, np.int32), (m.v_idx, np.int32), (m.xyz, np.float64), (m.zones, np.int32),
             (m.curve_el, np.int32), (m.curve_data, np.float64), (m.curve_type, np.int32))]
    el, vi, xyz, zo, ce, cd, ct = arrs
    if vi.shape != (el.shape[0], m.nv) or xyz.shape != (el.shape[0], m.nv, 3):
        raise ValueError("nmsh_t: v_idx / xyz do not match the element count and gdim")
    if zo.size and zo.shape[1] != 9:
        raise ValueError("nmsh_t: zones must be int32[9] records")
    check(lib().ntg_nmsh_write(os.fsencode(path), int(el.shape[0]), int(m.gdim), _vp(el), _vp(vi), _vp(xyz),
                               int(zo.shape[0]), _vp(zo), int(ce.shape[0]), _vp(ce), _vp(cd), _vp(ct)))


def coef_from_nmsh(m: nmsh_t, lx: int, device="cuda", curves: str = "error"):
    """A coef_t of a 3D .nmsh mesh at lx GLL points per direction: global
    node ids from the vertex ids (dofmap.dofmap_from_vertices, Neko's
    dofmap_t numbering), node coordinates trilinear in the vertices
    (ntg_nodes_from_vertices).  Curved sides are not applied: a mesh with
    curve records raises unless curves="ignore"."""
    from .api import _ptr, _stream, coef_t
    from .dofmap import dofmap_from_vertices
    if m.gdim != 3:
        raise ValueError("coef_from_nmsh: the solver takes 3D (hexahedral) meshes")
    if len(m.curve_el) and curves != "ignore":
        raise ValueError(f"coef_from_nmsh: {len(m.curve_el)} curved elements; pass curves='ignore' to use "
                         "straight sides")
    E = m.nelv
    gid = torch.from_numpy(dofmap_from_vertices(m.v_idx.astype(np.int64), lx)).to(device)
    xyz = torch.from_numpy(np.ascontiguousarray(m.xyz, dtype=np.float64)).to(device)
    n = E * lx ** 3
    x = torch.empty(n, dtype=torch.float64, device=device)
    y, z = torch.empty_like(x), torch.empty_like(x)
    check(lib().ntg_nodes_from_vertices(E, lx, _ptr(xyz, n=E * 24, name="xyz"), _ptr(x), _ptr(y), _ptr(z),
                                        _stream()))
    c = coef_t(E, lx, x, y, z, gid)
    c.nmsh = m
    return c


def face_mask(coef, faces, device=None):
    """Neko-style 1-based Dirichlet mask of every local node on the given
    element faces ((element, face) 0-based, faces r-, r+, s-, s+, t-, t+),
    all copies of each such node included."""
    lx = coef.lx
    N = lx - 1
    gid = coef.gid.cpu().numpy()
    sel = []
    s, t = np.meshgrid(np.arange(lx), np.arange(lx), indexing="xy")
    s, t = s.ravel(), t.ravel()
    for e, f in faces:
        d, nrm = f // 2, (N if f % 2 else 0)
        i, j, k = [(np.full_like(s, nrm), s, t), (s, np.full_like(s, nrm), t), (s, t, np.full_like(s, nrm))][d]
        sel.append(e * lx ** 3 + i + lx * (j + lx * k))
    if not sel:
        return torch.zeros(0, dtype=torch.int32, device=device or coef.device)
    g = np.unique(gid[np.concatenate(sel)])
    local = np.nonzero(np.isin(gid, g))[0] + 1
    return torch.from_numpy(local.astype(np.int32)).to(device or coef.device)
