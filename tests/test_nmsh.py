""".nmsh mesh files (neko-top_gb300/nmsh.py over ntg_nmsh_*): no GPU.

Pinned on the reference's own mesh files when the reference tree is present
(data/debugging_pipe.nmsh, a 3D hex pipe with labeled zones, and
examples/power_iterations/ext_cyl.nmsh, a 2D mesh with periodic zones and
curved sides): reading and writing them back reproduces every byte, and the
pipe's zones are exactly the faces no other element shares, with the face
numbering (r-, r+, s-, s+, t-, t+) of the tensor vertex order.  The rest
runs on the synthetic O-grid pipe of tests/meshgen.py."""
import os

import numpy as np
import pytest

import meshgen

REF = os.environ.get("NTG_REFERENCE_DIR", "/root/reference")
PIPE = os.path.join(REF, "data", "debugging_pipe.nmsh")
CYL = os.path.join(REF, "examples", "power_iterations", "ext_cyl.nmsh")
FACES = [[v for v in range(8) if (v >> (f // 2)) & 1 == f % 2] for f in range(6)]


@pytest.fixture(scope="module")
def nm(pkg):
    return pkg.nmsh


def boundary_faces(ev):
    cnt = {}
    for e in range(len(ev)):
        for f in range(6):
            k = tuple(sorted(ev[e, FACES[f]]))
            cnt[k] = cnt.get(k, 0) + 1
    return {(e + 1, f + 1) for e in range(len(ev)) for f in range(6) if cnt[tuple(sorted(ev[e, FACES[f]]))] == 1}


@pytest.mark.skipif(not os.path.exists(PIPE), reason="reference mesh files not present")
@pytest.mark.parametrize("path", [PIPE, CYL])
def test_reference_files_round_trip(nm, tmp_path, path):
    if not os.path.exists(path):
        pytest.skip("reference mesh file not present")
    m = nm.read(path)
    out = tmp_path / "rt.nmsh"
    nm.write(out, m)
    assert open(path, "rb").read() == out.read_bytes()


@pytest.mark.skipif(not os.path.exists(PIPE), reason="reference mesh files not present")
def test_reference_pipe_zones_are_its_boundary(nm):
    m = nm.read(PIPE)
    assert (m.nelv, m.gdim, len(m.zones), len(m.curve_el)) == (160, 3, 192, 0)
    # the same vertex id always has the same coordinates
    ids, xyz = m.v_idx.ravel(), m.xyz.reshape(-1, 3)
    o = np.argsort(ids, kind="stable")
    same = ids[o][1:] == ids[o][:-1]
    assert np.all(xyz[o][1:][same] == xyz[o][:-1][same])
    # zones = the unshared faces, numbered in the tensor frame
    assert {(int(e), int(f)) for e, f in m.zones[:, :2]} == boundary_faces(m.v_idx)
    # right-handed elements: positive corner Jacobians
    X = m.xyz
    for v in range(8):
        i, j, k = v & 1, (v >> 1) & 1, v >> 2
        d = [X[:, v ^ (1 << a)] - X[:, v] for a in range(3)]
        d = [dd * (1 if (i, j, k)[a] == 0 else -1) for a, dd in enumerate(d)]
        assert np.all(np.einsum("ei,ei->e", np.cross(d[0], d[1]), d[2]) > 0)
    # labeled zones carry the sidesets: 1, 2 at x = 0, 3 at x = 10, 4 the walls
    for lab, xs in ((1, 0.0), (2, 0.0), (3, 10.0)):
        for e, f in m.zone_faces(labels=[lab]):
            assert np.allclose(m.xyz[e, FACES[f], 0], xs)


def test_synthetic_round_trip(nm, tmp_path):
    ev, xyz, zones = meshgen.ogrid_pipe(2, 2, 3)
    m = nm.nmsh_t(3, np.arange(1, len(ev) + 1, dtype=np.int32), ev.astype(np.int32), xyz, zones)
    path = tmp_path / "ogrid.nmsh"
    nm.write(path, m)
    assert path.stat().st_size == 8 + len(ev) * 228 + 4 + len(zones) * 36 + 4
    r = nm.read(path)
    assert r.gdim == 3 and np.array_equal(r.v_idx, m.v_idx) and np.array_equal(r.xyz, m.xyz)
    assert np.array_equal(r.zones, zones) and np.array_equal(r.el_idx, m.el_idx)
    assert {(int(e), int(f)) for e, f in zones[:, :2]} == boundary_faces(ev)
    assert len(r.zone_faces(labels=[2])) == 20 and len(r.zone_faces(types=[7])) == len(zones)


def test_bad_files(nm, tmp_path, pkg):
    bad = tmp_path / "bad.nmsh"
    bad.write_bytes(b"\x02\x00\x00\x00\x05\x00\x00\x00")  # gdim 5
    with pytest.raises(pkg.NtgError):
        nm.read(bad)
    ev, xyz, zones = meshgen.ogrid_pipe(1, 1, 1)
    good = tmp_path / "good.nmsh"
    nm.write(good, nm.nmsh_t(3, np.arange(1, len(ev) + 1, dtype=np.int32), ev.astype(np.int32), xyz, zones))
    trunc = tmp_path / "trunc.nmsh"
    trunc.write_bytes(good.read_bytes()[:-3])
    with pytest.raises(pkg.NtgError):
        nm.read(trunc)
    with pytest.raises(pkg.NtgError):
        nm.read(tmp_path / "missing.nmsh")


def test_face_mask_covers_every_copy(nm, pkg):
    """nmsh.face_mask: every local copy of every node on the selected zone
    faces, 1-based, sorted (host arrays: the coefficients are not needed)."""
    import torch

    ev, xyz, zones = meshgen.ogrid_pipe(2, 1, 2)
    lx = 4
    gid = pkg.dofmap.dofmap_from_vertices(ev, lx)

    class Stub:
        pass

    c = Stub()
    c.lx, c.gid, c.device = lx, torch.from_numpy(gid), torch.device("cpu")
    m = nm.nmsh_t(3, np.arange(1, len(ev) + 1, dtype=np.int32), ev.astype(np.int32), xyz, zones)
    faces = m.zone_faces(labels=[2])
    mask = nm.face_mask(c, faces).numpy()
    # the nodes on those faces, by position: z = length
    X = meshgen.nodes_from_vertices(xyz, lx)
    on_face = np.isclose(X[2], 1.5)
    assert np.array_equal(np.sort(mask), np.nonzero(on_face)[0] + 1)
    assert mask.dtype == np.int32 and np.all(np.diff(mask) > 0)
    assert len(nm.face_mask(c, [])) == 0
