"""Field files (Nek5000 binary "#std" format of Neko's fld_file_t): written
from host arrays by the library and parsed here by an independent numpy
reader, in single and double precision; the library's reader round trip;
the .nek5000 index file.  Host code only (no GPU)."""
import numpy as np
import pytest


def parse(path):
    """Independent reader of the format (header, byte-order mark, element
    numbers, per-element blocks, per-element min/max)."""
    raw = open(path, "rb").read()
    hdr = raw[:132].decode()
    tok = hdr.split()
    assert tok[0] == "#std"
    wd, lx, ly, lz, nel, nelg = (int(t) for t in tok[1:7])
    time, step = float(tok[7]), int(tok[8])
    code = tok[11]
    assert np.frombuffer(raw[132:136], "<f4")[0] == np.float32(6.54321)
    el = np.frombuffer(raw[136:136 + 4 * nel], "<i4")
    off = 136 + 4 * nel
    dt = "<f4" if wd == 4 else "<f8"
    l3 = lx * ly * lz
    fields, i = {}, 0
    comps = []
    while i < len(code):
        c = code[i]
        if c in "XU":
            comps.append((c, 3))
            i += 1
        elif c in "PT":
            comps.append((c, 1))
            i += 1
        else:
            comps.append(("S", int(code[i + 1:i + 3])))
            i += 3
    for c, nc in comps:
        cnt = nel * nc * l3
        blk = np.frombuffer(raw[off:off + cnt * wd], dt).astype(np.float64)
        off += cnt * wd
        if c in "XU":
            fields[c] = blk.reshape(nel, nc, l3).transpose(1, 0, 2).reshape(nc, -1)
        else:
            fields[c] = blk.reshape(nc, nel * l3)
    meta = {}
    for c, nc in comps:
        cnt = nel * nc * 2
        m = np.frombuffer(raw[off:off + 4 * cnt], "<f4")
        off += 4 * cnt
        meta[c] = m.reshape(nel, nc, 2) if c in "XU" else m.reshape(nc, nel, 2)
    assert off == len(raw)
    return dict(wd=wd, lx=lx, nel=nel, nelg=nelg, time=time, step=step, code=code, el=el, fields=fields,
                meta=meta)


def fields(ne, lx, seed=0):
    rng = np.random.default_rng(seed)
    n = ne * lx ** 3
    return {k: rng.standard_normal(n) for k in ("x", "y", "z", "u", "v", "w", "p", "t")}, \
        [rng.standard_normal(n) for _ in range(2)]


@pytest.mark.parametrize("precision", ["sp", "dp"])
def test_written_file_parses_independently(pkg, tmp_path, precision):
    ne, lx = 5, 4
    f, s = fields(ne, lx)
    path = tmp_path / "field0.f00003"
    el = np.array([3, 1, 5, 2, 4])
    pkg.fld_file_t(path, precision).write(dict(f, s=s), lx, ne, t=0.125, tstep=30, glb_el=el)
    r = parse(path)
    assert (r["wd"], r["lx"], r["nel"], r["nelg"], r["step"]) == (4 if precision == "sp" else 8, lx, ne, ne, 30)
    assert r["time"] == 0.125 and r["code"] == "XUPTS02"
    assert np.array_equal(r["el"], el)
    cast = (lambda a: a.astype(np.float32).astype(np.float64)) if precision == "sp" else (lambda a: a)
    for c, keys in (("X", "xyz"), ("U", "uvw")):
        for q, k in enumerate(keys):
            assert np.array_equal(r["fields"][c][q], cast(f[k]))
    assert np.array_equal(r["fields"]["P"][0], cast(f["p"]))
    assert np.array_equal(r["fields"]["T"][0], cast(f["t"]))
    for q in range(2):
        assert np.array_equal(r["fields"]["S"][q], cast(s[q]))
    # per-element min/max of each component
    xe = f["x"].reshape(ne, -1)
    assert np.array_equal(r["meta"]["X"][:, 0, 0], xe.min(1).astype(np.float32))
    assert np.array_equal(r["meta"]["X"][:, 0, 1], xe.max(1).astype(np.float32))
    se = s[1].reshape(ne, -1)
    assert np.array_equal(r["meta"]["S"][1, :, 1], se.max(1).astype(np.float32))


def test_library_reader_round_trip(pkg, tmp_path):
    ne, lx = 3, 6
    f, s = fields(ne, lx, seed=1)
    path = tmp_path / "adj0.f00000"
    fl = pkg.fld_file_t(path, "dp")
    fl.write({"u": f["u"], "v": f["v"], "w": f["w"], "p": f["p"], "s": s[:1]}, lx, ne, t=2.5, tstep=7)
    r = fl.read()
    assert r["rdcode"] == "UPS01" and r["lx"] == lx and r["nelv"] == ne and r["time"] == 2.5
    for k in ("u", "v", "w", "p"):
        assert np.array_equal(r[k], f[k])
    assert np.array_equal(r["s"][0], s[0]) and list(r["glb_el"]) == [1, 2, 3]
    assert "x" not in r


def test_index_file(pkg, tmp_path):
    p = tmp_path / "field.nek5000"
    pkg.fld_file_t.write_index(p, "field", 0, 12)
    assert p.read_text() == "filetemplate: field%01d.f%05d\nfirsttimestep: 0\nnumtimesteps: 12\n"


def test_bad_arguments_are_refused(pkg, tmp_path):
    with pytest.raises(pkg.NtgError):
        pkg.fld_file_t(tmp_path / "a.f00000").write({"x": np.zeros(8)}, 2, 1)  # x without y, z
    with pytest.raises(pkg.NtgError):
        pkg.fld_file_t(tmp_path / "missing.f00000").info()
