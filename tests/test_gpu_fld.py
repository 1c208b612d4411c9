"""Field files written from device arrays are byte-identical to those
written from the same host arrays, and read back onto the device."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_device_fields_write_and_read(pkg, dev, tmp_path):
    ne, lx = 4, 8
    rng = np.random.default_rng(2)
    host = {k: rng.standard_normal(ne * lx ** 3) for k in ("x", "y", "z", "p")}
    devf = {k: torch.from_numpy(v).to(dev) for k, v in host.items()}
    a, b = tmp_path / "h0.f00000", tmp_path / "d0.f00000"
    pkg.fld_file_t(a).write(host, lx, ne, t=1.0, tstep=1)
    pkg.fld_file_t(b).write(devf, lx, ne, t=1.0, tstep=1)
    assert a.read_bytes() == b.read_bytes()
    r = pkg.fld_file_t(b, "sp").read(device=dev)
    assert r["rdcode"] == "XP"
    assert torch.equal(r["p"].cpu(), torch.from_numpy(host["p"].astype(np.float32).astype(np.float64)))
