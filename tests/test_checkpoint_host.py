"""Host side of the sequence checkpoint (no GPU): SolveSequence.state_dict
-> save -> load -> load_state_dict moves every piece of state unchanged,
and a checkpoint of another guess mode is refused.  The device side (the
basis, network and history copies) is tested bit for bit in
test_gpu_checkpoint.py."""
import pytest
import torch


class FakeProj:
    def __init__(self, m, xs, axs):
        self.m, self.xs, self.axs = m, xs, axs

    def state(self):
        return self.m, self.xs, self.axs

    def load_state(self, m, xs, axs):
        self.m, self.xs, self.axs = m, xs.clone(), axs.clone()


class FakeNet:
    def __init__(self, st):
        self.st = st

    def state(self):
        return self.st

    def load_state(self, st):
        self.st = {k: (v.clone() if isinstance(v, torch.Tensor) else list(v)) for k, v in st.items()}


def _seq(pkg, proj, net, guess="learned"):
    s = object.__new__(pkg.SolveSequence)
    s.guess, s.proj, s.net = guess, proj, net
    s.nsolved, s.training = 0, True
    return s


def test_state_round_trip(pkg, tmp_path):
    g = torch.Generator().manual_seed(0)
    xs, axs = torch.randn(3, 50, generator=g, dtype=torch.float64), torch.randn(3, 50, generator=g,
                                                                              dtype=torch.float64)
    net = {"buf": torch.randn(123, generator=g), "ints": [7, 2, 4, 0], "hrms": [0.5, 1.5] + [0.0] * 6}
    a = _seq(pkg, FakeProj(3, xs, axs), FakeNet(net))
    a.nsolved, a.training = 57, False
    path = str(tmp_path / "ck.pt")
    a.save(path)
    b = _seq(pkg, FakeProj(0, torch.zeros(0, 50), torch.zeros(0, 50)), FakeNet({}))
    b.load(path)
    assert (b.nsolved, b.training) == (57, False)
    assert b.proj.m == 3 and torch.equal(b.proj.xs, xs) and torch.equal(b.proj.axs, axs)
    assert torch.equal(b.net.st["buf"], net["buf"]) and b.net.st["ints"] == net["ints"]
    assert b.net.st["hrms"] == net["hrms"]
    c = _seq(pkg, None, None, guess="zero")
    with pytest.raises(ValueError):
        c.load(path)
