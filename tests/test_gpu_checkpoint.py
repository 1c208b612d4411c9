"""Checkpoint / resume of a solve sequence (the reference restarts from
checkpoint files at sources/adjoint/simulation_adjoint.f90:208-256): a
sequence stopped mid-way, saved to a file and restored into fresh objects
continues with bit-identical iterates -- projection basis, network weights,
Adam moments and step, solution history and counters all round-trip."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _case(pkg, dev):
    coef = pkg.coef_t.box(4, 3, 3, 8, amp=0.05, seed=4, device=dev)
    coef.set_mask(pkg.mask_face_xmax(4, 3, 3, 8, device=dev), base=1)
    rho = coef.field_blobs(3, 12, 0.1)
    chi = torch.empty_like(rho)
    pkg.RAMP_mapping_t(0.0, 1e4, 8.0, False).apply_forward(chi, 1.0 - rho)
    coef.set_coefs(h1c=1.0, h2=chi, ifh2=True)
    k, ph, amps = pkg.ar1_modes(5, 32, 12, rho=0.98)
    rhs = [coef.rhs_assemble(coef.field_modes(k, amps[t], ph)) for t in range(12)]
    return coef, rhs


@pytest.mark.parametrize("guess", ["learned", "projection"])
def test_resume_is_bit_identical(pkg, dev, tmp_path, guess):
    coef, rhs = _case(pkg, dev)

    def seq():
        return pkg.SolveSequence(coef, "cg_mixed", guess, rtol=1e-10, L=4, train_steps=5, seed=1, lr=1e-3,
                                 pc="jacobi", delta=0.1)

    ref = seq()
    xs_ref, it_ref = [], []
    for t in range(12):
        ref.training = t < 8
        x, mon, _, _ = ref.solve(rhs[t])
        xs_ref.append(x.clone())
        it_ref.append(mon.iter)
    del ref

    a = seq()
    for t in range(6):
        a.training = t < 8
        a.solve(rhs[t])
    path = str(tmp_path / "seq.pt")
    a.save(path)
    del a
    b = seq()
    b.load(path)
    assert b.nsolved == 6
    for t in range(6, 12):
        b.training = t < 8
        x, mon, _, _ = b.solve(rhs[t])
        assert mon.iter == it_ref[t], (t, mon.iter, it_ref[t])
        assert torch.equal(x, xs_ref[t]), t


def test_solve_log_lines(pkg, dev, tmp_path):
    import json
    coef, rhs = _case(pkg, dev)
    path = tmp_path / "solves.jsonl"
    s = pkg.SolveSequence(coef, "cg_mixed", "projection", rtol=1e-10, L=4, pc="jacobi", delta=0.1, log=str(path))
    for t in range(3):
        s.solve(rhs[t], extra={"t": t})
    s.close()
    lines = [json.loads(l) for l in open(path)]
    assert [l["solve"] for l in lines] == [0, 1, 2] and [l["t"] for l in lines] == [0, 1, 2]
    for l in lines:
        assert l["status"] == 0 and l["rel_res"] <= 1e-10 * (1 + 1e-9) and l["iter"] > 0
    assert lines[0]["guess"] == "projection"
