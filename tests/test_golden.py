"""The oracle still reproduces the frozen golden fixtures (tests/golden/,
made by tests/golden/make_golden.py).  Tolerances allow for OpenMP
reduction order in the oracle's dot products."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden.npz")


@pytest.fixture(scope="module")
def fresh(orc):
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "make_golden", os.path.join(os.path.dirname(GOLDEN), "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.cases()


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLDEN))


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def test_golden_operator_and_maps(fresh, gold):
    assert rel(fresh["ax_w"], gold["ax_w"]) < 1e-14
    assert rel(fresh["ax_w_gs"], gold["ax_w_gs"]) < 1e-14
    assert np.array_equal(fresh["gs_perm"], gold["gs_perm"])
    assert np.array_equal(fresh["gs_offs"], gold["gs_offs"])
    assert np.array_equal(fresh["mult"], gold["mult"])


def test_golden_solve_ramp_schwarz(fresh, gold):
    assert abs(int(fresh["cg_iters"][0]) - int(gold["cg_iters"][0])) <= 1
    assert np.linalg.norm(fresh["cg_x"] - gold["cg_x"]) <= 1e-9 * np.linalg.norm(gold["cg_x"])
    for k in ("ramp_fwd_0", "ramp_bwd_0", "ramp_fwd_1", "ramp_bwd_1"):
        assert rel(fresh[k], gold[k]) < 1e-15, k
    assert rel(fresh["sw_z"], gold["sw_z"]) < 1e-11
