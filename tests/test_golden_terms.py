"""The step-term and MMA oracles still reproduce their frozen fixtures
(tests/golden/golden_terms.npz, made by tests/golden/make_golden_terms.py),
and the MMA fixture ends near the optimum the reference's test states."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden_terms.npz")


@pytest.fixture(scope="module")
def fresh(orc):
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "make_golden_terms", os.path.join(os.path.dirname(GOLDEN), "make_golden_terms.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.cases()


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLDEN))


def test_same_keys(fresh, gold):
    assert set(fresh) == set(gold)


@pytest.mark.parametrize("prefix", ["vel_res", "prs_res", "adj", "lin", "adj_d", "lin_d", "md", "mma_toy"])
def test_oracle_reproduces_fixture(fresh, gold, prefix):
    keys = [k for k in gold if k.startswith(prefix) and (prefix != "adj" or k[3:].isdigit())
            and (prefix != "lin" or k[3:].isdigit())]
    assert keys
    for k in keys:
        a, b = fresh[k], gold[k]
        assert np.abs(a - b).max() <= 1e-11 * max(np.abs(b).max(), 1.0), k


def test_mma_fixture_reaches_the_stated_optimum(gold):
    assert np.allclose(gold["mma_toy1"][-1], gold["mma_toy1_stated_optimum"], atol=2e-3)
