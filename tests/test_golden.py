"""The oracle reproduces the committed golden fixtures (CPU)."""
import numpy as np
import pytest

from helpers import GOLDEN_CASES, load_golden, rel_l2


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_oracle_reproduces_golden(oracle, name):
    c, exp = load_golden(name)
    r = oracle.project(c)
    # assembly, right-hand side: bit for bit
    assert np.array_equal(r["pocoef"], exp["pocoef"])
    assert np.array_equal(r["matr"], exp["matr"])
    assert np.array_equal(r["rhm"], exp["rhm"])
    # direct FP64 solve and correction: to rounding
    assert rel_l2(r["Pp"], exp["Pp"]) < 1e-12
    assert rel_l2(r["u"], exp["u"]) < 1e-12
    assert rel_l2(r["v"], exp["v"]) < 1e-12
    assert np.abs(r["mres"] - exp["mres"]).max() < 1e-13
    assert r["row_residual"] <= 1e-10
