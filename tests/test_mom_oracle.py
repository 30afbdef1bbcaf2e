"""CPU checks of the momentum-predictor oracle (oracle/mom_oracle.c): the
restated SetMatrix / SetVectors system, its solves, and a closed-form case."""
import numpy as np
import pytest

from gen import synth

CASES = [lambda: synth.c1(n=48), lambda: synth.c4(n=64, instance=2),
         lambda: synth.random_instance(5, 40, 3)]


@pytest.mark.parametrize("comp", ["u", "v"])
@pytest.mark.parametrize("mk", CASES, ids=["c1_48", "c4_64", "r40"])
def test_solvers_agree_and_solve_the_system(oracle, mk, comp):
    mi = synth.momentum_inputs(mk(), comp)
    d = oracle.mom_predict(mi)
    assert not d["bad"]
    A, b, x = d["A"], d["b"], d["x"]
    assert np.linalg.norm(A @ x - b) <= 1e-13 * np.linalg.norm(b)
    e = oracle.mom_predict(mi, solver="bicgstab", rtol=1e-14)
    assert 0 < e["iters"] <= 20
    assert np.abs(e["pred"] - d["pred"]).max() <= 1e-12 * np.abs(d["pred"]).max()
    assert np.array_equal(e["Dp"], d["Dp"])


@pytest.mark.parametrize("comp", ["u", "v"])
def test_boundary_rules(oracle, comp):
    """U: no east/west diffusion coefficient on the first and last U cells
    and none north of the top row; V: none north of the top V row
    (src/PredictorUV_mod.f90:659-661, :675)."""
    mi = synth.momentum_inputs(synth.c1(n=40), comp)
    m = oracle.mom_operator(mi)["matr"]
    nx, ny = mi["nx"], mi["ny"]
    act = mi["posnu"][1:nx + 1, 1:ny + 1] != -1
    if comp == "u":
        assert np.all(m[0, :, 1] == 0) and np.all(m[nx - 2, :, 3] == 0)
        assert np.all(m[:nx - 1, ny - 1, 4] == 0)
        assert np.all(m[nx - 1, :, :] == 0)          # no U unknowns at i = nx
    else:
        assert np.all(m[:, ny - 2, 4] == 0)
        assert np.all(m[:, ny - 1, :] == 0)          # no V unknowns at j = ny
    rng = (slice(0, nx - 1), slice(None)) if comp == "u" else (slice(None), slice(0, ny - 1))
    assert np.all(m[rng][..., 2][act[rng]] > 0)


@pytest.mark.parametrize("comp", ["u", "v"])
def test_diagonal_system_closed_form(oracle, comp):
    """Without diffusion, skew fluxes and walls the operator is dx dy / dt on
    the diagonal: Pred = rhs dt / (dx dy) + dt GradP / dx / dy and Dp = dt."""
    c = synth.c1(n=32)
    mi = synth.momentum_inputs(c, comp)
    for k in ("difEW", "difNS", "edEW", "edNS", "WlLh"):
        mi[k] = np.zeros_like(mi[k], order="F")
    d = oracle.mom_predict(mi)
    nx, ny, iu, iv = mi["nx"], mi["ny"], mi["iu"], mi["iv"]
    dx, dy, dt = mi["dx"], mi["dy"], mi["dt"]
    act = mi["posnu"][1:nx + 1, 1:ny + 1] != -1
    rhs = -mi["flux"]
    if comp == "v":
        rhs = rhs - 1.0 / mi["fr"] ** 2 * dx * dy
    x = np.where(act, rhs / (dx * dy / dt), 0.0)
    exp = x + dt * mi["gradp"] / dx / dy
    got = d["pred"][1:nx + 1, 1:ny + 1]
    rng = (slice(0, nx - iu), slice(0, ny - iv))
    np.testing.assert_allclose(got[rng], exp[rng], rtol=1e-13, atol=1e-300)
    Dp = d["Dp"][1:nx + 1, 1:ny + 1]
    np.testing.assert_allclose(Dp[rng][act[rng]], dt, rtol=1e-14)
