"""GPU parity of the momentum-predictor solves (include/scf_mom.h) against
the oracle, through the C-ABI.

Operator, right-hand side and Dp bit for bit; the predicted velocity within
1e-11 (rel. L2) of the oracle's direct solve of the same system (the GPU
solve stops at relative residual 1e-14)."""
import numpy as np
import pytest

from simcoflow_gb300 import momentum as M
from gen import synth

pytestmark = pytest.mark.gpu

CASES = [lambda: synth.c1(), lambda: synth.c1(n=33), lambda: synth.c4(n=256, instance=3),
         lambda: synth.random_instance(5, 96, 9), lambda: synth.c5(instance=2, n=160)]
IDS = ["c1_128", "c1_33", "c4_256", "r96", "c5_160"]


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("comp", ["u", "v"])
@pytest.mark.parametrize("mk", CASES, ids=IDS)
def test_parity_vs_oracle(cuda, oracle, mk, comp):
    mi = synth.momentum_inputs(mk(), comp)
    exp = oracle.mom_predict(mi)
    g = M.predict(mi, rtol=1e-14)
    assert np.array_equal(g["matr"], exp["matr"])
    assert np.array_equal(g["rhm"], exp["rhm"])
    assert np.array_equal(g["Dp"], exp["Dp"])
    assert rel(g["pred"], exp["pred"]) <= 1e-11
    st = g["stats"]
    assert st["status"] == 0 and 0 < st["iters"] <= 20 and st["relres"] <= 1e-14
    assert st["launches"] >= 3 * st["iters"] + 3


def test_deterministic_and_device_pointers(cuda):
    import torch
    mi = synth.momentum_inputs(synth.c4(n=200, instance=1), "v")
    a = M.predict(mi)
    b = M.predict(mi)
    assert np.array_equal(a["pred"], b["pred"]) and np.array_equal(a["Dp"], b["Dp"])
    dev = torch.device("cuda", 0)
    T = lambda x: torch.from_numpy(np.ascontiguousarray(x.ravel(order="F"))).to(dev)
    s = M.MomentumSolver(mi["nx"], mi["ny"], device_ptrs=True)
    try:
        tin = {k: (T(v) if isinstance(v, np.ndarray) else v) for k, v in mi.items()}
        pred, Dp = T(mi["pred"]), T(mi["Dp"])
        s.solve("v", tin, pred, Dp)
        torch.cuda.synchronize()
    finally:
        s.close()
    shp = (mi["nx"] + 2, mi["ny"] + 2)
    assert np.array_equal(pred.cpu().numpy().reshape(shp, order="F"), a["pred"])
    assert np.array_equal(Dp.cpu().numpy().reshape(shp, order="F"), a["Dp"])


@pytest.mark.parametrize("comp", ["u", "v"])
def test_diagonal_system_closed_form(cuda, comp):
    mi = synth.momentum_inputs(synth.c1(n=64), comp)
    for k in ("difEW", "difNS", "edEW", "edNS", "WlLh"):
        mi[k] = np.zeros_like(mi[k], order="F")
    g = M.predict(mi)
    nx, ny, iu, iv = mi["nx"], mi["ny"], mi["iu"], mi["iv"]
    dx, dy, dt = mi["dx"], mi["dy"], mi["dt"]
    act = mi["posnu"][1:nx + 1, 1:ny + 1] != -1
    rhs = -mi["flux"] - (1.0 / mi["fr"] ** 2 * dx * dy if comp == "v" else 0.0)
    exp = np.where(act, rhs / (dx * dy / dt), 0.0) + dt * mi["gradp"] / dx / dy
    r = (slice(0, nx - iu), slice(0, ny - iv))
    np.testing.assert_allclose(g["pred"][1:nx + 1, 1:ny + 1][r], exp[r], rtol=1e-12, atol=1e-300)
    assert g["stats"]["iters"] <= 2


def test_zero_rhs_and_bad_arguments(cuda):
    mi = synth.momentum_inputs(synth.c1(n=32), "u")
    mi["flux"] = np.zeros_like(mi["flux"], order="F")
    mi["u"] = np.zeros_like(mi["u"], order="F")
    mi["gradp"] = np.zeros_like(mi["gradp"], order="F")
    g = M.predict(mi)
    assert g["stats"]["iters"] == 0 and g["stats"]["status"] == 0
    assert np.all(g["pred"][1:32, 1:33] == 0.0)
    s = M.MomentumSolver(32, 32)
    try:
        bad = dict(mi)
        bad["dx"] = np.zeros((31, 32), order="F")
        with pytest.raises(ValueError):
            s.solve("u", bad, mi["pred"].copy(order="F"), mi["Dp"].copy(order="F"))
    finally:
        s.close()


@pytest.mark.parametrize("comp", ["u", "v"])
@pytest.mark.parametrize("mk", [lambda: synth.c1(n=96), lambda: synth.c4(n=128, instance=3)],
                         ids=["c1_96", "c4_128"])
def test_multigrid_preconditioner_where_diffusion_dominates(cuda, oracle, mk, comp):
    """Reynolds number 0.01: the viscous couplings outweigh dx dy / dt by
    about a hundred, the diagonal preconditioner needs hundreds of
    iterations, the multigrid V-cycle (SCF_MOM_MG) a handful; the same
    operator bit for bit and the same solution as the oracle's direct solve."""
    mi = synth.momentum_inputs(mk(), comp, rey=0.01)
    exp = oracle.mom_predict(mi)
    mg = M.predict(mi, rtol=1e-13, maxit=100, mg=True)
    diag = M.predict(mi, rtol=1e-13, maxit=3000)
    for g in (mg, diag):
        assert np.array_equal(g["matr"], exp["matr"])
        assert np.array_equal(g["Dp"], exp["Dp"])
        assert g["stats"]["status"] == 0
        assert rel(g["pred"], exp["pred"]) <= 1e-10
    assert mg["stats"]["iters"] * 5 <= diag["stats"]["iters"]


def test_multigrid_preconditioner_on_the_predictor_workload(cuda, oracle):
    """At the benchmark's Reynolds number the diagonal already converges in
    a few iterations; the multigrid one matches it and the oracle."""
    mi = synth.momentum_inputs(synth.c4(n=256, instance=3), "u")
    exp = oracle.mom_predict(mi)
    g = M.predict(mi, rtol=1e-14, mg=True)
    assert np.array_equal(g["matr"], exp["matr"])
    assert rel(g["pred"], exp["pred"]) <= 1e-11
    assert g["stats"]["status"] == 0 and g["stats"]["iters"] <= 10
