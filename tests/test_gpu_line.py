"""Line smoother on stretched grids (the 4096^2 configuration's grid, scaled
down): GPU V-cycle against the oracle's, and full projections against the
oracle's direct solve, in both precisions, through the C-ABI."""
import numpy as np
import pytest

from helpers import rel_l2
from gen import synth
from simcoflow_gb300 import projection as P

pytestmark = pytest.mark.gpu

TOL_P = 1e-8
TOL_UV = 1e-9


def _active(c):
    return c["posnu_p"][1:c.nx + 1, 1:c.ny + 1] != -1


def _odd_stretched():
    from gen import geometry as G
    rng = np.random.Generator(np.random.PCG64(23))
    xf = G.axis(38, 0.0, 1.0)
    yf = G.axis(30, 0.0, 1.0, True, 0.45, 0.55, 12)
    solids = [G.Solid(G.SOLID_BOX, 0.5, 0.3, hw=0.2, hh=0.03, angle=np.deg2rad(10.0))]
    surf = G.Surface(0.5, [0.02], [2 * np.pi], [0.4])
    return synth.build_case("odd_stretched", xf, yf, solids, surf, synth._modes(rng, 8),
                            synth._modes(rng, 8), 1e-3, 800.0)


@pytest.mark.parametrize("coarse", [None, (1, 4)], ids=["one_step", "two_steps_from_1"])
@pytest.mark.parametrize("maker", [lambda: synth.c3(n=128), _odd_stretched],
                         ids=["c3_128", "odd37x29"])
def test_line_vcycle_matches_oracle(cuda, oracle, maker, coarse):
    """One alternating step per side everywhere, or two from level 1 down
    (the per-level kernels and the single-CTA tail)."""
    c = maker()
    matr, _ = oracle.matrix(c)
    rng = np.random.Generator(np.random.PCG64(7))
    b = np.asfortranarray(rng.normal(size=(c.nx, c.ny)) * _active(c))
    s = P.ProjectionSolver(c.nx, c.ny, smoother="line")
    try:
        s.setup_case(c)
        if coarse:
            s.set_coarse_sweeps(*coarse)
        xg = s.vcycle(b)
    finally:
        s.close()
    xo = oracle.vcycle(c, matr, b, npre=2, npost=2, omega=1.9, smoother="line", coarse=coarse)
    # partitioned line solves (Schur complement + cyclic reduction) against
    # the Thomas algorithm: the same exact line solves, other rounding
    assert rel_l2(xg, xo) < 1e-10


@pytest.mark.parametrize("coarse", [(0, 0), (1, 4)], ids=["one_step", "two_steps_from_1"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("maker", [lambda: synth.c3(n=256), _odd_stretched],
                         ids=["c3_256", "odd37x29"])
def test_line_projection_parity(cuda, oracle, maker, precision, coarse):
    c = maker()
    exp = oracle.project(c)
    g = P.project_case(c, precision=precision, rtol=1e-13, maxit=200, coarse_from=coarse[0],
                       coarse_sweeps=coarse[1])
    st = g["stats"]
    assert st["smoother"] == P.SMOOTHERS["line"]  # chosen automatically
    assert st["iters"] < 60
    assert rel_l2(g["Pp"], exp["Pp"]) <= TOL_P
    assert rel_l2(g["u"], exp["u"]) <= TOL_UV
    assert rel_l2(g["v"], exp["v"]) <= TOL_UV
    assert np.abs(g["mres"][_active(c)]).max() <= 1e-10


def test_point_smoother_stalls_where_lines_do_not(cuda):
    c = synth.c3(n=256)
    lines = P.project_case(c, precision="mixed", rtol=1e-8, maxit=400)["stats"]
    point = P.project_case(c, precision="mixed", rtol=1e-8, maxit=400, smoother="point")["stats"]
    assert lines["smoother"] == P.SMOOTHERS["line"]
    assert point["smoother"] == P.SMOOTHERS["point"]
    assert lines["iters"] * 4 < point["iters"]


def test_uniform_grid_keeps_point_smoother_and_lines_also_converge(cuda, oracle):
    c = synth.c4(n=128, instance=2)
    exp = oracle.project(c)
    auto = P.project_case(c, rtol=1e-13, maxit=200)
    line = P.project_case(c, rtol=1e-13, maxit=200, smoother="line")
    assert auto["stats"]["smoother"] == P.SMOOTHERS["point"]
    assert line["stats"]["smoother"] == P.SMOOTHERS["line"]
    for g in (auto, line):
        assert rel_l2(g["Pp"], exp["Pp"]) <= TOL_P
        assert rel_l2(g["u"], exp["u"]) <= TOL_UV


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_line_graph_and_graph_free_agree(cuda, precision):
    c = synth.c3(n=96)
    a = P.project_case(c, precision=precision, rtol=1e-12, maxit=200)
    b = P.project_case(c, precision=precision, rtol=1e-12, maxit=200, use_graph=False)
    for k in ("Pp", "u", "v", "p", "mres"):
        assert np.array_equal(a[k], b[k]), k


def test_coarse_steps_cut_iterations(cuda):
    """Two alternating steps per side on the coarse levels (the latency-bound
    ones) take fewer PCG iterations to 1e-8 on the stretched grid, in both
    precisions."""
    c = synth.c3(n=512)
    for precision in ("fp64", "mixed"):
        it = {}
        for coarse in ((0, 0), (2, 4)):
            g = P.project_case(c, precision=precision, rtol=1e-8, maxit=200,
                               coarse_from=coarse[0], coarse_sweeps=coarse[1])
            assert g["stats"]["status"] == 0
            it[coarse] = g["stats"]["iters"]
        assert it[(2, 4)] < it[(0, 0)], (precision, it)
