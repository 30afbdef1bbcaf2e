"""GPU parity of the projection path against the oracle, through the C-ABI.

Tolerances: pressure rel-L2 <= 1e-8, corrected velocity
rel-L2 <= 1e-9, when both sides are driven to the FP64 floor; assembly and
right-hand side bit for bit.
"""
import numpy as np
import pytest

from helpers import GOLDEN_CASES, load_golden, rel_l2, rel_l2_finite
from gen import synth
from simcoflow_gb300 import projection as P

pytestmark = pytest.mark.gpu

TOL_P = 1e-8
TOL_UV = 1e-9


def _active(c):
    return c["posnu_p"][1:c.nx + 1, 1:c.ny + 1] != -1


def _gpu_project(c, **kw):
    kw.setdefault("rtol", 1e-13)
    kw.setdefault("maxit", 500)
    return P.project_case(c, **kw)


def _asym_faces(matr):
    """Faces whose two rows carry different entries: a row's own W (S) entry
    against its west (south) neighbour's E (N) entry."""
    W, El = -matr[1:, :, 1], -matr[:-1, :, 3]
    S, Nl = -matr[:, 1:, 0], -matr[:, :-1, 4]
    return int((W != El).sum() + (S != Nl).sum())


def _check_operator(c, g, matr, rhm):
    """All five columns of the assembled rows bit for bit (S, W, diagonal,
    E, N of src/ProjectionP_Mod.f90:176-230), the right-hand side, and the
    count of faces whose two rows differ."""
    op = g["operator"]
    act = _active(c)
    cE = np.where(act, -matr[:, :, 3], 0.0) + 0.0
    cN = np.where(act, -matr[:, :, 4], 0.0) + 0.0
    dg = np.where(act, matr[:, :, 2], -1.0)
    assert np.array_equal(op["cE"], cE)
    assert np.array_equal(op["cN"], cN)
    assert np.array_equal(op["diag"], dg)
    assert np.array_equal(op["rhs"], rhm)
    for f in range(5):
        assert np.array_equal(g["matr"][:, :, f], matr[:, :, f]), f"matr(:,:,{f + 1})"
    assert g["asym_faces"] == _asym_faces(matr)
    assert g["stats"]["asym_faces"] == g["asym_faces"]


def _check_solution(c, g, exp):
    assert rel_l2(g["Pp"], exp["Pp"]) <= TOL_P
    assert rel_l2_finite(g["u"], exp["u"]) <= TOL_UV
    assert rel_l2_finite(g["v"], exp["v"]) <= TOL_UV
    assert rel_l2(g["p"], exp["p"]) <= TOL_P
    act = _active(c)
    assert np.abs(g["mres"][act]).max() <= 1e-10
    assert np.abs(g["mres"] - exp["mres"]).max() <= 1e-10


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_golden_fixture(cuda, name, precision):
    c, exp = load_golden(name)
    g = _gpu_project(c, precision=precision)
    _check_operator(c, g, exp["matr"], exp["rhm"])
    _check_solution(c, g, exp)
    assert g["stats"]["relres_true"] < 1e-11


@pytest.mark.parametrize("maker", [
    lambda: synth.c1(),
    lambda: synth.c1(n=33),
    lambda: synth.c4(n=40, instance=7),
    lambda: synth.random_instance(5, 9, 3),
    lambda: synth.c5(instance=1, n=96),
    lambda: synth.walls(64),
    lambda: synth.walls(128),
    lambda: synth.walls(97, ny=61),
    lambda: synth.walls(48),
], ids=["c1_128", "c1_33", "c4_40", "r9", "c5_96", "walls_64", "walls_128", "walls_97x61",
        "walls_48"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_parity_vs_oracle(cuda, oracle, maker, precision):
    c = maker()
    exp = oracle.project(c)
    g = _gpu_project(c, precision=precision)
    _check_operator(c, g, exp["matr"], exp["rhm"])
    _check_solution(c, g, exp)


def test_odd_rectangular_grid(cuda, oracle):
    from gen import geometry as G
    rng = np.random.Generator(np.random.PCG64(11))
    xf = G.axis(34, 0.0, 1.7)
    yf = G.axis(18, 0.0, 0.9)
    solids = [G.Solid(G.SOLID_CIRCLE, 0.8, 0.3, r=0.12)]
    surf = G.Surface(0.5, [0.04], [2 * np.pi / 1.7], [0.2])
    c = synth.build_case("odd", xf, yf, solids, surf, synth._modes(rng, 8), synth._modes(rng, 8),
                         1e-3, 50.0, vb=-0.02)
    exp = oracle.project(c)
    g = _gpu_project(c)
    _check_operator(c, g, exp["matr"], exp["rhm"])
    _check_solution(c, g, exp)


@pytest.mark.parametrize("coarse", [None, (1, 4), (2, 3)],
                         ids=["uniform", "four_from_1", "three_from_2"])
def test_vcycle_matches_oracle(cuda, oracle, coarse):
    """The point-smoothed V-cycle against the oracle's, with npre / npost on
    every level or a coarse-level schedule (an odd count changes which of
    the two iterate buffers holds each level's result)."""
    c = synth.c4(n=128, instance=4)
    matr, _ = oracle.matrix(c)
    rng = np.random.Generator(np.random.PCG64(5))
    b = np.asfortranarray(rng.normal(size=(c.nx, c.ny)) * _active(c))
    s = P.ProjectionSolver(c.nx, c.ny)
    try:
        s.setup_case(c)
        if coarse:
            s.set_coarse_sweeps(*coarse)
        xg = s.vcycle(b)
    finally:
        s.close()
    xo = oracle.vcycle(c, matr, b, npre=2, npost=2, omega=1.9, coarse=coarse)
    assert rel_l2(xg, xo) < 1e-11


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_deterministic_and_graph_free_path_agree(cuda, precision):
    c = synth.c4(n=96, instance=9)
    a = _gpu_project(c, precision=precision)
    b = _gpu_project(c, precision=precision)
    n = _gpu_project(c, use_graph=False, precision=precision)
    for k in ("Pp", "u", "v", "p", "mres"):
        assert np.array_equal(a[k], b[k]), k
        assert np.array_equal(a[k], n[k]), k
    assert a["stats"]["iters"] == n["stats"]["iters"]
    # launch counts: the graph loop's executed bodies are counted node by
    # node; the host-polled path runs whole chunks of bodies, so it launches
    # at least as many kernels
    la, ln = a["stats"]["launches"], n["stats"]["launches"]
    assert la == b["stats"]["launches"]
    assert 3 * a["stats"]["iters"] < la <= ln


_PDL_PROBE = r'''
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
from gen import synth
from simcoflow_gb300 import projection as P
c = synth.c4(n=320, instance=3)
for prec in ("fp64", "mixed"):
    g = P.project_case(c, precision=prec, rtol=1e-10, maxit=300)
    np.save(sys.argv[2] + "_" + prec + ".npy", g["Pp"])
'''


def test_programmatic_launch_does_not_change_results(cuda, tmp_path):
    """Kernels overlap their predecessors' tails under programmatic dependent
    launch; the results must be bit-identical to strictly serial launches."""
    import os
    import subprocess
    import sys
    from helpers import GOLDEN
    root = str(GOLDEN.parent.parent)
    for tag, env in (("on", {}), ("off", {"SCF_NO_PDL": "1"})):
        e = dict(os.environ)
        e.update(env)
        r = subprocess.run([sys.executable, "-c", _PDL_PROBE, root, str(tmp_path / tag)], env=e,
                           capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr[-2000:]
    for prec in ("fp64", "mixed"):
        a = np.load(tmp_path / f"on_{prec}.npy")
        b = np.load(tmp_path / f"off_{prec}.npy")
        assert np.array_equal(a, b), prec


def test_device_pointers_match_host(cuda):
    import torch
    c = synth.c1(n=64)
    host = _gpu_project(c, rtol=1e-10)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).to(cuda)
    s = P.ProjectionSolver(c.nx, c.ny, device_ptrs=True, rtol=1e-10, maxit=500)
    try:
        A = {k: dev(v) for k, v in c.arrays.items() if isinstance(v, np.ndarray)}
        s.set_grid(A["dx"], A["dy"], A["dxU"], A["dyV"])
        s.set_geometry(**{k: A[k] for k in P.GEOMETRY_ARGS})
        s.assemble(A["DpU"], A["DpV"], c.betaP, c.betaM, c.bc)
        u, v, p = A["u0"].clone(), A["v0"].clone(), A["p0"].clone()
        Pp = torch.zeros_like(A["p0"])
        mres = torch.zeros(c.nx * c.ny, dtype=torch.float64, device=cuda)
        _, _, st = s.update_puv(A["ustar"], A["vstar"], u, v, p, c.vb, Pp=Pp, mres=mres)
        torch.cuda.synchronize()
    finally:
        s.close()
    f = lambda t, shp: t.cpu().numpy().reshape(shp, order="F")
    n0 = (c.nx + 2, c.ny + 2)
    assert np.array_equal(f(Pp, n0), host["Pp"])
    assert np.array_equal(f(u, n0), host["u"])
    assert np.array_equal(f(v, n0), host["v"])
    assert np.array_equal(f(mres, (c.nx, c.ny)), host["mres"])


def test_zero_rhs_and_errors(cuda):
    c = synth.c1(n=32)
    s = P.ProjectionSolver(c.nx, c.ny)
    try:
        # solve before assemble: call-order error, nothing runs
        z = np.zeros((c.nx + 2, c.ny + 2), order="F")
        with pytest.raises(P.ProjectionError) as e:
            s.poisson_equation_solver(z, z)
        assert e.value.code == -7
        s.setup_case(c)
        Pp, st = s.poisson_equation_solver(z, z)
        assert st.iters == 0 and np.all(Pp == 0.0)
        bad = c["ustar"].copy(order="F")
        bad[5, 7] = np.nan
        with pytest.raises(P.ProjectionError) as e:
            s.poisson_equation_solver(bad, c["vstar"])
        assert e.value.code == -3
        # the handle stays usable after an error
        Pp, st = s.poisson_equation_solver(c["ustar"], c["vstar"])
        assert st.status == 0 and st.relres_true < 1e-8
    finally:
        s.close()
    s = P.ProjectionSolver(c.nx, c.ny, maxit=2, rtol=1e-14)
    try:
        s.setup_case(c)
        Pp, st = s.poisson_equation_solver(c["ustar"], c["vstar"], check=False)
        assert st.status == -4 and st.iters == 2
    finally:
        s.close()


def test_mixed_vcycle_is_close_to_fp64(cuda, oracle):
    """The FP32/BF16 V-cycle approximates the FP64 one to BF16 accuracy."""
    c = synth.c4(n=128, instance=4)
    rng = np.random.Generator(np.random.PCG64(6))
    b = np.asfortranarray(rng.normal(size=(c.nx, c.ny)) * _active(c))
    out = {}
    for prec in ("fp64", "mixed"):
        s = P.ProjectionSolver(c.nx, c.ny, precision=prec)
        try:
            s.setup_case(c)
            out[prec] = s.vcycle(b)
        finally:
            s.close()
    assert rel_l2(out["mixed"], out["fp64"]) < 3e-2


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_coarse_sweeps_point_smoother(cuda, oracle, precision):
    """More sweeps on the coarse levels: the same solution as the oracle's
    direct solve, in fewer PCG iterations on the 2048^2 configuration's
    workload scaled down."""
    c = synth.c2(n=512)
    exp = oracle.project(c)
    it = {}
    for coarse in ((0, 0), (1, 4)):
        g = _gpu_project(c, precision=precision, rtol=1e-13, maxit=200, coarse_from=coarse[0],
                         coarse_sweeps=coarse[1])
        _check_solution(c, g, exp)
        it[coarse] = g["stats"]["iters"]
    assert it[(1, 4)] < it[(0, 0)], it


def test_mixed_preconditioner_iterations(cuda):
    """The mixed preconditioner inside flexible PCG needs about as many
    iterations as the FP64 one."""
    c = synth.c4(n=256, instance=2)
    it = {}
    for prec in ("fp64", "mixed"):
        g = _gpu_project(c, precision=prec, rtol=1e-8, maxit=200)
        assert g["stats"]["status"] == 0 and g["stats"]["relres_true"] < 1.5e-8
        it[prec] = g["stats"]["iters"]
    assert it["mixed"] <= it["fp64"] + 3, it


@pytest.mark.slow
def test_full_size_c2(cuda, oracle):
    """2048^2 at the benchmark tolerance: FP64 relative residual 1e-8, mass
    residual at the reference's 1e-10 bound, and the pressure against a CPU
    FP64 MG-PCG oracle solve driven to 1e-13."""
    c = synth.c2()
    g = _gpu_project(c, rtol=1e-8, maxit=200)
    st = g["stats"]
    assert st["status"] == 0
    assert st["relres_true"] <= 1.5e-8
    act = _active(c)
    assert np.abs(g["mres"][act]).max() <= 1e-10
    matr, _ = oracle.matrix(c)
    rhm, _ = oracle.rhs(c)
    xi, it, rel, nlev = oracle.mgpcg(c, matr, rhm, rtol=1e-13, npre=2, npost=2, omega=1.9)
    assert rel < 1e-10  # the recomputed FP64 residual floors near 3e-12 at 2048^2
    err = rel_l2(g["Pp"][1:-1, 1:-1], xi)
    assert err < 1e-6, err
    for prec in ("fp64", "mixed"):
        g2 = _gpu_project(c, rtol=1e-12, maxit=400, precision=prec)
        assert rel_l2(g2["Pp"][1:-1, 1:-1], xi) <= TOL_P, prec
    gm = _gpu_project(c, rtol=1e-8, maxit=200, precision="mixed")
    assert gm["stats"]["status"] == 0 and gm["stats"]["relres_true"] <= 1.5e-8
    # full size, many CTAs per kernel: repeated solves are bit-identical
    gm2 = _gpu_project(c, rtol=1e-8, maxit=200, precision="mixed")
    assert np.array_equal(gm["Pp"], gm2["Pp"]) and gm["stats"]["iters"] == gm2["stats"]["iters"]
    g3 = _gpu_project(c, rtol=1e-8, maxit=200)
    assert np.array_equal(g["Pp"], g3["Pp"])


_TMA_PROBE = r'''
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
from gen import synth
from simcoflow_gb300 import projection as P
c = synth.c4(n=330, instance=5)
g = P.project_case(c, precision="mixed", rtol=1e-10, maxit=300)
np.save(sys.argv[2] + "_Pp.npy", g["Pp"])
np.save(sys.argv[2] + "_it.npy", np.array([g["stats"]["iters"]]))
'''


def test_tma_staged_sweep_matches_plain_sweep(cuda, tmp_path):
    """The TMA-staged sweep (bulk tensor copies of the tile window) computes
    the same cell updates in the same order as the sweep that loads through
    the cache hierarchy: results are bit-identical (330^2: partial tiles)."""
    import os
    import subprocess
    import sys
    from helpers import GOLDEN
    root = str(GOLDEN.parent.parent)
    for tag, env in (("tma", {}), ("plain", {"SCF_NO_TMA": "1"})):
        e = dict(os.environ)
        e.update(env)
        r = subprocess.run([sys.executable, "-c", _TMA_PROBE, root, str(tmp_path / tag)], env=e,
                           capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr[-2000:]
    assert np.array_equal(np.load(tmp_path / "tma_Pp.npy"), np.load(tmp_path / "plain_Pp.npy"))
    assert np.load(tmp_path / "tma_it.npy")[0] == np.load(tmp_path / "plain_it.npy")[0]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_wall_case_with_line_smoother(cuda, oracle, precision):
    """The rows that differ from their neighbours' (solids on the walls) with
    the line-smoothed preconditioner: same operator, same solution."""
    c = synth.walls(96, instance=2)
    exp = oracle.project(c)
    g = _gpu_project(c, precision=precision, smoother="line")
    assert g["stats"]["smoother"] == P.SMOOTHERS["line"]
    _check_operator(c, g, exp["matr"], exp["rhm"])
    _check_solution(c, g, exp)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_sweep_tiles_give_the_same_vcycle(cuda, oracle, precision):
    """The point smoother's two sweep tiles (64x32 with TMA staging on the
    larger FP32 levels, 32x32 with plain loads) recompute their halo rings
    exactly, so both give global red-black half-sweeps: the same V-cycle bit
    for bit.  The PCG's r.z is summed per tile, so beta and the iterates then
    differ in the last bits only: both projections meet the parity bar."""
    c = synth.c5(instance=3, n=288)
    rng = np.random.Generator(np.random.PCG64(3))
    b = np.asfortranarray(rng.normal(size=(c.nx, c.ny)) * _active(c))
    xs = []
    for tile in (0, 1):
        s = P.ProjectionSolver(c.nx, c.ny, precision=precision)
        try:
            s.set_tile(tile)
            s.setup_case(c)
            xs.append(s.vcycle(b))
        finally:
            s.close()
    assert np.array_equal(xs[0], xs[1])
    exp = oracle.project(c)
    for tile in (0, 1):
        g = _gpu_project(c, precision=precision, tile=tile)
        assert g["stats"]["smoother"] == P.SMOOTHERS["point"]
        _check_solution(c, g, exp)
