"""GPU Grid_Preprocess + NewCellFace for the P, U and V cells
(scf_grid_preprocess, include/scf_cutcell.h) against the literal
restatement (oracle/cutcell_literal.py), bit for bit, through the C-ABI."""
import numpy as np
import pytest

import cutcell_cases as CC
from simcoflow_gb300 import cutcell as CU
from simcoflow_gb300 import projection as P

pytestmark = pytest.mark.gpu

FIELDS = {"p": ["vofS", "nxS", "nyS", "aE", "aW", "aN", "aS", "FCE", "FCN", "WlLh", "posnu"],
          "u": ["vofS", "nxS", "nyS", "aE", "aW", "aN", "aS", "FCE", "FCN", "cent", "WlLh",
                "delh", "posnu", "moex", "msce", "SxE", "EtaE", "AlE", "DAlE", "SyN", "EtaN",
                "AlN", "DAlN"]}
FIELDS["v"] = FIELDS["u"]


def same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if a.dtype.kind == "f":
        return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))
    return a.shape == b.shape and np.array_equal(a, b)


def compare(got, lit):
    bad = []
    for f, names in FIELDS.items():
        for n in names:
            if not same(got[f][n], lit[f][n]):
                d = np.argwhere(~((np.asarray(got[f][n]) == np.asarray(lit[f][n])) |
                                  (np.isnan(np.asarray(got[f][n], dtype=float)) &
                                   np.isnan(np.asarray(lit[f][n], dtype=float)))))
                bad.append(f"{f}.{n} at {d[:3].tolist()}")
    assert not bad, bad


@pytest.mark.parametrize("nx,ny,stretch,seed", [(31, 27, 0.0, 1), (40, 36, 0.3, 2),
                                               (23, 45, 0.4, 3)])
def test_matches_literal(cuda, oracle, nx, ny, stretch, seed):
    grids, fams = CC.case(nx, ny, CC.CIRCLES, stretch=stretch, seed=seed)
    got, ms = CU.grid_preprocess(grids, fams)
    lit = oracle.grid_preprocess_literal(nx, ny, grids, fams)
    compare(got, lit)
    assert got["u"]["moex"].sum() > 0 and got["v"]["moex"].sum() > 0


def test_second_step_carries_the_inout_arrays(cuda, oracle):
    """AlE(0,j) takes the previous step's AlN(1,j); MsCe and the rows the
    loops skip keep their entry values."""
    nx, ny = 30, 26
    grids, fams = CC.case(nx, ny, CC.CIRCLES, stretch=0.2, seed=5)
    first, _ = CU.grid_preprocess(grids, fams)
    moved = [(cx + 0.013, cy - 0.007, r) for cx, cy, r in CC.CIRCLES]
    fams2 = CC.family_fields(grids, moved)
    state = {f: {k: first[f][k] for k in CU.INOUT} for f in ("u", "v")}
    got, _ = CU.grid_preprocess(grids, fams2, state=state)
    lit = oracle.grid_preprocess_literal(nx, ny, grids, fams2,
                                         aln_old={f: first[f]["AlN"] for f in ("u", "v")})
    for f in ("u", "v"):
        # the literal starts MsCe and the untouched rows from zeros: compare
        # where this step writes them
        m = lit[f]["moex"] == 1
        assert np.array_equal(got[f]["msce"][m], lit[f]["msce"][m])
        for k in ("SxE", "EtaE", "AlE", "DAlE"):
            assert same(got[f][k][:, 1:-1], lit[f][k][:, 1:-1]), (f, k)
        for k in ("SyN", "EtaN", "AlN", "DAlN"):
            assert same(got[f][k][1:-1, :], lit[f][k][1:-1, :]), (f, k)
        assert np.array_equal(got[f]["AlE"][0, 1:-1], first[f]["AlN"][1, 1:-1])


def test_p_family_matches_projection_geometry(cuda):
    """The P family equals what scf_proj_set_solid derives for the projection."""
    nx, ny = 48, 40
    grids, fams = CC.case(nx, ny, CC.CIRCLES, stretch=0.25, seed=7)
    got, _ = CU.grid_preprocess(grids, fams)
    g = grids["p"]
    s = P.ProjectionSolver(nx, ny)
    try:
        s.set_grid(g["dx"], g["dy"], grids["u"]["dx"], grids["v"]["dy"])
        z = np.zeros((nx, ny), order="F")
        fp = fams["p"]
        s.set_solid(z, z, fp["vofS"], fp["phiS"], fp["nxS"], fp["nyS"], fams["u"]["vofS"],
                    fams["v"]["vofS"], True)
        geo = s.get_geometry()
    finally:
        s.close()
    for k in ("aE", "aW", "aN", "aS", "WlLh", "vofS", "nyS"):
        assert same(got["p"][k], geo[k]), k
    assert np.array_equal(got["p"]["posnu"], geo["posnu_p"])
    assert np.array_equal(got["u"]["moex"], geo["moex_u"])


def test_argument_errors(cuda):
    grids, fams = CC.case(8, 8, CC.CIRCLES)
    grids["u"]["dx"] = np.zeros((8, 9), order="F")
    with pytest.raises(ValueError):
        CU.grid_preprocess(grids, fams)


def test_device_pointers_match_host(cuda):
    import torch
    nx, ny = 37, 33
    grids, fams = CC.case(nx, ny, CC.CIRCLES, stretch=0.2, seed=8)
    host, _ = CU.grid_preprocess(grids, fams)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).cuda()
    dev, _ = CU.grid_preprocess({f: {k: T(v) for k, v in g.items()} for f, g in grids.items()},
                                {f: {k: T(v) for k, v in g.items()} for f, g in fams.items()},
                                nx=nx, ny=ny)
    for f in ("p", "u", "v"):
        for k, a in host[f].items():
            b = dev[f][k].cpu().numpy()
            assert np.array_equal(np.asarray(a).ravel(order="F").view(np.uint8),
                                  b.view(np.uint8)), (f, k)


def test_headline_grid_family_inputs(cuda, oracle):
    """synth.cutcell_inputs on a small circles case: GPU equals the literal."""
    from gen import synth
    c = synth.c2(n=48)
    grids, fams = synth.cutcell_inputs(c)
    got, _ = CU.grid_preprocess(grids, fams)
    lit = oracle.grid_preprocess_literal(c.nx, c.ny, grids, fams)
    compare(got, lit)
