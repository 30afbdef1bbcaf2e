"""The literal restatement of Grid_Preprocess + NewCellFace for all three
families (oracle/cutcell_literal.py) on the CPU: its P family agrees with the
established literal of the projection's geometry, and its U/V outputs obey
the relations the reference's formulas imply."""
import numpy as np

import cutcell_cases as CC


def test_p_family_matches_projection_literal(oracle):
    nx, ny = 31, 27
    grids, fams = CC.case(nx, ny, CC.CIRCLES, stretch=0.3, seed=4)
    out = oracle.grid_preprocess_literal(nx, ny, grids, fams)
    g, fp = grids["p"], fams["p"]
    lit = oracle.geometry_literal(nx, ny, g["dx"], g["dy"], fp["vofS"], fp["phiS"], fp["nxS"],
                                  fp["nyS"], fams["u"]["vofS"], fams["v"]["vofS"])
    P, U, V = out["p"], out["u"], out["v"]
    for k in ("aE", "aW", "aN", "aS", "WlLh", "vofS", "nxS", "nyS"):
        assert np.array_equal(P[k], lit[k]), k
    assert np.array_equal(P["posnu"], lit["posnu_p"])
    assert np.array_equal(U["posnu"], lit["posnu_u"]) and np.array_equal(V["posnu"], lit["posnu_v"])
    assert np.array_equal(U["moex"], lit["moex_u"]) and np.array_equal(V["moex"], lit["moex_v"])
    assert np.array_equal(U["vofS"], lit["vofS_u"]) and np.array_equal(V["vofS"], lit["vofS_v"])


def test_uv_outputs_are_consistent(oracle):
    nx, ny = 34, 30
    grids, fams = CC.case(nx, ny, CC.CIRCLES, seed=2)
    out = oracle.grid_preprocess_literal(nx, ny, grids, fams)
    for f in ("u", "v"):
        T, g = out[f], grids[f]
        assert (T["moex"].sum() > 0), f  # the circles make exchange cells
        # cells with no solid part keep the zero centroid of Cell_Geo_Cal, so
        # delh is |phiS| there (the level set is linear in the cell)
        open_ = (fams[f]["vofS"] <= 1.0e-3) & (T["moex"] == 0)
        assert np.all(T["cent"][open_] == 0.0)
        assert np.array_equal(T["delh"][open_], np.abs(fams[f]["phiS"][open_]) + 1.0e-24)
        # interpolation weights inside the grid
        inside = T["posnu"][1:-1, 1:-1] != -1
        eta = T["EtaE"][1:-1, 1:-1][inside]
        assert np.all((eta > 0.0) & (eta <= 1.0))
        assert np.all(T["AlE"][1:-1, 1:-1] <= 2.0) and np.all(T["AlN"][1:-1, 1:-1] <= 2.0)
        # WlLh vanishes where all four faces are open or closed alike
        full = (T["aE"] == T["aW"])[1:-1, 1:-1] & (T["aN"] == T["aS"])[1:-1, 1:-1]
        assert np.all(T["WlLh"][full] == 0.0)
        assert np.all(T["delh"][T["moex"] == 1] == 1.0e-20)
