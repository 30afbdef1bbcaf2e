"""CPU tests of the oracle: the reference's built-in identities, analytic
known-answer cases, the literal-vs-intended coefficient rule, the geometry
restatement and the committed golden fixtures."""
import math

import numpy as np
import pytest

from gen import geometry as G
from gen import synth


def _nosolid_case(n, ratio=1000.0 / 1.2, amp=0.0, dt=1e-3):
    xf = G.axis(n + 1, 0.0, 1.0)
    yf = G.axis(n + 1, 0.0, 1.0)
    surf = G.Surface(0.5, [amp], [2 * np.pi], [0.0])
    zero = (np.zeros(1), np.ones(1, int), np.ones(1, int), np.zeros(1))
    return synth.build_case("kat", xf, yf, [], surf, zero, zero, dt, ratio)


def _set_velocity(case, us, vs):
    case.arrays["ustar"] = np.asfortranarray(us)
    case.arrays["vstar"] = np.asfortranarray(vs)
    case.arrays["u0"] = np.asfortranarray(us).copy(order="F")
    case.arrays["v0"] = np.asfortranarray(vs).copy(order="F")


def test_reference_identities_c1(oracle, built):
    """Per-row |A p - b| <= 1e-10 (src/ProjectionP_Mod.f90:86) and
    |mres| <= 1e-10 (src/ComputePUV_Mod.f90:193) on the 128^2 case."""
    c = synth.c1()
    r = oracle.project(c)
    assert r["row_residual"] <= 1e-10
    fluid = c["posnu_p"][1:-1, 1:-1] != -1
    assert np.abs(r["mres"][fluid]).max() <= 1e-10
    assert r["relres"] < 1e-12


def test_literal_loop_equals_intended_rule(oracle, built):
    """The dry/dry-south branch divides by a BetaD left from the previous
    cell (src/ProjectionP_Mod.f90:504-508); in the reference's loop order
    that value is always BetaP, so the literal loop gives the intended rule."""
    for case in (synth.c1(n=64), synth.c4(n=96, instance=2), synth.c5(instance=0, n=64)):
        assert np.array_equal(oracle.pocoef(case, literal=True), oracle.pocoef(case, literal=False))


def test_matrix_symmetric_positive_definite(oracle, built):
    c = synth.c4(n=24, instance=1)
    matr, A = oracle.matrix(c)
    As = A.toarray()
    asym = np.abs(As - As.T).max() / np.abs(As).max()
    assert asym < 1e-15
    w = np.linalg.eigvalsh(0.5 * (As + As.T))
    assert w.min() > 0.0


def test_divergence_free_velocity_gives_zero_pressure(oracle, built):
    """Known answer: a discretely divergence-free u* (from a stream function
    at cell corners, zero on the walls) needs no correction: p = 0, u = u*."""
    n = 32
    c = _nosolid_case(n)
    xf, yf = c.meta["xf"], c.meta["yf"]
    X, Y = np.meshgrid(xf, yf, indexing="ij")
    psi = np.sin(np.pi * X) * np.sin(0.5 * np.pi * Y)
    us = np.zeros((n + 2, n + 2)); vs = np.zeros((n + 2, n + 2))
    dy = np.diff(yf); dx = np.diff(xf)
    for i in range(0, n + 1):
        for j in range(1, n + 1):
            us[i, j] = (psi[i, j] - psi[i, j - 1]) / dy[j - 1]
    for i in range(1, n + 1):
        for j in range(0, n + 1):
            vs[i, j] = -(psi[i, j] - psi[i - 1, j]) / dx[i - 1]
    us[0, :] = 0.0; us[n, :] = 0.0; vs[:, 0] = 0.0
    _set_velocity(c, us, vs)
    r = oracle.project(c)
    assert np.abs(r["Pp"]).max() < 1e-10
    assert np.abs(r["u"] - us).max() < 1e-12
    assert np.abs(r["v"][:, :n] - vs[:, :n]).max() < 1e-12


def test_stratified_column_analytic_pressure(oracle, built):
    """Known answer: no solid, flat interface on a face, u* = 0, v* = V0 on all
    faces above the closed bottom.  The corrected field must vanish and the
    pressure follows face by face from the density-weighted coefficients."""
    n = 16
    V0 = 0.3
    c = _nosolid_case(n)
    us = np.zeros((n + 2, n + 2)); vs = np.zeros((n + 2, n + 2))
    vs[1:n + 1, 1:n + 1] = V0
    _set_velocity(c, us, vs)
    r = oracle.project(c)
    bP, bM, dt = c.betaP, c.betaM, c.dt
    dy = 1.0 / n
    # analytic column: top Dirichlet, dry top cell coefficient dt*dx/dy*betaM
    p = np.zeros(n + 2)
    p[n] = -V0 * dy / (dt * bM)
    phi = (np.arange(1, n + 1) - 0.5) * dy - 0.5
    for j in range(n - 1, 0, -1):
        wet_j, wet_n = phi[j - 1] < 0, phi[j] < 0
        if wet_j and wet_n:
            BW = bM
        elif (not wet_j) and (not wet_n):
            BW = bP
        else:
            lam = abs(phi[j - 1]) / (abs(phi[j - 1]) + abs(phi[j]) + 1e-24)
            BW = lam * bM + (1 - lam) * bP if wet_j else lam * bP + (1 - lam) * bM
        p[j] = p[j + 1] - V0 * dy * BW / (bM * bP * dt)
    Pp = r["Pp"]
    for i in range(1, n + 1):
        assert np.allclose(Pp[i, 1:n + 1], p[1:n + 1], rtol=1e-12, atol=1e-12 * abs(p).max())
    assert np.abs(r["v"][1:n + 1, 1:n + 1]).max() < 1e-12
    assert np.abs(r["mres"]).max() < 1e-12


def test_manufactured_solution_second_order(oracle, built):
    """Known answer: uniform density, no solid, u* = dt grad p_e for
    p_e = cos(pi x) cos(pi y / (2L)) (Neumann W/E/S).  The reference puts the
    Dirichlet ghost p = 0 one spacing dyV above the top cell centre
    (src/ProjectionP_Mod.f90:589, diagonal kept at :224), i.e. at
    y = L = 1 + dy/2; with p_e vanishing there the discrete pressure
    converges to p_e at second order."""
    errs = []
    for n in (16, 32, 64):
        c = _nosolid_case(n, ratio=1.0, dt=1e-3)
        xf, yf = c.meta["xf"], c.meta["yf"]
        xc, yc = 0.5 * (xf[1:] + xf[:-1]), 0.5 * (yf[1:] + yf[:-1])
        k = 0.5 * np.pi / (1.0 + 0.5 / n)
        us = np.zeros((n + 2, n + 2)); vs = np.zeros((n + 2, n + 2))
        for i in range(0, n + 1):
            us[i, 1:n + 1] = c.dt * (-np.pi * np.sin(np.pi * xf[i]) * np.cos(k * yc))
        for j in range(0, n + 1):
            vs[1:n + 1, j] = c.dt * (-k * np.cos(np.pi * xc) * np.sin(k * yf[j]))
        _set_velocity(c, us, vs)
        r = oracle.project(c)
        X, Y = np.meshgrid(xc, yc, indexing="ij")
        pe = np.cos(np.pi * X) * np.cos(k * Y)
        errs.append(np.abs(r["Pp"][1:n + 1, 1:n + 1] - pe).max())
    assert errs[0] / errs[1] > 3.5 and errs[1] / errs[2] > 3.5, errs


def test_oracle_mgpcg_matches_direct(oracle, built):
    c = synth.c4(n=128, instance=5)
    r = oracle.project(c)
    xi, it, rel, nlev = oracle.mgpcg(c, r["matr"], r["rhm"], rtol=1e-13)
    x = oracle.x_from_interior(c, xi)
    assert rel < 1e-12
    assert np.linalg.norm(x - r["x"]) / np.linalg.norm(r["x"]) < 1e-10


def _row_entries(matr):
    """(own W, west neighbour's E, own S, south neighbour's N) magnitudes."""
    return -matr[1:, :, 1], -matr[:-1, :, 3], -matr[:, 1:, 0], -matr[:, :-1, 4]


def test_wall_solids_make_rows_differ_and_mgpcg_solves_them(oracle, built):
    """Solids on the first / last rows and columns: the reference leaves those
    faces' apertures unaveraged (src/Cutcell_Mod.f90:161-204), so a row's own
    W / S entry (src/ProjectionP_Mod.f90:183,193) differs by per cent from
    the neighbour's E / N entry.  The MG-PCG, which applies the rows as
    written, agrees with the direct solve of the reference's CSR; solving the
    symmetrised rows instead misses it by far more than the tolerances."""
    c = synth.walls(64)
    r = oracle.project(c)
    W, El, S, Nl = _row_entries(r["matr"])
    worst = max(np.abs(W - El).max() / np.abs(W).max(), np.abs(S - Nl).max() / np.abs(S).max())
    assert worst > 1e-2
    xi, it, rel, _ = oracle.mgpcg(c, r["matr"], r["rhm"], rtol=1e-13)
    x = oracle.x_from_interior(c, xi)
    assert rel < 1e-12
    assert np.linalg.norm(x - r["x"]) / np.linalg.norm(r["x"]) < 1e-10
    # the symmetrised rows (W / S taken from the neighbours) give another solution
    m = r["matr"].copy(order="F")
    m[1:, :, 1] = m[:-1, :, 3]
    m[:, 1:, 0] = m[:, :-1, 4]
    act = c["posnu_p"][1:c.nx + 1, 1:c.ny + 1] != -1
    m[:, :, 0] *= act
    m[:, :, 1] *= act
    xs, _, _, _ = oracle.mgpcg(c, m, r["rhm"], rtol=1e-13)
    xs = oracle.x_from_interior(c, xs)
    assert np.linalg.norm(xs - r["x"]) / np.linalg.norm(r["x"]) > 1e-4


def test_interface_faces_differ_in_the_last_bits(oracle, built):
    """Away from walls the rows differ only where the interface's density
    weight is formed from either side (src/ProjectionP_Mod.f90:415-418
    against :493-498): a few faces, relative differences near rounding."""
    c = synth.c1(n=64)
    W, El, S, Nl = _row_entries(oracle.matrix(c)[0])
    n = int((W != El).sum() + (S != Nl).sum())
    assert n > 0
    assert max(np.abs(W - El).max() / np.abs(W).max(), np.abs(S - Nl).max() / np.abs(S).max()) < 1e-13


# ---- geometry: package builder vs the literal restatement ----

def _levelset_py(solids, x, y):
    best = (1e30, 0.0, 1.0)
    for s in solids:
        if s.kind == G.SOLID_CIRCLE:
            dx, dy = x - s.cx, y - s.cy
            r = math.sqrt(dx * dx + dy * dy)
            cand = (r - s.r, dx / r, dy / r)
        else:
            c, sn = math.cos(s.angle), math.sin(s.angle)
            px, py = x - s.cx, y - s.cy
            qx, qy = c * px + sn * py, -sn * px + c * py
            ddx, ddy = abs(qx) - s.hw, abs(qy) - s.hh
            sx, sy = (1.0 if qx >= 0 else -1.0), (1.0 if qy >= 0 else -1.0)
            if ddx > 0 and ddy > 0:
                d = math.sqrt(ddx * ddx + ddy * ddy)
                ph, lx, ly = d, sx * ddx / d, sy * ddy / d
            elif ddx > ddy:
                ph, lx, ly = ddx, sx, 0.0
            else:
                ph, lx, ly = ddy, 0.0, sy
            cand = (ph, c * lx - sn * ly, sn * lx + c * ly)
        if cand[0] < best[0]:
            best = cand
    return best


def _raw_vofS(oracle, solids, xc, yc, dxc, dyc):
    p, a, b = _levelset_py(solids, xc, yc)
    v = oracle.frac_literal(a, b, p, dxc, dyc)
    if v < 1e-14:
        v = 0.0
    if v >= 1.0 - 1e-14:
        v = 1.0
    return v, p, a, b


@pytest.mark.parametrize("which", ["circles", "box"])
def test_geometry_builder_matches_literal(oracle, built, which):
    nx, ny = 28, 22
    if which == "circles":
        solids = [G.Solid(G.SOLID_CIRCLE, 0.4, 0.42, r=0.17), G.Solid(G.SOLID_CIRCLE, 0.7, 0.5, r=0.09)]
        yf = G.axis(ny + 1, 0.0, 1.0)
    else:
        solids = [G.Solid(G.SOLID_BOX, 0.5, 0.4, hw=0.3, hh=0.05, angle=np.deg2rad(10.0))]
        yf = G.axis(ny + 1, 0.0, 1.0, True, 0.45, 0.55, 9)
    xf = G.axis(nx + 1, 0.0, 1.0)
    g = G.build(xf, yf, solids, G.Surface(0.55, [0.03], [2 * np.pi], [0.3]))
    raw = {k: np.zeros((nx, ny)) for k in ("vofS", "phiS", "nxS", "nyS", "vofS_u", "vofS_v")}
    for i in range(nx):
        for j in range(ny):
            x, y, dx, dy = g["x"][i, j], g["y"][i, j], g["dx"][i, j], g["dy"][i, j]
            v, p, a, b = _raw_vofS(oracle, solids, x, y, dx, dy)
            raw["vofS"][i, j], raw["phiS"][i, j], raw["nxS"][i, j], raw["nyS"][i, j] = v, p, a, b
            raw["vofS_u"][i, j] = _raw_vofS(oracle, solids, x + 0.5 * dx, y, g["dxU"][i, j], dy)[0]
            raw["vofS_v"][i, j] = _raw_vofS(oracle, solids, x, y + 0.5 * dy, dx, g["dyV"][i, j])[0]
    lit = oracle.geometry_literal(nx, ny, g["dx"], g["dy"], raw["vofS"], raw["phiS"], raw["nxS"],
                                  raw["nyS"], raw["vofS_u"], raw["vofS_v"])
    assert (g["posnu_p"][1:-1, 1:-1] == -1).sum() > 0
    for k in ("aE", "aW", "aN", "aS"):
        assert np.array_equal(g[k][1:-1, 1:-1], lit[k][1:-1, 1:-1]), k
    for k in ("WlLh", "vofS", "nyS", "vofS_u", "vofS_v"):
        assert np.array_equal(g[k], lit[k]), k
    for k in ("posnu_p", "posnu_u", "posnu_v"):
        assert np.array_equal(g[k][1:-1, 1:-1], lit[k][1:-1, 1:-1]), k
    for k in ("moex_u", "moex_v"):
        assert np.array_equal(g[k], lit[k]), k


def test_frac_known_areas(oracle):
    # half-plane through the centre: half the cell
    assert oracle.frac_literal(0.0, 1.0, 0.0, 1.0, 1.0) == 0.5
    # diagonal through the centre of a unit square
    s = 1 / math.sqrt(2)
    assert abs(oracle.frac_literal(s, s, 0.0, 1.0, 1.0) - 0.5) < 1e-15
    # corner triangle: x + y < 0.5 (shifted to cell coordinates) has area 1/8
    assert abs(oracle.frac_literal(s, s, (1.0 - 0.5) * s, 1.0, 1.0) - 0.125) < 1e-15
    assert oracle.frac_literal(0.0, 1.0, -2.0, 1.0, 1.0) == 1.0
    assert oracle.frac_literal(0.0, 1.0, 2.0, 1.0, 1.0) == 0.0


def test_geometry_top_row_keeps_open_faces(built):
    for inst in range(8):
        c = synth.c5(instance=inst, n=64)
        assert (c["aN"][1:-1, c.ny] > 0).all()


def test_oracle_line_smoother_on_stretched_grid(oracle, built):
    """The point smoother stalls on the stretched 4096^2 configuration's grid
    (scaled down); the line smoother converges in a grid-independent number
    of iterations and reaches the direct solution."""
    its = {}
    for n in (128, 256):
        c = synth.c3(n=n)
        r = oracle.project(c)
        xp, itp, _, _ = oracle.mgpcg(c, r["matr"], r["rhm"], rtol=1e-8, maxit=1000)
        xl, itl, rel, _ = oracle.mgpcg(c, r["matr"], r["rhm"], rtol=1e-12, maxit=200,
                                       smoother="line")
        pn = c["posnu_p"][1:n + 1, 1:n + 1] != -1
        xd = r["Pp"][1:n + 1, 1:n + 1]
        assert np.linalg.norm((xl - xd)[pn]) <= 1e-9 * np.linalg.norm(xd[pn])
        its[n] = (itp, itl)
    assert all(itl < 30 for _, itl in its.values())
    assert all(itp > 3 * itl for itp, itl in its.values())


def test_oracle_coarse_line_steps(oracle, built):
    """The line smoother's coarse schedule: two sweeps (one alternating
    step) from some level down is the default V-cycle bit for bit; four (two
    steps) on the coarse levels cut the MG-PCG iterations on the stretched
    grid and reach the same solution."""
    c = synth.c3(n=256)
    r = oracle.project(c)
    rng = np.random.Generator(np.random.PCG64(3))
    b = rng.normal(size=(c.nx, c.ny)) * (c["posnu_p"][1:c.nx + 1, 1:c.ny + 1] != -1)
    x0 = oracle.vcycle(c, r["matr"], b, smoother="line")
    assert np.array_equal(x0, oracle.vcycle(c, r["matr"], b, smoother="line", coarse=(1, 2)))
    assert not np.array_equal(x0, oracle.vcycle(c, r["matr"], b, smoother="line",
                                                coarse=(1, 4)))
    _, it1, _, _ = oracle.mgpcg(c, r["matr"], r["rhm"], rtol=1e-8, maxit=200, smoother="line")
    x2, it2, rel, _ = oracle.mgpcg(c, r["matr"], r["rhm"], rtol=1e-12, maxit=200,
                                   smoother="line", coarse=(1, 4))
    _, it2e, _, _ = oracle.mgpcg(c, r["matr"], r["rhm"], rtol=1e-8, maxit=200, smoother="line",
                                 coarse=(1, 4))
    assert it2e < it1
    pn = c["posnu_p"][1:c.nx + 1, 1:c.ny + 1] != -1
    xd = r["Pp"][1:c.nx + 1, 1:c.ny + 1]
    assert np.linalg.norm((x2 - xd)[pn]) <= 1e-9 * np.linalg.norm(xd[pn])


def test_whole_projection_in_c_matches_direct_solve(oracle, built):
    """The timed CPU baseline's path (every stage in C, the dense rows only,
    the MG-PCG on them) gives the direct solve's projection, with the
    literal loops' rows."""
    for c in (synth.c1(n=64), synth.walls(64), synth.c3(n=64)):
        d = oracle.project(c)
        m = oracle.project_mg(c, rtol=1e-13, maxit=300)
        assert np.array_equal(m["matr"], d["matr"])
        assert np.array_equal(m["rhm"], d["rhm"])
        assert m["relres"] < 1e-12
        for k, tol in (("Pp", 1e-10), ("u", 1e-11), ("v", 1e-11)):
            assert np.linalg.norm(m[k] - d[k]) / np.linalg.norm(d[k]) < tol, k
    assert oracle.project_mg(synth.c3(n=64))["smoother"] == "line"


def test_top_row_continuity_divides_by_a_closed_face(oracle, built):
    """A solid cell of the top row whose V cell is not solid enough to be
    zeroed: the reference's top-row continuity (src/ComputePUV_Mod.f90:177-182)
    divides by its closed north face, 0 / 0, and nothing clears the result
    (:227-245).  The restatement keeps that (one NaN in v here)."""
    c = synth.walls(48)
    d = oracle.project(c)
    bad = np.argwhere(~np.isfinite(d["v"]))
    assert bad.tolist() == [[13, 48]]
    i, j = bad[0]
    assert c["aN"][i, j] == 0.0 and c["posnu_p"][i, j] == -1
    assert np.isfinite(d["u"]).all() and np.isfinite(d["mres"]).all()
