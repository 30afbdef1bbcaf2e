"""The oracle's restatement of the CLSVOF sweeps (oracle/clsvof_oracle.c)
against a second, pure-Python transcription of the same Fortran loops,
statement by statement, on small grids: the level-set part of X_Sweep
(src/Clsvof_Mod.f90:1074-1123) and Y_Sweep (:1191-1244), and their VOF part
(:1004-1069, :1141-1189) with topflux .. leftflux, frac and CellGeoCal; frac
and CellGeoCal also against an independent polygon clipper."""
import math

import numpy as np
import pytest

from gen.synth import ls_fields


def py_sweep(dir, nx, ny, f, dtv, t):
    """The Fortran loops with 1-based indices (temls modified in place)."""
    t = t.copy(order="F")
    P = lambda i, j: f["phi"][i - 1, j - 1]
    D = lambda a, i, j: f[a][i - 1, j - 1]
    A = lambda a, i, j: f[a][i, j]
    if dir == 0:
        U = lambda i, j: f["ue"][i, j - 1]
        for j in range(1, ny + 1):
            for i in range(2, nx):
                if U(i, j) >= 0.0: l = (P(i + 1, j) + P(i - 1, j)) / 2.0
                elif i <= nx - 2: l = (P(i + 2, j) + P(i, j)) / 2.0
                else: l = (P(i + 1, j) + P(i - 1, j)) / 2.0
                fl = U(i, j) * l * dtv
                t[i - 1, j - 1] = t[i - 1, j - 1] - fl * A("aE", i, j) / D("dx", i, j)
                t[i, j - 1] = (t[i, j - 1] * (1.0 - D("vofS", i + 1, j)) +
                               fl * A("aW", i + 1, j) / D("dx", i + 1, j))
        for j in range(1, ny + 1):
            if U(1, j) >= 0.0:
                l = P(1, j) + D("dx", 1, j) / 2.0 * (1.0 - U(1, j) * dtv / D("dx", 1, j)) * \
                    (P(2, j) - P(1, j)) / (D("x", 2, j) - D("x", 1, j))
            else:
                l = P(2, j) - D("dx", 2, j) / 2.0 * (1.0 + U(1, j) * dtv / D("dx", 2, j)) * \
                    (P(3, j) - P(1, j)) / (2.0 * D("dx", 2, j))
            fl = l * U(1, j) * dtv
            t[0, j - 1] = t[0, j - 1] - fl * A("aE", 1, j) / D("dx", 1, j)
            t[1, j - 1] = t[1, j - 1] + fl * A("aE", 1, j) / D("dx", 2, j)
            t[0, j - 1] = t[0, j - 1] + P(1, j) * U(0, j) * dtv * A("aW", 1, j) / D("dx", 1, j)
            n = nx
            if U(n, j) > 0.0:
                l = P(n, j) + D("dx", n, j) / 2.0 * (1.0 - U(n, j) * dtv / D("dx", n, j)) * \
                    (P(n, j) - P(n - 1, j)) / (D("x", n, j) - D("x", n - 1, j))
            else:
                l = P(n, j) - D("dx", n - 1, j) / 2.0 * (1.0 + U(n, j) * dtv / D("dx", n - 1, j)) * \
                    (P(n, j) - P(n - 1, j)) / (D("x", n, j) - D("x", n - 1, j))
            fl = l * U(n, j) * dtv
            t[n - 1, j - 1] = t[n - 1, j - 1] - fl * A("aE", n, j) / D("dx", n, j)
    else:
        V = lambda i, j: f["ve"][i - 1, j]
        for j in range(2, ny):
            for i in range(1, nx + 1):
                if V(i, j) >= 0.0: l = (P(i, j + 1) + P(i, j - 1)) / 2.0
                elif j <= ny - 2: l = (P(i, j + 2) + P(i, j)) / 2.0
                else: l = (P(i, j + 1) + P(i, j - 1)) / 2.0
                fl = l * V(i, j) * dtv
                t[i - 1, j - 1] = t[i - 1, j - 1] - fl * A("aN", i, j) / D("dy", i, j)
                t[i - 1, j] = (t[i - 1, j] * (1.0 - D("vofS", i, j + 1)) +
                               fl * A("aS", i, j + 1) / D("dy", i, j + 1))
        for i in range(1, nx + 1):
            if V(i, 1) >= 0.0:
                l = P(i, 1) + D("dy", i, 1) / 2.0 * (1.0 - V(i, 1) * dtv / D("dy", i, 1)) * \
                    (P(i, 2) - P(i, 1)) / (D("y", i, 2) - D("y", i, 1))
            else:
                l = P(i, 2) - D("dy", i, 2) / 2.0 * (1.0 + V(i, 1) * dtv / D("dy", i, 2)) * \
                    (P(i, 3) - P(i, 1)) / (D("y", i, 3) - D("y", i, 1))
            fl = l * V(i, 1) * dtv
            t[i - 1, 0] = t[i - 1, 0] - fl * A("aN", i, 1) / D("dy", i, 1)
            t[i - 1, 1] = t[i - 1, 1] + fl * A("aN", i, 1) / D("dy", i, 2)
            t[i - 1, 0] = t[i - 1, 0] + P(i, 1) * V(i, 0) * dtv * A("aS", i, 1) / D("dy", i, 1)
            n = ny
            if V(i, n) > 0.0:
                l = P(i, n) + D("dy", i, n) / 2.0 * (1.0 - V(i, n) * dtv / D("dy", i, n)) * \
                    (P(i, n) - P(i, n - 1)) / (D("y", i, n) - D("y", i, n - 1))
            else:
                l = P(i, n) - D("dy", i, n - 1) / 2.0 * (1.0 + V(i, n) * dtv / D("dy", i, n - 1)) * \
                    (P(i, n) - P(i, n - 1)) / (D("y", i, n) - D("y", i, n - 1))
            fl = l * V(i, n) * dtv
            t[i - 1, n - 1] = t[i - 1, n - 1] - fl / D("dy", i, n)
    return t


@pytest.mark.parametrize("dir", [0, 1])
@pytest.mark.parametrize("nx,ny", [(3, 3), (4, 7), (9, 5)])
def test_ls_sweep_oracle_matches_transcription(oracle, dir, nx, ny):
    rng = np.random.default_rng(100 * nx + 10 * ny + dir)
    f = ls_fields(rng, nx, ny)
    t = np.asfortranarray(rng.standard_normal((nx, ny)))
    got = oracle.ls_sweep(dir, nx, ny, f, 1e-2, t)
    assert np.array_equal(got, py_sweep(dir, nx, ny, f, 1e-2, t))


def test_ls_sweep_at_rest_changes_nothing(oracle):
    """No velocity and no solid: the update leaves temls as it was."""
    rng = np.random.default_rng(3)
    nx, ny = 12, 10
    f = ls_fields(rng, nx, ny)
    f["ue"][:] = 0.0
    f["ve"][:] = 0.0
    f["vofS"][:] = 0.0
    t = np.asfortranarray(rng.standard_normal((nx, ny)))
    for d in (0, 1):
        assert np.array_equal(oracle.ls_sweep(d, nx, ny, f, 1e-2, t), t)


# ---------------------------------------------------------------------------
# VOF part: X_Sweep (src/Clsvof_Mod.f90:1004-1069), Y_Sweep (:1141-1189)
# ---------------------------------------------------------------------------
VOFEPS, EPSI, TOLDENO = 1e-14, 1e-3, 1e-24


def py_frac(nx, ny, diss, dx, dy):
    """frac (:1371-1404), statement by statement."""
    tnx, tny = abs(nx), abs(ny)
    if diss + 0.5 * (tnx * dx + tny * dy) <= 0.0: return 1.0
    if diss - 0.5 * (tnx * dx + tny * dy) >= 0.0: return 0.0
    if tnx <= 1e-20: return 0.5 - diss / dy
    if tny <= 1e-20: return 0.5 - diss / dx
    xx = (0.5 * tny * dy - diss) / dx / tnx + 0.5
    yy = (0.5 * tnx * dx - diss) / dy / tny + 0.5
    total = 0.5 * xx * yy
    top = ((yy - 1.0) / yy) * ((yy - 1.0) / yy) if yy > 1.0 else 0.0
    right = ((xx - 1.0) / xx) * ((xx - 1.0) / xx) if xx > 1.0 else 0.0
    return total * (1.0 - top - right)


def py_cellgeocal(nxs, nys, phis, nxl, nyl, phil, dx, dy):
    """CellGeoCal (:2159-2253), statement by statement."""
    dx2, dy2 = dx / 2.0, dy / 2.0
    d = [dx2 * nxs - dy2 * nys + phis, -(dx2 * nxs) - dy2 * nys + phis,
         -(dx2 * nxs) + dy2 * nys + phis, dx2 * nxs + dy2 * nys + phis]
    node = []
    if d[0] >= 0.0: node.append((dx2, -dy2))
    if d[0] * d[1] < 0.0: node.append(((dy2 * nys - phis) / nxs, -dy2))
    if d[1] >= 0.0: node.append((-dx2, -dy2))
    if d[1] * d[2] < 0.0: node.append((-dx2, (dx2 * nxs - phis) / nys))
    if d[2] >= 0.0: node.append((-dx2, dy2))
    if d[2] * d[3] < 0.0: node.append(((-(dy2 * nys) - phis) / nxs, dy2))
    if d[3] >= 0.0: node.append((dx2, dy2))
    if d[3] * d[0] < 0.0: node.append((dx2, (-(dx2 * nxs) - phis) / nys))
    m = len(node)
    node.append(node[0] if m else (0.0, 0.0))
    vol, pdt = 0.0, []
    for k in range(m):
        vol = vol + 0.5 * (node[k][0] * node[k + 1][1] - node[k + 1][0] * node[k][1])
        pdt.append(node[k][0] * nxl + node[k][1] * nyl + phil)
    vols = 1.0 - abs(vol / (dx * dy))
    if m: pdt.append(pdt[0])
    nodel = []
    for k in range(m):
        if pdt[k] <= 0.0: nodel.append(node[k])
        if pdt[k] * pdt[k + 1] < 0.0:
            w = abs(pdt[k]), abs(pdt[k]) + abs(pdt[k + 1])
            nodel.append((node[k][0] + (node[k + 1][0] - node[k][0]) * w[0] / w[1],
                          node[k][1] + (node[k + 1][1] - node[k][1]) * w[0] / w[1]))
    ml = len(nodel)
    if ml: nodel.append(nodel[0])
    vol = 0.0
    for k in range(ml):
        vol = vol + 0.5 * (nodel[k][0] * nodel[k + 1][1] - nodel[k + 1][0] * nodel[k][1])
    return vols, abs(vol / (dx * dy))


def py_face(side, fn, nxx, nyy, diss, volf, nxss, nyss, phiss, vols, dx, dy, vdt):
    """topflux (fn 'y', side -1), bottomflux ('y', +1), rightflux ('x', -1),
    leftflux ('x', +1) (:1416-1522)."""
    if vdt == 0.0: return 0.0
    h, nl, ns = (dy, nyy, nyss) if fn == "y" else (dx, nxx, nxss)
    sh = 0.5 * (vdt - h)
    dl = diss - sh * nl if side < 0 else diss + sh * nl
    ds = phiss - sh * ns if side < 0 else phiss + sh * ns
    sx, sy = (dx, vdt) if fn == "y" else (vdt, dy)
    if vols < EPSI:
        flux = py_frac(nxx, nyy, dl, sx, sy)
    elif vols >= 1.0 - EPSI:
        return volf
    else:
        volss, flux = py_cellgeocal(nxss, nyss, ds, nxx, nyy, dl, sx, sy)
        if volf / (1.0 - vols) >= 1.0 - VOFEPS: flux = 1.0 - volss
        flux = flux / (1.0 - volss + TOLDENO)
        if volf + vols > 1.0 - 1e-14: flux = 1.0
    return flux * vdt


def py_vof_sweep(dir, nx, ny, f, v, dtv, t, wave=None):
    """The Fortran loops with 1-based indices (temvf modified in place)."""
    t = t.copy(order="F")
    D = lambda a, i, j: (v[a] if a in v else f[a])[i - 1, j - 1]
    A = lambda a, i, j: f[a][i, j]
    for j in range(1, ny + 1):
        for i in range(1, nx + 1):
            if D("vofS", i, j) < 1.0 - VOFEPS:
                t[i - 1, j - 1] = t[i - 1, j - 1] / (1.0 - D("vofS", i, j))

    def cell_flux(vel, i, j, side, fn):
        vf = D("vof", i, j)
        if vf >= 1.0 - VOFEPS or vf <= VOFEPS:
            fl = vf * vel * dtv
            if vf >= 1.0: fl = vel * dtv
            if vf < 0.0: fl = 0.0
            return fl
        args = [D(k, i, j) for k in ("nxv", "nyv", "dis", "vof", "nxs", "nys", "phiS", "vofS",
                                     "dx", "dy")]
        if side < 0:
            return py_face(-1, fn, *args, vel * dtv)
        return -py_face(+1, fn, *args, -vel * dtv)

    if dir == 0:
        U = lambda i, j: f["ue"][i, j - 1]
        xwu = D("x", 1, 1) - D("dx", 1, 1) / 2.0
        for j in range(1, ny + 1):
            for i in range(1, nx + 1):
                u = U(i, j)
                if u >= 0.0:
                    fl = cell_flux(u, i, j, -1, "x")
                    if A("aE", i, j) > 1.0 - VOFEPS and D("vofS", i, j) > 1.0 - VOFEPS:
                        fl = 1.0 * u * dtv
                elif i < nx:
                    fl = cell_flux(u, i + 1, j, +1, "x")
                    if A("aW", i + 1, j) > 1.0 - VOFEPS and D("vofS", i + 1, j) > 1.0 - VOFEPS:
                        fl = 1.0 * u * dtv
                else:
                    fl = D("vof", i, j) * u * dtv
                t[i - 1, j - 1] = t[i - 1, j - 1] - fl * A("aE", i, j) / D("dx", i, j)
                if i <= nx - 1:
                    t[i, j - 1] = (t[i, j - 1] * (1.0 - D("vofS", i + 1, j)) +
                                   fl * A("aW", i + 1, j) / D("dx", i + 1, j))
            fl = 0.0
            if wave is not None:
                etau = wave[0] * math.sin(wave[1] * xwu - wave[2] * (wave[4] + wave[5] * dtv))
                if D("y", 1, j) - D("dy", 1, j) / 2.0 < wave[3] + etau:
                    fl = D("vof", 1, j) * U(0, j) * dtv
            t[0, j - 1] = t[0, j - 1] + fl * A("aW", 1, j) / D("dx", 1, j)
    else:
        V = lambda i, j: f["ve"][i - 1, j]
        for i in range(1, nx + 1):
            for j in range(1, ny + 1):
                w = V(i, j)
                if w > 0.0:
                    fl = cell_flux(w, i, j, -1, "y")
                    if A("aN", i, j) > 1.0 - VOFEPS and D("vofS", i, j) > 1.0 - VOFEPS:
                        fl = 1.0 * w * dtv
                elif j < ny:
                    fl = cell_flux(w, i, j + 1, +1, "y")
                    if A("aS", i, j + 1) > 1.0 - VOFEPS and D("vofS", i, j + 1) > 1.0 - VOFEPS:
                        fl = 1.0 * w * dtv
                else:
                    fl = D("vof", i, j) * w * dtv
                t[i - 1, j - 1] = t[i - 1, j - 1] - fl * A("aN", i, j) / D("dy", i, j)
                if j <= ny - 1:
                    t[i - 1, j] = (t[i - 1, j] * (1.0 - D("vofS", i, j + 1)) +
                                   fl * A("aS", i, j + 1) / D("dy", i, j + 1))
            t[i - 1, 0] = t[i - 1, 0] + D("vof", i, 1) * V(i, 0) * dtv * A("aS", i, 1) / D("dy", i, 1)
    return t


def _vof_case(seed, nx, ny):
    from gen.synth import vof_fields, wave_inlet
    rng = np.random.default_rng(seed)
    f = ls_fields(rng, nx, ny)
    v = vof_fields(rng, nx, ny, f)
    t = np.asfortranarray(v["vof"] + 0.1 * rng.standard_normal((nx, ny)))
    return f, v, t, wave_inlet(f)


@pytest.mark.parametrize("dir", [0, 1])
@pytest.mark.parametrize("nx,ny", [(1, 1), (2, 2), (3, 3), (4, 7), (9, 5), (16, 12)])
def test_vof_sweep_oracle_matches_transcription(oracle, dir, nx, ny):
    f, v, t, wave = _vof_case(1000 * nx + 10 * ny + dir, nx, ny)
    for w in (wave, None):
        got = oracle.vof_sweep(dir, nx, ny, f, v, 0.3, t, w)
        want = py_vof_sweep(dir, nx, ny, f, v, 0.3, t, w)
        assert np.array_equal(got, want, equal_nan=True)


def _clip(poly, a, b, c):
    """Sutherland-Hodgman: the part of poly with a x + b y + c <= 0."""
    out = []
    for k in range(len(poly)):
        p, q = poly[k], poly[(k + 1) % len(poly)]
        fp, fq = a * p[0] + b * p[1] + c, a * q[0] + b * q[1] + c
        if fp <= 0: out.append(p)
        if fp * fq < 0:
            s = fp / (fp - fq)
            out.append((p[0] + s * (q[0] - p[0]), p[1] + s * (q[1] - p[1])))
    return out


def _area(poly):
    return abs(sum(poly[k][0] * poly[(k + 1) % len(poly)][1] -
                   poly[(k + 1) % len(poly)][0] * poly[k][1] for k in range(len(poly)))) / 2.0


def test_frac_and_cellgeocal_measure_the_clipped_areas(oracle):
    """frac is the part of the cell with |nx| x + |ny| y + d <= 0; CellGeoCal's
    vols the part outside nxs x + nys y + phis >= 0 and volf the liquid
    (nxl x + nyl y + phil <= 0) part of the rest -- checked against an
    independent polygon clipper, and the C restatement against the Python
    one bit for bit."""
    rng = np.random.default_rng(17)
    for _ in range(400):
        dx, dy = rng.uniform(0.3, 2.0, 2)
        box = [(-dx / 2, -dy / 2), (dx / 2, -dy / 2), (dx / 2, dy / 2), (-dx / 2, dy / 2)]
        th = rng.uniform(0, 2 * np.pi)
        nx, ny = math.cos(th), math.sin(th)
        d = rng.uniform(-1.0, 1.0) * math.hypot(dx, dy) / 2
        want = _area(_clip(box, abs(nx), abs(ny), d)) / (dx * dy)
        got = oracle.frac(nx, ny, d, dx, dy)
        assert got == py_frac(nx, ny, d, dx, dy)
        assert abs(got - want) < 1e-12
        ts = rng.uniform(0, 2 * np.pi)
        nxs, nys = math.cos(ts), math.sin(ts)
        ps = rng.uniform(-0.5, 0.5) * math.hypot(dx, dy)
        vols, volf = oracle.cellgeocal(nxs, nys, ps, nx, ny, d, dx, dy)
        assert (vols, volf) == py_cellgeocal(nxs, nys, ps, nx, ny, d, dx, dy)
        fluid = _clip(box, -nxs, -nys, -ps)
        assert abs(vols - (1.0 - (_area(fluid) if len(fluid) > 2 else 0.0) / (dx * dy))) < 1e-12
        liq = _clip(fluid, nx, ny, d) if len(fluid) > 2 else []
        assert abs(volf - (_area(liq) if len(liq) > 2 else 0.0) / (dx * dy)) < 1e-12


def test_vof_sweep_conserves_liquid_without_solid(oracle):
    """No solid, open apertures, closed first and last faces of every line:
    one X or Y sweep only moves liquid between the cells of a line, so each
    line's liquid volume (sum of temvf * dx, or * dy) is kept to rounding."""
    nx, ny = 24, 20
    f, v, _, _ = _vof_case(5, nx, ny)
    f["vofS"][:] = 0.0
    for k in ("aE", "aW", "aN", "aS"):
        f[k][:] = 1.0
    f["ue"][0, :] = f["ue"][nx, :] = 0.0
    f["ve"][:, 0] = f["ve"][:, ny] = 0.0
    t = np.asfortranarray(v["vof"].copy())
    moved = 0
    for d in (0, 1):
        out = oracle.vof_sweep(d, nx, ny, f, v, 0.05, t, None)
        h = f["dx"] if d == 0 else f["dy"]
        before, after = (t * h).sum(axis=d), (out * h).sum(axis=d)
        assert np.allclose(after, before, rtol=0, atol=1e-12)
        moved += int((np.abs(out - t) > 1e-6).sum())
    assert moved > nx * ny // 4
