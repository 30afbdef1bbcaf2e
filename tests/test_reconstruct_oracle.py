"""The oracle's restatement of Interface_Reconstruct (oracle/clsvof_oracle.c:
src/Clsvof_Mod.f90:1250-1321 with Normal_Vector_Irre :1710-1919, distance
:1323-1369, DistanceFluidCalculate :1957-2042, zriddr :2044-2105 and
LiqFuncVol :2107-2155) against a second, pure-Python transcription of the
same Fortran, statement by statement, and against the geometry it stands
for: the PLIC line of a two-phase cell cuts off the cell's liquid fraction,
and that of a three-phase cell the liquid fraction of the part outside the
solid."""
import math

import numpy as np
import pytest

from gen.synth import reconstruct_fields
from test_clsvof_oracle import _area, _clip, py_frac

VOFEPS, EPSI = 1e-14, 1e-3
# Vset as Coupled_LS_VOF leaves it (src/Clsvof_Mod.f90:746-753)
VSET = [(0.0, 1.0), (0.0, 0.0), (-1.0, 0.0), (-1.0, -1.0), (-1.0, 1.0), (1.0, 0.0), (1.0, -1.0),
        (1.0, 1.0)]


def py_distance(v, dx, dy, nxx, nyy):
    nx, ny = abs(nxx), abs(nyy)
    if nx < 1e-20: return (0.5 - v) * dy
    if ny < 1e-20: return (0.5 - v) * dx
    dll = 0.5 * (nx * dx + ny * dy)
    dul = 0.5 * (nx * dx - ny * dy)
    dlr, dur = -dul, -dll
    vful, vflr = py_frac(nx, ny, dul, dx, dy), py_frac(nx, ny, dlr, dx, dy)
    if v <= vful and v <= vflr:
        if vful > vflr: vful, vflr, dul, dlr = vflr, vful, dlr, dul
        return dll - math.sqrt(((dul - dll) * (dul - dll)) * v / vful)
    if v >= vful and v >= vflr:
        if vflr < vful: vful, vflr, dul, dlr = vflr, vful, dlr, dul
        return dur + math.sqrt((dlr - dur) * (dlr - dur) * (1.0 - v) / (1.0 - vflr))
    if abs(vflr - vful) < 1e-20: return 0.5 * (dul + dlr)
    th = (v - vful) / (vflr - vful)
    return dlr * th + dul * (1.0 - th)


def py_liqfuncvol(node6, nxf, nyf, volf, dx, dy, xf, ev):
    phil = -(nxf * xf[0] + nyf * xf[1])
    temp = 0
    for k in range(1, 7):
        if abs(node6[k - 1][0]) > 1e-14 or abs(node6[k - 1][1]) > 1e-14: temp = k
    if temp == 0:
        ev[0] += 1
        return volf - 0.0
    pdt = [node6[k][0] * nxf + node6[k][1] * nyf + phil for k in range(temp - 1)]
    pdt.append(pdt[0])
    nodel = []
    for k in range(temp - 1):
        if pdt[k] <= 0.0: nodel.append(node6[k])
        if pdt[k] * pdt[k + 1] < 0.0:
            a, b = abs(pdt[k]), abs(pdt[k]) + abs(pdt[k + 1])
            nodel.append((node6[k][0] + (node6[k + 1][0] - node6[k][0]) * a / b,
                          node6[k][1] + (node6[k + 1][1] - node6[k][1]) * a / b))
    vol = 0.0
    for k in range(len(nodel)):
        p, q = nodel[k], nodel[(k + 1) % len(nodel)]
        vol = vol + 0.5 * (p[0] * q[1] - q[0] * p[1])
    return volf - abs(vol / (dx * dy))


def py_dfc(nxss, nyss, phiss, nxf, nyf, volf, dx, dy, phif, ev):
    """(phif, assigned)."""
    dx2, dy2 = dx / 2.0, dy / 2.0
    d = [dx2 * nxss - dy2 * nyss + phiss, -(dx2 * nxss) - dy2 * nyss + phiss,
         -(dx2 * nxss) + dy2 * nyss + phiss, dx2 * nxss + dy2 * nyss + phiss]
    node = []
    if d[0] >= 0.0: node.append((dx2, -dy2))
    if d[0] * d[1] < 0.0: node.append(((dy2 * nyss - phiss) / nxss, -dy2))
    if d[1] >= 0.0: node.append((-dx2, -dy2))
    if d[1] * d[2] < 0.0: node.append((-dx2, (dx2 * nxss - phiss) / nyss))
    if d[2] >= 0.0: node.append((-dx2, dy2))
    if d[2] * d[3] < 0.0: node.append(((-(dy2 * nyss) - phiss) / nxss, dy2))
    if d[3] >= 0.0: node.append((dx2, dy2))
    if d[3] * d[0] < 0.0: node.append((dx2, (-(dx2 * nxss) - phiss) / nyss))
    m = len(node)
    node6 = node + [node[0] if m else (0.0, 0.0)] + [(0.0, 0.0)] * 8
    maxd, mind = -2.0 * math.sqrt(dx * dx + dy * dy), 2.0 * math.sqrt(dx * dx + dy * dy)
    mx = mn = (0.0, 0.0)
    for k in range(m):
        t = nxf * node[k][0] + nyf * node[k][1]
        if t > maxd: maxd, mx = t, node[k]
        if t < mind: mind, mn = t, node[k]
    x2 = (mx[0] + mx[0] * nxf * EPSI, mx[1] + mx[1] * nyf * EPSI)
    x1 = (mn[0] - mn[0] * nxf * EPSI, mn[1] - mn[1] * nyf * EPSI)
    if m == 0 or (abs(node6[0][0]) < 1e-14 and abs(node6[0][1]) < 1e-14): ev[0] += 1
    F = lambda xf: py_liqfuncvol(node6, nxf, nyf, volf, dx, dy, xf, ev)
    tol = 1e-14
    fl, fh = F(x1), F(x2)
    ph = lambda a: -(nxf * a[0] + nyf * a[1])
    if (fl > tol and fh < -tol) or (fl < -tol and fh > tol):
        xl, xh, ans = x1, x2, (-1.11e-30, -1.11e-30)
        for _ in range(1000):
            xm = (0.5 * (xl[0] + xh[0]), 0.5 * (xl[1] + xh[1]))
            fm = F(xm)
            s = math.sqrt(fm * fm - fl * fh)
            if s == 0.0: ev[0] += 1
            sg = math.copysign(1.0, fl - fh)
            xn = (xm[0] + (xm[0] - xl[0]) * sg * fm / s, xm[1] + (xm[1] - xl[1]) * sg * fm / s)
            if math.sqrt((xn[0] - ans[0]) * (xn[0] - ans[0]) + (xn[1] - ans[1]) * (xn[1] - ans[1])) <= tol:
                return ph(ans), True
            ans = xn
            fn = F(ans)
            if abs(fn) <= tol: return ph(ans), True
            if math.copysign(fm, fn) != fm: xl, fl, xh, fh = xm, fm, ans, fn
            elif math.copysign(fl, fn) != fl: xh, fh = ans, fn
            elif math.copysign(fh, fn) != fh: xl, fl = ans, fn
            else: ev[0] += 1
            if math.sqrt((xh[0] - xl[0]) * (xh[0] - xl[0]) + (xh[1] - xl[1]) * (xh[1] - xl[1])) <= tol:
                return ph(ans), True
        return ph(ans), True
    if -tol < fl < tol: return ph(x1), True
    if -tol < fh < tol: return ph(x2), True
    return phif, False


def py_reconstruct(nx, ny, f):
    """Interface_Reconstruct's loop, 1-based, with the loop's locals kept
    from cell to cell as in the Fortran."""
    P = lambda i, j: f["phi"][i - 1, j - 1]
    X = lambda i, j: f["x"][i - 1, j - 1]
    Y = lambda i, j: f["y"][i - 1, j - 1]
    S = lambda i, j: f["vofS"][i - 1, j - 1]
    gx = lambda a, b, j: (P(a, j) - P(b, j)) / (X(a, j) - X(b, j))
    gy = lambda i, a, b: (P(i, a) - P(i, b)) / (Y(i, a) - Y(i, b))
    q = lambda vx, vy: abs(1.0 - math.sqrt(vx * vx + vy * vy))
    ev = [0]

    def parallel(i, j, imv):
        vx, vy = gx(i + 1, i - 1, j), gy(i, j + 1, j - 1)
        mv = 0.0
        for ii in range(1, 9):
            a, b = VSET[ii - 1]
            cp = abs(a * vx + b * vy) / (math.sqrt(a * a + b * b) * math.sqrt(vx * vx + vy * vy)) \
                if (a * a + b * b) * (vx * vx + vy * vy) != 0 else math.nan
            if cp >= mv: mv, imv = cp, ii
        if imv == 0:
            ev[0] += 1
            imv = 1
        v1 = (-VSET[imv - 1][1], VSET[imv - 1][0])
        if v1[0] == -1: vx1, vx2 = gx(i, i - 1, j), gx(i + 1, i, j)
        elif v1[0] == 0: vx1 = vx2 = gx(i + 1, i - 1, j)
        else: vx1, vx2 = gx(i + 1, i, j), gx(i, i - 1, j)
        if v1[1] == -1: vy1, vy2 = gy(i, j, j - 1), gy(i, j + 1, j)
        elif v1[1] == 0: vy1 = vy2 = gy(i, j + 1, j - 1)
        else: vy1, vy2 = gy(i, j + 1, j), gy(i, j, j - 1)
        return (vx1, vy1) if q(vx1, vy1) < q(vx2, vy2) + 0.075 / 8.0 else (vx2, vy2)

    def choose(qm, q0, qp):
        eta = 0.075
        if qm < eta and qp >= eta: return -1
        if qm >= eta and qp < eta: return 1
        if qm < eta and q0 < eta and qp < eta: return 0
        if qm >= eta and q0 >= eta and qp >= eta: return 0
        return None

    def normal(i, j):
        if S(i, j) >= EPSI:
            if S(i + 1, j) < 1.0 - EPSI and S(i - 1, j) < 1.0 - EPSI: a = gx(i + 1, i - 1, j)
            elif S(i + 1, j) >= 1.0 - EPSI: a = gx(i, i - 1, j)
            else: a = gx(i + 1, i, j)
            if S(i, j + 1) < 1.0 - EPSI and S(i, j - 1) < 1.0 - EPSI: b = gy(i, j + 1, j - 1)
            elif S(i, j + 1) > 1.0 - EPSI: b = gy(i, j, j - 1)
            else: b = gy(i, j + 1, j)
            return a, b
        qm = q(gx(i, i - 2, j) if i >= 3 else gx(i, i - 1, j), gy(i - 1, j + 1, j - 1))
        q0 = q(gx(i + 1, i - 1, j), gy(i, j + 1, j - 1))
        qp = q(gx(i + 2, i, j) if i <= nx - 2 else gx(i + 1, i, j), gy(i + 1, j + 1, j - 1))
        dxs = choose(qm, q0, qp)
        if dxs is None: return parallel(i, j, 0)
        qm = q(gx(i + 1, i - 1, j - 1), gy(i, j, j - 2) if j >= 3 else gy(i, j, j - 1))
        q0 = q(gx(i + 1, i - 1, j), gy(i, j + 1, j - 1))
        qp = q(gx(i + 1, i - 1, j + 1), gy(i, j + 2, j) if j <= ny - 2 else gy(i, j + 1, j))
        dys = choose(qm, q0, qp)
        if dys is None: return parallel(i, j, 1)
        a = {-1: gx(i, i - 1, j), 1: gx(i + 1, i, j), 0: gx(i + 1, i - 1, j)}[dxs]
        b = {-1: gy(i, j, j - 1), 1: gy(i, j + 1, j), 0: gy(i, j + 1, j - 1)}[dys]
        return a, b

    out = {k: np.zeros((nx, ny), order="F") for k in ("nxv", "nyv", "dis")}
    nxx = nyy = diss = 0.0
    for i in range(1, nx + 1):
        for j in range(1, ny + 1):
            v, s = f["vof"][i - 1, j - 1], S(i, j)
            flag = 0
            if v >= VOFEPS and v < (1.0 - VOFEPS - s) and s < EPSI: flag = 1
            if v >= VOFEPS and v < (1.0 - VOFEPS - s) and s >= EPSI and s < 1.0 - EPSI: flag = 2
            if flag:
                if 1 < i < nx and 1 < j < ny:
                    nxx, nyy = normal(i, j)
                else:
                    if i == 1: nxx = gx(i + 1, i, j)
                    elif i == nx: nxx = gx(i, i - 1, j)
                    if j == 1: nyy = gy(i, j + 1, j)
                    elif j == ny: nyy = gy(i, j, j - 1)
                t = math.sqrt(nxx * nxx + nyy * nyy)
                if t < 1e-14: nxx, nyy = 0.0, 1.0
                else: nxx, nyy = nxx / t, nyy / t
                c = (f[k][i - 1, j - 1] for k in ("nxs", "nys", "phiS"))
                if flag == 1:
                    diss = py_distance(v, f["dx"][i - 1, j - 1], f["dy"][i - 1, j - 1], nxx, nyy)
                else:
                    diss, _ = py_dfc(*c, nxx, nyy, v, f["dx"][i - 1, j - 1], f["dy"][i - 1, j - 1],
                                     diss, ev)
            else:
                nxx, nyy = 0.0, 1.0
                if 1.0 - s > VOFEPS: diss = (0.5 - v / (1.0 - s)) * f["dy"][i - 1, j - 1]
                else: diss = (0.0 - v) * f["dy"][i - 1, j - 1]
            out["nxv"][i - 1, j - 1], out["nyv"][i - 1, j - 1] = nxx, nyy
            out["dis"][i - 1, j - 1] = diss
    return out, ev[0]


def _same(a, b):
    return np.array_equal(a, b, equal_nan=True)


@pytest.mark.parametrize("nx,ny,band", [(3, 3, 3.0), (4, 9, 3.0), (17, 12, 3.0), (40, 43, 1e9),
                                        (64, 61, 3.0)])
def test_reconstruct_oracle_matches_transcription(oracle, nx, ny, band):
    f = reconstruct_fields(np.random.default_rng(nx * 7 + ny), nx, ny, band)
    got, ev = oracle.interface_reconstruct(nx, ny, f)
    want, ev2 = py_reconstruct(nx, ny, f)
    for k in ("nxv", "nyv", "dis"):
        assert _same(got[k], want[k]), k
    assert ev == ev2


def test_reconstructed_lines_cut_off_the_liquid_fraction(oracle):
    """Two-phase interface cells: frac of the PLIC line is the cell's liquid
    fraction.  Three-phase cells whose Ridders bracket holds: the liquid
    part of the non-solid polygon (independent clipper) is the liquid
    fraction of the whole cell."""
    nx, ny = 120, 97
    f = reconstruct_fields(np.random.default_rng(12), nx, ny, band=1e9)
    out, _ = oracle.interface_reconstruct(nx, ny, f)
    v, s = f["vof"], f["vofS"]
    inter = (v >= VOFEPS) & (v < (1.0 - VOFEPS) - s)
    two, three = inter & (s < EPSI), inter & (s >= EPSI) & (s < 1.0 - EPSI)
    assert two.sum() > 1000 and three.sum() > 50
    # (frac divides by the smaller normal component: nearly axis-aligned
    # normals, below 1e-6, are ill-conditioned there and left out)
    well = two & (np.minimum(np.abs(out["nxv"]), np.abs(out["nyv"])) > 1e-6)
    assert well.sum() > 1000
    for i, j in zip(*np.nonzero(well)):
        got = oracle.frac(out["nxv"][i, j], out["nyv"][i, j], out["dis"][i, j], f["dx"][i, j],
                          f["dy"][i, j])
        assert abs(got - v[i, j]) < 1e-10
    checked = 0
    for i, j in zip(*np.nonzero(three)):
        dx, dy = f["dx"][i, j], f["dy"][i, j]
        p, assigned, _ = oracle.dfc(f["nxs"][i, j], f["nys"][i, j], f["phiS"][i, j],
                                    out["nxv"][i, j], out["nyv"][i, j], v[i, j], dx, dy)
        if not assigned:
            continue
        box = [(-dx / 2, -dy / 2), (dx / 2, -dy / 2), (dx / 2, dy / 2), (-dx / 2, dy / 2)]
        fluid = _clip(box, -f["nxs"][i, j], -f["nys"][i, j], -f["phiS"][i, j])
        liq = _clip(fluid, out["nxv"][i, j], out["nyv"][i, j], out["dis"][i, j])
        assert abs((_area(liq) if len(liq) > 2 else 0.0) / (dx * dy) - v[i, j]) < 1e-9
        checked += 1
    assert checked > 50


def test_boundary_cells_keep_the_previous_cells_normal_component(oracle):
    """A flagged cell of column 1 (rows 2..ny-1) has no formula for nyy in
    the reference and keeps the previous cell's; row 1 (columns 2..nx-1)
    keeps the previous cell's nxx -- the last cell of the column before."""
    nx, ny = 6, 7
    f = reconstruct_fields(np.random.default_rng(4), nx, ny, band=1e9)
    f["vofS"][:] = 0.0
    f["vof"][:] = 0.4
    out, _ = oracle.interface_reconstruct(nx, ny, f)
    P, X, Y = f["phi"], f["x"], f["y"]
    # column 1, row 2: nxx from the i == 1 formula, nyy = ny(1,1)
    a = (P[1, 1] - P[0, 1]) / (X[1, 1] - X[0, 1])
    b = out["nyv"][0, 0]
    t = math.sqrt(a * a + b * b)
    assert out["nxv"][0, 1] == a / t and out["nyv"][0, 1] == b / t
    # row 1, column 2: nxx = nx(1, ny), nyy from the j == 1 formula
    a = out["nxv"][0, ny - 1]
    b = (P[1, 1] - P[1, 0]) / (Y[1, 1] - Y[1, 0])
    t = math.sqrt(a * a + b * b)
    assert out["nxv"][1, 0] == a / t and out["nyv"][1, 0] == b / t


def test_failed_brackets_keep_the_previous_distance(oracle):
    """Three-phase cells whose liquid fraction exceeds the non-solid polygon
    have no Ridders bracket; the reference's diss then keeps the value of
    the cell before it in the loop -- the restatement against the
    transcription, and the carried values themselves."""
    nx, ny = 48, 40
    f = reconstruct_fields(np.random.default_rng(21), nx, ny, band=1e9)
    cut = (f["vofS"] >= 0.05) & (f["vofS"] < 1 - 1e-3)
    f["vofS"][cut] = 2e-3
    f["vof"][cut] = 0.99
    got, ev = oracle.interface_reconstruct(nx, ny, f)
    want, ev2 = py_reconstruct(nx, ny, f)
    for k in ("nxv", "nyv", "dis"):
        assert _same(got[k], want[k]), k
    flat = got["dis"].ravel(order="C")  # the loop's order: i outer, j inner
    idx = np.flatnonzero(cut.ravel(order="C"))
    assert len(idx) > 20
    for k in idx:  # each failed cell holds the dis of the cell before it
        assert k > 0 and flat[k] == flat[k - 1]
