"""The oracle's restatement of Redistance (oracle/clsvof_oracle.c:
src/Clsvof_Mod.f90:1525-1708 with isinsiderect :1921-1955) against a second,
pure-Python transcription of the same Fortran, statement by statement, and
against what it stands for: near the interface, |phi| is a distance to the
PLIC segments of the band's interface cells."""
import math

import numpy as np
import pytest

from gen.synth import reconstruct_fields

VOFEPS, EPSI, BAND, TOL = 1e-14, 1e-3, 4, 1e-24


def py_inside(xp, yp, dx, dy):
    c = [(-0.5 * dx, 0.5 * dy), (0.5 * dx, 0.5 * dy), (0.5 * dx, -0.5 * dy), (-0.5 * dx, -0.5 * dy)]
    b = [math.sqrt((cx - xp) * (cx - xp) + (cy - yp) * (cy - yp)) for cx, cy in c]
    side = [dx, dy, dx, dy]
    tot = 0.0
    for k in range(4):
        u = 0.5 * (side[k] + b[k] + b[(k + 1) % 4])
        w = u * (u - side[k]) * (u - b[k]) * (u - b[(k + 1) % 4])
        tot = tot + (math.sqrt(w) if w >= 0 else math.nan)
    return abs(tot - dx * dy) < 1e-10


def py_redistance(nx, ny, f, phi_in):
    g = lambda k, i, j: f[k][i - 1, j - 1]
    phi = phi_in.copy(order="F")
    aux = np.full((nx, ny), 1e4)
    fix = np.zeros((nx, ny), dtype=int)
    ev = 0
    sgn = lambda a: math.copysign(1.0, a)

    def two_ifs(pa, deuc, vT, sT):
        if abs(deuc) < abs(pa) and vT >= 1.0 - VOFEPS - sT: pa = -abs(deuc)
        if abs(deuc) < abs(pa) and vT < VOFEPS: pa = abs(deuc)
        return pa

    for i in range(1, nx + 1):
        for j in range(1, ny + 1):
            if not ((0.0 + VOFEPS) < g("vof", i, j) < (1.0 - VOFEPS - g("vofS", i, j))):
                continue
            aux[i - 1, j - 1] = g("dis", i, j)
            fix[i - 1, j - 1] = 1
            dxs, dys = g("dx", i, j), g("dy", i, j)
            ns = (g("nxs", i, j), g("nys", i, j), g("phiS", i, j))
            n1, n2, d1 = g("nxv", i, j), g("nyv", i, j), g("dis", i, j)
            solid = lambda a, b: ns[0] * a + ns[1] * b + ns[2]
            for ii in range(-BAND, BAND + 1):
                for jj in range(-BAND, BAND + 1):
                    p, q = i + ii, j + jj
                    if not (1 <= p <= nx and 1 <= q <= ny): continue
                    vT, sT = g("vof", p, q), g("vofS", p, q)
                    if not (vT < 0.0 + VOFEPS or vT >= 1.0 - VOFEPS - sT): continue
                    fix[p - 1, q - 1] = 1
                    pa = aux[p - 1, q - 1]
                    l, m = max(-1, min(1, ii)), max(-1, min(1, jj))
                    xv, yv = dxs * float(l) / 2.0, dys * float(m) / 2.0
                    if solid(xv, yv) < 0.0:
                        if abs(yv) < VOFEPS:
                            yv = dys / 2.0
                            if solid(xv, yv) < 0.0:
                                yv = -dys / 2.0
                                if solid(xv, yv) < 0.0:
                                    xv = dxs * (0.0 - float(l)) / 2.0
                                    if solid(xv, yv) < 0.0: yv = dys / 2.0
                        elif abs(xv) < VOFEPS:
                            xv = dxs / 2.0
                            if solid(xv, yv) < 0.0:
                                xv = -dxs / 2.0
                                if solid(xv, yv) < 0.0:
                                    yv = dys * (0.0 - float(m)) / 2.0
                                    if solid(xv, yv) < 0.0: xv = dxs / 2.0
                        else:
                            yv = dys * (0.0 - float(m)) / 2.0
                            if solid(xv, yv) < 0.0:
                                xv, yv = dxs * (0.0 - float(l)) / 2.0, dys * float(m) / 2.0
                                if solid(xv, yv) < 0.0: yv = dys * (0.0 - float(m)) / 2.0
                    rx, ry = g("x", p, q) - g("x", i, j), g("y", p, q) - g("y", i, j)
                    dv = n1 * xv + n2 * yv + d1
                    dist = lambda a, b: math.sqrt((rx - a) * (rx - a) + (ry - b) * (ry - b))
                    if dv * sgn(phi_in[p - 1, q - 1]) <= 0.0:
                        deuc = dist(xv, yv)
                        if sT < EPSI: pa = sgn(0.5 - vT) * min(deuc, abs(pa))
                        else: pa = two_ifs(pa, deuc, vT, sT)
                    else:
                        dij1 = n1 * rx + n2 * ry + d1
                        xp, yp = rx - dij1 * n1, ry - dij1 * n2
                        inside = py_inside(xp, yp, dxs, dys)
                        if inside and sT < EPSI:
                            pa = sgn(0.5 - vT) * min(dist(xp, yp), abs(pa))
                        elif inside and EPSI <= sT < 1.0 - EPSI:
                            pa = two_ifs(pa, dist(xp, yp), vT, sT)
                        elif sT >= 1.0 - EPSI:
                            if g("vofS", i, j) < EPSI:
                                deuc = dist(xp, yp)
                                if abs(deuc) < abs(pa): pa = sgn(dij1) * deuc
                        else:
                            xoff = max(abs(xp) - 0.5 * dxs, 0.0)
                            yoff = max(abs(yp) - 0.5 * dys, 0.0)
                            xfc, yfc = sgn(xp) * 0.5 * dxs, sgn(yp) * 0.5 * dys
                            if xoff * abs(n1 + TOL) >= yoff * abs(n2 + TOL):
                                xs = xfc
                                ys = (d1 + n1 * xs) / (-n2 + TOL)
                            else:
                                ys = yfc
                                xs = (d1 + n2 * ys) / (-n1 + TOL)
                            deuc = dist(xs, ys)
                            if solid(xs, ys) >= 0.0:
                                if sT < EPSI: pa = sgn(0.5 - vT) * min(deuc, abs(pa))
                                else: pa = two_ifs(pa, deuc, vT, sT)
                    aux[p - 1, q - 1] = pa
                    if pa > 9.999e3: fix[p - 1, q - 1] = 0
    for i in range(1, nx + 1):
        for j in range(1, ny + 1):
            v, s = g("vof", i, j), g("vofS", i, j)
            h = math.sqrt(g("dx", i, j) * g("dx", i, j) + g("dy", i, j) * g("dy", i, j))
            if fix[i - 1, j - 1] == 1:
                if aux[i - 1, j - 1] > 1e3: ev += 1
                phi[i - 1, j - 1] = aux[i - 1, j - 1]
            elif v <= VOFEPS:
                phi[i - 1, j - 1] = float(BAND + 1) * h
            elif v >= 1.0 - VOFEPS - s:
                phi[i - 1, j - 1] = -float(BAND + 1) * h
            if v < VOFEPS and phi[i - 1, j - 1] < -VOFEPS and s < 1.0 - EPSI: ev += 1
    return phi, ev


def _case(seed, nx, ny, band=3.0):
    return reconstruct_fields(np.random.default_rng(seed), nx, ny, band)


@pytest.mark.parametrize("nx,ny,band", [(3, 3, 3.0), (9, 7, 3.0), (24, 21, 1e9), (40, 37, 3.0)])
def test_redistance_oracle_matches_transcription(oracle, nx, ny, band):
    f = _case(nx * 3 + ny, nx, ny, band)
    rec, _ = oracle.interface_reconstruct(nx, ny, f)
    g = dict(f)
    g.update(rec)
    got, ev = oracle.redistance(nx, ny, g, f["phi"])
    want, ev2 = py_redistance(nx, ny, g, f["phi"])
    assert np.array_equal(got, want, equal_nan=True)
    assert ev == ev2


def test_redistance_gives_the_distance_to_a_straight_interface(oracle):
    """A straight liquid surface y = c through a uniform grid without solid:
    the interface cells' PLIC lines are that line, and phi within the band
    becomes the signed distance to it (negative in the liquid), exactly the
    vertical distance here."""
    nx, ny = 30, 40
    x = np.asfortranarray(np.broadcast_to((np.arange(nx) + 0.5)[:, None], (nx, ny)).copy())
    y = np.asfortranarray(np.broadcast_to((np.arange(ny) + 0.5)[None, :], (nx, ny)).copy())
    c = 17.3
    ones = lambda: np.ones((nx, ny), order="F")
    zeros = lambda: np.zeros((nx, ny), order="F")
    vof = np.asfortranarray(np.clip(c - (y - 0.5), 0.0, 1.0))
    f = {"x": x, "y": y, "dx": ones(), "dy": ones(), "vof": vof, "vofS": zeros(),
         "nxs": zeros(), "nys": ones(), "phiS": np.asfortranarray(ones() * 1e3),
         "phi": np.asfortranarray(y - c)}
    rec, _ = oracle.interface_reconstruct(nx, ny, f)
    g = dict(f)
    g.update(rec)
    phi, ev = oracle.redistance(nx, ny, g, f["phi"])
    near = np.abs(y - c) < 3.0
    assert ev == 0
    assert np.allclose(phi[near], (y - c)[near], atol=1e-12)
    far = np.abs(y - c) > 6.0
    assert np.all(np.abs(phi[far]) == 5.0 * math.sqrt(2.0))
