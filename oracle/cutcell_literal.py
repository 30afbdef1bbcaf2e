"""Literal pure-Python restatement of SIMCOFlow's per-step cut-cell geometry
for all three cell families -- TEST INFRASTRUCTURE ONLY (the package never
imports it).

Follows, loop by loop and in the reference's operation order:
  Grid_Preprocess      src/Cutcell_Mod.f90:18-32
  Cell_Geo_Cal         src/Cutcell_Mod.f90:34-300 (with Edge_Geo_Cal :302-337)
  NumberExternalCell   src/Cutcell_Mod.f90:340-358
  DefineMomentumExchangeCell  src/Cutcell_Mod.f90:360-397
  NewCellFace          src/Cutcell_Mod.f90:399-549 (with CellLinking :702-725,
                       EastFaceInterpolationInf :551-616,
                       NorthFaceInterpolationInf :618-700)
Python floats are IEEE binary64 with every operation rounded, the same
arithmetic as the Fortran without FMA contraction.  Meant for grids of a
few thousand cells.

Conventions where the reference reads memory it never writes:
  * ghost apertures (i = 0, nx+1 or j = 0, ny+1) are 0: the reference only
    ever writes zeros there, into freshly allocated arrays;
  * Posnu of the cells outside the numbering loops (U cells at i = nx, V
    cells at j = ny) is -1;
  * a moving-body exchange cell on the domain edge would let CellLinking
    read vofS outside the grid; such a neighbour counts as solid (1.0);
  * AlE(0,j) takes AlN(1,j) as it was before this step's
    NorthFaceInterpolationInf (the reference's assignment, :612): the
    previous AlN is an input (zeros on the first step).
Arrays in and out are numpy arrays indexed [i, j] with the reference's
Fortran bounds shifted to 0-based storage:
  (nx,ny) fields: a[i-1, j-1];  (0:nx+1,0:ny+1) fields: a[i, j];
  face centres FCE / FCN: (nx+2, ny+2, 2);  Cell_Cent, MsCe: (nx, ny, 2).
"""
from __future__ import annotations

import math

import numpy as np

EPSI, EPSIF, RND = 1.0e-3, 1.0e-2, 1.0e-24


def _sign(a, b):
    """Fortran SIGN(A,B) for reals: |A| with B's sign bit."""
    return math.copysign(abs(a), b)


def _edge(p1, p2, nxx, nyy, diss):
    """Edge_Geo_Cal (:302-337): solid fraction of the edge p1-p2 and the
    centre of the edge's solid part."""
    l1 = nxx * p1[0] + nyy * p1[1] + diss
    l2 = nxx * p2[0] + nyy * p2[1] + diss
    eps = 1.0e-14
    fx = 0.5 * (p1[0] + p2[0])
    fy = 0.5 * (p1[1] + p2[1])
    area = None
    if l1 >= eps and l2 >= eps:
        area = 0.0
    elif l1 < eps and l2 < eps:
        area = 1.0
    elif l1 >= eps and l2 < eps:
        area = abs(l2) / (abs(l1) + abs(l2))
        if abs(p1[0] - p2[0]) <= 1.0e-10:
            fy = p2[1] - 0.5 * area * (p2[1] - p1[1])
        else:
            fx = p2[0] - 0.5 * area * (p2[0] - p1[0])
    elif l1 < eps and l2 >= eps:
        area = abs(l1) / (abs(l1) + abs(l2))
        if abs(p1[0] - p2[0]) <= 1.0e-10:
            fy = p1[1] - 0.5 * area * (p1[1] - p2[1])
        else:
            fx = p1[0] - 0.5 * area * (p1[0] - p2[0])
    else:  # a NaN level set: Edge_Area keeps its previous value (0 here)
        area = 0.0
    return area, fx, fy


def cell_geo_cal(nx, ny, g, fam, icorprob=True):
    """Cell_Geo_Cal (:34-300) of one family.  g: dx, dy, x, y (nx,ny);
    fam: vofS, phiS, nxS, nyS (nx,ny) as Initial_Clsvof leaves them.
    Family 'p' has neither MsCe nor MoExCell nor delh allocated (the
    degenerate-cell rule and the corner rule apply, delh does not); 'u' and
    'v' have all three."""
    dxa, dya, xa, ya = g["dx"], g["dy"], g["x"], g["y"]
    is_p = fam["family"] == "p"
    E = np.zeros((nx + 2, ny + 2)); W = np.zeros_like(E); N = np.zeros_like(E); S = np.zeros_like(E)
    FCE = np.zeros((nx + 2, ny + 2, 2)); FCN = np.zeros_like(FCE)
    FCW = np.zeros((nx + 1, ny + 1, 2)); FCS = np.zeros_like(FCW)  # [i, j], 1-based
    cent = np.zeros((nx, ny, 2))
    vs = np.array(fam["vofS"], dtype=float).copy()
    nxs = np.array(fam["nxS"], dtype=float).copy()
    nys = np.array(fam["nyS"], dtype=float).copy()
    phs = np.array(fam["phiS"], dtype=float)
    WL = np.zeros((nx, ny))
    delh = None if is_p else np.zeros((nx, ny))
    dx = lambda i, j: dxa[i - 1, j - 1]
    dy = lambda i, j: dya[i - 1, j - 1]
    for i in range(1, nx + 1):
        for j in range(1, ny + 1):
            a, b, p = nxs[i - 1, j - 1], nys[i - 1, j - 1], phs[i - 1, j - 1]
            pt = {(ii, jj): (-dx(i, j) * (0.5 - float(ii)), -dy(i, j) * (0.5 - float(jj)))
                  for ii in (0, 1) for jj in (0, 1)}
            W[i, j], FCW[i, j, 0], FCW[i, j, 1] = _edge(pt[0, 0], pt[0, 1], a, b, p)
            N[i, j], FCN[i, j, 0], FCN[i, j, 1] = _edge(pt[0, 1], pt[1, 1], a, b, p)
            E[i, j], FCE[i, j, 0], FCE[i, j, 1] = _edge(pt[1, 1], pt[1, 0], a, b, p)
            S[i, j], FCS[i, j, 0], FCS[i, j, 1] = _edge(pt[1, 0], pt[0, 0], a, b, p)
    for i in range(1, nx + 1):
        for j in range(1, ny + 1):
            a_ = (E[i, j] - W[i, j]) * dx(i, j)
            b_ = (N[i, j] - S[i, j]) * dy(i, j)
            WL[i - 1, j - 1] = math.sqrt(a_ * a_ + b_ * b_)
    # ghost face centres (:91-112), whole-column / whole-row assignments in order
    for j in range(0, ny + 2):
        FCE[0, j, 0] = FCE[1, j, 0] - dx(1, 1)
        FCE[0, j, 1] = FCE[1, j, 1]
        FCE[nx + 1, j, 0] = FCE[nx, j, 0] + dx(nx, 1)
        FCE[nx + 1, j, 1] = FCE[nx, j, 1]
    for j in range(0, ny + 2):
        FCN[0, j, 0] = FCN[1, j, 0] - dx(1, 1)
        FCN[0, j, 1] = FCN[1, j, 1]
        FCN[nx + 1, j, 0] = FCN[nx, j, 0] + dx(nx, 1)
        FCN[nx + 1, j, 1] = FCN[nx, j, 1]
    for i in range(0, nx + 2):
        FCE[i, 0, 0] = FCE[i, 1, 0]
        FCE[i, 0, 1] = FCE[i, 1, 1] - dy(1, 1)
        FCE[i, ny + 1, 0] = FCE[i, ny, 0]
        FCE[i, ny + 1, 1] = FCE[i, ny, 1] + dy(1, ny)
    for i in range(0, nx + 2):
        FCN[i, 0, 0] = FCE[i, 1, 0]
        FCN[i, 0, 1] = FCE[i, 1, 1] - dy(1, 1)
        FCN[i, ny + 1, 0] = FCE[i, ny, 0]
        FCN[i, ny + 1, 1] = FCE[i, ny, 1] + dy(1, ny)
    # solid fractions -> open fractions, solid-part face centres -> open-part ones
    for i in range(1, nx + 1):
        for j in range(1, ny + 1):
            W[i, j] = 1.0 - W[i, j]; E[i, j] = 1.0 - E[i, j]
            N[i, j] = 1.0 - N[i, j]; S[i, j] = 1.0 - S[i, j]
            if abs(FCE[i, j, 1]) < EPSI:
                FCE[i, j, 1] = 0.0
            else:
                FCE[i, j, 1] = (0.5 - E[i, j] / 2.0) * _sign(1.0, -FCE[i, j, 1]) * dy(i, j)
            if E[i, j] < EPSIF:
                FCE[i, j, 1] = 0.0
            if abs(FCW[i, j, 1]) < EPSI:
                FCW[i, j, 1] = 0.0
            else:
                FCW[i, j, 1] = (0.5 - W[i, j] / 2.0) * _sign(1.0, -FCW[i, j, 1]) * dy(i, j)
            if W[i, j] < EPSIF:
                FCW[i, j, 1] = 0.0
            if abs(FCN[i, j, 0]) < EPSI:
                FCN[i, j, 0] = 0.0
            else:
                FCN[i, j, 0] = (0.5 - N[i, j] / 2.0) * _sign(1.0, -FCN[i, j, 0]) * dx(i, j)
            if N[i, j] < EPSIF:
                FCN[i, j, 0] = 0.0
            if abs(FCS[i, j, 0]) < EPSI:
                FCS[i, j, 0] = 0.0
            else:
                FCS[i, j, 0] = (0.5 - S[i, j] / 2.0) * _sign(1.0, -FCS[i, j, 0]) * dx(i, j)
            if S[i, j] < EPSIF:
                FCS[i, j, 0] = 0.0
    # shared faces: harmonic mean of the two open fractions, weighted centres
    for i in range(2, nx):
        for j in range(2, ny):
            av = 2.0 * N[i, j] * S[i, j + 1] / (N[i, j] + S[i, j + 1] + RND)
            FCN[i, j, 0] = ((FCN[i, j, 0] * N[i, j] + FCS[i, j + 1, 0] * S[i, j + 1]) /
                            (N[i, j] + S[i, j + 1] + RND))
            FCN[i, j, 1] = ((FCN[i, j, 1] * N[i, j] + (FCS[i, j + 1, 1] +
                             (ya[i - 1, j] - ya[i - 1, j - 1])) * S[i, j + 1]) /
                            (N[i, j] + S[i, j + 1] + RND))
            if N[i, j] < EPSIF and S[i, j + 1] < EPSIF:
                FCN[i, j, 1] = dy(i, j) / 2.0
            N[i, j] = av; S[i, j + 1] = av
            av = 2.0 * E[i, j] * W[i + 1, j] / (E[i, j] + W[i + 1, j] + RND)
            FCE[i, j, 0] = ((FCE[i, j, 0] * E[i, j] + (FCW[i + 1, j, 0] +
                             (xa[i, j - 1] - xa[i - 1, j - 1])) * W[i + 1, j]) /
                            (E[i, j] + W[i + 1, j] + RND))
            FCE[i, j, 1] = ((FCE[i, j, 1] * E[i, j] + FCW[i + 1, j, 1] * W[i + 1, j]) /
                            (E[i, j] + W[i + 1, j] + RND))
            if E[i, j] < EPSIF and W[i + 1, j] < EPSIF:
                FCE[i, j, 0] = dx(i, j) / 2.0
            E[i, j] = av; W[i + 1, j] = av
    V = lambda i, j: vs[i - 1, j - 1]

    def close(i, j):
        vs[i - 1, j - 1] = 1.0
        W[i, j] = E[i, j] = N[i, j] = S[i, j] = 0.0
        E[i - 1, j] = 0.0; N[i, j - 1] = 0.0; W[i + 1, j] = 0.0; S[i, j + 1] = 0.0

    for i in range(1, nx + 1):
        for j in range(1, ny + 1):
            if V(i, j) > 1.0 - EPSI:
                close(i, j)
            if (is_p and (W[i, j] + E[i, j] < RND or S[i, j] + N[i, j] < RND)
                    and V(i, j) < 1.0 - EPSI):
                close(i, j)
    for i in range(1, nx + 1):
        for j in range(1, ny + 1):
            if abs(V(i, j) - 1.0) < RND:
                if W[i, j] == 0.0 or E[i, j] == 0.0:
                    WL[i - 1, j - 1] = dy(i, j)
                    if delh is not None:
                        delh[i - 1, j - 1] = dx(i, j) / 2.0
                if N[i, j] == 0.0 or S[i, j] == 0.0:
                    WL[i - 1, j - 1] = dx(i, j)
                    if delh is not None:
                        delh[i - 1, j - 1] = dy(i, j) / 2.0
    if icorprob and is_p:
        for i in range(1, nx + 1):
            for j in range(1, ny - 3):
                if -EPSI < V(i, j) < EPSI:
                    if 0.6 - EPSI < V(i, j + 1) < 0.6 + EPSI and 0.6 - EPSI < V(i, j + 2) < 0.6 + EPSI:
                        N[i, j] = 0.4; S[i, j + 1] = 0.4
                        FCN[i, j, 0] = -0.3 * dx(i, j)
                        FCN[i, j, 1] = 0.5 * dy(i, j)
                        WL[i - 1, j - 1] = 0.6 * dx(i, j)
                        nys[i - 1, j - 1] = -1.0; nxs[i - 1, j - 1] = 0.0
                    if 1.0 - EPSI < V(i, j + 1) < 1.0 + EPSI:
                        WL[i - 1, j - 1] = dx(i, j)
                        nys[i - 1, j - 1] = -1.0; nxs[i - 1, j - 1] = 0.0
    out = {"aE": E, "aW": W, "aN": N, "aS": S, "FCE": FCE, "FCN": FCN, "cent": cent,
           "vofS": vs, "nxS": nxs, "nyS": nys, "phiS": phs, "WlLh": WL}
    if delh is not None:
        out["delh"] = delh
    return out


def _exchange_cells(nx, ny, P, U, V):
    """DefineMomentumExchangeCell (:360-397)."""
    mu = np.zeros((nx, ny), dtype=np.int32); mv = np.zeros((nx, ny), dtype=np.int32)
    vp, vu, vv = P["vofS"], U["vofS"], V["vofS"]
    for i in range(1, nx + 1):
        for j in range(1, ny + 1):
            if EPSI <= vu[i - 1, j - 1] < 1.0 - EPSI:
                if i < nx:
                    if (vp[i - 1, j - 1] >= 1.0 - EPSI or vp[i, j - 1] >= 1.0 - EPSI
                            or P["aE"][i, j] < EPSIF):
                        mu[i - 1, j - 1] = 1; P["aE"][i, j] = 0.0; P["aW"][i + 1, j] = 0.0
                elif vp[i - 1, j - 1] >= 1.0 - EPSI:
                    mu[i - 1, j - 1] = 1
            if EPSI <= vv[i - 1, j - 1] < 1.0 - EPSI:
                if j < ny:
                    if (vp[i - 1, j - 1] >= 1.0 - EPSI or vp[i - 1, j] >= 1.0 - EPSI
                            or P["aN"][i, j] < EPSIF):
                        mv[i - 1, j - 1] = 1; P["aN"][i, j] = 0.0; P["aS"][i, j + 1] = 0.0
                elif vp[i - 1, j - 1] >= 1.0 - EPSI:
                    mv[i - 1, j - 1] = 1
    U["moex"], V["moex"] = mu, mv


def _number(nx, ny, T, iu, iv):
    """NumberExternalCell (:340-358): j fastest; -1 elsewhere."""
    pn = -np.ones((nx + 2, ny + 2), dtype=np.int32)
    c = 0
    for i in range(1, nx - iu + 1):
        for j in range(1, ny - iv + 1):
            if T["vofS"][i - 1, j - 1] < 1.0 - EPSI:
                pn[i, j] = c; c += 1
    T["posnu"] = pn


def _cell_linking(nx, ny, T, i, j):
    """CellLinking (:702-725)."""
    ii = i + int(_sign(1.0, T["nxS"][i - 1, j - 1]))
    jj = j + int(_sign(1.0, T["nyS"][i - 1, j - 1]))
    vs = lambda a, b: T["vofS"][a - 1, b - 1] if 1 <= a <= nx and 1 <= b <= ny else 1.0
    if vs(ii, j) < vs(i, jj):
        T["msce"][i - 1, j - 1] = (ii, j)
    else:
        T["msce"][i - 1, j - 1] = (i, jj)


def _east(nx, ny, T, tg, bdx, iu, aln_old):
    """EastFaceInterpolationInf (:551-616); bdx: BGrid%dx."""
    SxE = T["SxE"]; EtaE = T["EtaE"]; AlE = T["AlE"]; DAlE = T["DAlE"]
    c, F, pn = T["cent"], T["FCE"], T["posnu"]
    nxs, nys, phs = T["nxS"], T["nyS"], T["phiS"]
    C = lambda i, j, k: c[i - 1, j - 1, k]
    f = lambda a, i, j: a[i - 1, j - 1]
    for j in range(1, ny + 1):
        for i in range(1, nx):
            B = f(bdx, i + iu, j)
            if pn[i, j] != -1 and pn[i + 1, j] != -1:
                SxE[i, j] = C(i + 1, j, 0) + B - C(i, j, 0)
                sy = C(i + 1, j, 1) - C(i, j, 1)
                EtaE[i, j] = _div(abs(F[i, j, 0] - C(i, j, 0)), SxE[i, j])
                if EtaE[i, j] >= 1.0:
                    EtaE[i, j] = 0.5
                xf = (1.0 - EtaE[i, j]) * C(i, j, 0) + EtaE[i, j] * (C(i + 1, j, 0) + B)
                yf = (1.0 - EtaE[i, j]) * C(i, j, 1) + EtaE[i, j] * C(i + 1, j, 1)
                if abs(sy) > 0.0001 * f(tg["dy"], i, j):
                    nyf = 0.5 * (f(nys, i, j) + f(nys, i + 1, j))
                    ipd = 0.5 * (abs(xf * f(nxs, i, j) + yf * f(nys, i, j) + f(phs, i, j)) +
                                 abs((xf - B) * f(nxs, i + 1, j) + yf * f(nys, i + 1, j) +
                                     f(phs, i + 1, j)))
                    fcd = 0.5 * (abs(F[i, j, 0] * f(nxs, i, j) + F[i, j, 1] * f(nys, i, j) +
                                     f(phs, i, j)) +
                                 abs((F[i, j, 0] - B) * f(nxs, i + 1, j) +
                                     F[i, j, 1] * f(nys, i + 1, j) + f(phs, i + 1, j)))
                    AlE[i, j] = _div(abs(fcd), abs(ipd))
                    DAlE[i, j] = _div(sy * nyf, SxE[i, j] * abs(ipd))
                    if abs(ipd) < 1.0e-5:
                        DAlE[i, j] = 0.0; AlE[i, j] = 1.0
                    if AlE[i, j] >= 2.0:
                        AlE[i, j] = 2.0
                else:
                    DAlE[i, j] = 0.0; AlE[i, j] = 1.0
            else:
                AlE[i, j] = 1.0; DAlE[i, j] = 0.0; SxE[i, j] = B; EtaE[i, j] = 0.5
        i = nx
        SxE[i, j] = SxE[i - 1, j]; EtaE[i, j] = EtaE[i - 1, j]
        DAlE[i, j] = DAlE[i - 1, j]; AlE[i, j] = AlE[i - 1, j]
        SxE[0, j] = SxE[1, j]; EtaE[0, j] = EtaE[1, j]; DAlE[0, j] = DAlE[1, j]
        AlE[0, j] = aln_old[1, j]


def _north(nx, ny, T, tg, bdy, iv):
    """NorthFaceInterpolationInf (:618-700); bdy: BGrid%dy."""
    SyN = T["SyN"]; EtaN = T["EtaN"]; AlN = T["AlN"]; DAlN = T["DAlN"]
    c, F, pn = T["cent"], T["FCN"], T["posnu"]
    nxs, nys, phs = T["nxS"], T["nyS"], T["phiS"]
    C = lambda i, j, k: c[i - 1, j - 1, k]
    f = lambda a, i, j: a[i - 1, j - 1]
    for i in range(1, nx + 1):
        for j in range(1, ny):
            B = f(bdy, i, j + iv)
            if pn[i, j] != -1 and pn[i, j + 1] != -1:
                SyN[i, j] = C(i, j + 1, 1) + B - C(i, j, 1)
                sx = C(i, j + 1, 0) - C(i, j, 0)
                EtaN[i, j] = _div(abs(F[i, j, 1] - C(i, j, 1)), SyN[i, j])
                if EtaN[i, j] >= 1.0:
                    EtaN[i, j] = 0.5
                xf = (1.0 - EtaN[i, j]) * C(i, j, 0) + EtaN[i, j] * C(i, j + 1, 0)
                yf = (1.0 - EtaN[i, j]) * C(i, j, 1) + EtaN[i, j] * (C(i, j + 1, 1) + B)
                if abs(sx) >= 0.0001 * f(tg["dx"], i, j):
                    nxf = 0.5 * (f(nxs, i, j) + f(nxs, i, j + 1))
                    ipd = 0.5 * (abs(xf * f(nxs, i, j) + yf * f(nys, i, j) + f(phs, i, j)) +
                                 abs(xf * f(nxs, i, j + 1) + (yf - B) * f(nys, i, j + 1) +
                                     f(phs, i, j + 1)))
                    fcd = 0.5 * (abs(F[i, j, 0] * f(nxs, i, j) + F[i, j, 1] * f(nys, i, j) +
                                     f(phs, i, j)) +
                                 abs(F[i, j, 0] * f(nxs, i, j + 1) +
                                     (F[i, j, 1] - B) * f(nys, i, j + 1) + f(phs, i, j + 1)))
                    AlN[i, j] = _div(abs(ipd), abs(fcd))
                    DAlN[i, j] = _div(sx * nxf, SyN[i, j] * abs(ipd))
                    if abs(ipd) < 1.0e-5:
                        DAlN[i, j] = 0.0; AlN[i, j] = 1.0
                    if AlN[i, j] >= 2.0:
                        AlN[i, j] = 2.0
                else:
                    DAlN[i, j] = 0.0; AlN[i, j] = 1.0
            else:
                EtaN[i, j] = 0.5; AlN[i, j] = 1.0; DAlN[i, j] = 0.0; SyN[i, j] = B
        j = ny
        SyN[i, j] = SyN[i, j - 1]; EtaN[i, j] = EtaN[i, j - 1]
        DAlN[i, j] = DAlN[i, j - 1]; AlN[i, j] = AlN[i, j - 1]
        SyN[i, 0] = SyN[i, 1]; EtaN[i, 0] = EtaN[i, 1]; DAlN[i, 0] = DAlN[i, 1]
        AlN[i, 0] = AlN[i, 1]


def _div(a, b):
    """IEEE division (Python raises on /0)."""
    if b == 0.0:
        if a == 0.0 or math.isnan(a):
            return math.nan
        return math.copysign(math.inf, a) * (math.copysign(1.0, b))
    return a / b


def _new_cell_face(nx, ny, P, U, V, gp, gu, gv, aln_old):
    """NewCellFace (:399-549)."""
    tol = 1.0e-24
    for T in (U, V):
        T["msce"] = np.zeros((nx, ny, 2), dtype=np.int32)
    for i in range(1, nx + 1):
        for j in range(1, ny + 1):
            if U["moex"][i - 1, j - 1] != 1 and U["vofS"][i - 1, j - 1] > EPSI:
                U["cent"][i - 1, j - 1, 0] = P["FCE"][i, j, 0] - gp["dx"][i - 1, j - 1] / 2.0
                U["cent"][i - 1, j - 1, 1] = P["FCE"][i, j, 1]
            if V["moex"][i - 1, j - 1] != 1 and V["vofS"][i - 1, j - 1] > EPSI:
                V["cent"][i - 1, j - 1, 0] = P["FCN"][i, j, 0]
                V["cent"][i - 1, j - 1, 1] = P["FCN"][i, j, 1] - gp["dy"][i - 1, j - 1] / 2.0
    for i in range(1, nx + 1):
        for j in range(1, ny + 1):
            for T in (U, V):
                if T["moex"][i - 1, j - 1] != 1:
                    continue
                if T["vofS"][i - 1, j - 1] < 1.0 - EPSI:
                    aN, aE, FN, FE = T["aN"], T["aE"], T["FCN"], T["FCE"]
                    c = T["cent"][i - 1, j - 1]
                    nxs, nys, phs = (T["nxS"][i - 1, j - 1], T["nyS"][i - 1, j - 1],
                                     T["phiS"][i - 1, j - 1])
                    if aN[i, j] * aN[i, j - 1] == 0.0:
                        c[0] = (FN[i, j, 0] * aN[i, j] / (aN[i, j] + tol) +
                                FN[i, j - 1, 0] * aN[i, j - 1] / (aN[i, j - 1] + tol))
                    else:
                        c[1] = (FE[i, j, 1] * aE[i, j] / (aE[i, j] + tol) +
                                FE[i - 1, j, 1] * aE[i - 1, j] / (aE[i - 1, j] + tol))
                        c[0] = _div(-(nys * c[1] + phs), nxs + tol)
                    if aE[i, j] * aE[i - 1, j] == 0.0:
                        c[1] = (FE[i, j, 1] * aE[i, j] / (aE[i, j] + tol) +
                                FE[i - 1, j, 1] * aE[i - 1, j] / (aE[i - 1, j] + tol))
                    else:
                        c[1] = _div(-(nxs * c[0] + phs), nys + tol)
                _cell_linking(nx, ny, T, i, j)
    for i in range(1, nx + 1):
        for j in range(1, ny + 1):
            for T, g in ((U, gu), (V, gv)):
                c = T["cent"][i - 1, j - 1]
                T["delh"][i - 1, j - 1] = abs(c[0] * T["nxS"][i - 1, j - 1] +
                                              c[1] * T["nyS"][i - 1, j - 1] +
                                              T["phiS"][i - 1, j - 1]) + tol
                if T["moex"][i - 1, j - 1] == 1:
                    T["delh"][i - 1, j - 1] = 1.0e-20
            for T, g in ((U, gu), (V, gv)):
                a_ = (T["aE"][i, j] - T["aW"][i, j]) * g["dx"][i - 1, j - 1]
                b_ = (T["aN"][i, j] - T["aS"][i, j]) * g["dy"][i - 1, j - 1]
                T["WlLh"][i - 1, j - 1] = math.sqrt(a_ * a_ + b_ * b_)
    for T in (U, V):
        for k in ("SxE", "EtaE", "AlE", "DAlE", "SyN", "EtaN", "AlN", "DAlN"):
            T[k] = np.zeros((nx + 2, ny + 2))
    _east(nx, ny, U, gu, gp["dx"], 1, aln_old["u"])
    _north(nx, ny, U, gu, gv["dy"], 0)
    _east(nx, ny, V, gv, gu["dx"], 0, aln_old["v"])
    _north(nx, ny, V, gv, gp["dy"], 1)


def grid_preprocess(nx, ny, grids, fams, icorprob=True, aln_old=None):
    """Grid_Preprocess + NewCellFace for the P, U and V families.
    grids[f] = {dx, dy, x, y}; fams[f] = {vofS, phiS, nxS, nyS} for f in
    'p', 'u', 'v'.  aln_old[f] (f = 'u', 'v'): AlN (nx+2,ny+2) before this
    step (zeros if None).  Returns {f: outputs}."""
    out = {}
    for f in ("p", "u", "v"):
        out[f] = cell_geo_cal(nx, ny, grids[f], dict(fams[f], family=f), icorprob)
    P, U, V = out["p"], out["u"], out["v"]
    _exchange_cells(nx, ny, P, U, V)
    _number(nx, ny, P, 0, 0)
    _number(nx, ny, U, 1, 0)
    _number(nx, ny, V, 0, 1)
    if aln_old is None:
        aln_old = {"u": np.zeros((nx + 2, ny + 2)), "v": np.zeros((nx + 2, ny + 2))}
    _new_cell_face(nx, ny, P, U, V, grids["p"], grids["u"], grids["v"], aln_old)
    return out
