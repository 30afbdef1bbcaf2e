"""Oracle of the projection path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py may
import this module.  The simcoflow_gb300 package never does.

Parity status: UNPINNED.  The reference (Fortran 90 + HYPRE + MPI) cannot be
compiled here or on the GPU host (no Fortran compiler, MPI or HYPRE) and ships
no tests or golden vectors.  The restatement is pinned instead against the
reference's built-in identities (per-row |A p - b| <= 1e-10,
src/ProjectionP_Mod.f90:70-93; mass residual, src/ComputePUV_Mod.f90:184-216)
and analytic known-answer cases (tests/test_oracle.py).

Pieces:
  C restatement (scf_oracle.c, via ctypes)
    pocoef      ComputePossionMatrixCoefficient  src/ProjectionP_Mod.f90:395-580
    matrix      SetPoissonMatrix                 src/ProjectionP_Mod.f90:137-273
    rhs         SetPoissonVectors                src/ProjectionP_Mod.f90:275-354
    scatter     DeltaPressureGetValues + BC      src/ProjectionP_Mod.f90:356-393, 582-595
    correct     UpdatePUV correction .. zeroing  src/ComputePUV_Mod.f90:59-245
    mgpcg       CPU FP64 MG-PCG (same algorithm as the CUDA path)
  solve_direct  the HYPRE PCG/BoomerAMG solve replaced by SuperLU on the same
                CSR matrix (an exact FP64 solve; HYPRE is not available)
  geometry_literal  pure-Python restatement of Cell_Geo_Cal, frac, numbering
                and DefineMomentumExchangeCell for small grids, to check the
                package's geometry builder.
  C restatement of the momentum predictor's implicit solves (mom_oracle.c)
    mom_predict SetMatrix, SetVectors, solve, DeltaGetValues, gradient update,
                Dp copies              src/PredictorUV_mod.f90:507-563, 622-885
                (solve: SuperLU, or the C BiCGStab of the CPU baseline)
  C restatement of the Tecplot result files (out_oracle.c)
  cutcell_literal.grid_preprocess   pure-Python Grid_Preprocess + NewCellFace
                for the P, U and V families (src/Cutcell_Mod.f90:18-725)
    tecplot_pcell / tecplot_vcell   Print_Result_Tecplot_PCent / _UCent /
                _VCent                 src/PrintResult.f90:39-168
    f24_14      the "(f24.14)" number format
    vtr         Print_Result_VTK_2D's ParaView file   src/PrintResult.f90:165-190,
                src/VTR_mod.f90:79-379
    e15_8       its list-directed REAL(4) value text (15 characters)
  C restatement of the CLSVOF sweeps after Interface_Reconstruct (clsvof_oracle.c)
    ls_sweep    X_Sweep / Y_Sweep temls update   src/Clsvof_Mod.f90:1074-1123,
                1191-1244
    vof_sweep   X_Sweep / Y_Sweep temvf update   src/Clsvof_Mod.f90:1004-1069,
                1141-1189, with topflux .. leftflux (:1416-1522)
    frac, cellgeocal                             src/Clsvof_Mod.f90:1371-1404,
                2159-2253
    interface_reconstruct  Interface_Reconstruct with Normal_Vector_Irre,
                distance, DistanceFluidCalculate, zriddr, LiqFuncVol
                                                 src/Clsvof_Mod.f90:1250-1369,
                1710-1919, 1957-2155
    redistance  Redistance with isinsiderect     src/Clsvof_Mod.f90:1525-1708,
                1921-1955
    clsvof_step Coupled_LS_VOF with a fixed solid  src/Clsvof_Mod.f90:730-973
"""
from __future__ import annotations

import ctypes as C
import math
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
import build as _build  # noqa: E402

_P = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int32)
_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(str(path))
        L.oracle_pocoef.argtypes = [C.c_int, C.c_int, C.c_int] + [_P] * 9 + [C.c_double, C.c_double, _P]
        L.oracle_matrix.restype = C.c_int
        L.oracle_matrix.argtypes = [C.c_int, C.c_int, _P, _P, _P, _P, _P, _I, C.c_int, C.c_int,
                                    C.c_int, C.c_int, _P, _I, _I, _P]
        L.oracle_rhs.argtypes = [C.c_int, C.c_int] + [_P] * 10 + [_I, C.c_double, _P, _P]
        L.oracle_scatter.argtypes = [C.c_int, C.c_int, _I, _P, C.c_int, C.c_int, C.c_int,
                                     C.c_int, _P]
        L.oracle_correct.argtypes = ([C.c_int, C.c_int] + [_P] * 3 + [_P] * 3 + [_P] * 2 +
                                     [_P] * 4 + [_I, _I, _I, _P, _I, _I, _P] + [_P] * 6 +
                                     [C.c_double, C.c_double, C.c_double, _P, _P, _P, _P])
        L.oracle_row_residual.restype = C.c_double
        L.oracle_row_residual.argtypes = [C.c_int, C.c_int, _P, _P, _P, _I]
        L.oracle_mgpcg.restype = C.c_int
        L.oracle_mgpcg.argtypes = [C.c_int, C.c_int, _P, _P, _P, _P, _P, _P, _P, C.c_double, C.c_int,
                                   C.c_int, C.c_int, C.c_double, C.c_int, _P, C.POINTER(C.c_int),
                                   C.c_int]
        L.oracle_mgpcg_matr.restype = C.c_int
        L.oracle_mgpcg_matr.argtypes = [C.c_int, C.c_int, _P, _P, _I, _P, C.c_double, C.c_int,
                                        C.c_int, C.c_int, C.c_double, C.c_int, _P,
                                        C.POINTER(C.c_int), C.c_int]
        L.oracle_scatter_interior.argtypes = [C.c_int, C.c_int, _I, _P, C.c_int, C.c_int,
                                              C.c_int, C.c_int, _P]
        L.oracle_vcycle.argtypes = [C.c_int, C.c_int, _P, _P, _P, _P, _P, C.c_int, C.c_int,
                                    C.c_double, C.c_int, C.c_int]
        L.oracle_mom_matrix.restype = C.c_int
        L.oracle_mom_matrix.argtypes = ([C.c_int] * 4 + [_P, _P, _I] + [_P] * 10 +
                                        [_P, _P, _P, _P, _P])
        L.oracle_mom_vectors.argtypes = ([C.c_int] * 4 + [_I, _P, _P, _P, _P, _P, _P, _P,
                                         C.c_double, _P])
        L.oracle_mom_finish.argtypes = ([C.c_int] * 4 + [_I, _P, _P, _P, _P, C.c_double, _P,
                                        _P])
        L.oracle_mom_bicgstab.restype = C.c_int
        L.oracle_mom_bicgstab.argtypes = ([C.c_int] * 4 + [_I, _P, _P, C.c_double, C.c_int, _P,
                                          C.POINTER(C.c_double)])
        L.oracle_num_threads.restype = C.c_int
        L.oracle_set_threads.argtypes = [C.c_int]
        L.oracle_set_coarse_sweeps.argtypes = [C.c_int, C.c_int]
        L.oracle_format_many.argtypes = [_P, C.c_int64, C.c_char_p]
        L.oracle_tecplot_pcell.restype = C.c_int64
        L.oracle_tecplot_pcell.argtypes = [C.c_int, C.c_int] + [_P] * 13 + [C.c_char_p]
        L.oracle_tecplot_vcell.restype = C.c_int64
        L.oracle_tecplot_vcell.argtypes = [C.c_int, C.c_int, C.c_int] + [_P] * 7 + [C.c_char_p]
        L.oracle_format_e15_8.argtypes = [_P, C.c_int64, C.c_char_p]
        L.oracle_vtr.restype = C.c_int64
        L.oracle_vtr.argtypes = [C.c_int, C.c_int] + [_P] * 9 + [C.c_char_p]
        L.oracle_ls_sweep.argtypes = [C.c_int] * 3 + [_P] * 12 + [C.c_double, _P]
        L.oracle_frac.restype = C.c_double
        L.oracle_frac.argtypes = [C.c_double] * 5
        L.oracle_cellgeocal.argtypes = [C.c_double] * 8 + [_P, _P]
        L.oracle_vof_sweep.argtypes = [C.c_int] * 3 + [_P] * 11 + [_P] * 7 + [_P, C.c_double, _P]
        L.oracle_interface_reconstruct.restype = C.c_int
        L.oracle_interface_reconstruct.argtypes = [C.c_int, C.c_int] + [_P] * 10 + [_P] * 3
        L.oracle_redistance.restype = C.c_int
        L.oracle_redistance.argtypes = [C.c_int, C.c_int] + [_P] * 12 + [_P, _P, _I]
        L.oracle_clsvof_step.restype = C.c_int
        L.oracle_clsvof_step.argtypes = [C.c_int, C.c_int] + [_P] * 14 + [_P, C.c_double] + [_P] * 6
        L.oracle_plic_distance.restype = C.c_double
        L.oracle_plic_distance.argtypes = [C.c_double] * 5
        L.oracle_dfc.restype = C.c_int
        L.oracle_dfc.argtypes = [C.c_double] * 8 + [_P, C.POINTER(C.c_int)]
        _lib = L
    return _lib


def _p(a):
    if a is None:
        return None
    assert a.flags["F_CONTIGUOUS"] or a.ndim == 1, "arrays must be Fortran ordered"
    return a.ctypes.data_as(_P if a.dtype == np.float64 else _I)


def pocoef(case, literal=False) -> np.ndarray:
    a = case.arrays
    pc = np.zeros((case.nx, case.ny, 4), order="F")
    lib().oracle_pocoef(case.nx, case.ny, int(literal), _p(a["vof"]), _p(a["phi"]), _p(a["vofS"]),
                        _p(a["dx"]), _p(a["dy"]), _p(a["dxU"]), _p(a["dyV"]), _p(a["DpU"]),
                        _p(a["DpV"]), case.betaP, case.betaM, _p(pc))
    return pc


def matrix(case, pc=None, csr=True):
    """Returns (matr (nx,ny,5), scipy CSR in Posnu numbering); with
    csr=False only the dense copy matr is built (and None returned for A)."""
    a = case.arrays
    if pc is None:
        pc = pocoef(case)
    nx, ny = case.nx, case.ny
    nmax = nx * ny
    matr = np.zeros((nx, ny, 5), order="F")
    if not csr:
        wb, eb, sb, nb = case.bc
        lib().oracle_matrix(nx, ny, _p(pc), _p(a["aE"]), _p(a["aW"]), _p(a["aN"]), _p(a["aS"]),
                            _p(a["posnu_p"]), wb, eb, sb, nb, _p(matr), None, None, None)
        return matr, None
    import scipy.sparse as sp
    rowptr = np.zeros(nmax + 1, dtype=np.int32)
    cols = np.zeros(5 * nmax, dtype=np.int32)
    vals = np.zeros(5 * nmax)
    wb, eb, sb, nb = case.bc
    nrows = lib().oracle_matrix(nx, ny, _p(pc), _p(a["aE"]), _p(a["aW"]), _p(a["aN"]), _p(a["aS"]),
                                _p(a["posnu_p"]), wb, eb, sb, nb, _p(matr), _p(rowptr), _p(cols),
                                _p(vals))
    nnz = rowptr[nrows]
    A = sp.csr_matrix((vals[:nnz], cols[:nnz], rowptr[: nrows + 1]), shape=(nrows, nrows))
    return matr, A


def rhs(case, ustar=None, vstar=None, vb=None):
    a = case.arrays
    nx, ny = case.nx, case.ny
    us = a["ustar"] if ustar is None else ustar
    vs = a["vstar"] if vstar is None else vstar
    vb = case.vb if vb is None else vb
    rhm = np.zeros((nx, ny), order="F")
    n = int((a["posnu_p"][1:nx + 1, 1:ny + 1] != -1).sum())
    b = np.zeros(max(n, 1))
    lib().oracle_rhs(nx, ny, _p(us), _p(vs), _p(a["aE"]), _p(a["aW"]), _p(a["aN"]), _p(a["aS"]),
                     _p(a["dx"]), _p(a["dy"]), _p(a["nyS"]), _p(a["WlLh"]), _p(a["posnu_p"]), vb,
                     _p(rhm), _p(b))
    return rhm, b[:n]


def scatter(case, x) -> np.ndarray:
    Pp = np.zeros((case.nx + 2, case.ny + 2), order="F")
    x = np.ascontiguousarray(x, dtype=np.float64)
    wb, eb, sb, nb = case.bc
    lib().oracle_scatter(case.nx, case.ny, _p(case["posnu_p"]), x.ctypes.data_as(_P), wb, eb, sb,
                         nb, _p(Pp))
    return Pp


def correct(case, Pp, u0=None, v0=None, p0=None, vb=None):
    a = case.arrays
    nx, ny = case.nx, case.ny
    u = (a["u0"] if u0 is None else u0).copy(order="F")
    v = (a["v0"] if v0 is None else v0).copy(order="F")
    p = (a["p0"] if p0 is None else p0).copy(order="F")
    mres = np.zeros((nx, ny), order="F")
    vb = case.vb if vb is None else vb
    lib().oracle_correct(nx, ny, _p(Pp), _p(a["ustar"]), _p(a["vstar"]), _p(a["vof"]),
                         _p(a["phi"]), _p(a["vofS"]), _p(a["nyS"]), _p(a["WlLh"]), _p(a["aE"]),
                         _p(a["aW"]), _p(a["aN"]), _p(a["aS"]), _p(a["posnu_p"]),
                         _p(a["posnu_u"]), _p(a["moex_u"]), _p(a["vofS_u"]), _p(a["posnu_v"]),
                         _p(a["moex_v"]), _p(a["vofS_v"]), _p(a["dx"]), _p(a["dy"]),
                         _p(a["dxU"]), _p(a["dyV"]), _p(a["DpU"]), _p(a["DpV"]), case.betaP,
                         case.betaM, vb, _p(u), _p(v), _p(p), _p(mres))
    return u, v, p, mres


def row_residual(case, matr, Pp, rhm) -> float:
    return lib().oracle_row_residual(case.nx, case.ny, _p(matr), _p(Pp), _p(rhm),
                                     _p(case["posnu_p"]))


def solve_direct(A, b) -> np.ndarray:
    """FP64 direct solve of the reference's own matrix (SuperLU)."""
    import scipy.sparse.linalg as spla
    if A.shape[0] == 0:
        return np.zeros(0)
    return spla.spsolve(A.tocsc(), b)


def symmetric_operator(case, matr):
    """The symmetric 5-point storage of the multigrid built from matr:
    cE = -matr(.,.,4), cN = -matr(.,.,5), dg = matr(.,.,3) (-1 without an
    unknown), in 0-based C order (ny, nx) flattened."""
    nx, ny = case.nx, case.ny
    act = case["posnu_p"][1:nx + 1, 1:ny + 1] != -1
    cE = np.where(act, -matr[:, :, 3], 0.0) + 0.0
    cN = np.where(act, -matr[:, :, 4], 0.0) + 0.0
    dg = np.where(act, matr[:, :, 2], -1.0)
    f = lambda a: np.ascontiguousarray(a.T).ravel()
    return f(cE), f(cN), f(dg)


def own_west_south(case, matr):
    """Each row's own west and south couplings, -matr(.,.,2) and
    -matr(.,.,1) (src/ProjectionP_Mod.f90:183,193), in the same 0-based
    order; the PCG applies the rows with them."""
    nx, ny = case.nx, case.ny
    act = case["posnu_p"][1:nx + 1, 1:ny + 1] != -1
    cW = np.where(act, -matr[:, :, 1], 0.0) + 0.0
    cS = np.where(act, -matr[:, :, 0], 0.0) + 0.0
    f = lambda a: np.ascontiguousarray(a.T).ravel()
    return f(cW), f(cS)


SMOOTHERS = {"point": 0, "line": 1}


class _coarse_sweeps:
    """The coarse-level schedule (level, sweeps) for the calls in a
    with-block; None or sweeps 0: npre / npost on every level."""

    def __init__(self, coarse):
        self.c = coarse or (0, 0)

    def __enter__(self):
        lib().oracle_set_coarse_sweeps(int(self.c[0]), int(self.c[1]))

    def __exit__(self, *a):
        lib().oracle_set_coarse_sweeps(0, 0)


def mgpcg(case, matr, rhm, rtol=1e-13, maxit=500, npre=2, npost=2, omega=1.9, coarse_max=64,
          threads=0, smoother="point", coarse=None):
    """CPU FP64 MG-PCG: the PCG applies the assembled rows as written (own
    west / south entries), the V-cycle preconditioner the symmetric storage.
    Returns (Pp-interior x as (nx,ny) Fortran array, iterations, true relres,
    levels).  smoother: 'point' (red-black Gauss-Seidel) or 'line'
    (alternating zebra lines)."""
    nx, ny = case.nx, case.ny
    cE, cN, dg = symmetric_operator(case, matr)
    cW, cS = own_west_south(case, matr)
    b = np.ascontiguousarray(rhm.T).ravel()
    x = np.zeros(nx * ny)
    rel = C.c_double(0.0)
    nlev = C.c_int(0)
    if threads:
        lib().oracle_set_threads(threads)
    with _coarse_sweeps(coarse):
        it = lib().oracle_mgpcg(nx, ny, cE.ctypes.data_as(_P), cN.ctypes.data_as(_P),
                                dg.ctypes.data_as(_P), cW.ctypes.data_as(_P),
                                cS.ctypes.data_as(_P), b.ctypes.data_as(_P),
                                x.ctypes.data_as(_P), rtol, maxit, npre, npost, omega,
                                coarse_max, C.byref(rel), C.byref(nlev), SMOOTHERS[smoother])
    return np.asfortranarray(x.reshape(ny, nx).T), it, rel.value, nlev.value


def vcycle(case, matr, b_f, npre=2, npost=2, omega=1.9, coarse_max=64,
           smoother="point", coarse=None) -> np.ndarray:
    nx, ny = case.nx, case.ny
    cE, cN, dg = symmetric_operator(case, matr)
    b = np.ascontiguousarray(b_f.T).ravel()
    x = np.zeros(nx * ny)
    with _coarse_sweeps(coarse):
        lib().oracle_vcycle(nx, ny, cE.ctypes.data_as(_P), cN.ctypes.data_as(_P),
                            dg.ctypes.data_as(_P), b.ctypes.data_as(_P), x.ctypes.data_as(_P),
                            npre, npost, omega, coarse_max, SMOOTHERS[smoother])
    return np.asfortranarray(x.reshape(ny, nx).T)


def line_smoother_wanted(case) -> bool:
    """The library's automatic smoother choice: lines when some cell's aspect
    ratio exceeds 2."""
    dx, dy = case["dx"], case["dy"]
    return bool(max((dx / dy).max(), (dy / dx).max()) > 2.0)


def project_mg(case, rtol=1e-8, maxit=500, npre=2, npost=2, omega=1.9, coarse_max=64,
               smoother=None, threads=0, coarse=None) -> dict:
    """The whole projection in C on all host threads, as the timed CPU
    baseline runs it: pocoef, the dense rows, the right-hand side, the FP64
    MG-PCG to rtol (the PCG on the rows as written, the V-cycle on their
    symmetric part; maxit < 0 encodes cycles per application, see
    oracle_mgpcg), scatter and correction.  smoother None picks lines where
    the library would."""
    if threads:
        lib().oracle_set_threads(threads)
    if smoother is None:
        smoother = "line" if line_smoother_wanted(case) else "point"
    nx, ny = case.nx, case.ny
    pc = pocoef(case)
    matr, _ = matrix(case, pc, csr=False)
    rhm, _ = rhs(case)
    xint = np.zeros((nx, ny), order="F")
    rel = C.c_double(0.0)
    nlev = C.c_int(0)
    with _coarse_sweeps(coarse):
        it = lib().oracle_mgpcg_matr(nx, ny, _p(matr), _p(rhm), _p(case["posnu_p"]), _p(xint),
                                     rtol, maxit, npre, npost, omega, coarse_max, C.byref(rel),
                                     C.byref(nlev), SMOOTHERS[smoother])
    Pp = np.zeros((nx + 2, ny + 2), order="F")
    wb, eb, sb, nb = case.bc
    lib().oracle_scatter_interior(nx, ny, _p(case["posnu_p"]), _p(xint), wb, eb, sb, nb, _p(Pp))
    u, v, p, mres = correct(case, Pp)
    return {"Pp": Pp, "u": u, "v": v, "p": p, "mres": mres, "matr": matr, "rhm": rhm,
            "iters": it, "relres": rel.value, "levels": nlev.value, "smoother": smoother}


def x_from_interior(case, xint):
    """Posnu-ordered vector from an (nx,ny) interior field."""
    pn = case["posnu_p"][1:case.nx + 1, 1:case.ny + 1]
    n = int((pn != -1).sum())
    x = np.zeros(n)
    m = pn != -1
    x[pn[m]] = xint[m]
    return x


def project(case, solver="direct", **kw) -> dict:
    """The whole reference projection on the CPU: assembly, RHS, FP64 solve,
    scatter, correction.  solver='direct' (SuperLU) or 'mg' (CPU MG-PCG)."""
    pc = pocoef(case)
    matr, A = matrix(case, pc)
    rhm, b = rhs(case)
    if solver == "direct":
        x = solve_direct(A, b)
    else:
        xi, it, rel, nlev = mgpcg(case, matr, rhm, **kw)
        x = x_from_interior(case, xi)
    Pp = scatter(case, x)
    u, v, p, mres = correct(case, Pp)
    res = row_residual(case, matr, Pp, rhm)
    bn = float(np.linalg.norm(b))
    relres = float(np.linalg.norm(A @ x - b) / bn) if bn > 0 else 0.0
    return {"pocoef": pc, "matr": matr, "A": A, "rhm": rhm, "b": b, "x": x, "Pp": Pp, "u": u,
            "v": v, "p": p, "mres": mres, "row_residual": res, "relres": relres}


# ---------------------------------------------------------------------------
# Literal pure-Python restatement of the geometry pipeline (small grids only)
# ---------------------------------------------------------------------------

def frac_literal(nx, ny, diss, dx, dy):
    """frac, src/Clsvof_Mod.f90:1371-1404."""
    slop_eps = 1.0e-20
    tnx, tny = abs(nx), abs(ny)
    if diss + 0.5 * (tnx * dx + tny * dy) <= 0.0:
        return 1.0
    if diss - 0.5 * (tnx * dx + tny * dy) >= 0.0:
        return 0.0
    if tnx <= slop_eps:
        return 0.5 - diss / dy
    if tny <= slop_eps:
        return 0.5 - diss / dx
    xx = (0.5 * tny * dy - diss) / dx / tnx + 0.5
    yy = (0.5 * tnx * dx - diss) / dy / tny + 0.5
    totalarea = 0.5 * xx * yy
    topvf = ((yy - 1.0) / yy) ** 2.0 if yy > 1.0 else 0.0
    rightvf = ((xx - 1.0) / xx) ** 2.0 if xx > 1.0 else 0.0
    return totalarea * (1.0 - topvf - rightvf)


def _edge(p1, p2, nxx, nyy, diss):
    """Edge_Geo_Cal, src/Cutcell_Mod.f90:302-337 (edge solid fraction)."""
    l1 = nxx * p1[0] + nyy * p1[1] + diss
    l2 = nxx * p2[0] + nyy * p2[1] + diss
    e = 1.0e-14
    if l1 >= e and l2 >= e:
        return 0.0
    if l1 < e and l2 < e:
        return 1.0
    if l1 >= e and l2 < e:
        return abs(l2) / (abs(l1) + abs(l2))
    return abs(l1) / (abs(l1) + abs(l2))


def geometry_literal(nx, ny, dxP, dyP, vofS_in, phiS, nxS, nyS, vofS_u_in, vofS_v_in,
                     icorprob=True):
    """Cell_Geo_Cal (P, U, V), DefineMomentumExchangeCell and
    NumberExternalCell (src/Cutcell_Mod.f90:34-358) on (nx,ny) inputs given
    as dicts/arrays indexed [i, j] 1-based via helper.  Returns a dict with
    the same keys and layouts as simcoflow_gb300.geometry.build."""
    epsi, epsiF, rnd = 1.0e-3, 1.0e-2, 1.0e-24
    E = np.zeros((nx + 2, ny + 2)); W = np.zeros_like(E); N = np.zeros_like(E); S = np.zeros_like(E)
    vs = np.array(vofS_in, dtype=float).copy()
    ny_s = np.array(nyS, dtype=float).copy()
    nx_s = np.array(nxS, dtype=float).copy()
    WL = np.zeros((nx, ny))
    for i in range(1, nx + 1):
        for j in range(1, ny + 1):
            dx, dy = dxP[i - 1, j - 1], dyP[i - 1, j - 1]
            a, b, p = nx_s[i - 1, j - 1], ny_s[i - 1, j - 1], phiS[i - 1, j - 1]
            P00, P01, P10, P11 = (-dx * 0.5, -dy * 0.5), (-dx * 0.5, dy * 0.5), (dx * 0.5, -dy * 0.5), (dx * 0.5, dy * 0.5)
            W[i, j] = _edge(P00, P01, a, b, p)
            N[i, j] = _edge(P01, P11, a, b, p)
            E[i, j] = _edge(P11, P10, a, b, p)
            S[i, j] = _edge(P10, P00, a, b, p)
    for i in range(1, nx + 1):
        for j in range(1, ny + 1):
            WL[i - 1, j - 1] = math.sqrt(((E[i, j] - W[i, j]) * dxP[i - 1, j - 1]) ** 2.0 +
                                         ((N[i, j] - S[i, j]) * dyP[i - 1, j - 1]) ** 2.0)
    for i in range(1, nx + 1):
        for j in range(1, ny + 1):
            W[i, j] = 1.0 - W[i, j]; E[i, j] = 1.0 - E[i, j]
            N[i, j] = 1.0 - N[i, j]; S[i, j] = 1.0 - S[i, j]
    for i in range(2, nx):
        for j in range(2, ny):
            av = 2.0 * N[i, j] * S[i, j + 1] / (N[i, j] + S[i, j + 1] + rnd)
            N[i, j] = av; S[i, j + 1] = av
            av = 2.0 * E[i, j] * W[i + 1, j] / (E[i, j] + W[i + 1, j] + rnd)
            E[i, j] = av; W[i + 1, j] = av
    V = lambda i, j: vs[i - 1, j - 1]
    for i in range(1, nx + 1):
        for j in range(1, ny + 1):
            if V(i, j) > 1.0 - epsi:
                vs[i - 1, j - 1] = 1.0
                W[i, j] = E[i, j] = N[i, j] = S[i, j] = 0.0
                E[i - 1, j] = 0.0; N[i, j - 1] = 0.0; W[i + 1, j] = 0.0; S[i, j + 1] = 0.0
            if (W[i, j] + E[i, j] < rnd or S[i, j] + N[i, j] < rnd) and V(i, j) < 1.0 - epsi:
                vs[i - 1, j - 1] = 1.0
                W[i, j] = E[i, j] = N[i, j] = S[i, j] = 0.0
                E[i - 1, j] = 0.0; N[i, j - 1] = 0.0; W[i + 1, j] = 0.0; S[i, j + 1] = 0.0
    for i in range(1, nx + 1):
        for j in range(1, ny + 1):
            if abs(V(i, j) - 1.0) < rnd:
                if W[i, j] == 0.0 or E[i, j] == 0.0:
                    WL[i - 1, j - 1] = dyP[i - 1, j - 1]
                if N[i, j] == 0.0 or S[i, j] == 0.0:
                    WL[i - 1, j - 1] = dxP[i - 1, j - 1]
    if icorprob:
        for i in range(1, nx + 1):
            for j in range(1, ny - 3):
                if -epsi < V(i, j) < epsi:
                    if 0.6 - epsi < V(i, j + 1) < 0.6 + epsi and 0.6 - epsi < V(i, j + 2) < 0.6 + epsi:
                        N[i, j] = 0.4; S[i, j + 1] = 0.4
                        WL[i - 1, j - 1] = 0.6 * dxP[i - 1, j - 1]
                        ny_s[i - 1, j - 1] = -1.0; nx_s[i - 1, j - 1] = 0.0
                    if 1.0 - epsi < V(i, j + 1) < 1.0 + epsi:
                        WL[i - 1, j - 1] = dxP[i - 1, j - 1]
                        ny_s[i - 1, j - 1] = -1.0; nx_s[i - 1, j - 1] = 0.0
    vsu = np.where(np.asarray(vofS_u_in) > 1.0 - epsi, 1.0, vofS_u_in)
    vsv = np.where(np.asarray(vofS_v_in) > 1.0 - epsi, 1.0, vofS_v_in)
    mu = np.zeros((nx, ny), dtype=np.int32); mv = np.zeros((nx, ny), dtype=np.int32)
    for i in range(1, nx + 1):
        for j in range(1, ny + 1):
            if epsi <= vsu[i - 1, j - 1] < 1.0 - epsi:
                if i < nx:
                    if V(i, j) >= 1.0 - epsi or V(i + 1, j) >= 1.0 - epsi or E[i, j] < epsiF:
                        mu[i - 1, j - 1] = 1; E[i, j] = 0.0; W[i + 1, j] = 0.0
                elif V(i, j) >= 1.0 - epsi:
                    mu[i - 1, j - 1] = 1
            if epsi <= vsv[i - 1, j - 1] < 1.0 - epsi:
                if j < ny:
                    if V(i, j) >= 1.0 - epsi or V(i, j + 1) >= 1.0 - epsi or N[i, j] < epsiF:
                        mv[i - 1, j - 1] = 1; N[i, j] = 0.0; S[i, j + 1] = 0.0
                elif V(i, j) >= 1.0 - epsi:
                    mv[i - 1, j - 1] = 1
    pp = -np.ones((nx + 2, ny + 2), dtype=np.int32)
    pu = -np.ones_like(pp); pv = -np.ones_like(pp)
    c = 0
    for i in range(1, nx + 1):
        for j in range(1, ny + 1):
            if V(i, j) < 1.0 - epsi:
                pp[i, j] = c; c += 1
    c = 0
    for i in range(1, nx):
        for j in range(1, ny + 1):
            if vsu[i - 1, j - 1] < 1.0 - epsi:
                pu[i, j] = c; c += 1
    c = 0
    for i in range(1, nx + 1):
        for j in range(1, ny):
            if vsv[i - 1, j - 1] < 1.0 - epsi:
                pv[i, j] = c; c += 1
    return {"aE": E, "aW": W, "aN": N, "aS": S, "WlLh": WL, "vofS": vs, "nyS": ny_s, "nxS": nx_s,
            "posnu_p": pp, "posnu_u": pu, "posnu_v": pv, "moex_u": mu, "moex_v": mv,
            "vofS_u": vsu, "vofS_v": vsv}


# ---------------------------------------------------------------------------
# Momentum predictor: implicit solve of one velocity component
# ---------------------------------------------------------------------------
def mom_operator(mi) -> dict:
    """SetMatrix + SetVectors on the inputs of synth.momentum_inputs:
    matr (nx,ny,5: S,W,P,E,N), rhm, Dp (assembled cells), CWE, CSN."""
    L = lib()
    nx, ny, iu, iv = mi["nx"], mi["ny"], mi["iu"], mi["iv"]
    cst = np.array([mi["dt"], mi["beta_vis"], mi["nua"], mi["nuw"], mi["nuref"], mi["rey"]])
    matr = np.zeros((nx, ny, 5), order="F")
    Dp = mi["Dp"].copy(order="F")
    cwe = np.zeros((ny, 2), order="F")
    csn = np.zeros((nx, 2), order="F")
    rc = L.oracle_mom_matrix(nx, ny, iu, iv, _p(mi["dx"]), _p(mi["dy"]), _p(mi["posnu"]),
                             _p(mi["vof"]), _p(mi["vofS"]), _p(mi["etaE"]), _p(mi["etaN"]),
                             _p(mi["WlLh"]), _p(mi["delh"]), _p(mi["difEW"]), _p(mi["difNS"]),
                             _p(mi["edEW"]), _p(mi["edNS"]), _p(cst), _p(Dp), _p(cwe),
                             _p(csn), _p(matr))
    rhm = np.zeros((nx, ny), order="F")
    L.oracle_mom_vectors(nx, ny, iu, iv, _p(mi["posnu"]), _p(mi["dx"]), _p(mi["dy"]),
                         _p(mi["flux"]), _p(cwe), _p(csn), _p(mi["u"]), _p(mi["v"]),
                         mi["fr"], _p(rhm))
    return {"matr": matr, "rhm": rhm, "Dp": Dp, "cwe": cwe, "csn": csn, "bad": rc != 0}


def mom_csr(mi, matr):
    """The system of the numbered cells (Posnu order) as a CSR matrix."""
    import scipy.sparse as sp
    nx, ny = mi["nx"], mi["ny"]
    pn = mi["posnu"][1:nx + 1, 1:ny + 1]
    act = pn != -1
    n = int(act.sum())
    rows, cols, vals = [], [], []
    idx = np.argwhere(act)
    r = pn[act]
    I, J = idx[:, 0], idx[:, 1]
    for f, (di, dj) in enumerate([(0, -1), (-1, 0), (0, 0), (1, 0), (0, 1)]):
        ii, jj = I + di, J + dj
        ok = (ii >= 0) & (ii < nx) & (jj >= 0) & (jj < ny)
        c = np.full(len(I), -1)
        c[ok] = pn[ii[ok], jj[ok]]
        ok &= c != -1
        rows.append(r[ok]); cols.append(c[ok]); vals.append(matr[I[ok], J[ok], f])
    A = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(n, n))
    return A, r, I, J


def mom_predict(mi, solver="direct", rtol=1e-14, maxit=500) -> dict:
    """The whole implicit step of one component: operator, right-hand side,
    solve (SuperLU, or the C BiCGStab), Pred and Dp with their boundary
    copies.  Returns pred, Dp, matr, rhm, x (by unknown), iterations."""
    L = lib()
    op = mom_operator(mi)
    nx, ny, iu, iv = mi["nx"], mi["ny"], mi["iu"], mi["iv"]
    A, r, I, J = mom_csr(mi, op["matr"])
    b = np.zeros(A.shape[0])
    b[r] = op["rhm"][I, J]
    its = 0
    if solver == "direct":
        x = solve_direct(A, b)
    else:
        xg = np.zeros((nx, ny), order="F")
        rel = C.c_double(0.0)
        its = L.oracle_mom_bicgstab(nx, ny, iu, iv, _p(mi["posnu"]), _p(op["matr"]),
                                    _p(op["rhm"]), rtol, maxit, _p(xg), C.byref(rel))
        x = np.zeros(A.shape[0])
        x[r] = xg[I, J]
    xv = np.ascontiguousarray(x, dtype=np.float64)
    pred = mi["pred"].copy(order="F")
    Dp = op["Dp"]
    L.oracle_mom_finish(nx, ny, iu, iv, _p(mi["posnu"]), _p(xv), _p(mi["gradp"]),
                        _p(mi["dx"]), _p(mi["dy"]), mi["dt"], _p(pred), _p(Dp))
    return {"pred": pred, "Dp": Dp, "matr": op["matr"], "rhm": op["rhm"], "x": x,
            "A": A, "b": b, "iters": its, "bad": op["bad"]}


# ---------------------------------------------------------------------------
# Tecplot result files (out_oracle.c; src/PrintResult.f90:39-168)
# ---------------------------------------------------------------------------
PCELL_FIELDS = ["x", "y", "p", "u", "v", "phi", "vof", "phiS", "vofS", "mres", "flux", "nxS",
                "nyS"]
VCELL_FIELDS = ["x", "y", "vel", "phi", "vof", "phiS", "vofS"]


def f24_14(values) -> bytes:
    """F24.14 text of every value, 24 bytes each, no line ends."""
    v = np.ascontiguousarray(values, dtype=np.float64).ravel()
    out = C.create_string_buffer(24 * v.size + 1)
    lib().oracle_format_many(v.ctypes.data_as(_P), v.size, out)
    return out.raw[:24 * v.size]


def tecplot_size(nvar, nx, ny) -> int:
    return 200 + nvar * nx * ny * 25


def tecplot_pcell(nx, ny, f) -> bytes:
    """The text of Print_Result_Tecplot_PCent's file (without particles)."""
    buf = C.create_string_buffer(tecplot_size(15, nx, ny))
    n = lib().oracle_tecplot_pcell(nx, ny, *[_p(f[k]) for k in PCELL_FIELDS], buf)
    return buf.raw[:n]


def tecplot_vcell(comp, nx, ny, f) -> bytes:
    """The text of Print_Result_Tecplot_UCent (comp 0) / _VCent (comp 1)."""
    buf = C.create_string_buffer(tecplot_size(8, nx, ny))
    n = lib().oracle_tecplot_vcell(comp, nx, ny, *[_p(f[k]) for k in VCELL_FIELDS], buf)
    return buf.raw[:n]


VTR_FIELDS = ["x", "y", "u", "v", "p", "phi", "phiS", "vof", "vofS"]


def e15_8(values) -> bytes:
    """The 15-character REAL(4) text of every value, no separators."""
    v = np.ascontiguousarray(values, dtype=np.float64).ravel()
    out = C.create_string_buffer(15 * v.size + 1)
    lib().oracle_format_e15_8(v.ctypes.data_as(_P), v.size, out)
    return out.raw[:15 * v.size]


def vtr_size(nx, ny) -> int:
    n = 10 * nx * ny + nx + ny + 1
    return 2000 + 16 * n + n // 5 + 10


def vtr(nx, ny, f) -> bytes:
    """The text of Print_Result_VTK_2D's FlowField_<iter>.vtr."""
    buf = C.create_string_buffer(vtr_size(nx, ny))
    n = lib().oracle_vtr(nx, ny, *[_p(f[k]) for k in VTR_FIELDS], buf)
    return buf.raw[:n]


LS_FIELDS = ["phi", "vofS", "dx", "dy", "x", "y", "aE", "aW", "aN", "aS", "ue", "ve"]


def ls_sweep(dir, nx, ny, f, dtv, temls):
    """X_Sweep (dir 0) / Y_Sweep (dir 1) level-set update of a copy of
    temls (Fortran-ordered (nx,ny)); returns the new array."""
    out = np.asfortranarray(np.array(temls, dtype=np.float64))
    lib().oracle_ls_sweep(dir, nx, ny, *[_p(f[k]) for k in LS_FIELDS], dtv, _p(out))
    return out


VOF_LS_FIELDS = ["vofS", "dx", "dy", "x", "y", "aE", "aW", "aN", "aS", "ue", "ve"]
VOF_FIELDS = ["vof", "nxv", "nyv", "dis", "nxs", "nys", "phiS"]


def vof_sweep(dir, nx, ny, f, v, dtv, temvf, wave=None):
    """X_Sweep (dir 0) / Y_Sweep (dir 1) VOF update of a copy of temvf
    (Fortran-ordered (nx,ny)) after Interface_Reconstruct; v holds vof,
    nxv, nyv, dis, nxs, nys, phiS; wave the X inlet's {Amp0, kw, omew,
    Depthw, NondiT, k} (None: no inlet flux).  Returns the new array."""
    out = np.asfortranarray(np.array(temvf, dtype=np.float64))
    w = None if wave is None else np.ascontiguousarray(wave, dtype=np.float64)
    lib().oracle_vof_sweep(dir, nx, ny, *[_p(f[k]) for k in VOF_LS_FIELDS],
                           *[_p(v[k]) for k in VOF_FIELDS], _p(w), dtv, _p(out))
    return out


def frac(nx, ny, diss, dx, dy) -> float:
    return lib().oracle_frac(nx, ny, diss, dx, dy)


def cellgeocal(nxs, nys, phis, nxl, nyl, phil, dx, dy):
    """(vols, volf) of CellGeoCal."""
    a, b = C.c_double(), C.c_double()
    lib().oracle_cellgeocal(nxs, nys, phis, nxl, nyl, phil, dx, dy, C.byref(a), C.byref(b))
    return a.value, b.value


IR_FIELDS = ["vof", "vofS", "phi", "nxs", "nys", "phiS", "x", "y", "dx", "dy"]


def interface_reconstruct(nx, ny, f):
    """Interface_Reconstruct (UpdateNorVec = 1) on the (nx,ny) fields of f
    (vof, vofS, phi, nxs, nys, phiS, x, y, dx, dy); returns
    ({"nxv", "nyv", "dis"}, events)."""
    out = {k: np.zeros((nx, ny), order="F") for k in ("nxv", "nyv", "dis")}
    ev = lib().oracle_interface_reconstruct(nx, ny, *[_p(f[k]) for k in IR_FIELDS],
                                            _p(out["nxv"]), _p(out["nyv"]), _p(out["dis"]))
    return out, ev


RD_FIELDS = ["vof", "vofS", "nxs", "nys", "phiS", "x", "y", "dx", "dy", "nxv", "nyv", "dis"]


def redistance(nx, ny, f, phi):
    """Redistance of a copy of phi (Fortran-ordered (nx,ny)) from the
    interface (nxv, nyv, dis) of Interface_Reconstruct; returns (phi,
    events)."""
    out = np.asfortranarray(np.array(phi, dtype=np.float64))
    aux = np.zeros((nx, ny), order="F")
    fix = np.zeros((nx, ny), dtype=np.int32, order="F")
    ev = lib().oracle_redistance(nx, ny, *[_p(f[k]) for k in RD_FIELDS], _p(out), _p(aux),
                                 fix.ctypes.data_as(_I))
    return out, ev


STEP_FIELDS = ["vofS", "nxs", "nys", "phiS", "dx", "dy", "x", "y", "aE", "aW", "aN", "aS", "ue",
               "ve"]


def clsvof_step(nx, ny, f, dt, vof, phi, wave=None):
    """Coupled_LS_VOF with a fixed solid on copies of vof and phi; wave the X
    inlet's {Amp0, kw, omew, Depthw, NondiT} or None.  Returns ({"vof",
    "phi", "nxv", "nyv", "dis"}, events)."""
    out = {"vof": np.asfortranarray(np.array(vof, dtype=np.float64)),
           "phi": np.asfortranarray(np.array(phi, dtype=np.float64))}
    for k in ("nxv", "nyv", "dis"):
        out[k] = np.zeros((nx, ny), order="F")
    work = np.zeros(6 * nx * ny)
    w = None if wave is None else np.ascontiguousarray(wave[:5], dtype=np.float64)
    ev = lib().oracle_clsvof_step(nx, ny, *[_p(f[k]) for k in STEP_FIELDS], _p(w), dt,
                                  _p(out["vof"]), _p(out["phi"]), _p(out["nxv"]), _p(out["nyv"]),
                                  _p(out["dis"]), _p(work))
    return out, ev


def plic_distance(v, dx, dy, nxx, nyy) -> float:
    return lib().oracle_plic_distance(v, dx, dy, nxx, nyy)


def dfc(nxss, nyss, phiss, nxf, nyf, volf, dx, dy, phif=0.0):
    """DistanceFluidCalculate: (phif or the given one when unassigned,
    assigned, events)."""
    p, e = C.c_double(phif), C.c_int(0)
    a = lib().oracle_dfc(nxss, nyss, phiss, nxf, nyf, volf, dx, dy, C.byref(p), C.byref(e))
    return p.value, bool(a), e.value


def grid_preprocess_literal(nx, ny, grids, fams, icorprob=True, aln_old=None):
    """Grid_Preprocess + NewCellFace for all three families (see
    cutcell_literal)."""
    import cutcell_literal
    return cutcell_literal.grid_preprocess(nx, ny, grids, fams, icorprob, aln_old)
