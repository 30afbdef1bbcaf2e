"""ctypes binding of libscf_gen.so (gen/scf_geom.h): builds the cut-cell
geometry of a synthetic projection case in the reference's Fortran layouts.

Restates, for synthetic solids and free surfaces, Initial_Grid/InitialUVGrid
(src/Mesh_Mod.f90:54-175), Initial_Clsvof (src/Clsvof_Mod.f90:39-400) and
Grid_Preprocess (src/Cutcell_Mod.f90:18-397).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

_LIB = Path(__file__).resolve().parent / "_lib" / "libscf_gen.so"
_lib = None

SOLID_CIRCLE = 0
SOLID_BOX = 1
MAXMODES = 8


class _Solid(C.Structure):
    _fields_ = [("kind", C.c_int), ("cx", C.c_double), ("cy", C.c_double), ("r", C.c_double),
                ("hw", C.c_double), ("hh", C.c_double), ("angle", C.c_double)]


class _Surface(C.Structure):
    _fields_ = [("y0", C.c_double), ("nmodes", C.c_int), ("amp", C.c_double * MAXMODES),
                ("k", C.c_double * MAXMODES), ("phase", C.c_double * MAXMODES)]


_P = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int32)


class _Out(C.Structure):
    _fields_ = [(n, _P) for n in ("x", "y", "dx", "dy", "dxU", "dyV", "vof", "phi", "vofS",
                                  "phiS", "nxS", "nyS", "WlLh", "aE", "aW", "aN", "aS")] + \
               [(n, _I) for n in ("posnu_p", "posnu_u", "posnu_v", "moex_u", "moex_v")] + \
               [(n, _P) for n in ("vofS_u", "vofS_v", "vofS_in", "nxS_in", "nyS_in",
                                  "vofS_u_in", "vofS_v_in")]


def use_library(path) -> None:
    """Load the generator from another build of geometry.cpp (the CPU arm of
    the benchmark uses the oracle's copy); call before the first case."""
    global _LIB, _lib
    if _lib is not None and Path(path) != _LIB:
        raise RuntimeError("the generator library is already loaded")
    _LIB = Path(path)


def _load():
    global _lib
    if _lib is None:
        if not _LIB.exists():
            from . import build
            build.build()
        lib = C.CDLL(str(_LIB))
        lib.scf_geom_axis.restype = C.c_int
        lib.scf_geom_axis.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int, C.c_double,
                                      C.c_double, C.c_int, _P]
        lib.scf_geom_build.restype = C.c_int
        lib.scf_geom_build.argtypes = [C.c_int, C.c_int, _P, _P, C.c_int, C.POINTER(_Solid),
                                       C.POINTER(_Surface), C.c_int, C.POINTER(_Out)]
        _lib = lib
    return _lib


@dataclass
class Solid:
    kind: int
    cx: float
    cy: float
    r: float = 0.0
    hw: float = 0.0
    hh: float = 0.0
    angle: float = 0.0


@dataclass
class Surface:
    y0: float
    amp: list = field(default_factory=list)
    k: list = field(default_factory=list)
    phase: list = field(default_factory=list)


def axis(npts: int, s0: float, s1: float, nonuniform: bool = False, r0: float = 0.0,
         r1: float = 0.0, nrec: int = 0) -> np.ndarray:
    """Face coordinates of one axis (Initial_Grid, src/Mesh_Mod.f90:54-137)."""
    out = np.zeros(npts, dtype=np.float64)
    rc = _load().scf_geom_axis(npts, s0, s1, int(nonuniform), r0, r1, nrec,
                               out.ctypes.data_as(_P))
    if rc != 0:
        raise ValueError("scf_geom_axis: bad arguments")
    return out


def _ptr(a):
    return a.ctypes.data_as(_P if a.dtype == np.float64 else _I)


def build(xf: np.ndarray, yf: np.ndarray, solids: list[Solid], surface: Surface,
          icorprob: bool = True) -> dict:
    """Geometry of an nx-by-ny grid with face coordinates xf (nx+1), yf (ny+1).

    Returns a dict of Fortran-ordered arrays with the reference's bounds:
    (nx, ny) arrays for (1:nx,1:ny) and (nx+2, ny+2) for (0:nx+1,0:ny+1).
    """
    xf = np.ascontiguousarray(xf, dtype=np.float64)
    yf = np.ascontiguousarray(yf, dtype=np.float64)
    nx, ny = len(xf) - 1, len(yf) - 1
    f1 = lambda dt=np.float64: np.zeros((nx, ny), dtype=dt, order="F")
    f0 = lambda dt=np.float64: np.zeros((nx + 2, ny + 2), dtype=dt, order="F")
    g = {k: f1() for k in ("x", "y", "dx", "dy", "dxU", "dyV", "vof", "phi", "vofS", "phiS",
                           "nxS", "nyS", "WlLh", "vofS_u", "vofS_v", "vofS_in", "nxS_in",
                           "nyS_in", "vofS_u_in", "vofS_v_in")}
    g.update({k: f0() for k in ("aE", "aW", "aN", "aS")})
    g.update({k: f0(np.int32) for k in ("posnu_p", "posnu_u", "posnu_v")})
    g.update({k: f1(np.int32) for k in ("moex_u", "moex_v")})
    out = _Out(**{k: _ptr(v) for k, v in g.items()})
    arr = (_Solid * max(1, len(solids)))()
    for n, s in enumerate(solids):
        arr[n] = _Solid(s.kind, s.cx, s.cy, s.r, s.hw, s.hh, s.angle)
    if len(surface.amp) > MAXMODES:
        raise ValueError("at most %d surface modes" % MAXMODES)
    surf = _Surface()
    surf.y0 = surface.y0
    surf.nmodes = len(surface.amp)
    for m in range(len(surface.amp)):
        surf.amp[m] = surface.amp[m]
        surf.k[m] = surface.k[m]
        surf.phase[m] = surface.phase[m]
    n = _load().scf_geom_build(nx, ny, xf.ctypes.data_as(_P), yf.ctypes.data_as(_P),
                               len(solids), arr, C.byref(surf), int(icorprob), C.byref(out))
    if n < 0:
        raise ValueError("scf_geom_build: bad arguments")
    g["n_unknowns"] = int(n)
    g["xf"], g["yf"] = xf, yf
    return g
