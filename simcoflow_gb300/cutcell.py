"""Python host API over scf_grid_preprocess (include/scf_cutcell.h): the
per-step cut-cell geometry of the P, U and V cells (Grid_Preprocess and
NewCellFace, src/Cutcell_Mod.f90:18-725) on the GPU.

grids[f] = {dx, dy, x, y} and fams[f] = {vofS, phiS, nxS, nyS} for f in
'p', 'u', 'v': Fortran-ordered (nx,ny) float64 arrays.  Returns per family a
dict of numpy arrays in the reference's layouts (Fortran order):
(nx,ny), (nx+2,ny+2), (nx,ny,2) for cent / msce, (nx+2,ny+2,2) for FCE / FCN.
`state` (optional, per U/V family) gives the in/out arrays' entry values
(msce and the interpolation coefficients, AlN's supplying AlE(0,j)); zeros
otherwise.  No CPU fallback.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import projection as P

EXPORTS = ["scf_grid_preprocess"]
FAMILIES = ("p", "u", "v")
GRID = ["dx", "dy", "x", "y"]
SOLID = ["vofS", "phiS", "nxS", "nyS"]
# (name, shape kind, dtype): "1" (nx,ny), "0" (nx+2,ny+2), "c" (nx,ny,2), "f" (nx+2,ny+2,2)
GEOM = [("vofS", "1", "d"), ("nxS", "1", "d"), ("nyS", "1", "d"), ("aE", "0", "d"),
        ("aW", "0", "d"), ("aN", "0", "d"), ("aS", "0", "d"), ("FCE", "f", "d"),
        ("FCN", "f", "d"), ("cent", "c", "d"), ("WlLh", "1", "d"), ("delh", "1", "d"),
        ("posnu", "0", "i"), ("moex", "1", "i"), ("msce", "c", "i"), ("SxE", "0", "d"),
        ("EtaE", "0", "d"), ("AlE", "0", "d"), ("DAlE", "0", "d"), ("SyN", "0", "d"),
        ("EtaN", "0", "d"), ("AlN", "0", "d"), ("DAlN", "0", "d")]
UV_ONLY = {"delh", "moex", "msce", "SxE", "EtaE", "AlE", "DAlE", "SyN", "EtaN", "AlN", "DAlN"}
INOUT = {"msce", "SxE", "EtaE", "AlE", "DAlE", "SyN", "EtaN", "AlN", "DAlN"}


class CellGrid(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in GRID]


class CellSolid(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in SOLID]


class CellGeom(C.Structure):
    _fields_ = [(n, C.c_void_p) for n, _, _ in GEOM]


def load():
    L = P.load()
    if not getattr(L, "_cutcell_bound", False):
        L.scf_grid_preprocess.argtypes = [C.c_int, C.c_int, C.POINTER(CellGrid),
                                          C.POINTER(CellSolid), C.POINTER(CellGeom), C.c_int,
                                          C.c_int, C.c_int, C.POINTER(C.c_double)]
        L.scf_grid_preprocess.restype = C.c_int
        L._cutcell_bound = True
    return L


def _shape(kind, nx, ny):
    return {"1": (nx, ny), "0": (nx + 2, ny + 2), "c": (nx, ny, 2), "f": (nx + 2, ny + 2, 2)}[kind]


def _arr(a, shape, name, dev):
    if dev:
        import torch
        if not (isinstance(a, torch.Tensor) and a.is_cuda and a.is_contiguous()
                and a.dtype == torch.float64 and a.numel() == int(np.prod(shape))):
            raise ValueError(f"{name}: expected a contiguous CUDA float64 tensor of "
                             f"{int(np.prod(shape))} elements")
        return a, a.data_ptr()
    a = np.asarray(a)
    if a.shape != shape or a.dtype != np.float64 or not a.flags["F_CONTIGUOUS"]:
        raise ValueError(f"{name}: expected a Fortran-ordered float64{shape}")
    return a, a.ctypes.data


def grid_preprocess(grids: dict, fams: dict, icorprob: bool = True, state: dict | None = None,
                    device: int = 0, nx: int | None = None, ny: int | None = None):
    """Grid_Preprocess + NewCellFace on the GPU; returns ({f: outputs}, ms).
    With CUDA torch tensors as inputs (flat, Fortran element order; give nx
    and ny) everything stays on the device and the outputs are CUDA tensors
    with the same element counts as the Fortran arrays."""
    import importlib
    dev = not isinstance(grids["p"]["dx"], np.ndarray)
    if not dev:
        nx, ny = grids["p"]["dx"].shape
    elif nx is None or ny is None:
        raise ValueError("device inputs need nx and ny")
    torch = importlib.import_module("torch") if dev else None
    G = (CellGrid * 3)()
    S = (CellSolid * 3)()
    O = (CellGeom * 3)()
    keep, out = [], {}
    for k, f in enumerate(FAMILIES):
        for n in GRID:
            a, ptr = _arr(grids[f][n], (nx, ny), f"{f}.{n}", dev)
            keep.append(a)
            setattr(G[k], n, ptr)
        for n in SOLID:
            a, ptr = _arr(fams[f][n], (nx, ny), f"{f}.{n}", dev)
            keep.append(a)
            setattr(S[k], n, ptr)
        out[f] = {}
        for n, kind, dt in GEOM:
            if f == "p" and n in UV_ONLY:
                continue
            shape = _shape(kind, nx, ny)
            if dev:
                a = torch.zeros(int(np.prod(shape)),
                                dtype=torch.float64 if dt == "d" else torch.int32,
                                device=grids["p"]["dx"].device)
                if state and f in state and n in INOUT and n in state[f]:
                    a.copy_(state[f][n])
                ptr = a.data_ptr()
            else:
                a = np.zeros(shape, dtype=np.float64 if dt == "d" else np.int32, order="F")
                if state and f in state and n in INOUT and n in state[f]:
                    a[...] = state[f][n]
                ptr = a.ctypes.data
            out[f][n] = a
            setattr(O[k], n, ptr)
    ms = C.c_double(0.0)
    P._check(load().scf_grid_preprocess(nx, ny, G, S, O, 1 if icorprob else 0, 1 if dev else 0,
                                        device, C.byref(ms)), "scf_grid_preprocess")
    return out, ms.value
