"""Python host API over the momentum-predictor solves of libscf_proj.so
(include/scf_mom.h).

MomentumSolver.solve(comp, ...) is the implicit step of Predictor_UV for one
velocity component (src/PredictorUV_mod.f90:507-563): SetMatrix, SetVectors,
the linear solve, DeltaGetValues, the pressure-gradient update, the Dp
boundary copies and (for v) the open top.  Arrays are the Fortran arrays of
the reference, Fortran ordered: (nx,ny) for (1:Isize,1:Jsize), (nx+2,ny+2)
for (0:Isize+1,0:Jsize+1), (nx+1,ny) for the east-west face fluxes
(1:Isize+1,1:Jsize) and (nx,ny+1) for the north-south ones.  numpy arrays
are host pointers; with device_ptrs=True every array is a contiguous CUDA
torch tensor with the same element count.  No CPU fallback.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import projection as P

# every symbol declared in include/scf_mom.h
EXPORTS = ["scf_mom_create", "scf_mom_destroy", "scf_mom_set_stream", "scf_mom_solve",
           "scf_mom_get_system"]

COMPONENTS = {"u": 0, "v": 1}

# (name in scf_mom_in, shape kind): 1 = (nx,ny), 0 = (nx+2,ny+2), e = (nx+1,ny), n = (nx,ny+1)
ARRAYS = [("dx", "1"), ("dy", "1"), ("posnu", "0"), ("vof", "1"), ("vofS", "1"),
          ("WlLh", "1"), ("delh", "1"), ("etaE", "0"), ("etaN", "0"), ("difEW", "e"),
          ("edEW", "e"), ("difNS", "n"), ("edNS", "n"), ("flux", "1"), ("gradp", "1"),
          ("u", "0"), ("v", "0")]
SCALARS = ["dt", "beta_vis", "nua", "nuw", "nuref", "rey", "fr"]


MOM_MG = 4  # scf_mom_create flag: multigrid preconditioner (include/scf_mom.h)


class MomIn(C.Structure):
    _fields_ = ([(n, C.c_void_p) for n, _ in ARRAYS] + [(n, C.c_double) for n in SCALARS])


def load():
    L = P.load()
    if not getattr(L, "_mom_bound", False):
        vp = C.c_void_p
        L.scf_mom_create.argtypes = [C.POINTER(vp), C.c_int, C.c_int, C.c_int, C.c_int]
        L.scf_mom_create.restype = C.c_int
        L.scf_mom_destroy.argtypes = [vp]
        L.scf_mom_destroy.restype = None
        L.scf_mom_set_stream.argtypes = [vp, vp]
        L.scf_mom_set_stream.restype = C.c_int
        L.scf_mom_solve.argtypes = [vp, C.c_int, C.POINTER(MomIn), vp, vp, C.c_double, C.c_int,
                                    C.POINTER(P.Stats)]
        L.scf_mom_solve.restype = C.c_int
        L.scf_mom_get_system.argtypes = [vp, vp, vp]
        L.scf_mom_get_system.restype = C.c_int
        L._mom_bound = True
    return L


class MomentumSolver:
    """Implicit momentum solves on an nx-by-ny grid (a handle of the C-ABI)."""

    def __init__(self, nx: int, ny: int, device_ptrs: bool = False, device: int = 0,
                 mg: bool = False):
        """mg: precondition the BiCGStab solves with a multigrid V-cycle
        (SCF_MOM_MG) instead of the diagonal."""
        self.nx, self.ny, self.device_ptrs = nx, ny, device_ptrs
        self._h = C.c_void_p()
        flags = (P.FLAG_DEVICE_PTRS if device_ptrs else 0) | (MOM_MG if mg else 0)
        P._check(load().scf_mom_create(C.byref(self._h), nx, ny, flags, device),
                 "scf_mom_create")
        self._keep = []

    def close(self):
        if self._h:
            load().scf_mom_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream: int):
        P._check(load().scf_mom_set_stream(self._h, C.c_void_p(stream)), "scf_mom_set_stream")

    def _shape(self, kind):
        nx, ny = self.nx, self.ny
        return {"1": (nx, ny), "0": (nx + 2, ny + 2), "e": (nx + 1, ny), "n": (nx, ny + 1)}[kind]

    def _ptr(self, a, shape, dtype, name, writable=False):
        if self.device_ptrs:
            import torch
            if not (isinstance(a, torch.Tensor) and a.is_cuda and a.is_contiguous()):
                raise TypeError(f"{name}: device_ptrs=True needs a contiguous CUDA tensor")
            tdt = {np.float64: torch.float64, np.int32: torch.int32}[dtype]
            if a.dtype != tdt or a.numel() != int(np.prod(shape)):
                raise ValueError(f"{name}: expected {np.prod(shape)} {tdt}")
            return a.data_ptr()
        if (not isinstance(a, np.ndarray) or a.shape != tuple(shape) or a.dtype != dtype
                or not a.flags["F_CONTIGUOUS"]):
            raise ValueError(f"{name}: expected a Fortran-ordered {dtype.__name__}{tuple(shape)}")
        if writable and not a.flags["WRITEABLE"]:
            raise ValueError(f"{name}: array is read-only")
        return a.ctypes.data

    def solve(self, comp: str, inputs: dict, pred, Dp, rtol: float = 1e-13, maxit: int = 200):
        """The implicit step of component comp ('u' or 'v'); pred and Dp are
        updated in place.  inputs: the fields of scf_mom_in by name (as made
        by synth.momentum_inputs).  Returns the solve statistics."""
        mi = MomIn()
        for name, kind in ARRAYS:
            dt = np.int32 if name == "posnu" else np.float64
            setattr(mi, name, self._ptr(inputs[name], self._shape(kind), dt, name))
        for name in SCALARS:
            setattr(mi, name, float(inputs[name]))
        st = P.Stats()
        rc = load().scf_mom_solve(self._h, COMPONENTS[comp], C.byref(mi),
                                  self._ptr(pred, self._shape("0"), np.float64, "pred", True),
                                  self._ptr(Dp, self._shape("0"), np.float64, "Dp", True),
                                  rtol, maxit, C.byref(st))
        if rc not in (P.SCF_OK, P.SCF_ERR_NOT_CONVERGED):
            raise P.ProjectionError(rc, "scf_mom_solve")
        return st

    def system(self):
        """(matr (nx,ny,5): S, W, P, E, N; rhm (nx,ny)) of the last solve."""
        matr = np.zeros((self.nx, self.ny, 5), order="F")
        rhm = np.zeros((self.nx, self.ny), order="F")
        P._check(load().scf_mom_get_system(self._h, matr.ctypes.data, rhm.ctypes.data),
                 "scf_mom_get_system")
        return matr, rhm


def predict(inputs: dict, rtol: float = 1e-13, maxit: int = 200, mg: bool = False) -> dict:
    """One component's implicit step on host arrays (a fresh handle)."""
    s = MomentumSolver(inputs["nx"], inputs["ny"], mg=mg)
    try:
        pred = inputs["pred"].copy(order="F")
        Dp = inputs["Dp"].copy(order="F")
        st = s.solve(inputs["comp"], inputs, pred, Dp, rtol=rtol, maxit=maxit)
        matr, rhm = s.system()
    finally:
        s.close()
    return {"pred": pred, "Dp": Dp, "matr": matr, "rhm": rhm, "stats": st.as_dict()}
