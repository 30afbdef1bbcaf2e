"""Python host API over the CLSVOF sweeps of libscf_proj.so
(include/scf_clsvof.h): X_Sweep / Y_Sweep after Interface_Reconstruct
(src/Clsvof_Mod.f90:989-1124, 1126-1245) on the GPU -- the level-set part
alone (sweep) or the VOF part with, optionally, the level-set part in the
same kernel (clsvof_sweep); and Interface_Reconstruct (src/Clsvof_Mod.f90:
1250-1321), which each sweep calls first (interface_reconstruct), and
Redistance (src/Clsvof_Mod.f90:1525-1708, redistance); and the whole
Coupled_LS_VOF step with a fixed solid (src/Clsvof_Mod.f90:730-973,
clsvof_step).

Fields are the reference's Fortran arrays (Fortran-ordered numpy float64):
(nx,ny) phi, vofS, dx, dy, x, y; (nx+2,ny+2) aE, aW, aN, aS; ue (nx+1,ny)
for ue(0:nx,1:ny); ve (nx,ny+1) for ve(1:nx,0:ny); with device_ptrs=True,
contiguous CUDA float64 tensors with those element counts.  No CPU fallback.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import projection as P

EXPORTS = ["scf_ls_sweep", "scf_clsvof_sweep", "scf_interface_reconstruct", "scf_redistance",
           "scf_clsvof_step"]
X, Y = 0, 1
DEVICE_PTRS = 1
FIELDS = [("phi", "1"), ("vofS", "1"), ("dx", "1"), ("dy", "1"), ("x", "1"), ("y", "1"),
          ("aE", "0"), ("aW", "0"), ("aN", "0"), ("aS", "0"), ("ue", "u"), ("ve", "v")]


VOF_FIELDS = ["vof", "nxv", "nyv", "dis", "nxs", "nys", "phiS"]


class LsFields(C.Structure):
    _fields_ = [(n, C.c_void_p) for n, _ in FIELDS]


class VofFields(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in VOF_FIELDS]


IR_FIELDS = ["vof", "vofS", "phi", "nxs", "nys", "phiS", "x", "y", "dx", "dy"]


class IrFields(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in IR_FIELDS]


RD_FIELDS = ["vof", "vofS", "nxs", "nys", "phiS", "x", "y", "dx", "dy", "nxv", "nyv", "dis"]


class RdFields(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in RD_FIELDS]


STEP_FIELDS = [("vofS", "1"), ("nxs", "1"), ("nys", "1"), ("phiS", "1"), ("x", "1"), ("y", "1"),
               ("dx", "1"), ("dy", "1"), ("aE", "0"), ("aW", "0"), ("aN", "0"), ("aS", "0"),
               ("ue", "u"), ("ve", "v")]


class StepFields(C.Structure):
    _fields_ = [(n, C.c_void_p) for n, _ in STEP_FIELDS]


class VofWave(C.Structure):
    _fields_ = [("amp0", C.c_double), ("kw", C.c_double), ("omew", C.c_double),
                ("depthw", C.c_double), ("nondit", C.c_double), ("k", C.c_int)]


def load():
    L = P.load()
    if not getattr(L, "_ls_bound", False):
        L.scf_ls_sweep.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_double, C.c_void_p,
                                   C.c_int, C.c_int, C.POINTER(C.c_double)]
        L.scf_ls_sweep.restype = C.c_int
        L.scf_clsvof_sweep.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.c_int,
                                       C.c_int, C.POINTER(C.c_double)]
        L.scf_clsvof_sweep.restype = C.c_int
        L.scf_interface_reconstruct.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                                C.c_void_p, C.c_void_p, C.POINTER(C.c_int),
                                                C.c_int, C.c_int, C.POINTER(C.c_double)]
        L.scf_interface_reconstruct.restype = C.c_int
        L.scf_redistance.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                     C.POINTER(C.c_int), C.c_int, C.c_int,
                                     C.POINTER(C.c_double)]
        L.scf_redistance.restype = C.c_int
        L.scf_clsvof_step.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_double,
                                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.POINTER(C.c_int), C.c_int, C.c_int,
                                      C.POINTER(C.c_double)]
        L.scf_clsvof_step.restype = C.c_int
        L._ls_bound = True
    return L


def _pack(nx, ny, f, device_ptrs, fields=FIELDS, cls=LsFields, optional=()):
    st, keep = cls(), []
    for name, sk in fields:
        a = f.get(name)
        if a is None and name in optional:
            continue
        shape = {"1": (nx, ny), "0": (nx + 2, ny + 2), "u": (nx + 1, ny), "v": (nx, ny + 1)}[sk]
        if device_ptrs:
            import torch
            if not (isinstance(a, torch.Tensor) and a.is_cuda and a.is_contiguous()
                    and a.dtype == torch.float64 and a.numel() == int(np.prod(shape))):
                raise ValueError(f"{name}: expected a contiguous CUDA float64 tensor of "
                                 f"{int(np.prod(shape))} elements")
            ptr = a.data_ptr()
        else:
            if (not isinstance(a, np.ndarray) or a.shape != shape or a.dtype != np.float64
                    or not a.flags["F_CONTIGUOUS"]):
                raise ValueError(f"{name}: expected a Fortran-ordered float64{shape}")
            ptr = a.ctypes.data
        keep.append(a)
        setattr(st, name, ptr)
    return st, keep


def sweep(dir: int, nx: int, ny: int, fields: dict, dtv: float, temls, device_ptrs: bool = False,
          device: int = 0) -> float:
    """Apply one sweep's level-set update to temls in place (a Fortran-ordered
    (nx,ny) float64 array, or a CUDA tensor with device_ptrs); returns the
    call's elapsed milliseconds."""
    st, keep = _pack(nx, ny, fields, device_ptrs)
    if device_ptrs:
        ptr = temls.data_ptr()
    else:
        if (not isinstance(temls, np.ndarray) or temls.shape != (nx, ny)
                or temls.dtype != np.float64 or not temls.flags["F_CONTIGUOUS"]):
            raise ValueError("temls: expected a Fortran-ordered float64 (nx,ny)")
        ptr = temls.ctypes.data
    ms = C.c_double(0.0)
    P._check(load().scf_ls_sweep(dir, nx, ny, C.byref(st), float(dtv), ptr,
                                 DEVICE_PTRS if device_ptrs else 0, device, C.byref(ms)),
             "scf_ls_sweep")
    return ms.value


def _target(a, nx, ny, device_ptrs, name):
    if device_ptrs:
        import torch
        if not (isinstance(a, torch.Tensor) and a.is_cuda and a.is_contiguous()
                and a.dtype == torch.float64 and a.numel() == nx * ny):
            raise ValueError(f"{name}: expected a contiguous CUDA float64 tensor of {nx * ny} "
                             "elements")
        return a.data_ptr()
    if (not isinstance(a, np.ndarray) or a.shape != (nx, ny) or a.dtype != np.float64
            or not a.flags["F_CONTIGUOUS"]):
        raise ValueError(f"{name}: expected a Fortran-ordered float64 (nx,ny)")
    return a.ctypes.data


def clsvof_sweep(dir: int, nx: int, ny: int, fields: dict, vof: dict, dtv: float, temvf,
                 temls=None, wave=None, device_ptrs: bool = False, device: int = 0) -> float:
    """One whole X_Sweep (dir X) or Y_Sweep (dir Y) after Interface_Reconstruct:
    the VOF update of temvf and, when temls is given, the level-set update
    of temls, in place.  fields as for sweep() (phi only needed with temls);
    vof holds (nx,ny) vof, nxv, nyv, dis (Interface_Reconstruct's normal and
    distance), nxs, nys, phiS; wave the X inlet's (Amp0, kw, omew, Depthw,
    NondiT, k) or None (no inflow through face 0 of X).  Returns the call's
    elapsed milliseconds."""
    st, keep = _pack(nx, ny, fields, device_ptrs, optional=("phi",) if temls is None else ())
    vs, keep2 = _pack(nx, ny, vof, device_ptrs, [(n, "1") for n in VOF_FIELDS], VofFields)
    pv = _target(temvf, nx, ny, device_ptrs, "temvf")
    pl = None if temls is None else _target(temls, nx, ny, device_ptrs, "temls")
    w = None
    if wave is not None:
        a, k, o, d, t, kk = wave
        w = VofWave(float(a), float(k), float(o), float(d), float(t), int(kk))
    ms = C.c_double(0.0)
    P._check(load().scf_clsvof_sweep(dir, nx, ny, C.byref(st), C.byref(vs),
                                     None if w is None else C.byref(w), float(dtv), pv, pl,
                                     DEVICE_PTRS if device_ptrs else 0, device, C.byref(ms)),
             "scf_clsvof_sweep")
    return ms.value


def interface_reconstruct(nx: int, ny: int, fields: dict, out: dict | None = None,
                          device_ptrs: bool = False, device: int = 0):
    """Interface_Reconstruct (UpdateNorVec = 1) on the GPU: fields holds the
    (nx,ny) arrays vof, vofS, phi, nxs, nys, phiS, x, y, dx, dy.  Returns
    ({"nxv", "nyv", "dis"}, events, elapsed ms); out, when given, supplies
    the three output arrays (required with device_ptrs)."""
    st, keep = _pack(nx, ny, fields, device_ptrs, [(n, "1") for n in IR_FIELDS], IrFields)
    if out is None:
        if device_ptrs:
            raise ValueError("out: the three output tensors are required with device_ptrs")
        out = {k: np.zeros((nx, ny), order="F") for k in ("nxv", "nyv", "dis")}
    ptrs = [_target(out[k], nx, ny, device_ptrs, k) for k in ("nxv", "nyv", "dis")]
    ev, ms = C.c_int(0), C.c_double(0.0)
    P._check(load().scf_interface_reconstruct(nx, ny, C.byref(st), *ptrs, C.byref(ev),
                                              DEVICE_PTRS if device_ptrs else 0, device,
                                              C.byref(ms)),
             "scf_interface_reconstruct")
    return out, ev.value, ms.value


def redistance(nx: int, ny: int, fields: dict, phi, device_ptrs: bool = False,
               device: int = 0):
    """Redistance on the GPU: phi (in place) rebuilt from the interface
    (nxv, nyv, dis) of interface_reconstruct; fields holds the (nx,ny)
    arrays vof, vofS, nxs, nys, phiS, x, y, dx, dy, nxv, nyv, dis.  Returns
    (events, elapsed ms)."""
    st, keep = _pack(nx, ny, fields, device_ptrs, [(n, "1") for n in RD_FIELDS], RdFields)
    ptr = _target(phi, nx, ny, device_ptrs, "phi")
    ev, ms = C.c_int(0), C.c_double(0.0)
    P._check(load().scf_redistance(nx, ny, C.byref(st), ptr, C.byref(ev),
                                   DEVICE_PTRS if device_ptrs else 0, device, C.byref(ms)),
             "scf_redistance")
    return ev.value, ms.value


def clsvof_step(nx: int, ny: int, fields: dict, dt: float, vof, phi, wave=None,
                out: dict | None = None, device_ptrs: bool = False, device: int = 0):
    """One Coupled_LS_VOF step (six sub-steps of dt/6) with the solid held
    fixed, on the GPU: vof and phi in place.  fields holds vofS, nxs, nys,
    phiS, x, y, dx, dy ((nx,ny)), aE, aW, aN, aS ((nx+2,ny+2)), ue
    ((nx+1,ny)), ve ((nx,ny+1)); wave the X inlet's (Amp0, kw, omew, Depthw,
    NondiT) or None.  Returns ({"nxv", "nyv", "dis"} of the last
    reconstruction, events, elapsed ms); out supplies those three arrays
    (required with device_ptrs)."""
    st, keep = _pack(nx, ny, fields, device_ptrs, STEP_FIELDS, StepFields)
    if out is None:
        if device_ptrs:
            raise ValueError("out: the three output tensors are required with device_ptrs")
        out = {k: np.zeros((nx, ny), order="F") for k in ("nxv", "nyv", "dis")}
    pv, pp = _target(vof, nx, ny, device_ptrs, "vof"), _target(phi, nx, ny, device_ptrs, "phi")
    ptrs = [_target(out[k], nx, ny, device_ptrs, k) for k in ("nxv", "nyv", "dis")]
    w = None
    if wave is not None:
        w = VofWave(float(wave[0]), float(wave[1]), float(wave[2]), float(wave[3]),
                    float(wave[4]), 0)
    ev, ms = C.c_int(0), C.c_double(0.0)
    P._check(load().scf_clsvof_step(nx, ny, C.byref(st), None if w is None else C.byref(w),
                                    float(dt), pv, pp, *ptrs, C.byref(ev),
                                    DEVICE_PTRS if device_ptrs else 0, device, C.byref(ms)),
             "scf_clsvof_step")
    return out, ev.value, ms.value
