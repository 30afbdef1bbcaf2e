"""Python host API over the result-file writers of libscf_proj.so
(include/scf_out.h): Print_Result_Tecplot_PCent / _UCent / _VCent
(src/PrintResult.f90:39-168) and Print_Result_VTK_2D's ParaView file
(:165-190, src/VTR_mod.f90:79-379), with the text formatted on the GPU.

Fields are the reference's Fortran arrays (Fortran-ordered numpy float64):
(nx,ny) for (1:Isize,1:Jsize), (nx+2,ny+2) for (0:Isize+1,0:Jsize+1) and
(nx+2,ny+2,2) for Flux_n1; with device_ptrs=True, contiguous CUDA torch
tensors with the same element counts.  No CPU fallback.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import projection as P

EXPORTS = ["scf_tecplot_size", "scf_tecplot_text", "scf_tecplot_write", "scf_tecplot_format",
           "scf_format_f24_14", "scf_vtr_size", "scf_vtr_text", "scf_vtr_write",
           "scf_format_e15_8"]

PCELL, UCELL, VCELL = 0, 1, 2
DEVICE_PTRS = 1
# (field, shape kind): "1" = (nx,ny), "0" = (nx+2,ny+2), "f" = (nx+2,ny+2,2)
PCELL_FIELDS = [("x", "1"), ("y", "1"), ("p", "0"), ("u", "0"), ("v", "0"), ("phi", "1"),
                ("vof", "1"), ("phiS", "1"), ("vofS", "1"), ("mres", "1"), ("flux", "f"),
                ("nxS", "1"), ("nyS", "1")]
VCELL_FIELDS = [("x", "1"), ("y", "1"), ("vel", "0"), ("phi", "1"), ("vof", "1"),
                ("phiS", "1"), ("vofS", "1")]
VTR_FIELDS = [("x", "1"), ("y", "1"), ("u", "0"), ("v", "0"), ("p", "0"), ("phi", "1"),
              ("phiS", "1"), ("vof", "1"), ("vofS", "1")]


class PCellFields(C.Structure):
    _fields_ = [(n, C.c_void_p) for n, _ in PCELL_FIELDS]


class VCellFields(C.Structure):
    _fields_ = [(n, C.c_void_p) for n, _ in VCELL_FIELDS]


class VtrFields(C.Structure):
    _fields_ = [(n, C.c_void_p) for n, _ in VTR_FIELDS]


def load():
    L = P.load()
    if not getattr(L, "_out_bound", False):
        vp = C.c_void_p
        L.scf_tecplot_size.argtypes = [C.c_int, C.c_int, C.c_int]
        L.scf_tecplot_size.restype = C.c_int64
        L.scf_tecplot_text.argtypes = [C.c_int, C.c_int, C.c_int, vp, C.c_int, vp, C.c_int64,
                                       C.POINTER(C.c_int64), C.c_int]
        L.scf_tecplot_text.restype = C.c_int
        L.scf_tecplot_write.argtypes = [C.c_int, C.c_int, C.c_int, vp, C.c_int, C.c_int64,
                                        C.c_char_p, C.c_int, C.POINTER(C.c_double)]
        L.scf_tecplot_write.restype = C.c_int
        L.scf_tecplot_format.argtypes = [C.c_int, C.c_int, C.c_int, vp, vp, vp]
        L.scf_tecplot_format.restype = C.c_int
        L.scf_format_f24_14.argtypes = [vp, C.c_int64, vp, C.c_int]
        L.scf_format_f24_14.restype = C.c_int
        L.scf_vtr_size.argtypes = [C.c_int, C.c_int]
        L.scf_vtr_size.restype = C.c_int64
        L.scf_vtr_text.argtypes = [C.c_int, C.c_int, vp, C.c_int, vp, C.c_int64,
                                   C.POINTER(C.c_int64), C.c_int]
        L.scf_vtr_text.restype = C.c_int
        L.scf_vtr_write.argtypes = [C.c_int, C.c_int, vp, C.c_int, C.c_int64, C.c_char_p,
                                    C.c_int, C.POINTER(C.c_double)]
        L.scf_vtr_write.restype = C.c_int
        L.scf_format_e15_8.argtypes = [vp, C.c_int64, vp, C.c_int]
        L.scf_format_e15_8.restype = C.c_int
        L._out_bound = True
    return L


def _fields(kind, nx, ny, fields, device_ptrs):
    if kind == PCELL:
        return _pack(PCELL_FIELDS, PCellFields, nx, ny, fields, device_ptrs)
    return _pack(VCELL_FIELDS, VCellFields, nx, ny, fields, device_ptrs)


def _pack(table, cls, nx, ny, fields, device_ptrs):
    st = cls()
    keep = []
    for name, sk in table:
        a = fields[name]
        shape = {"1": (nx, ny), "0": (nx + 2, ny + 2), "f": (nx + 2, ny + 2, 2)}[sk]
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


def _kind(kind):
    return {"p": PCELL, "u": UCELL, "v": VCELL}.get(kind, kind)


def text(kind, nx: int, ny: int, fields: dict, device_ptrs: bool = False,
         device: int = 0) -> bytes:
    """The whole file text of `kind` ('p', 'u' or 'v') as bytes."""
    k = _kind(kind)
    L = load()
    st, keep = _fields(k, nx, ny, fields, device_ptrs)
    size = L.scf_tecplot_size(k, nx, ny)
    if size < 0:
        raise ValueError("bad kind or size")
    buf = C.create_string_buffer(size)
    n = C.c_int64(0)
    P._check(L.scf_tecplot_text(k, nx, ny, C.byref(st), DEVICE_PTRS if device_ptrs else 0,
                                buf, size, C.byref(n), device), "scf_tecplot_text")
    return buf.raw[:n.value]


def write(kind, nx: int, ny: int, fields: dict, iter: int, dir: str,
          device_ptrs: bool = False, device: int = 0) -> float:
    """Write dir/Tecplot/<Pressure|Uvelocity|Vvelocity>_<iter>.dat; returns
    the elapsed milliseconds."""
    k = _kind(kind)
    L = load()
    st, keep = _fields(k, nx, ny, fields, device_ptrs)
    ms = C.c_double(0.0)
    P._check(L.scf_tecplot_write(k, nx, ny, C.byref(st), DEVICE_PTRS if device_ptrs else 0,
                                 int(iter), dir.encode(), device, C.byref(ms)),
             "scf_tecplot_write")
    return ms.value


def nvars(kind) -> int:
    return 15 if _kind(kind) == PCELL else 8


def format_device(kind, nx: int, ny: int, fields: dict, out, stream: int = 0) -> None:
    """The records of `kind` into the CUDA uint8 tensor `out`
    (nvars * nx * ny * 25 bytes), enqueued on `stream`; device fields."""
    import torch
    k = _kind(kind)
    if not (isinstance(out, torch.Tensor) and out.is_cuda and out.dtype == torch.uint8
            and out.numel() >= nvars(k) * nx * ny * 25):
        raise ValueError("out: a CUDA uint8 tensor of nvars*nx*ny*25 bytes")
    st, keep = _fields(k, nx, ny, fields, True)
    P._check(load().scf_tecplot_format(k, nx, ny, C.byref(st), out.data_ptr(),
                                       C.c_void_p(stream)), "scf_tecplot_format")


def f24_14(values, device: int = 0) -> bytes:
    """F24.14 text of every value (24 bytes each), formatted on the GPU."""
    v = np.ascontiguousarray(values, dtype=np.float64).ravel()
    out = C.create_string_buffer(24 * v.size + 1)
    P._check(load().scf_format_f24_14(v.ctypes.data, v.size, out, device), "scf_format_f24_14")
    return out.raw[:24 * v.size]


def vtr_text(nx: int, ny: int, fields: dict, device_ptrs: bool = False,
             device: int = 0) -> bytes:
    """The whole text of Print_Result_VTK_2D's FlowField_<iter>.vtr."""
    L = load()
    st, keep = _pack(VTR_FIELDS, VtrFields, nx, ny, fields, device_ptrs)
    size = L.scf_vtr_size(nx, ny)
    if size < 0:
        raise ValueError("bad size")
    buf = C.create_string_buffer(size)
    n = C.c_int64(0)
    P._check(L.scf_vtr_text(nx, ny, C.byref(st), DEVICE_PTRS if device_ptrs else 0, buf, size,
                            C.byref(n), device), "scf_vtr_text")
    return buf.raw[:n.value]


def vtr_write(nx: int, ny: int, fields: dict, iter: int, dir: str, device_ptrs: bool = False,
              device: int = 0) -> float:
    """Write dir/Paraview/FlowField_<iter>.vtr; returns the elapsed
    milliseconds."""
    L = load()
    st, keep = _pack(VTR_FIELDS, VtrFields, nx, ny, fields, device_ptrs)
    ms = C.c_double(0.0)
    P._check(L.scf_vtr_write(nx, ny, C.byref(st), DEVICE_PTRS if device_ptrs else 0, int(iter),
                             dir.encode(), device, C.byref(ms)), "scf_vtr_write")
    return ms.value


def e15_8(values, device: int = 0) -> bytes:
    """The 15-character REAL(4) text of every value, formatted on the GPU."""
    v = np.ascontiguousarray(values, dtype=np.float64).ravel()
    out = C.create_string_buffer(15 * v.size + 1)
    P._check(load().scf_format_e15_8(v.ctypes.data, v.size, out, device), "scf_format_e15_8")
    return out.raw[:15 * v.size]
