"""Python host API over libscf_proj.so (include/scf_proj.h).

Mirrors the reference's projection entry points:

  ProjectionSolver.poisson_equation_solver  PoissonEquationSolver
                                            (src/ProjectionP_Mod.f90:26-99)
  ProjectionSolver.update_puv               projection part of UpdatePUV
                                            (src/ComputePUV_Mod.f90:56-218)

Arguments are the arrays the Fortran code holds, in the same layouts
((nx,ny) for (1:Isize,1:Jsize), (nx+2,ny+2) for (0:Isize+1,0:Jsize+1),
Fortran order).  numpy arrays are passed as host pointers; with
device_ptrs=True every array must be a CUDA torch tensor (Fortran-ordered
data, i.e. a tensor whose storage is the transpose (ny, nx) in C order, or
any 1-D tensor with the right element count) and stays on the GPU.

There is no CPU fallback: if libscf_proj.so cannot be loaded or a CUDA call
fails, an exception is raised.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from pathlib import Path

import numpy as np

_LIB = Path(__file__).resolve().parent / "_lib" / "libscf_proj.so"
_lib = None

SCF_OK = 0
SCF_ERR_NOT_CONVERGED = -4
ERRORS = {-1: "SCF_ERR_ARG", -2: "SCF_ERR_CUDA", -3: "SCF_ERR_NAN", -4: "SCF_ERR_NOT_CONVERGED",
          -5: "SCF_ERR_STALL", -6: "SCF_ERR_TIMEOUT", -7: "SCF_ERR_STATE", -8: "SCF_ERR_NOMEM",
          -9: "SCF_ERR_IO"}
PREC = {"fp64": 0, "mixed": 1}
FLAG_DEVICE_PTRS = 1
FLAG_NO_GRAPH = 2

# every symbol declared in include/scf_proj.h
EXPORTS = ["scf_opts_default", "scf_proj_create", "scf_proj_destroy", "scf_proj_set_stream",
           "scf_proj_set_grid", "scf_proj_set_geometry", "scf_proj_assemble",
           "scf_proj_poisson_solve", "scf_proj_update_puv", "scf_proj_get_operator",
           "scf_proj_vcycle", "scf_proj_time_kernel", "scf_rhs_norm_noalloc", "scf_strerror",
           "scf_proj_set_network", "scf_proj_solve_rhs", "scf_proj_set_opts",
           "scf_batch_create", "scf_batch_set_io", "scf_batch_run", "scf_batch_destroy",
           "scf_proj_set_solid", "scf_proj_get_geometry", "scf_diag_divide", "scf_diag_sqrt",
           "scf_proj_get_matrix", "scf_diag_tma_timeout", "scf_proj_set_tile",
           "scf_proj_set_coarse_sweeps"]
# every symbol declared in include/scf_unet.h
UNET_EXPORTS = ["scf_unet_num_params", "scf_unet_create", "scf_unet_destroy",
                "scf_unet_set_stream", "scf_unet_set_params", "scf_unet_get_params",
                "scf_unet_features", "scf_unet_target", "scf_unet_set_input", "scf_unet_forward",
                "scf_unet_loss", "scf_unet_set_dz", "scf_unet_backward", "scf_unet_get_grads",
                "scf_unet_adam", "scf_unet_set_engine", "scf_unet_conv"]


class Opts(C.Structure):
    _fields_ = [("precision", C.c_int), ("flags", C.c_int), ("device", C.c_int),
                ("maxit", C.c_int), ("rtol", C.c_double), ("npre", C.c_int),
                ("npost", C.c_int), ("omega", C.c_double), ("coarse_max", C.c_int),
                ("smoother", C.c_int), ("precond", C.c_int), ("coarse_sweeps", C.c_int),
                ("coarse_from", C.c_int), ("reserved", C.c_int * 4)]


class Stats(C.Structure):
    _fields_ = [("iters", C.c_int), ("status", C.c_int), ("levels", C.c_int),
                ("fallbacks", C.c_int), ("bnorm", C.c_double), ("relres", C.c_double),
                ("relres_true", C.c_double), ("mres_max", C.c_double), ("ms_h2d", C.c_double),
                ("ms_assemble", C.c_double), ("ms_solve", C.c_double),
                ("ms_correct", C.c_double), ("ms_d2h", C.c_double), ("ms_total", C.c_double),
                ("smoother", C.c_int), ("learned_iters", C.c_int), ("launches", C.c_int),
                ("asym_faces", C.c_int)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class ProjectionError(RuntimeError):
    def __init__(self, code: int, where: str):
        self.code = code
        msg = load().scf_strerror(code).decode() if _lib is not None else ERRORS.get(code, "?")
        super().__init__(f"{where}: {ERRORS.get(code, code)} ({msg})")


def load():
    """Load libscf_proj.so (built by simcoflow_gb300.build); raises if absent."""
    global _lib
    if _lib is None:
        if not _LIB.exists():
            raise ImportError(f"{_LIB} is missing: run simcoflow_gb300.build.build_all() "
                              "(there is no CPU fallback)")
        L = C.CDLL(str(_LIB))
        vp, dp, ip = C.c_void_p, C.c_void_p, C.c_void_p
        L.scf_opts_default.argtypes = [C.POINTER(Opts)]
        L.scf_opts_default.restype = None
        L.scf_strerror.argtypes = [C.c_int]
        L.scf_strerror.restype = C.c_char_p
        L.scf_proj_create.argtypes = [C.POINTER(vp), C.c_int, C.c_int, C.POINTER(Opts)]
        L.scf_proj_destroy.argtypes = [vp]
        L.scf_proj_set_stream.argtypes = [vp, vp]
        L.scf_proj_set_grid.argtypes = [vp, dp, dp, dp, dp]
        L.scf_proj_set_geometry.argtypes = [vp] + [dp] * 9 + [ip, ip, ip, dp, ip, ip, dp]
        L.scf_proj_assemble.argtypes = [vp, dp, dp, C.c_double, C.c_double, C.c_int, C.c_int,
                                        C.c_int, C.c_int]
        L.scf_proj_poisson_solve.argtypes = [vp, dp, dp, C.c_double, dp, C.POINTER(Stats)]
        L.scf_proj_update_puv.argtypes = [vp, dp, dp, C.c_double, dp, dp, dp, dp, dp,
                                          C.POINTER(Stats)]
        L.scf_proj_get_operator.argtypes = [vp, dp, dp, dp, dp]
        L.scf_proj_get_matrix.argtypes = [vp, dp, C.POINTER(C.c_int), C.POINTER(C.c_double)]
        L.scf_proj_vcycle.argtypes = [vp, dp, dp]
        L.scf_proj_time_kernel.argtypes = [vp, C.c_int, C.c_int, C.POINTER(C.c_double)]
        L.scf_rhs_norm_noalloc.argtypes = [C.c_int, C.c_int] + [dp] * 10 + [ip, C.c_double, dp,
                                                                            dp, vp]
        L.scf_rhs_norm_noalloc.restype = C.c_int
        L.scf_proj_set_network.argtypes = [vp, vp, C.c_int]
        L.scf_proj_solve_rhs.argtypes = [vp, dp, dp, dp, C.c_int, C.POINTER(Stats)]
        L.scf_proj_set_opts.argtypes = [vp, C.c_int, C.c_int, C.c_double]
        L.scf_proj_set_tile.argtypes = [vp, C.c_int]
        L.scf_proj_set_coarse_sweeps.argtypes = [vp, C.c_int, C.c_int]
        L.scf_batch_create.argtypes = [C.POINTER(vp), C.POINTER(vp), C.c_int]
        L.scf_batch_set_io.argtypes = [vp, C.c_int, dp, dp, C.c_double, dp, dp, dp, dp, dp]
        L.scf_batch_run.argtypes = [vp, vp, C.POINTER(Stats)]
        L.scf_batch_destroy.argtypes = [vp]
        L.scf_proj_set_solid.argtypes = [vp] + [dp] * 8 + [C.c_int]
        L.scf_proj_get_geometry.argtypes = [vp] + [dp] * 8 + [ip] * 5 + [dp, dp]
        L.scf_diag_divide.argtypes = [dp, dp, dp, C.c_int64, C.c_int]
        L.scf_diag_divide.restype = C.c_int
        L.scf_diag_sqrt.argtypes = [dp, dp, C.c_int64, C.c_int]
        L.scf_diag_sqrt.restype = C.c_int
        L.scf_diag_tma_timeout.argtypes = [C.c_int, C.c_int, C.c_int]
        L.scf_diag_tma_timeout.restype = C.c_int
        for name in EXPORTS:
            f = getattr(L, name)
            if f.restype is C.c_int or name.startswith("scf_proj"):
                f.restype = C.c_int
        _lib = L
    return _lib


def _check(rc: int, where: str):
    if rc != SCF_OK:
        raise ProjectionError(rc, where)


# multigrid smoother (scf_opts.smoother / scf_stats.smoother)
SMOOTHERS = {"auto": 0, "point": 1, "line": 2}
# preconditioner (scf_opts.precond)
PRECONDS = {"mg": 0, "learned": 1}

GEOMETRY_ARGS = ("vof", "phi", "vofS", "nyS", "WlLh", "aE", "aW", "aN", "aS", "posnu_p",
                 "posnu_u", "moex_u", "vofS_u", "posnu_v", "moex_v", "vofS_v")


class ProjectionSolver:
    """One projection solver for an nx-by-ny grid (a handle of the C-ABI)."""

    def __init__(self, nx: int, ny: int, precision: str = "fp64", device: int = 0,
                 device_ptrs: bool = False, use_graph: bool = True, maxit: int = 200,
                 rtol: float = 1e-8, npre: int = 2, npost: int = 2, omega: float = 1.9,
                 coarse_max: int = 64, smoother: str = "auto", precond: str = "mg",
                 coarse_sweeps: int = 0, coarse_from: int = 0):
        L = load()
        o = Opts()
        L.scf_opts_default(C.byref(o))
        o.precision = PREC[precision]
        o.flags = (FLAG_DEVICE_PTRS if device_ptrs else 0) | (0 if use_graph else FLAG_NO_GRAPH)
        o.device, o.maxit, o.rtol = device, maxit, rtol
        o.npre, o.npost, o.omega, o.coarse_max = npre, npost, omega, coarse_max
        o.smoother = SMOOTHERS[smoother]
        o.precond = PRECONDS[precond]
        o.coarse_sweeps, o.coarse_from = coarse_sweeps, coarse_from
        self.nx, self.ny, self.device_ptrs = nx, ny, device_ptrs
        self.opts = o
        h = C.c_void_p()
        _check(L.scf_proj_create(C.byref(h), nx, ny, C.byref(o)), "scf_proj_create")
        self._h = h
        self._keep = {}

    def close(self):
        if getattr(self, "_h", None):
            load().scf_proj_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- pointers ---------------------------------------------------------
    def _ptr(self, a, shape, dtype, name, writable=False):
        if a is None:
            return None
        if self.device_ptrs:
            import torch
            if not (isinstance(a, torch.Tensor) and a.is_cuda):
                raise TypeError(f"{name}: device_ptrs=True needs a CUDA tensor")
            if a.numel() != int(np.prod(shape)):
                raise ValueError(f"{name}: expected {np.prod(shape)} elements, got {a.numel()}")
            tdt = {np.float64: torch.float64, np.int32: torch.int32}[dtype]
            if a.dtype != tdt or not a.is_contiguous():
                raise TypeError(f"{name}: needs a contiguous {tdt} tensor")
            return a.data_ptr()
        if not isinstance(a, np.ndarray):
            raise TypeError(f"{name}: expected a numpy array")
        if a.shape != tuple(shape) or a.dtype != dtype or not a.flags["F_CONTIGUOUS"]:
            raise ValueError(f"{name}: expected Fortran-ordered {dtype.__name__}{tuple(shape)}, "
                             f"got {a.dtype}{a.shape}")
        if writable and not a.flags["WRITEABLE"]:
            raise ValueError(f"{name}: array is read-only")
        return a.ctypes.data

    def _n1(self):
        return (self.nx, self.ny)

    def _n0(self):
        return (self.nx + 2, self.ny + 2)

    # -- API --------------------------------------------------------------
    def set_stream(self, stream_ptr: int):
        _check(load().scf_proj_set_stream(self._h, C.c_void_p(stream_ptr)), "scf_proj_set_stream")

    def set_grid(self, dx, dy, dxU, dyV):
        f = lambda a, n: self._ptr(a, self._n1(), np.float64, n)
        self._keep["grid"] = (dx, dy, dxU, dyV)
        _check(load().scf_proj_set_grid(self._h, f(dx, "dx"), f(dy, "dy"), f(dxU, "dxU"),
                                        f(dyV, "dyV")), "scf_proj_set_grid")

    def set_geometry(self, **g):
        shapes = {"aE": 0, "aW": 0, "aN": 0, "aS": 0, "posnu_p": 0, "posnu_u": 0, "posnu_v": 0}
        ptrs = []
        for k in GEOMETRY_ARGS:
            dt = np.int32 if k.startswith(("posnu", "moex")) else np.float64
            shp = self._n0() if k in shapes else self._n1()
            ptrs.append(self._ptr(g[k], shp, dt, k))
        self._keep["geom"] = [g[k] for k in GEOMETRY_ARGS]
        _check(load().scf_proj_set_geometry(self._h, *ptrs), "scf_proj_set_geometry")

    def set_solid(self, vof, phi, vofS, phiS, nxS, nyS, vofS_u, vofS_v, icorprob=True):
        """The cut-cell geometry computed on the GPU from the cells' solid
        level-set fields (Grid_Preprocess), in place of set_geometry."""
        args = (vof, phi, vofS, phiS, nxS, nyS, vofS_u, vofS_v)
        names = ("vof", "phi", "vofS", "phiS", "nxS", "nyS", "vofS_u", "vofS_v")
        ptrs = [self._ptr(a, self._n1(), np.float64, n) for a, n in zip(args, names)]
        self._keep["geom"] = list(args)
        _check(load().scf_proj_set_solid(self._h, *ptrs, int(bool(icorprob))),
               "scf_proj_set_solid")

    def get_geometry(self) -> dict:
        """The geometry the handle holds, as host arrays (set_geometry's
        keys plus nxS after set_solid)."""
        n1, n0 = self._n1(), self._n0()
        out = {k: np.zeros(n1, order="F") for k in ("vofS", "nxS", "nyS", "WlLh", "vofS_u",
                                                       "vofS_v")}
        out.update({k: np.zeros(n0, order="F") for k in ("aE", "aW", "aN", "aS")})
        out.update({k: np.zeros(n0, dtype=np.int32, order="F")
                    for k in ("posnu_p", "posnu_u", "posnu_v")})
        out.update({k: np.zeros(n1, dtype=np.int32, order="F") for k in ("moex_u", "moex_v")})
        order = ("vofS", "nxS", "nyS", "WlLh", "aE", "aW", "aN", "aS", "posnu_p", "posnu_u",
                 "posnu_v", "moex_u", "moex_v", "vofS_u", "vofS_v")
        rc = load().scf_proj_get_geometry(self._h, *[out[k].ctypes.data for k in order])
        if rc == -7:  # nxS only exists for GPU-built geometry
            del out["nxS"]
            order = tuple(k for k in order if k != "nxS")
            rc = load().scf_proj_get_geometry(self._h, *[out[k].ctypes.data if k in out else None
                                                         for k in ("vofS", "nxS", "nyS", "WlLh",
                                                                   "aE", "aW", "aN", "aS",
                                                                   "posnu_p", "posnu_u",
                                                                   "posnu_v", "moex_u", "moex_v",
                                                                   "vofS_u", "vofS_v")])
        _check(rc, "scf_proj_get_geometry")
        return out

    def assemble(self, DpU, DpV, betaP: float, betaM: float, bc=(1, 1, 1, 0)):
        f = lambda a, n: self._ptr(a, self._n0(), np.float64, n)
        self._keep["dp"] = (DpU, DpV)
        _check(load().scf_proj_assemble(self._h, f(DpU, "DpU"), f(DpV, "DpV"), betaP, betaM,
                                        *bc), "scf_proj_assemble")

    def poisson_equation_solver(self, ustar, vstar, vb: float = 0.0, Pp=None,
                                check: bool = True):
        """PoissonEquationSolver: returns (Pp, stats)."""
        if Pp is None:
            Pp = np.zeros(self._n0(), order="F")
        st = Stats()
        rc = load().scf_proj_poisson_solve(
            self._h, self._ptr(ustar, self._n0(), np.float64, "ustar"),
            self._ptr(vstar, self._n0(), np.float64, "vstar"), vb,
            self._ptr(Pp, self._n0(), np.float64, "Pp", True), C.byref(st))
        if check:
            _check(rc, "scf_proj_poisson_solve")
        return Pp, st

    def update_puv(self, ustar, vstar, u, v, p, vb: float = 0.0, Pp=None, mres=None,
                   check: bool = True):
        """Projection part of UpdatePUV: corrects u, v, p in place and returns
        (Pp, mres, stats)."""
        if Pp is None and not self.device_ptrs:
            Pp = np.zeros(self._n0(), order="F")
        if mres is None:
            mres = np.zeros(self._n1(), order="F")
        st = Stats()
        rc = load().scf_proj_update_puv(
            self._h, self._ptr(ustar, self._n0(), np.float64, "ustar"),
            self._ptr(vstar, self._n0(), np.float64, "vstar"), vb,
            self._ptr(Pp, self._n0(), np.float64, "Pp", True),
            self._ptr(p, self._n0(), np.float64, "p", True),
            self._ptr(u, self._n0(), np.float64, "u", True),
            self._ptr(v, self._n0(), np.float64, "v", True),
            self._ptr(mres, self._n1(), np.float64, "mres", True), C.byref(st))
        if check:
            _check(rc, "scf_proj_update_puv")
        return Pp, mres, st

    def get_operator(self):
        n1 = self._n1()
        out = [np.zeros(n1, order="F") for _ in range(4)]
        _check(load().scf_proj_get_operator(self._h, *[a.ctypes.data for a in out]),
               "scf_proj_get_operator")
        return dict(zip(("cE", "cN", "diag", "rhs"), out))

    def get_matrix(self):
        """The assembled rows as the reference's matr(Isize,Jsize,5) (S, W,
        diagonal, E, N; Fortran order), the number of faces whose two rows
        carry different entries and their largest relative difference."""
        m = np.zeros((self.nx, self.ny, 5), order="F")
        na, mx = C.c_int(0), C.c_double(0.0)
        _check(load().scf_proj_get_matrix(self._h, m.ctypes.data, C.byref(na), C.byref(mx)),
               "scf_proj_get_matrix")
        return m, na.value, mx.value

    def set_schedule(self, npre: int, npost: int, omega: float):
        """V-cycle schedule of this handle (rebuilds its graph)."""
        _check(load().scf_proj_set_opts(self._h, npre, npost, omega), "scf_proj_set_opts")
        self.opts.npre, self.opts.npost, self.opts.omega = npre, npost, omega

    def set_coarse_sweeps(self, coarse_from: int, sweeps: int):
        """Sweeps before / after the coarse correction on level coarse_from
        (0: the finest) and every coarser one, counted as npre / npost count
        them; 0 for npre / npost there too (rebuilds the handle's graph)."""
        _check(load().scf_proj_set_coarse_sweeps(self._h, int(coarse_from), int(sweeps)),
               "scf_proj_set_coarse_sweeps")
        self.opts.coarse_from, self.opts.coarse_sweeps = int(coarse_from), int(sweeps)

    def set_tile(self, tile: int):
        """Sweep tile of the point smoother: 0 = 64x32 (TMA-staged on large
        FP32 levels), 1 = 32x32 (plain loads); rebuilds the handle's graph."""
        _check(load().scf_proj_set_tile(self._h, int(tile)), "scf_proj_set_tile")
        self.tile = int(tile)

    def set_network(self, params):
        """Weights of the learned preconditioner (float32 array of
        scf_unet_num_params() values, order of include/scf_unet.h)."""
        p = np.ascontiguousarray(params, dtype=np.float32)
        _check(load().scf_proj_set_network(self._h, p.ctypes.data, p.size), "scf_proj_set_network")

    def solve_rhs(self, b, x=None, r=None, maxit=None, check=True):
        """A x = b for an (nx,ny) right-hand side; returns (x, r, stats).  With
        device_ptrs, b/x/r are CUDA float64 tensors of nx*ny elements (x and r
        allocated when not given); else Fortran-ordered numpy arrays."""
        maxit = self.opts.maxit if maxit is None else maxit
        if self.device_ptrs:
            import torch
            if x is None:
                x = torch.zeros(self.nx * self.ny, dtype=torch.float64, device=b.device)
            if r is None:
                r = torch.zeros(self.nx * self.ny, dtype=torch.float64, device=b.device)
        else:
            b = np.asfortranarray(b, dtype=np.float64)
            x = np.zeros(self._n1(), order="F") if x is None else x
            r = np.zeros(self._n1(), order="F") if r is None else r
        st = Stats()
        f = lambda a, n, w=False: self._ptr(a, self._n1(), np.float64, n, w)
        rc = load().scf_proj_solve_rhs(self._h, f(b, "b"), f(x, "x", True), f(r, "r", True),
                                       maxit, C.byref(st))
        if check and rc != SCF_ERR_NOT_CONVERGED:
            _check(rc, "scf_proj_solve_rhs")
        return x, r, st

    def vcycle(self, b):
        x = np.zeros(self._n1(), order="F")
        b = np.asfortranarray(b, dtype=np.float64)
        _check(load().scf_proj_vcycle(self._h, b.ctypes.data, x.ctypes.data), "scf_proj_vcycle")
        return x

    # -- convenience --------------------------------------------------------
    def setup_case(self, case):
        """set_grid + set_geometry + assemble from a synth.Case (host arrays)."""
        a = case.arrays
        self.set_grid(a["dx"], a["dy"], a["dxU"], a["dyV"])
        self.set_geometry(**{k: a[k] for k in GEOMETRY_ARGS})
        self.assemble(a["DpU"], a["DpV"], case.betaP, case.betaM, case.bc)


TMA_SPINS_DEFAULT = 1 << 20


def inject_tma_timeout(cta: int, spins: int, device: int = 0):
    """Test-only fault injection (scf_diag_tma_timeout): CTA `cta` of the
    TMA-staged sweeps arms its barrier without issuing copies and waits at
    most `spins` polls; cta=-1 with the default spins turns it off."""
    _check(load().scf_diag_tma_timeout(device, cta, spins), "scf_diag_tma_timeout")


def divide(a, b, device: int = 0):
    """a / b elementwise by the library's FP64 division (the one its
    bit-exact kernels use), on the GPU; numpy float64 arrays in and out."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    if a.shape != b.shape:
        raise ValueError("a and b need the same shape")
    q = np.empty_like(a)
    _check(load().scf_diag_divide(a.ctypes.data, b.ctypes.data, q.ctypes.data, a.size, device),
           "scf_diag_divide")
    return q


def sqrt(a, device: int = 0):
    """sqrt(a) elementwise by the library's FP64 square root (the one its
    CLSVOF kernels use), on the GPU; numpy float64 arrays in and out."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    q = np.empty_like(a)
    _check(load().scf_diag_sqrt(a.ctypes.data, q.ctypes.data, a.size, device), "scf_diag_sqrt")
    return q


def project_case(case, tile=None, **opts):
    """Full projection of a synth.Case through the C-ABI with host arrays:
    returns dict(Pp, u, v, p, mres, stats).  tile: sweep tile of the point
    smoother (None: the default)."""
    s = ProjectionSolver(case.nx, case.ny, **opts)
    try:
        if tile is not None:
            s.set_tile(tile)
        s.setup_case(case)
        a = case.arrays
        u, v, p = a["u0"].copy(order="F"), a["v0"].copy(order="F"), a["p0"].copy(order="F")
        Pp, mres, st = s.update_puv(a["ustar"], a["vstar"], u, v, p, case.vb)
        m, na, mx = s.get_matrix()
        return {"Pp": Pp, "u": u, "v": v, "p": p, "mres": mres, "stats": st.as_dict(),
                "operator": s.get_operator(), "matr": m, "asym_faces": na, "asym_max": mx}
    finally:
        s.close()
