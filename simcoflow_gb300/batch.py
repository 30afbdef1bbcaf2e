"""Batched uneven projections in one graph launch, with an autotuned V-cycle
schedule per grid-size class (the many-instance path of the library).

    bp = BatchProjector(cases, precision="mixed")   # uploads, assembles, tunes
    stats, ms = bp.run()                            # ONE cudaGraphLaunch
    bp.result(i)                                    # Pp, u, v, p, mres of instance i

Every instance is a handle of the C-ABI in device-pointer mode; the batch
graph (scf_batch_* in include/scf_proj.h) holds one independent branch per
instance: operator setup, right-hand side, the PCG loop as a conditional
WHILE node, the correction.  The autotuner times each candidate schedule
(pre/post sweeps, coarse-correction scale) with each sweep tile shape on one
representative instance of every size class and keeps the fastest time to
the tolerance.
"""
from __future__ import annotations

import ctypes as C
import json
import math
import time

import numpy as np

from . import projection as P

# candidate schedules: (npre, npost, omega)
# candidates of the batch autotuner (one representative instance per size
# class), and of a single large projection, which also tries omega 1.97
BATCH_SCHEDULES = [(1, 1, 1.9), (2, 2, 1.9), (2, 2, 1.95), (2, 1, 1.9), (3, 3, 1.9), (1, 2, 1.9)]
SCHEDULES = BATCH_SCHEDULES + [(2, 2, 1.97)]
# sweep tiles of the point smoother (scf_proj_set_tile): 64 x 32 cells per
# CTA (TMA-staged on the larger FP32 levels) and 32 x 32 (plain loads)
TILES = {"64x32": 0, "32x32": 1}
# coarse-level schedules (scf_proj_set_coarse_sweeps): (first level, sweeps)
# on the latency-bound coarse levels, or None for npre / npost everywhere
COARSE = [None, (1, 4), (2, 4)]


def size_class(nx: int, ny: int) -> int:
    """log2 bucket of the cell count (256^2 -> 16, 512^2 -> 18, ...)."""
    return int(round(math.log2(max(1, nx * ny))))


def _device_arrays(case, dev):
    import torch
    return {k: torch.from_numpy(np.ascontiguousarray(v.ravel(order="F"))).to(dev)
            for k, v in case.arrays.items() if isinstance(v, np.ndarray)}


class _Instance:
    def __init__(self, case, precision, rtol, maxit, dev):
        import torch
        self.case = case
        self.t = _device_arrays(case, dev)
        t = self.t
        self.s = P.ProjectionSolver(case.nx, case.ny, precision=precision, device_ptrs=True,
                                    rtol=rtol, maxit=maxit, device=dev.index or 0)
        self.s.set_grid(t["dx"], t["dy"], t["dxU"], t["dyV"])
        self.s.set_geometry(**{k: t[k] for k in P.GEOMETRY_ARGS})
        self.s.assemble(t["DpU"], t["DpV"], case.betaP, case.betaM, case.bc)
        n0, n1 = (case.nx + 2) * (case.ny + 2), case.nx * case.ny
        self.Pp = torch.zeros(n0, dtype=torch.float64, device=dev)
        self.mres = torch.zeros(n1, dtype=torch.float64, device=dev)
        self.reset()

    def reset(self):
        """Velocity and pressure back to the case's old time level."""
        if not hasattr(self, "u"):
            self.u, self.v, self.p = (self.t[k].clone() for k in ("u0", "v0", "p0"))
        else:
            for k, a in (("u0", self.u), ("v0", self.v), ("p0", self.p)):
                a.copy_(self.t[k])

    def solve_once(self):
        """One projection through the single-instance entry point (tuning)."""
        self.reset()
        return self.s.update_puv(self.t["ustar"], self.t["vstar"], self.u, self.v, self.p,
                                 self.case.vb, Pp=self.Pp, mres=self.mres)[2]

    def close(self):
        self.s.close()


def autotune(insts, schedules=BATCH_SCHEDULES, tiles=TILES, coarse=COARSE, reps=3, log=None):
    """Fastest schedule, sweep tile and coarse-level schedule per size
    class: {class: (npre, npost, omega, tile name, coarse)}.  Every schedule
    is timed with every tile and coarse schedule on one representative
    instance of the class."""
    import torch
    table = {}
    reps_by_class = {}
    for inst in insts:
        reps_by_class.setdefault(size_class(inst.case.nx, inst.case.ny), inst)
    for cls, inst in sorted(reps_by_class.items()):
        best = None
        for tname, tile in tiles.items():
            inst.s.set_tile(tile)
            for co in coarse:
                inst.s.set_coarse_sweeps(*(co or (0, 0)))
                for sch in schedules:
                    inst.s.set_schedule(*sch)
                    inst.solve_once()  # warm (graph build)
                    torch.cuda.synchronize()
                    t0 = time.perf_counter()
                    for _ in range(reps):
                        st = inst.solve_once()
                    torch.cuda.synchronize()
                    ms = (time.perf_counter() - t0) / reps * 1e3
                    if st.status == 0 and (best is None or ms < best[0]):
                        best = (ms, (*sch, tname, co), st.iters)
        table[cls] = best[1]
        if log:
            log(f"autotune class 2^{cls}: {best[1]} {best[0]:.2f} ms, {best[2]} iterations")
    return table


class BatchProjector:
    def __init__(self, cases, precision="mixed", rtol=1e-8, maxit=200, device=0, tune=True,
                 table=None, log=None):
        import torch
        self.dev = torch.device("cuda", device)
        self.insts = [_Instance(c, precision, rtol, maxit, self.dev) for c in cases]
        self.table = dict(table or {})
        if tune:
            self.table.update(autotune(self.insts, log=log))
        for inst in self.insts:
            sch = self.table.get(size_class(inst.case.nx, inst.case.ny))
            if sch is not None:
                inst.s.set_schedule(*sch[:3])
                inst.s.set_tile(TILES[sch[3]] if len(sch) > 3 else 0)
                inst.s.set_coarse_sweeps(*((sch[4] if len(sch) > 4 else None) or (0, 0)))
        L = P.load()
        handles = (C.c_void_p * len(self.insts))(*[i.s._h.value for i in self.insts])
        b = C.c_void_p()
        P._check(L.scf_batch_create(C.byref(b), handles, len(self.insts)), "scf_batch_create")
        self._b = b
        for k, inst in enumerate(self.insts):
            t = inst.t
            P._check(L.scf_batch_set_io(b, k, t["ustar"].data_ptr(), t["vstar"].data_ptr(),
                                        inst.case.vb, inst.Pp.data_ptr(), inst.p.data_ptr(),
                                        inst.u.data_ptr(), inst.v.data_ptr(),
                                        inst.mres.data_ptr()), "scf_batch_set_io")
        self.stream = torch.cuda.Stream(self.dev)

    def run(self, reset=True):
        """Solve every instance (one graph launch); returns (stats list, ms)."""
        if reset:
            for inst in self.insts:
                inst.reset()
        import torch
        torch.cuda.synchronize(self.dev)
        st = (P.Stats * len(self.insts))()
        rc = P.load().scf_batch_run(self._b, C.c_void_p(self.stream.cuda_stream), st)
        P._check(rc, "scf_batch_run")
        out = [st[i].as_dict() for i in range(len(self.insts))]
        return out, out[0]["ms_total"]

    def result(self, i):
        """Host copies of instance i: Pp, u, v, p ((nx+2,ny+2) Fortran) and mres."""
        inst = self.insts[i]
        c = inst.case
        f0 = lambda a: a.cpu().numpy().reshape((c.nx + 2, c.ny + 2), order="F")
        return {"Pp": f0(inst.Pp), "u": f0(inst.u), "v": f0(inst.v), "p": f0(inst.p),
                "mres": inst.mres.cpu().numpy().reshape((c.nx, c.ny), order="F")}

    def close(self):
        if getattr(self, "_b", None):
            P.load().scf_batch_destroy(self._b)
            self._b = None
        for inst in self.insts:
            inst.close()
        self.insts = []

    def table_json(self) -> str:
        return json.dumps({str(k): v for k, v in self.table.items()})
