#!/usr/bin/env python
"""Benchmark: milliseconds per pressure projection solved to FP64 relative
residual 1e-8, on the 2048x2048 two-phase cut-cell workload (three seeded
circles, density ratio 1000:1.2), one GB300.

One step = one full projection of SIMCOFlow's UpdatePUV projection part:
operator assembly + multigrid setup, right-hand side, PCG solve to
||b - A x||_2 <= 1e-8 ||b||_2, velocity correction, mass residual.

  value  device-resident: every input already in HBM (device pointers
         through the C-ABI), CUDA events on the solver's stream
  e2e    the same projection through the C-ABI with pinned host buffers:
         host->device copies of all inputs and device->host copies of all
         outputs inside the timed region
  --impl reference  the CPU restatement of the reference path (the oracle,
         C + OpenMP on all host cores), same workload and metric

Prints one JSON line (rank 0).  Under torchrun each rank solves its own
seeded instance (replicas, no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "ms/projection to FP64 rel. residual 1e-8: learned+mixed FPCG vs plain MG-PCG"
UNIT = "ms/projection"
FALLBACK_HBM_GBS = 6800.0


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return float(d["hbm_gbs"]), "measured"
        except Exception:
            pass
    return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []  # (arrival time, csv line)
        self.window = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.monotonic()  # the timed region starts once samples flow
            while not self.lines and time.monotonic() - t0 < 5.0:
                time.sleep(0.01)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.monotonic(), line.strip()))

    def mark(self, start: float, end: float):
        """Host times bracketing the timed region (synchronised on both sides)."""
        self.window = (start, end)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = [ln for _, ln in self.lines]
        if self.window:  # samples taken in the region (one period of slack after it)
            a, b = self.window
            inside = [ln for t, ln in self.lines if a <= t <= b + 0.1]
            if inside:
                lines = inside
        for ln in lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def reduce_max(x: float, pg, device) -> float:
    """Max of x over the ranks of process group module pg (None: one rank).
    The timed region's length is the slowest replica's."""
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def make_case(name: str, rank: int):
    from gen import synth
    return synth.make_case(name, instance=rank)


WORKLOADS = {
    "c2": "2048x2048 cut-cell two-phase projection, 3 seeded circles, density 1000:1.2, "
          "32-mode u*, dt 5e-4 (plain FP64 MG-PCG)",
    "c1": "128x128 cut-cell two-phase projection, circle r=0.1, density 1000:1.2",
    "c3": "4096x4096 y-stretched grid, rotated plate, density 1000:1.2 (plain FP64 MG-PCG)",
}

# compulsory bytes per fine cell of each measured kernel, per precision:
# sweep = one red-black iteration (both colours)
# in one pass; resid_restrict = sweep + residual + 2x2 restriction;
# prolong = prolongation fused into a sweep.
KERNEL_BYTES = {
    "fp64": {"sweep": 48, "pupdate_spmv": 56, "update_xr": 48, "resid_restrict": 58,
             "prolong": 50},
    # fine level of the mixed path: x, b (FP32 copy of r), di FP32; BF16 couplings;
    # FP32 search direction p of the outer PCG
    "mixed": {"sweep": 20, "pupdate_spmv": 44, "update_xr": 52, "resid_restrict": 25,
              "prolong": 21},
}
KERNEL_IDS = (("sweep", 0), ("pupdate_spmv", 1), ("update_xr", 2), ("resid_restrict", 3),
              ("prolong", 4), ("vcycle", 6), ("setup", 7))


def cpu_projection_ms(case, threads: int, rtol: float = 1e-8):
    """One projection through the oracle's C restatement (assembly, RHS,
    FP64 MG-PCG to rtol, correction) on `threads` host threads.  Returns
    (ms, info, solution)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    O.lib().oracle_set_threads(threads)
    t0 = time.perf_counter()
    pc = O.pocoef(case)
    matr, A = O.matrix(case, pc)
    rhm, b = O.rhs(case)
    xi, it, rel, nlev = O.mgpcg(case, matr, rhm, rtol=rtol, maxit=500, npre=2, npost=2,
                                omega=1.9, threads=threads)
    x = O.x_from_interior(case, xi)
    Pp = O.scatter(case, x)
    u, v, p, mres = O.correct(case, Pp)
    ms = (time.perf_counter() - t0) * 1e3
    return ms, {"iters": it, "relres": rel, "levels": nlev}, {"Pp": Pp, "u": u, "v": v}


def _rel(a, b):
    d = np.linalg.norm(np.asarray(a) - np.asarray(b))
    n = np.linalg.norm(np.asarray(b))
    return float(d / n) if n > 0 else float(d)


def extra_learned(case, tdev, dev, local, args):
    """The headline case with the learned preconditioner (shipped weights)."""
    import torch
    from simcoflow_gb300 import learned as Lr, projection as P
    params, meta = Lr.load_weights()
    nx, ny = case.nx, case.ny
    s = P.ProjectionSolver(nx, ny, precision="mixed", precond="learned", device=local,
                           device_ptrs=True, rtol=1e-8, maxit=200)
    try:
        s.set_network(params)
        s.set_grid(tdev["dx"], tdev["dy"], tdev["dxU"], tdev["dyV"])
        s.set_geometry(**{k: tdev[k] for k in P.GEOMETRY_ARGS})
        u, v, p = tdev["u0"].clone(), tdev["v0"].clone(), tdev["p0"].clone()
        Pp = torch.zeros_like(tdev["p0"])
        m = torch.zeros(nx * ny, dtype=torch.float64, device=dev)

        def step():
            s.assemble(tdev["DpU"], tdev["DpV"], case.betaP, case.betaM, case.bc)
            return s.update_puv(tdev["ustar"], tdev["vstar"], u, v, p, case.vb, Pp=Pp, mres=m)[2]

        step()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        reps = max(1, min(args.steps, 3))
        for _ in range(reps):
            st = step()
        torch.cuda.synchronize(dev)
        ms = (time.perf_counter() - t0) / reps * 1e3
        return {"ms": round(ms, 3), "iters": st.iters, "learned_iters": st.learned_iters,
                "fallback_to_vcycle": bool(st.fallbacks), "relres_true": st.relres_true,
                "training": {k: meta.get(k) for k in ("instances", "iters", "size", "steps",
                                                      "batch", "loss_first", "loss_last")}}
    finally:
        s.close()


def extra_stretched(local, args):
    """The 4096^2 y-stretched configuration (line smoother), mixed and plain FP64."""
    import torch
    from gen import synth
    from simcoflow_gb300 import projection as P
    case = synth.c3()
    dev = torch.device("cuda", local)
    t = {k: torch.from_numpy(np.ascontiguousarray(v.ravel(order="F"))).to(dev)
         for k, v in case.arrays.items() if isinstance(v, np.ndarray)}
    out = {"workload": WORKLOADS["c3"], "nx": case.nx, "ny": case.ny}
    for prec in ("mixed", "fp64"):
        s = P.ProjectionSolver(case.nx, case.ny, precision=prec, device=local, device_ptrs=True,
                               rtol=1e-8, maxit=300)
        try:
            s.set_grid(t["dx"], t["dy"], t["dxU"], t["dyV"])
            s.set_geometry(**{k: t[k] for k in P.GEOMETRY_ARGS})
            u, v, p = t["u0"].clone(), t["v0"].clone(), t["p0"].clone()
            Pp = torch.zeros_like(t["p0"])
            m = torch.zeros(case.nx * case.ny, dtype=torch.float64, device=dev)

            def step():
                s.assemble(t["DpU"], t["DpV"], case.betaP, case.betaM, case.bc)
                return s.update_puv(t["ustar"], t["vstar"], u, v, p, case.vb, Pp=Pp,
                                    mres=m)[2]

            # each arm at its fastest V-cycle schedule (the autotuner's candidates;
            # the line smoother uses only the coarse-correction weight)
            schedule = None
            if not args.no_tune:
                from simcoflow_gb300 import batch as Bt
                best = None
                for sch in sorted({(2, 2, sc[2]) for sc in Bt.SCHEDULES}):
                    s.set_schedule(*sch)
                    step()
                    torch.cuda.synchronize(dev)
                    t0 = time.perf_counter()
                    stt = step()
                    torch.cuda.synchronize(dev)
                    ms_t = time.perf_counter() - t0
                    if stt.status == 0 and (best is None or ms_t < best[0]):
                        best = (ms_t, sch)
                schedule = best[1]
                s.set_schedule(*schedule)
            step()
            torch.cuda.synchronize(dev)
            e0, e1 = torch.cuda.Event(True), torch.cuda.Event(True)
            e0.record()
            reps = 2
            for _ in range(reps):
                st = step()
            e1.record()
            torch.cuda.synchronize(dev)
            out[prec] = {"ms": round(e0.elapsed_time(e1) / reps, 3), "iters": st.iters,
                         "relres_true": st.relres_true, "schedule": schedule,
                         "smoother": {1: "point", 2: "line"}.get(st.smoother)}
        finally:
            s.close()
    out["speedup_mixed_vs_plain"] = round(out["fp64"]["ms"] / out["mixed"]["ms"], 3)
    return out


def extra_momentum(case, local, args):
    """The momentum predictor's implicit solves (u and v) on the headline
    workload's cells: device-resident GPU time against the C restatement
    (operator, right-hand side, BiCGStab, scatter) on all host cores."""
    import torch
    from simcoflow_gb300 import momentum as M
    from gen import synth
    dev = torch.device("cuda", local)
    out = {"workload": f"u and v implicit solves on the {case.nx}x{case.ny} cells of the "
                       "headline workload (seeded face fluxes, Re 1e5)"}
    T = lambda x: torch.from_numpy(np.ascontiguousarray(x.ravel(order="F"))).to(dev)
    mis = {c: synth.momentum_inputs(case, c) for c in ("u", "v")}
    s = M.MomentumSolver(case.nx, case.ny, device_ptrs=True, device=local)
    try:
        tin = {c: {k: (T(v) if isinstance(v, np.ndarray) else v) for k, v in mi.items()}
               for c, mi in mis.items()}
        work = {c: (T(mi["pred"]), T(mi["Dp"])) for c, mi in mis.items()}

        def step():
            sts = []
            for c in ("u", "v"):
                pred, Dp = work[c]
                sts.append(s.solve(c, tin[c], pred, Dp, rtol=1e-13))
            return sts

        for _ in range(3):
            step()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        reps = 10
        for _ in range(reps):
            sts = step()
        torch.cuda.synchronize(dev)
        ms = (time.perf_counter() - t0) / reps * 1e3
    finally:
        s.close()
    out["gpu"] = {"ms_u_plus_v": round(ms, 3), "iters": [st.iters for st in sts],
                  "relres": [st.relres for st in sts], "launches": sum(st.launches for st in sts),
                  "timing": "host clock around 10 steps (each solve ends with a host poll)"}
    if not args.no_cpu:
        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle as O
        threads = os.cpu_count() or 1
        O.lib().oracle_set_threads(threads)
        t0 = time.perf_counter()
        its = [O.mom_predict(mis[c], solver="bicgstab", rtol=1e-13)["iters"] for c in ("u", "v")]
        cpu_ms = (time.perf_counter() - t0) * 1e3
        out["cpu"] = {"ms_u_plus_v": round(cpu_ms, 1), "cores": threads, "kind": "port",
                      "iters": its, "sample": "one u and one v solve (C restatement, OpenMP)"}
        out["speedup_vs_cpu"] = round(cpu_ms / ms, 1)
    return out


def extra_tecplot(case, local, args):
    """Print_Result_Tecplot_PCent's file of the headline workload (15 blocks
    of nx*ny "(f24.14)" records) from device-resident fields: the formatting
    kernel alone (CUDA events), the text into a host buffer, and the whole
    file written to the box's temporary directory; against the C
    restatement's formatting into a host buffer on all host cores."""
    import ctypes
    import tempfile
    import torch
    from simcoflow_gb300 import output as Out
    nx, ny = case.nx, case.ny
    rng = np.random.default_rng(17)
    F = lambda a: np.asfortranarray(a)
    A = case.arrays
    f = {"x": A["x"], "y": A["y"], "p": F(rng.standard_normal((nx + 2, ny + 2))),
         "u": A["u0"], "v": A["v0"], "phi": A["phi"], "vof": A["vof"],
         "phiS": F(rng.standard_normal((nx, ny))), "vofS": A["vofS"],
         "mres": F(rng.standard_normal((nx, ny)) * 1e-12),
         "flux": F(rng.standard_normal((nx + 2, ny + 2, 2))),
         "nxS": F(rng.uniform(-1, 1, (nx, ny))), "nyS": F(rng.uniform(-1, 1, (nx, ny)))}
    f = {k: F(np.asarray(v, dtype=np.float64)) for k, v in f.items()}
    dev = torch.device("cuda", local)
    tf = {k: torch.from_numpy(np.ascontiguousarray(v.ravel(order="F"))).to(dev)
          for k, v in f.items()}
    L = Out.load()
    size = L.scf_tecplot_size(Out.PCELL, nx, ny)
    cells = nx * ny
    out = {"workload": f"Tecplot P-cell file of the {nx}x{ny} headline workload "
                       f"(15 variables, {size / 1e9:.2f} GB of text)"}
    # formatting kernel alone
    body = torch.empty(15 * cells * 25, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    for _ in range(3):
        Out.format_device("p", nx, ny, tf, body, stream.cuda_stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 10
    e0.record(stream)
    for _ in range(reps):
        Out.format_device("p", nx, ny, tf, body, stream.cuda_stream)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    ms_kernel = e0.elapsed_time(e1) / reps
    # algorithmic bytes: 15 x 8 B read (neighbour values of the averages come
    # from cache) and 15 x 25 B of text written per cell
    alg = cells * 15 * (8 + 25)
    peak, peak_kind = _peaks()
    # the text into a host buffer (C-ABI call only; the buffer is made once)
    st, keep = Out._fields(Out.PCELL, nx, ny, tf, True)
    buf = ctypes.create_string_buffer(size)
    n = ctypes.c_int64(0)

    def text_once():
        rc = L.scf_tecplot_text(Out.PCELL, nx, ny, ctypes.byref(st), Out.DEVICE_PTRS, buf, size,
                                ctypes.byref(n), local)
        if rc != 0:
            raise RuntimeError(f"scf_tecplot_text {rc}")

    for _ in range(2):
        text_once()
    t0 = time.perf_counter()
    for _ in range(3):
        text_once()
    ms_text = (time.perf_counter() - t0) / 3 * 1e3
    with tempfile.TemporaryDirectory() as d:
        os.makedirs(os.path.join(d, "Tecplot"))
        ms_file = min(Out.write("p", nx, ny, tf, 1, d + "/", device_ptrs=True, device=local)
                      for _ in range(3))
    out["gpu"] = {
        "ms_format_kernel": round(ms_kernel, 3),
        "roofline": {"bound": "hbm", "achieved": round(alg / (ms_kernel * 1e-3) / 1e9, 1),
                     "peak": peak, "unit": "GB/s",
                     "frac": round(alg / (ms_kernel * 1e-3) / 1e9 / peak, 3),
                     "peak_kind": peak_kind, "bytes_per_cell": 15 * (8 + 25)},
        "ms_text_in_host_memory": round(ms_text, 2),
        "ms_file_write": round(ms_file, 2),
        "timing": "kernel: CUDA events; text: host clock around scf_tecplot_text "
                  "(kernel, pinned 16 MiB chunks, 4 copy threads); file: host clock around "
                  "scf_tecplot_write (one writer thread) into the temporary directory"}
    if not args.no_cpu:
        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle as O
        threads = os.cpu_count() or 1
        O.lib().oracle_set_threads(threads)
        cbuf = ctypes.create_string_buffer(size + 256)
        args_ = [O._p(f[k]) for k in O.PCELL_FIELDS]
        t0 = time.perf_counter()
        m = O.lib().oracle_tecplot_pcell(nx, ny, *args_, cbuf)
        cpu_ms = (time.perf_counter() - t0) * 1e3
        out["cpu"] = {"ms_text_in_host_memory": round(cpu_ms, 1), "cores": threads,
                      "kind": "port", "sample": "the whole file text (C restatement, "
                      "snprintf %24.14f per record, OpenMP over rows) into a host buffer"}
        out["identical_to_oracle"] = bool(m == n.value and
                                          ctypes.string_at(cbuf, m) == ctypes.string_at(buf, m))
        out["speedup_text_vs_cpu"] = round(cpu_ms / ms_text, 1)
    return out


def extra_vtr(case, local, args):
    """Print_Result_VTK_2D's ParaView file of the headline workload (X, Y, Z
    coordinates, the 3-component velocity, its two components and five
    scalars: 10 nx*ny REAL(4) values) from device-resident fields: the text
    into a host buffer and the file written to the box's temporary directory;
    against the C restatement's formatting into a host buffer on all host
    cores."""
    import ctypes
    import tempfile
    import torch
    from simcoflow_gb300 import output as Out
    nx, ny = case.nx, case.ny
    rng = np.random.default_rng(23)
    F = lambda a: np.asfortranarray(np.asarray(a, dtype=np.float64))
    A = case.arrays
    f = {"x": A["x"], "y": A["y"], "u": A["u0"], "v": A["v0"],
         "p": rng.standard_normal((nx + 2, ny + 2)), "phi": A["phi"],
         "phiS": rng.standard_normal((nx, ny)), "vof": A["vof"], "vofS": A["vofS"]}
    f = {k: F(v) for k, v in f.items()}
    dev = torch.device("cuda", local)
    tf = {k: torch.from_numpy(np.ascontiguousarray(v.ravel(order="F"))).to(dev)
          for k, v in f.items()}
    L = Out.load()
    size = L.scf_vtr_size(nx, ny)
    out = {"workload": f"ParaView VTR file of the {nx}x{ny} headline workload "
                       f"({10 * nx * ny / 1e6:.1f} M REAL(4) values, {size / 1e9:.2f} GB of text)"}
    st, keep = Out._pack(Out.VTR_FIELDS, Out.VtrFields, nx, ny, tf, True)
    buf = ctypes.create_string_buffer(size)
    n = ctypes.c_int64(0)

    def text_once():
        rc = L.scf_vtr_text(nx, ny, ctypes.byref(st), Out.DEVICE_PTRS, buf, size, ctypes.byref(n),
                            local)
        if rc != 0:
            raise RuntimeError(f"scf_vtr_text {rc}")

    for _ in range(2):
        text_once()
    t0 = time.perf_counter()
    for _ in range(3):
        text_once()
    ms_text = (time.perf_counter() - t0) / 3 * 1e3
    with tempfile.TemporaryDirectory() as d:
        os.makedirs(os.path.join(d, "Paraview"))
        ms_file = min(Out.vtr_write(nx, ny, tf, 1, d + "/", device_ptrs=True, device=local)
                      for _ in range(3))
    out["gpu"] = {"ms_text_in_host_memory": round(ms_text, 2), "ms_file_write": round(ms_file, 2),
                  "timing": "text: host clock around scf_vtr_text (literal records, one "
                            "formatting kernel, pinned 16 MiB chunks, 4 copy threads); file: host "
                            "clock around scf_vtr_write (one writer thread) into the temporary "
                            "directory"}
    if not args.no_cpu:
        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle as O
        threads = os.cpu_count() or 1
        O.lib().oracle_set_threads(threads)
        cbuf = ctypes.create_string_buffer(size + 2048)
        args_ = [O._p(f[k]) for k in O.VTR_FIELDS]
        t0 = time.perf_counter()
        m = O.lib().oracle_vtr(nx, ny, *args_, cbuf)
        cpu_ms = (time.perf_counter() - t0) * 1e3
        out["cpu"] = {"ms_text_in_host_memory": round(cpu_ms, 1), "cores": threads,
                      "kind": "port", "sample": "the whole file text (C restatement, snprintf "
                      "%.8E per value, OpenMP over values) into a host buffer"}
        out["identical_to_oracle"] = bool(m == n.value and
                                          ctypes.string_at(cbuf, m) == ctypes.string_at(buf, m))
        out["speedup_text_vs_cpu"] = round(cpu_ms / ms_text, 1)
    return out


def extra_lsweep(case, local, args):
    """The level-set part of one X_Sweep and one Y_Sweep on the headline grid
    with device-resident fields, against the C restatement on one core."""
    import torch
    from simcoflow_gb300 import clsvof as CL
    from gen.synth import ls_fields
    nx, ny = case.nx, case.ny
    f = ls_fields(np.random.default_rng(29), nx, ny)
    t0 = np.asfortranarray(np.random.default_rng(30).standard_normal((nx, ny)))
    dev = torch.device("cuda", local)
    tf = {k: torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).to(dev)
          for k, a in f.items()}
    tt = torch.from_numpy(np.ascontiguousarray(t0.ravel(order="F"))).to(dev)
    for _ in range(3):
        CL.sweep(CL.X, nx, ny, tf, 1e-4, tt, device_ptrs=True, device=local)
    reps = 10
    ms = 0.0
    for _ in range(reps):
        ms += CL.sweep(CL.X, nx, ny, tf, 1e-4, tt, device_ptrs=True, device=local)
        ms += CL.sweep(CL.Y, nx, ny, tf, 1e-4, tt, device_ptrs=True, device=local)
    out = {"workload": f"level-set update of one X_Sweep and one Y_Sweep, {nx}x{ny}",
           "gpu": {"ms_x_plus_y": round(ms / reps, 3),
                   "timing": "host clock around scf_ls_sweep (device pointers; each call "
                             "creates a stream, launches one kernel and synchronises)"}}
    if not args.no_cpu:
        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle as O
        t1 = time.perf_counter()
        O.ls_sweep(1, nx, ny, f, 1e-4, O.ls_sweep(0, nx, ny, f, 1e-4, t0))
        cpu_ms = (time.perf_counter() - t1) * 1e3
        out["cpu"] = {"ms_x_plus_y": round(cpu_ms, 1), "cores": 1, "kind": "port",
                      "sample": "the literal sequential loops (C restatement)"}
    return out


def extra_cutcell(case, local, args):
    """The per-step cut-cell geometry of the P, U and V cells
    (Grid_Preprocess + NewCellFace, scf_grid_preprocess) on the headline
    workload's grid and bodies, device-resident."""
    import torch
    from simcoflow_gb300 import cutcell as CU
    from gen import synth
    grids, fams = synth.cutcell_inputs(case)
    dev = torch.device("cuda", local)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).to(dev)
    tg = {f: {k: T(v) for k, v in g.items()} for f, g in grids.items()}
    tf = {f: {k: T(v) for k, v in g.items()} for f, g in fams.items()}
    for _ in range(2):
        CU.grid_preprocess(tg, tf, nx=case.nx, ny=case.ny, device=local)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    reps = 5
    for _ in range(reps):
        out, _ = CU.grid_preprocess(tg, tf, nx=case.nx, ny=case.ny, device=local)
    torch.cuda.synchronize(dev)
    ms = (time.perf_counter() - t0) / reps * 1e3
    return {"workload": f"P, U and V cut-cell geometry of the {case.nx}x{case.ny} headline "
                        "grid (3 circles)",
            "gpu": {"ms": round(ms, 3), "moex_u": int(out["u"]["moex"].sum().item()),
                    "moex_v": int(out["v"]["moex"].sum().item()),
                    "timing": "host clock around scf_grid_preprocess with device-resident "
                              "inputs (includes its device allocation and output copies)"}}


def extra_batch(local):
    """64 uneven instances in one graph launch with autotuned schedules."""
    from gen import synth
    from simcoflow_gb300 import batch as Bt
    cases = [synth.c5(instance=i) for i in range(64)]
    bp = Bt.BatchProjector(cases, precision="mixed", rtol=1e-8, maxit=300, device=local)
    try:
        bp.run()
        times = []
        for _ in range(3):
            st, ms = bp.run()
            times.append(ms)
        ms = min(times)
        return {"workload": "64 instances, sides 256..1024 (log-uniform, multiples of 32), "
                            "density ratio log-U[10,1000], 0-4 circles, 16-mode u*, dt 1e-3",
                "cells": int(sum(c.nx * c.ny for c in cases)), "ms_per_batch": round(ms, 3),
                "solves_per_s": round(64 / (ms * 1e-3), 1),
                "iters_min_max": [min(x["iters"] for x in st), max(x["iters"] for x in st)],
                "max_relres_true": max(x["relres_true"] for x in st),
                "launch": "one CUDA graph (64 branches, conditional-while PCG per branch)",
                "autotune": json.loads(bp.table_json())}
    finally:
        bp.close()


def run_reference(args):
    world, rank, local = _dist()
    if rank != 0:
        return 0
    case = make_case(args.config, 0)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_projection_ms(case, threads)
    times, info = [], {}
    for _ in range(args.steps):
        ms, info, _ = cpu_projection_ms(case, threads)
        times.append(ms)
    ms = float(np.mean(times))
    line = {"impl": "reference", "metric": METRIC, "value": ms, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded, shapes and distributions of the named config)",
            "config": {"workload": WORKLOADS.get(args.config, args.config), "name": args.config,
                       "nx": case.nx, "ny": case.ny},
            "cpu_baseline": {"value": ms, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"one full {case.nx}x{case.ny} projection per step "
                                       f"(C restatement + OpenMP; Fortran+HYPRE reference "
                                       f"unbuildable: no Fortran compiler, MPI or HYPRE)",
                             "iters": info.get("iters")},
            "e2e": {"value": ms, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import ctypes
    import torch
    world, rank, local = _dist()
    from simcoflow_gb300 import build as B
    B.build_all()
    from simcoflow_gb300 import projection as P
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
        pg = dist
    case = make_case(args.config, rank)
    A = case.arrays
    nx, ny = case.nx, case.ny
    cells = nx * ny
    stream = torch.cuda.Stream(device=dev)

    def barrier():
        if pg:
            pg.barrier()
        torch.cuda.synchronize(dev)

    def max_over_ranks(x):
        return reduce_max(x, pg, dev)

    tdev = {k: torch.from_numpy(np.ascontiguousarray(v.ravel(order="F"))).to(dev)
            for k, v in A.items() if isinstance(v, np.ndarray)}

    def device_arm(precision, sample_clocks):
        """Device-resident projections: inputs in HBM, device pointers."""
        s = P.ProjectionSolver(nx, ny, precision=precision, device=local, device_ptrs=True,
                               rtol=1e-8, maxit=200, use_graph=not args.no_graph)
        s.set_stream(stream.cuda_stream)
        s.set_grid(tdev["dx"], tdev["dy"], tdev["dxU"], tdev["dyV"])
        s.set_geometry(**{k: tdev[k] for k in P.GEOMETRY_ARGS})
        u, v, p = tdev["u0"].clone(), tdev["v0"].clone(), tdev["p0"].clone()
        Pp = torch.zeros_like(tdev["p0"])
        mres = torch.zeros(cells, dtype=torch.float64, device=dev)

        def step():
            s.assemble(tdev["DpU"], tdev["DpV"], case.betaP, case.betaM, case.bc)
            _, _, st = s.update_puv(tdev["ustar"], tdev["vstar"], u, v, p, case.vb, Pp=Pp,
                                    mres=mres)
            return st

        # V-cycle schedule from the project's autotuner (same candidates as the
        # batch path), chosen by time to the tolerance on this workload
        schedule = None
        if not args.no_tune:
            from simcoflow_gb300 import batch as Bt
            best = None
            for sch in Bt.SCHEDULES:
                s.set_schedule(*sch)
                step()
                torch.cuda.synchronize(dev)
                t0 = time.perf_counter()
                for _ in range(2):
                    stt = step()
                torch.cuda.synchronize(dev)
                ms_t = (time.perf_counter() - t0) / 2
                if stt.status == 0 and (best is None or ms_t < best[0]):
                    best = (ms_t, sch)
            schedule = best[1]
            s.set_schedule(*schedule)
        for _ in range(args.warmup):
            st = step()
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        iters, relres, nlaunch = [], [], []
        clk = ClockSampler(local) if sample_clocks else None
        if clk:
            clk.__enter__()
        barrier()
        h0 = time.monotonic()
        e0.record(stream)
        for _ in range(args.steps):
            st = step()
            iters.append(st.iters)
            relres.append(st.relres_true)
            nlaunch.append(st.launches)
        e1.record(stream)
        barrier()
        if clk:
            clk.mark(h0, time.monotonic())
            clk.__exit__()
        ms = max_over_ranks(e0.elapsed_time(e1)) / args.steps
        kt = {}
        for name, kid in KERNEL_IDS:  # live per-kernel timing on the same data
            out = ctypes.c_double(0.0)
            if P.load().scf_proj_time_kernel(s._h, kid, 50, ctypes.byref(out)) == 0:
                kt[name] = out.value
        s.close()
        return {"ms": ms, "iters": iters, "relres": relres, "levels": st.levels, "kt": kt,
                "launches": nlaunch,
                "clk": clk.summary() if clk else None, "schedule": schedule}

    plain = device_arm("fp64", False)
    mixed = device_arm("mixed", True)

    # ---- end-to-end: the headline (mixed) path through host (pinned) buffers ----
    def pinned(a):
        t = torch.empty(a.size, dtype=torch.float64 if a.dtype == np.float64 else torch.int32)
        t = t.pin_memory()
        arr = t.numpy().reshape(a.shape, order="F")
        arr[...] = a
        return arr, t

    hp = {k: pinned(v) for k, v in A.items() if isinstance(v, np.ndarray)}
    H = {k: v[0] for k, v in hp.items()}
    hs = P.ProjectionSolver(nx, ny, precision="mixed", device=local, rtol=1e-8, maxit=200,
                            use_graph=not args.no_graph)
    hs.set_stream(stream.cuda_stream)
    hu, hv, hpp = pinned(A["u0"])[0], pinned(A["v0"])[0], pinned(A["p0"])[0]
    hPp = pinned(np.zeros((nx + 2, ny + 2), order="F"))[0]
    hm = pinned(np.zeros((nx, ny), order="F"))[0]
    # the grid is fixed for a whole run (Initial_Grid, src/Mesh_Mod.f90:54-175): set once;
    # everything the time step changes is copied in and out every step
    in_keys = [*P.GEOMETRY_ARGS, "DpU", "DpV", "ustar", "vstar"]
    h2d = sum(H[k].nbytes for k in in_keys) + hu.nbytes + hv.nbytes + hpp.nbytes
    d2h = hPp.nbytes + hu.nbytes + hv.nbytes + hpp.nbytes + hm.nbytes
    hs.set_grid(H["dx"], H["dy"], H["dxU"], H["dyV"])

    def e2e_step():
        hs.set_geometry(**{k: H[k] for k in P.GEOMETRY_ARGS})
        hs.assemble(H["DpU"], H["DpV"], case.betaP, case.betaM, case.bc)
        _, _, st_ = hs.update_puv(H["ustar"], H["vstar"], hu, hv, hpp, case.vb, Pp=hPp, mres=hm)
        return st_.mres_max  # the step's result (max |mres|), read on the host

    for _ in range(args.warmup):
        e2e_step()
    barrier()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    f1.record(stream)
    barrier()
    e2e_ms = max_over_ranks(f0.elapsed_time(f1)) / args.steps

    # the same step with the cut-cell geometry derived on the GPU
    # (scf_proj_set_solid): only the solid level-set fields cross
    solid_keys = ["vof", "phi", "vofS_in", "phiS", "nxS_in", "nyS_in", "vofS_u_in", "vofS_v_in"]
    h2d_solid = (sum(H[k].nbytes for k in solid_keys + ["DpU", "DpV", "ustar", "vstar"]) +
                 hu.nbytes + hv.nbytes + hpp.nbytes)

    def e2e_solid_step():
        hs.set_solid(*[H[k] for k in solid_keys])
        hs.assemble(H["DpU"], H["DpV"], case.betaP, case.betaM, case.bc)
        _, _, st_ = hs.update_puv(H["ustar"], H["vstar"], hu, hv, hpp, case.vb, Pp=hPp, mres=hm)
        return st_.mres_max

    for _ in range(args.warmup):
        e2e_solid_step()
    barrier()
    f0.record(stream)
    for _ in range(args.steps):
        e2e_solid_step()
    f1.record(stream)
    barrier()
    e2e_solid_ms = max_over_ranks(f0.elapsed_time(f1)) / args.steps
    hs.close()

    if rank != 0:
        if pg:
            pg.destroy_process_group()
        return 0

    peak, peak_kind = _peaks()

    def kernel_table(arm, prec):
        out = {}
        for k, v in arm["kt"].items():
            out[k] = {"ms": round(v, 5)}
            if k in KERNEL_BYTES[prec]:
                out[k]["GBps"] = round(KERNEL_BYTES[prec][k] * cells / (v * 1e-3) / 1e9, 1)
        return out

    # dominant kernel of the headline path: the fine-level sweep (4 of them per
    # V-cycle on the fine grid, plus the fused restrict / prolong variants)
    dom = "sweep"
    roof = None
    if dom in mixed["kt"] and mixed["kt"][dom] > 0:
        bytes_launch = KERNEL_BYTES["mixed"][dom] * cells
        achieved = bytes_launch / (mixed["kt"][dom] * 1e-3) / 1e9
        traffic = None
        tf = ROOT / "profiles" / "traffic.json"
        if tf.exists():
            try:
                traffic = json.loads(tf.read_text()).get(f"mixed_{dom}_{args.config}")
            except Exception:
                traffic = None
        roof = {"bound": "hbm",
                "kernel": "k_sweep_tma<FIRST=1,ZERO=0,PROLONG=0,RESTRICT=0,RZ=0,ITER=1> "
                          "(TMA-staged FP32/BF16 red-black iteration, fine grid)",
                "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                "bytes_per_launch": bytes_launch, "ms_per_launch": mixed["kt"][dom],
                "traffic": traffic,
                "kernel_timing": "CUDA events around 50 back-to-back launches on the solver "
                                 "stream, right after the timed region, same data"}
    # kernel launches of the timed steps as the library counts them (direct
    # launches plus the kernel nodes of each executed graph loop body)
    launches = sum(mixed["launches"])
    cpu = None
    err = None
    if world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        ms_cpu, info, _ = cpu_projection_ms(case, threads)
        cpu = {"value": round(ms_cpu, 2), "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"one full {nx}x{ny} projection (C restatement of the reference path, "
                         f"OpenMP, {info['iters']} MG-PCG iterations)"}
        # error statement of the headline result against the FP64 oracle driven
        # to its floor (checker only; not timed)
        _, info13, ref = cpu_projection_ms(case, threads, rtol=1e-13)
        err = {"p_rel_l2": _rel(hPp, ref["Pp"]),
               "uv_rel_l2": _rel(np.concatenate([hu.ravel(), hv.ravel()]),
                                 np.concatenate([ref["u"].ravel(), ref["v"].ravel()])),
               "oracle": f"C restatement, FP64 MG-PCG to relres {info13['relres']:.1e}"}
    extras = {}
    if world == 1 and not args.no_extras:
        for name, fn in (("learned", lambda: extra_learned(case, tdev, dev, local, args)),
                         ("stretched_4096", lambda: extra_stretched(local, args)),
                         ("batch_64", lambda: extra_batch(local)),
                         ("momentum_2048", lambda: extra_momentum(case, local, args)),
                         ("tecplot_2048", lambda: extra_tecplot(case, local, args)),
                         ("vtr_2048", lambda: extra_vtr(case, local, args)),
                         ("ls_sweep_2048", lambda: extra_lsweep(case, local, args)),
                         ("cutcell_2048", lambda: extra_cutcell(case, local, args))):
            try:
                extras[name] = fn()
            except Exception as e:  # an extra must not hide the headline line
                extras[name] = {"error": f"{type(e).__name__}: {e}"}
    ms_step = mixed["ms"]
    line = {
        "metric": METRIC, "value": round(ms_step, 4), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 4),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded; shapes and distributions of the named config)",
        "config": {"workload": WORKLOADS.get(args.config, args.config), "name": args.config,
                   "nx": nx, "ny": ny,
                   "path": "FP64 flexible PCG + FP32/BF16 multigrid (mixed)",
                   "parallelism": f"replicas x{world}",
                   "launch": "direct launches" if args.no_graph else "CUDA graph (conditional while)",
                   "l2": "inputs larger than L2 (about 1.3 GB of arrays per projection)"},
        "solves_per_s": round(1e3 * world / ms_step, 2),
        "iters": mixed["iters"][-1], "relres_true": mixed["relres"][-1],
        "levels": mixed["levels"],
        "schedule": {"npre_npost_omega": mixed["schedule"],
                     "source": "autotuner (simcoflow_gb300.batch.SCHEDULES), per arm"},
        "plain_fp64_mg_pcg": {"ms": round(plain["ms"], 4), "iters": plain["iters"][-1],
                              "relres_true": plain["relres"][-1],
                              "schedule": plain["schedule"],
                              "kernels": kernel_table(plain, "fp64")},
        "speedup_vs_plain": round(plain["ms"] / ms_step, 3),
        "e2e": {"value": round(e2e_ms, 4), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "e2e_gpu_geometry": {"value": round(e2e_solid_ms, 4), "unit": UNIT,
                             "h2d_bytes_per_step": int(h2d_solid),
                             "d2h_bytes_per_step": int(d2h),
                             "path": "scf_proj_set_solid: Grid_Preprocess's derived geometry "
                                     "computed on the GPU from the solid level-set fields"},
        "roofline": roof, "kernels": kernel_table(mixed, "mixed"),
        "gpu_launches": int(launches), "cpu_baseline": cpu, "clocks": mixed["clk"],
        "err_vs_fp64_oracle": err, **extras,
    }
    print(json.dumps(line), flush=True)
    if pg:
        pg.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", default="c2")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-tune", action="store_true",
                    help="default V-cycle schedule instead of the autotuned one")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the learned, 4096^2 stretched and 64-instance batch lines")
    ap.add_argument("--no-graph", action="store_true",
                    help="launch the same kernels one by one instead of through the CUDA graph "
                         "(profilers cannot see kernel nodes of graphs with conditional nodes)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
