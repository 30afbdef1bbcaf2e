#!/usr/bin/env python
"""Benchmark: milliseconds per pressure projection solved to FP64 relative
residual 1e-8 on one GB300, on the 4096x4096 configuration the metric is
quoted on: a y-stretched grid (geometric ratio 1.01 outside the band
y in [0.45, 0.55]) with a thin rotated plate, a two-mode free surface and
density ratio 1000:1.2.

One step = one full projection of SIMCOFlow's UpdatePUV projection part:
operator assembly + multigrid setup, right-hand side, PCG solve to
||b - A x||_2 <= 1e-8 ||b||_2, velocity correction, mass residual.

  value  device-resident: every input already in HBM (device pointers
         through the C-ABI), CUDA events on the solver's stream; the
         mixed-precision path (FP64 flexible PCG, FP32/BF16 multigrid), each
         arm at its autotuned V-cycle schedule.  The same line carries the
         plain FP64 MG-PCG arm and the learned + mixed arm on the same
         workload, each with its error against an FP64 oracle solve
  e2e    the same projection through the C-ABI with pinned host buffers:
         host->device copies of all inputs and device->host copies of all
         outputs inside the timed region
  --impl reference  the CPU restatement of the reference path (the oracle,
         C + OpenMP on all host cores), same workload, config and metric;
         it loads nothing of the product package

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
FALLBACK_BF16_TFLOPS = 1900.0


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return float(d["hbm_gbs"]), "measured"
        except Exception:
            pass
    return FALLBACK_HBM_GBS, "fallback"


def _bf16_peak():
    """Dense BF16 tensor peak (TFLOP/s, burst) and where it comes from."""
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["bf16_tflops"]), "measured"
        except Exception:
            pass
    return FALLBACK_BF16_TFLOPS, "fallback"


def unet_forward_times(sizes=((1024, 1024), (4096, 4096)), reps=10):
    """The learned preconditioner's network on its own: one forward pass
    (14 3x3 convolutions, pooling, head) of one image, shipped weights and
    seeded inputs, CUDA events around `reps` back-to-back passes after two
    warm-ups, on both convolution engines (tcgen05 with TMEM accumulators,
    the default; the mma.sync kernels, for comparison).  FLOPs: 2 x 9 x
    cin x cout per pixel of each convolution at its level."""
    import torch
    from simcoflow_gb300 import learned as Lr
    peak, kind = _bf16_peak()
    params, _ = Lr.load_weights()
    rng = np.random.Generator(np.random.PCG64(5))
    out = {}
    for (h, w) in sizes:
        flop = 2 * 9 * sum(ci * co / 4 ** lvl for (ci, co), lvl in zip(
            Lr.LAYERS, (0, 0, 1, 1, 2, 2, 3, 3, 2, 2, 1, 1, 0, 0))) * h * w
        net = Lr.UNet(1, h, w)
        try:
            net.set_params(params)
            net.set_input(rng.normal(size=(1, h, w, 5)).astype(np.float32))
            z = torch.empty((1, h, w), dtype=torch.float32, device="cuda")
            r = {}
            for name, eng in (("tcgen05", 1), ("mma_sync", 0)):
                net.set_engine(eng)
                for _ in range(2):
                    net.forward(z)
                torch.cuda.synchronize()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record()
                for _ in range(reps):
                    net.forward(z)
                b.record()
                torch.cuda.synchronize()
                ms = a.elapsed_time(b) / reps
                r[name] = {"ms": round(ms, 4), "tflops": round(flop / (ms * 1e-3) / 1e12, 1),
                           "frac_of_bf16_peak": round(flop / (ms * 1e-3) / 1e12 / peak, 4)}
            net.set_engine(1)
        finally:
            net.close()
        out[f"{h}x{w}"] = {**r, "gflop": round(flop / 1e9, 2),
                           "speedup_tcgen05": round(r["mma_sync"]["ms"] / r["tcgen05"]["ms"], 3)}
    out["peak"] = {"bf16_tflops": peak, "source": kind}
    out["timing"] = ("CUDA events on the default stream around back-to-back forward passes "
                     "(each ends with a 4-byte status read)")
    return out


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


def make_case(name: str, rank: int, **kw):
    from gen import synth
    return synth.make_case(name, instance=rank, **kw)


WORKLOADS = {
    "c3": "4096x4096 y-stretched grid (geometric ratio 1.01 outside the band y in "
          "[0.45,0.55]), 0.3x0.02 plate rotated 10 degrees at (0.5,0.35), two-mode free "
          "surface (0.02, 0.01), density 1000:1.2, 64 seeded u* modes + Gaussian vortex 0.5, "
          "dt 2.5e-4",
    "c2": "2048x2048 uniform grid, three seeded circles r U(0.04,0.1), surface "
          "0.5+0.03 sin(4 pi x + theta), density 1000:1.2, 32 seeded u* modes, dt 5e-4",
    "c1": "128x128 uniform grid, circle r=0.1 at (0.5,0.35), surface 0.5+0.02 sin(2 pi x), "
          "density 1000:1.2, 8 seeded u* modes, dt 1e-3",
}

# Compulsory DRAM bytes per fine cell of each timed kernel (each array element
# the launch touches counted once), per precision.
#   pupdate_spmv  p = z + beta p, q = A p, p.q: z, p_old, p_new, dg, cE, cN, q
#   update_xr     x += alpha p, r -= alpha q, FP32 copy of r, r.r, r.z
#   line          one parity of x-lines: relaxed rows dg, b, cE, cN, x written
#                 (16 B), the other rows' x and cN (6 B); 22 B per two cells
#   fine_pre      first pre-smoothing launch: zero start, fused iterations,
#                 residual + restriction: b, inverse diagonal, cE, cN, x
#                 written, a quarter of the coarse b written
#   fine_post     last post-smoothing launch: x, b, inverse diagonal, cE, cN,
#                 a quarter of the coarse x read, x written
#   assemble      14 FP64 / int32 input fields read, cE, cN, dg, own W and S
#                 entries written (Fortran inputs with their ghost rings)
KERNEL_BYTES = {
    "fp64": {"pupdate_spmv": 56, "update_xr": 48, "fine_pre": 40, "fine_post": 48,
             "assemble": 152},
    "mixed": {"pupdate_spmv": 44, "update_xr": 52, "line": 11, "fine_pre": 17, "fine_post": 21,
              "assemble": 152},
}
KERNEL_IDS = {"pupdate_spmv": 1, "update_xr": 2, "assemble": 5, "vcycle": 6, "setup": 7,
              "line": 8, "fine_pre": 9, "fine_post": 10}
# the dominant kernel of each smoother's path by share of the launch list
# (profiles/launches_c3_4096_mixed.md, profiles/launches_c2_mixed.md): its
# name as ncu lists it and the scf_proj_time_kernel id that launches it
DOMINANT = {
    "line": ("line", "k_line<float, __nv_bfloat16, 8, 0, 0>",
             "one parity of the fine level's x-lines (zebra line relaxation, FP32 iterate, "
             "BF16 couplings)"),
    "point": ("fine_pre", "k_sweep_tma<0, 1, 0, 1, 0, 2>",
              "the fine level's pre-smoothing launch (two red-black iterations from zero, "
              "residual and 2x2 restriction, TMA-staged)"),
}


# DRAM bytes per launch of the roofline kernel from an ncu capture of the
# same kernel (bench.py runs no profiler, so the line's `traffic` stays null):
# the capture, the workload it ran on and the scaling to a full launch
TRAFFIC_PROFILE = {
    ("c3", "line"): {"bytes_per_launch": 152.1e6, "source": "profiles/k_line_mixed_c3.md",
                     "how": "dram__bytes_read.sum + dram__bytes_write.sum of 3 launches on the "
                            "2048x2048 case of this workload (38.0 MB), x4 for the cells of a "
                            "4096x4096 launch"},
}


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    m = np.isfinite(a) & np.isfinite(b)
    d = np.linalg.norm(a[m] - b[m])
    n = np.linalg.norm(b[m])
    return float(d / n) if n > 0 else float(d)


def _oracle():
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    return O


def cpu_projection(case, threads: int, rtol: float = 1e-8, maxit: int = 500):
    """One projection through the oracle's C restatement (PoCoef, the dense
    rows, RHS, FP64 MG-PCG to rtol, scatter, correction) on `threads` host
    threads.  Returns (ms, result)."""
    O = _oracle()
    O.lib().oracle_set_threads(threads)
    t0 = time.perf_counter()
    r = O.project_mg(case, rtol=rtol, maxit=maxit)
    return (time.perf_counter() - t0) * 1e3, r


def errors_vs(out, ref):
    """Relative L2 errors of a projection's outputs against the FP64 oracle."""
    return {"p_rel_l2": _rel(out["Pp"], ref["Pp"]),
            "u_rel_l2": _rel(out["u"], ref["u"]), "v_rel_l2": _rel(out["v"], ref["v"])}


def _tdev(case, dev):
    import torch
    return {k: torch.from_numpy(np.ascontiguousarray(v.ravel(order="F"))).to(dev)
            for k, v in case.arrays.items() if isinstance(v, np.ndarray)}


def _host(t, shape):
    return t.cpu().numpy().reshape(shape, order="F")


# the coarse-level schedules the autotuner tries: (first level, sweeps) --
# more sweeps on the latency-bound coarse levels (line smoother: two to four
# alternating steps per side) -- or None (the fine level's schedule
# everywhere)
LINE_COARSE = [None, (1, 4), (2, 4), (3, 4), (1, 6), (2, 6), (2, 8)]
POINT_COARSE = [None, (1, 4), (2, 4), (2, 6)]


def apply_schedule(s, schedule):
    """(npre, npost, omega, extras...) on a solver: an extra is the point
    smoother's sweep tile (a name in TILES) or the coarse-level schedule
    (first level, sweeps); without one, npre / npost on every level."""
    from simcoflow_gb300 import batch as Bt
    s.set_schedule(*schedule[:3])
    coarse = (0, 0)
    for extra in schedule[3:]:
        if isinstance(extra, str):
            s.set_tile(Bt.TILES[extra])
        elif extra is not None:
            coarse = tuple(extra)
    s.set_coarse_sweeps(*coarse)


def device_arm(case, tdev, local, precision, *, steps, warmup, precond="mg", schedule=None,
               tune=True, sample_clocks=False, stream=None, use_graph=True, pg=None,
               kernels=True):
    """Device-resident projections (inputs in HBM, device pointers through
    the C-ABI), timed with CUDA events on the solver's stream.  Returns the
    per-step time, statistics, the autotuned schedule, live per-kernel
    times and the last step's outputs (host copies)."""
    import ctypes
    import torch
    from simcoflow_gb300 import projection as P
    dev = torch.device("cuda", local)
    stream = stream or torch.cuda.Stream(device=dev)
    nx, ny = case.nx, case.ny
    s = P.ProjectionSolver(nx, ny, precision=precision, device=local, device_ptrs=True,
                           rtol=1e-8, maxit=300, use_graph=use_graph, precond=precond)
    try:
        if precond == "learned":
            from simcoflow_gb300 import learned as Lr
            params, _ = Lr.load_weights()
            s.set_network(params)
        s.set_stream(stream.cuda_stream)
        s.set_grid(tdev["dx"], tdev["dy"], tdev["dxU"], tdev["dyV"])
        s.set_geometry(**{k: tdev[k] for k in P.GEOMETRY_ARGS})
        u, v, p = tdev["u0"].clone(), tdev["v0"].clone(), tdev["p0"].clone()
        Pp = torch.zeros_like(tdev["p0"])
        mres = torch.zeros(nx * ny, dtype=torch.float64, device=dev)

        # u, v, p are corrected in place; the faces a projection corrects
        # do not read their old value and the others keep it, so every step
        # gives the first step's result
        def step():
            s.assemble(tdev["DpU"], tdev["DpV"], case.betaP, case.betaM, case.bc)
            return s.update_puv(tdev["ustar"], tdev["vstar"], u, v, p, case.vb, Pp=Pp,
                                mres=mres)[2]

        st = step()
        smoother = {1: "point", 2: "line"}.get(st.smoother)
        # V-cycle schedule from the project's autotuner, by time to the
        # tolerance on this workload (sweeps, omega, the coarse levels'
        # sweeps and, for the point smoother, the sweep tile)
        if schedule is None and tune:
            from simcoflow_gb300 import batch as Bt
            # point smoother: every schedule with every sweep tile
            cands = ([(*sc, tn, co) for tn in Bt.TILES for sc in Bt.SCHEDULES
                      for co in POINT_COARSE]
                     if smoother == "point" else
                     [(2, 2, om, co) for om in sorted({sc[2] for sc in Bt.SCHEDULES})
                      for co in LINE_COARSE])
            best = None
            for sch in cands:
                apply_schedule(s, sch)
                step()
                torch.cuda.synchronize(dev)
                t0 = time.perf_counter()
                for _ in range(2):
                    stt = step()
                torch.cuda.synchronize(dev)
                ms_t = (time.perf_counter() - t0) / 2
                if stt.status == 0 and (best is None or ms_t < best[0]):
                    best = (ms_t, sch)
            schedule = best[1] if best else None
        if schedule is not None:
            apply_schedule(s, schedule)
        for _ in range(warmup):
            st = step()
        if pg:
            pg.barrier()
        torch.cuda.synchronize(dev)
        clk = ClockSampler(local) if sample_clocks else None
        if clk:
            clk.__enter__()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        iters, relres, nlaunch, lit = [], [], [], []
        if pg:
            pg.barrier()
        torch.cuda.synchronize(dev)
        h0 = time.monotonic()
        e0.record(stream)
        for _ in range(steps):
            st = step()
            iters.append(st.iters)
            relres.append(st.relres_true)
            nlaunch.append(st.launches)
            lit.append(st.learned_iters)
        e1.record(stream)
        if pg:
            pg.barrier()
        torch.cuda.synchronize(dev)
        if clk:
            clk.mark(h0, time.monotonic())
            clk.__exit__()
        ms = e0.elapsed_time(e1) / steps
        if pg:
            ms = reduce_max(ms, pg, dev)
        out = {"Pp": _host(Pp, (nx + 2, ny + 2)), "u": _host(u, (nx + 2, ny + 2)),
               "v": _host(v, (nx + 2, ny + 2)), "mres": _host(mres, (nx, ny))}
        kt = {}
        if kernels:
            for name, kid in KERNEL_IDS.items():  # live per-kernel timing on the same data
                if name == "line" and smoother != "line":
                    continue
                if name in ("fine_pre", "fine_post") and smoother != "point":
                    continue
                o = ctypes.c_double(0.0)
                if P.load().scf_proj_time_kernel(s._h, kid, 50, ctypes.byref(o)) == 0:
                    kt[name] = o.value
        return {"ms": ms, "iters": iters, "relres": relres, "levels": st.levels,
                "launches": nlaunch, "learned_iters": lit, "fallbacks": st.fallbacks,
                "asym_faces": st.asym_faces, "smoother": smoother, "schedule": schedule,
                "kt": kt, "clk": clk.summary() if clk else None, "out": out}
    finally:
        s.close()


def kernel_table(arm, prec, cells, peak):
    out = {}
    for k, v in arm["kt"].items():
        out[k] = {"ms": round(v, 5)}
        if k in KERNEL_BYTES[prec]:
            gbs = KERNEL_BYTES[prec][k] * cells / (v * 1e-3) / 1e9
            out[k]["GBps"] = round(gbs, 1)
            out[k]["frac"] = round(gbs / peak, 3)
    return out


def e2e_arm(case, local, stream, *, steps, warmup, schedule, pg=None, solid=False):
    """The mixed projection through the C-ABI with pinned host buffers: every
    input copied host->device and every output device->host inside the timed
    region (the grid, fixed for a run, is set once)."""
    import torch
    from simcoflow_gb300 import projection as P
    dev = torch.device("cuda", local)
    A = case.arrays
    nx, ny = case.nx, case.ny

    def pinned(a):
        t = torch.empty(a.size, dtype=torch.float64 if a.dtype == np.float64 else torch.int32)
        t = t.pin_memory()
        arr = t.numpy().reshape(a.shape, order="F")
        arr[...] = a
        return arr

    solid_keys = ["vof", "phi", "vofS_in", "phiS", "nxS_in", "nyS_in", "vofS_u_in", "vofS_v_in"]
    geo_keys = solid_keys if solid else list(P.GEOMETRY_ARGS)
    H = {k: pinned(A[k]) for k in set(geo_keys) | {"dx", "dy", "dxU", "dyV", "DpU", "DpV",
                                                    "ustar", "vstar"}}
    hu, hv, hpp = pinned(A["u0"]), pinned(A["v0"]), pinned(A["p0"])
    hPp = pinned(np.zeros((nx + 2, ny + 2), order="F"))
    hm = pinned(np.zeros((nx, ny), order="F"))
    hs = P.ProjectionSolver(nx, ny, precision="mixed", device=local, rtol=1e-8, maxit=300)
    try:
        hs.set_stream(stream.cuda_stream)
        if schedule:
            apply_schedule(hs, schedule)
        hs.set_grid(H["dx"], H["dy"], H["dxU"], H["dyV"])
        h2d = (sum(H[k].nbytes for k in geo_keys + ["DpU", "DpV", "ustar", "vstar"]) +
               hu.nbytes + hv.nbytes + hpp.nbytes)
        d2h = hPp.nbytes + hu.nbytes + hv.nbytes + hpp.nbytes + hm.nbytes

        def step():
            if solid:
                hs.set_solid(*[H[k] for k in solid_keys])
            else:
                hs.set_geometry(**{k: H[k] for k in P.GEOMETRY_ARGS})
            hs.assemble(H["DpU"], H["DpV"], case.betaP, case.betaM, case.bc)
            _, _, st = hs.update_puv(H["ustar"], H["vstar"], hu, hv, hpp, case.vb, Pp=hPp,
                                     mres=hm)
            return st.mres_max  # the step's result (max |mres|), read on the host

        for _ in range(warmup):
            step()
        if pg:
            pg.barrier()
        torch.cuda.synchronize(dev)
        # host clock: every call returns once its outputs are in host memory
        t0 = time.perf_counter()
        for _ in range(steps):
            step()
        tot = time.perf_counter() - t0
        ms = tot / steps * 1e3
        if pg:
            ms = reduce_max(ms, pg, dev)
        return {"value": round(ms, 4), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h),
                "out": {"Pp": hPp.copy(order="F"), "u": hu.copy(order="F"),
                        "v": hv.copy(order="F")}}
    finally:
        hs.close()


def extra_c4_eval(local, args, threads):
    """The learned preconditioner's evaluation on unseen instances of the
    fourth configuration (1024^2 and 4096^2, uniform grids, density ratio
    log-uniform in [10,1000]): learned + mixed against the mixed V-cycle and
    the plain FP64 arm, each with its error against the FP64 oracle."""
    import torch
    from gen import synth
    out = {"workload": "unseen c4 instances (0-4 circles r U(0.03,0.12), surface amplitude "
                       "U(0,0.05) wavenumber 1-6, density ratio log-U[10,1000], 16 u* modes), "
                       "FP64 relres 1e-8"}
    dev = torch.device("cuda", local)
    for n, inst in ((1024, 1001), (4096, 1002)):
        case = synth.c4(n=n, instance=inst)
        t = _tdev(case, dev)
        row = {"ratio": round(case.meta["ratio"], 2), "circles": case.meta["ncirc"]}
        ref = None
        if not args.no_cpu:
            _, ref = cpu_projection(case, threads, rtol=1e-12)
            row["oracle_relres"] = ref["relres"]
        for name, prec, pre in (("mixed", "mixed", "mg"), ("learned_mixed", "mixed", "learned"),
                                ("plain_fp64", "fp64", "mg")):
            a = device_arm(case, t, local, prec, steps=3, warmup=1, precond=pre, tune=False,
                           kernels=False)
            r = {"ms": round(a["ms"], 3), "iters": a["iters"][-1],
                 "relres_true": a["relres"][-1]}
            if pre == "learned":
                r["learned_iters"] = a["learned_iters"][-1]
                r["fallback_to_vcycle"] = bool(a["fallbacks"])
            if ref is not None:
                r["err_vs_fp64_oracle"] = errors_vs(a["out"], ref)
            row[name] = r
        out[f"{n}x{n}"] = row
        del t
        torch.cuda.empty_cache()
    return out


def extra_batch(local, args, threads):
    """64 uneven instances in one graph launch with autotuned schedules and
    sweep tiles, with every instance's error against the FP64 oracle."""
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
        res = {"workload": "64 instances, sides 256..1024 (log-uniform, multiples of 32), "
                           "density ratio log-U[10,1000], 0-4 circles, 16-mode u*, dt 1e-3",
               "cells": int(sum(c.nx * c.ny for c in cases)), "ms_per_batch": round(ms, 3),
               "solves_per_s": round(64 / (ms * 1e-3), 1),
               "iters_min_max": [min(x["iters"] for x in st), max(x["iters"] for x in st)],
               "max_relres_true": max(x["relres_true"] for x in st),
               "launch": "one CUDA graph (64 branches, conditional-while PCG per branch)",
               "autotune": json.loads(bp.table_json())}
        if not args.no_cpu:
            O = _oracle()
            O.lib().oracle_set_threads(threads)
            errs = []
            for i, c in enumerate(cases):
                ref = O.project_mg(c, rtol=1e-12, maxit=500)
                e = errors_vs(bp.result(i), ref)
                errs.append({"side": c.nx, "ratio": round(c.meta["ratio"], 1),
                             "iters": st[i]["iters"], "p": float(f"{e['p_rel_l2']:.3e}"),
                             "uv": float(f"{max(e['u_rel_l2'], e['v_rel_l2']):.3e}")})
            res["per_instance_err_vs_fp64_oracle"] = errs
            res["max_err_p"] = max(x["p"] for x in errs)
            res["max_err_uv"] = max(x["uv"] for x in errs)
        return res
    finally:
        bp.close()


def extra_c2(local, args, threads, peak):
    """The 2048^2 configuration (uniform grid, point smoother): mixed and
    plain FP64, device-resident, with errors against the FP64 oracle."""
    import torch
    case = make_case("c2", 0)
    dev = torch.device("cuda", local)
    t = _tdev(case, dev)
    out = {"workload": WORKLOADS["c2"]}
    ref = None
    if not args.no_cpu:
        _, ref = cpu_projection(case, threads, rtol=1e-12)
    for name, prec in (("mixed", "mixed"), ("plain_fp64", "fp64")):
        a = device_arm(case, t, local, prec, steps=max(3, min(args.steps, 10)), warmup=3)
        r = {"ms": round(a["ms"], 4), "iters": a["iters"][-1], "relres_true": a["relres"][-1],
             "schedule": a["schedule"], "kernels": kernel_table(a, prec, case.nx * case.ny, peak)}
        if ref is not None:
            r["err_vs_fp64_oracle"] = errors_vs(a["out"], ref)
        out[name] = r
    out["speedup_mixed_vs_plain"] = round(out["plain_fp64"]["ms"] / out["mixed"]["ms"], 3)
    return out, case


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
    # the multigrid preconditioner (SCF_MOM_MG) against the diagonal: on this
    # workload (Re 1e5) and where diffusion dominates (Re 0.01, the u solve)
    mg = {}
    for rey, comps in ((1.0e5, ("u", "v")), (0.01, ("u",))):
        mi_r = {c: synth.momentum_inputs(case, c, rey=rey) for c in comps}
        for prec in ("diagonal", "multigrid"):
            sm = M.MomentumSolver(case.nx, case.ny, device_ptrs=True, device=local,
                                  mg=prec == "multigrid")
            try:
                ti = {c: {k: (T(v) if isinstance(v, np.ndarray) else v) for k, v in mi.items()}
                      for c, mi in mi_r.items()}
                best, sts = None, []
                for rep in range(3):
                    sts = []
                    w = {c: (T(mi["pred"]), T(mi["Dp"])) for c, mi in mi_r.items()}
                    torch.cuda.synchronize(dev)
                    t0 = time.perf_counter()
                    for c in comps:
                        sts.append(sm.solve(c, ti[c], w[c][0], w[c][1], rtol=1e-10,
                                            maxit=20000))
                    torch.cuda.synchronize(dev)
                    ms_r = (time.perf_counter() - t0) * 1e3
                    best = ms_r if best is None else min(best, ms_r)
            finally:
                sm.close()
            mg[f"re_{rey:g}_{prec}"] = {"components": list(comps), "ms": round(best, 2),
                                        "iters": [st.iters for st in sts],
                                        "relres": [st.relres for st in sts]}
    out["preconditioners_rtol_1e-10"] = mg
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
    """The CLSVOF transport on the headline grid with device-resident fields:
    one whole Coupled_LS_VOF step (six sub-steps: reconstruction, both
    sweeps, the updates, Redistance) on a drop beside a solid wall, its
    parts, and the sweeps on an every-cell-an-interface stress case;
    against the C restatement on one core."""
    import torch
    from simcoflow_gb300 import clsvof as CL
    from gen.synth import clsvof_step_fields, ls_fields, vof_fields, wave_inlet
    nx, ny = case.nx, case.ny
    dev = torch.device("cuda", local)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).to(dev)
    f, vof, phi, dt, wave = clsvof_step_fields(np.random.default_rng(33), nx, ny)
    tf = {k: T(a) for k, a in f.items()}
    z = lambda: torch.zeros(nx * ny, dtype=torch.float64, device=dev)
    out = {k: z() for k in ("nxv", "nyv", "dis")}

    def step():
        tv, tp = T(vof), T(phi)
        torch.cuda.synchronize(dev)
        return CL.clsvof_step(nx, ny, tf, dt, tv, tp, wave=wave, out=out, device_ptrs=True,
                              device=local)[2]
    for _ in range(2):
        step()
    reps = 5
    ms_step = sorted(step() for _ in range(reps))[reps // 2]
    # the parts, on the step's starting fields
    irf = {k: tf[k] for k in ("vofS", "nxs", "nys", "phiS", "x", "y", "dx", "dy")}
    irf.update({"vof": T(vof), "phi": T(phi)})
    rec = {k: z() for k in ("nxv", "nyv", "dis")}
    ms_ir = sorted(CL.interface_reconstruct(nx, ny, irf, out=rec, device_ptrs=True,
                                            device=local)[2] for _ in range(reps))[reps // 2]
    sf = dict(tf)
    sf["phi"] = irf["phi"]
    vf = {"vof": irf["vof"], "nxv": rec["nxv"], "nyv": rec["nyv"], "dis": rec["dis"],
          "nxs": tf["nxs"], "nys": tf["nys"], "phiS": tf["phiS"]}
    tv, tl = T(vof), T(phi)
    ms_sw = []
    for _ in range(reps):
        a = CL.clsvof_sweep(CL.X, nx, ny, sf, vf, dt / 6, tv, temls=tl,
                            wave=list(wave) + [1], device_ptrs=True, device=local)
        b = CL.clsvof_sweep(CL.Y, nx, ny, sf, vf, dt / 6, tv, temls=tl, device_ptrs=True,
                            device=local)
        ms_sw.append(a + b)
    rdf = dict(irf)
    rdf.update(rec)
    ms_rd = sorted(CL.redistance(nx, ny, rdf, T(phi), device_ptrs=True, device=local)[1]
                   for _ in range(reps))[reps // 2]
    # every cell an interface cell: the sweeps' worst case
    fs = ls_fields(np.random.default_rng(29), nx, ny)
    vs = vof_fields(np.random.default_rng(31), nx, ny, fs)
    tfs, tvs = {k: T(a) for k, a in fs.items()}, {k: T(a) for k, a in vs.items()}
    ttv, ttl = T(vs["vof"]), T(fs["phi"])
    ms_stress = []
    for _ in range(reps):
        a = CL.clsvof_sweep(CL.X, nx, ny, tfs, tvs, 1e-4, ttv, temls=ttl,
                            wave=wave_inlet(fs), device_ptrs=True, device=local)
        b = CL.clsvof_sweep(CL.Y, nx, ny, tfs, tvs, 1e-4, ttv, temls=ttl, device_ptrs=True,
                            device=local)
        ms_stress.append(a + b)
    out_ = {"workload": f"one Coupled_LS_VOF step (6 sub-steps, fixed solid) on {nx}x{ny}: a "
                        "drop of radius 0.25 L beside a solid half-plane, solid-body rotation, "
                        "sub-step Courant number 0.2",
            "gpu": {"ms_step": round(ms_step, 3),
                    "ms_interface_reconstruct": round(ms_ir, 3),
                    "ms_sweeps_x_plus_y": round(sorted(ms_sw)[reps // 2], 3),
                    "ms_redistance": round(ms_rd, 3),
                    "ms_sweeps_x_plus_y_every_cell_interface": round(sorted(ms_stress)[reps // 2],
                                                                     3),
                    "timing": "host clock around each C-ABI call with device pointers (each "
                              "call allocates its scratch, creates a stream and synchronises); "
                              "median of 5"}}
    if not args.no_cpu:
        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle as O
        t1 = time.perf_counter()
        O.clsvof_step(nx, ny, f, dt, vof, phi, wave)
        cpu_ms = (time.perf_counter() - t1) * 1e3
        out_["cpu"] = {"ms_step": round(cpu_ms, 1), "cores": 1, "kind": "port",
                       "sample": "the same step, the reference's loops as written (C "
                                 "restatement)"}
        out_["speedup_step_vs_cpu"] = round(cpu_ms / ms_step, 1)
    return out_


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


def _config(case, name):
    """The line's config: identical in both arms (workload and sizes only)."""
    return {"workload": WORKLOADS.get(name, name), "name": name, "nx": case.nx, "ny": case.ny,
            "l2": "inputs larger than L2 (no flush needed)"}


def cpu_reference_settings(case, threads):
    """Bounded sample of the reference's own solver settings on the CPU
    restatement: PCG with 10 V-cycles per preconditioner application
    (BoomerAMG MaxIter 10, src/ProjectionP_Mod.f90:130) and, with rtol 1e-20
    (:111), 50 iterations (:108).  After an untimed warm-up, one and three
    iterations are timed; the 50-iteration projection is projected from their
    difference."""
    O = _oracle()
    O.lib().oracle_set_threads(threads)
    O.project_mg(case, rtol=1e-20, maxit=-(10 * 1000 + 1))  # warm-up (untimed)
    t = []
    for its in (1, 3):
        t0 = time.perf_counter()
        r = O.project_mg(case, rtol=1e-20, maxit=-(10 * 1000 + its))
        t.append((time.perf_counter() - t0) * 1e3)
    per_it = (t[1] - t[0]) / 2
    return {"ms_1_iteration": round(t[0], 1), "ms_3_iterations": round(t[1], 1),
            "ms_per_iteration": round(per_it, 1),
            "ms_50_iterations_projected": round(t[0] + 49 * per_it, 1),
            "relres_after_3": r["relres"], "cores": threads,
            "settings": "PCG maxit 50, rtol 1e-20, 10 V-cycles per application "
                        "(src/ProjectionP_Mod.f90:106-133); sample: 1 and 3 iterations"}


def run_reference(args):
    world, rank, local = _dist()
    if rank != 0:
        return 0
    # the generator built by the oracle's recipe: nothing of the product loads
    O = _oracle()
    import build as oracle_build  # oracle/build.py
    from gen import geometry
    geometry.use_library(oracle_build.geom_lib())
    case = make_case(args.config, 0)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_projection(case, threads)
    times, r = [], None
    for _ in range(args.steps):
        ms, r = cpu_projection(case, threads)
        times.append(ms)
    ms = float(np.mean(times))
    line = {"impl": "reference", "metric": METRIC, "value": round(ms, 3), "unit": UNIT,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms, 3), "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded; shapes and distributions of the named config)",
            "config": _config(case, args.config),
            "cpu_baseline": {"value": round(ms, 3), "unit": UNIT, "cores": threads,
                             "kind": "port",
                             "sample": f"one full {case.nx}x{case.ny} projection per step: the "
                                       f"oracle's C restatement (PoCoef, rows, RHS, FP64 "
                                       f"MG-PCG to relres 1e-8 with the {r['smoother']} "
                                       f"smoother, correction), OpenMP; the Fortran+HYPRE "
                                       f"reference is unbuildable (no Fortran compiler, MPI "
                                       f"or HYPRE)",
                             "iters": r["iters"], "relres": r["relres"]},
            "e2e": {"value": round(ms, 3), "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    del O
    return 0


def run_ours(args):
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
    P.load()
    case = make_case(args.config, rank)
    nx, ny = case.nx, case.ny
    cells = nx * ny
    stream = torch.cuda.Stream(device=dev)
    tdev = _tdev(case, dev)
    peak, peak_kind = _peaks()
    use_graph = not args.no_graph

    mixed = device_arm(case, tdev, local, "mixed", steps=args.steps, warmup=args.warmup,
                       tune=not args.no_tune, sample_clocks=True, stream=stream,
                       use_graph=use_graph, pg=pg)
    plain = device_arm(case, tdev, local, "fp64", steps=args.steps, warmup=args.warmup,
                       tune=not args.no_tune, stream=stream, use_graph=use_graph, pg=pg)
    learned = None
    if not args.no_learned:
        learned = device_arm(case, tdev, local, "mixed", precond="learned",
                             steps=max(1, min(args.steps, 5)), warmup=1,
                             schedule=mixed["schedule"], stream=stream, use_graph=use_graph,
                             pg=pg, kernels=False)
    del tdev
    torch.cuda.empty_cache()
    e2e = e2e_arm(case, local, stream, steps=args.steps, warmup=args.warmup,
                  schedule=mixed["schedule"], pg=pg)
    e2e_solid = e2e_arm(case, local, stream, steps=args.steps, warmup=args.warmup,
                        schedule=mixed["schedule"], pg=pg, solid=True)
    if rank != 0:
        if pg:
            pg.destroy_process_group()
        return 0

    # roofline: the dominant kernel of the headline path, timed live (CUDA
    # events around 50 back-to-back launches on the solver's stream, same
    # data) right after the timed region
    dkey, dname, ddesc = DOMINANT[mixed["smoother"]]
    roof = None
    if dkey in mixed["kt"] and mixed["kt"][dkey] > 0:
        bytes_launch = KERNEL_BYTES["mixed"][dkey] * cells
        achieved = bytes_launch / (mixed["kt"][dkey] * 1e-3) / 1e9
        roof = {"bound": "hbm", "kernel": dname, "what": ddesc,
                "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": f"{peak_kind} (hbm_gbs)",
                "bytes_per_launch": bytes_launch,
                "bytes_model": f"{KERNEL_BYTES['mixed'][dkey]} B per fine cell "
                               "(compulsory: each element the launch touches once)",
                "ms_per_launch": round(mixed["kt"][dkey], 5),
                "traffic": None,
                "traffic_profile": TRAFFIC_PROFILE.get((args.config, dkey)),
                "kernel_timing": "CUDA events around 50 back-to-back launches on the solver "
                                 "stream after the timed region, same data"}
    threads = os.cpu_count() or 1
    cpu = err = ref_settings = None
    if world == 1 and not args.no_cpu:
        ms_cpu, rc = cpu_projection(case, threads)
        cpu = {"value": round(ms_cpu, 1), "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"one full {nx}x{ny} projection (the oracle's C restatement: PoCoef, "
                         f"rows, RHS, FP64 MG-PCG to relres 1e-8 with the {rc['smoother']} "
                         f"smoother ({rc['iters']} iterations), correction; OpenMP)"}
        # the FP64 oracle solve every result's error is stated against
        # (checker only; outside every timed region)
        _, ref = cpu_projection(case, threads, rtol=1e-12)
        err = {"oracle": f"C restatement, FP64 MG-PCG to relres {ref['relres']:.1e} "
                         f"({ref['iters']} iterations)",
               "mixed": errors_vs(mixed["out"], ref), "plain_fp64": errors_vs(plain["out"], ref),
               "e2e": errors_vs(e2e["out"], ref), "e2e_gpu_geometry": errors_vs(e2e_solid["out"],
                                                                                 ref)}
        if learned:
            err["learned_mixed"] = errors_vs(learned["out"], ref)
        if not args.no_ref_settings:
            ref_settings = cpu_reference_settings(case, threads)
    extras = {}
    if world == 1 and not args.no_extras:
        c2line = None

        def c2():
            nonlocal c2line
            r, c2line = extra_c2(local, args, threads, peak)
            return r
        steps = [("c2_2048", c2),
                 ("c4_eval", lambda: extra_c4_eval(local, args, threads)),
                 ("batch_64", lambda: extra_batch(local, args, threads)),
                 ("momentum_2048", lambda: extra_momentum(c2line, local, args)),
                 ("tecplot_2048", lambda: extra_tecplot(c2line, local, args)),
                 ("vtr_2048", lambda: extra_vtr(c2line, local, args)),
                 ("clsvof_step_2048", lambda: extra_lsweep(c2line, local, args)),
                 ("cutcell_2048", lambda: extra_cutcell(c2line, local, args))]
        for name, fn in steps:
            try:
                extras[name] = fn()
            except Exception as e:  # an extra must not hide the headline line
                extras[name] = {"error": f"{type(e).__name__}: {e}"}
            torch.cuda.empty_cache()
    ms_step = mixed["ms"]

    def arm_line(a, prec):
        return {"ms": round(a["ms"], 4), "iters": a["iters"][-1], "relres_true": a["relres"][-1],
                "schedule": a["schedule"], "smoother": a["smoother"],
                "kernels": kernel_table(a, prec, cells, peak)}
    line = {
        "metric": METRIC, "value": round(ms_step, 4), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 4),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64+f32/bf16",
        "precision": "FP64 outer PCG (operator, residuals, dot products, alpha/beta, true "
                     "residual, correction); FP32 multigrid iterate with BF16 couplings "
                     "rescaled per level; FP64 coarsest solve",
        "data": "synthetic (seeded; shapes and distributions of the named config)",
        "config": _config(case, args.config),
        "path": "mixed: FP64 flexible PCG + FP32/BF16 multigrid V-cycle "
                f"({mixed['smoother']} smoother), one CUDA graph with a conditional while "
                "node" if use_graph else "direct launches",
        "parallelism": f"replicas x{world}",
        "solves_per_s": round(1e3 * world / ms_step, 2),
        "iters": mixed["iters"][-1], "relres_true": mixed["relres"][-1],
        "levels": mixed["levels"], "asym_faces": mixed["asym_faces"],
        "schedule": {"npre_npost_omega": mixed["schedule"],
                     "source": "autotuner (simcoflow_gb300.batch.SCHEDULES; TILES for the "
                               "point smoother; the coarse levels' schedule, [first level, "
                               "sweeps], from bench.LINE_COARSE / POINT_COARSE), per arm"},
        "plain_fp64_mg_pcg": arm_line(plain, "fp64"),
        "speedup_vs_plain_fp64": round(plain["ms"] / ms_step, 3),
        "e2e": {k: v for k, v in e2e.items() if k != "out"},
        "e2e_gpu_geometry": {**{k: v for k, v in e2e_solid.items() if k != "out"},
                             "path": "scf_proj_set_solid: Grid_Preprocess's derived geometry "
                                     "computed on the GPU from the solid level-set fields"},
        "roofline": roof, "kernels": kernel_table(mixed, "mixed", cells, peak),
        "gpu_launches": int(sum(mixed["launches"])), "cpu_baseline": cpu,
        "cpu_reference_settings": ref_settings, "clocks": mixed["clk"],
        "err_vs_fp64_oracle": err, **extras,
    }
    if learned:
        line["learned_mixed"] = {"ms": round(learned["ms"], 4), "iters": learned["iters"][-1],
                                 "learned_iters": learned["learned_iters"][-1],
                                 "fallback_to_vcycle": bool(learned["fallbacks"]),
                                 "relres_true": learned["relres"][-1],
                                 "speedup_vs_plain_fp64": round(plain["ms"] / learned["ms"], 3)}
        try:
            line["unet_forward"] = unet_forward_times()
        except Exception as e:  # must not hide the headline line
            line["unet_forward"] = {"error": f"{type(e).__name__}: {e}"}
    print(json.dumps(line), flush=True)
    if pg:
        pg.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", default="c3")
    ap.add_argument("--no-cpu", action="store_true",
                    help="skip the CPU baseline and the oracle error statements")
    ap.add_argument("--no-ref-settings", action="store_true",
                    help="skip the CPU sample of the reference's 10-cycle solver settings")
    ap.add_argument("--no-tune", action="store_true",
                    help="default V-cycle schedule instead of the autotuned one")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned + mixed arm")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the 2048^2, c4 evaluation, batch and file-format lines")
    ap.add_argument("--no-graph", action="store_true",
                    help="launch the same kernels one by one instead of through the CUDA graph "
                         "(profilers cannot see kernel nodes of graphs with conditional nodes)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
