"""Kernel micro-benchmark and profiling driver of the projection path.

Sets up one workload through the C-ABI (device-resident inputs), runs one
projection so that every work vector holds real data, then runs the
selected work inside an NVTX range named "kernels" and prints its time.  A
profiler can restrict itself to that range (ncu --nvtx --nvtx-include
"kernels/").  Work items:

  sweep, pupdate_spmv, update_xr, resid_restrict, prolong, assemble, vcycle,
  setup, line, fine_pre, fine_post
            one kernel (or the captured V-cycle / setup) launched back to
            back through scf_proj_time_kernel (line: one fine-level pass of
            the line smoother; fine_pre / fine_post: the point smoother's
            first and last fine-level launches of a V-cycle)
  projection  --reps whole projections (assembly, right-hand side, PCG,
            correction) with direct launches, no graph: the launch list of
            the path
  unet      --reps forward passes of the learned preconditioner's network on
            the workload's operator and right-hand side (shipped weights)
  cutcell   --reps GPU builds of the P, U and V cells' cut-cell geometry
            (scf_grid_preprocess) from the workload's circles, device-resident
  tecplot   --reps formattings of the P-cell Tecplot records into a device
            buffer (scf_tecplot_format)
  momentum  --reps pairs of momentum-predictor solves (u then v) on the
            workload's cells (seeded face fluxes), device-resident
  geometry  --reps GPU builds of the cut-cell geometry (scf_proj_set_solid)
            from the workload's solid level-set fields, device-resident
  clsvof    --reps Coupled_LS_VOF steps (scf_clsvof_step: six sub-steps of
            reconstruction, sweeps, updates and Redistance) on a drop beside a
            solid wall, --n cells a side (default 2048), device-resident

    python -m simcoflow_gb300.profile_kernels --config c2 --kernel sweep --precision mixed
    python -m simcoflow_gb300.profile_kernels --config c3 --n 2048 --kernel projection
"""
from __future__ import annotations

import argparse
import ctypes
import json
import time

import numpy as np

from . import projection as P
from gen import synth

KERNELS = {"sweep": (0, {"fp64": 48, "mixed": 20}), "pupdate_spmv": (1, {"fp64": 56, "mixed": 44}),
           "update_xr": (2, {"fp64": 48, "mixed": 52}),
           "resid_restrict": (3, {"fp64": 58, "mixed": 25}),
           "prolong": (4, {"fp64": 50, "mixed": 21}), "assemble": (5, {"fp64": 200, "mixed": 200}),
           "vcycle": (6, {"fp64": 0, "mixed": 0}), "setup": (7, {"fp64": 0, "mixed": 0}),
           "projection": (None, {"fp64": 0, "mixed": 0}), "unet": (None, {"fp64": 0, "mixed": 0}),
           "momentum": (None, {"fp64": 0, "mixed": 0}), "geometry": (None, {"fp64": 0, "mixed": 0}),
           "cutcell": (None, {"fp64": 0, "mixed": 0}), "tecplot": (None, {"fp64": 0, "mixed": 0}),
           "clsvof": (None, {"fp64": 0, "mixed": 0}),
           "line": (8, {"fp64": 0, "mixed": 11}), "fine_pre": (9, {"fp64": 40, "mixed": 17}),
           "fine_post": (10, {"fp64": 48, "mixed": 21})}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="c2")
    ap.add_argument("--n", type=int, default=None, help="grid side (default: the config's)")
    ap.add_argument("--kernel", default="sweep", choices=sorted(KERNELS))
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--omega", type=float, default=1.9, help="coarse-correction weight")
    ap.add_argument("--coarse", type=int, nargs=2, default=(0, 0), metavar=("LEVEL", "SWEEPS"),
                    help="line smoother: SWEEPS before / after the coarse correction from "
                         "LEVEL down (0 0: the fine schedule everywhere)")
    ap.add_argument("--engine", type=int, default=1, choices=[0, 1, 2],
                    help="unet: tcgen05 with TMA staging (1), with thread staging (2), mma.sync (0)")
    args = ap.parse_args()
    import torch
    dev = torch.device("cuda", 0)
    if args.kernel == "clsvof":
        from . import clsvof as CL
        n = args.n or 2048
        f, vof, phi, dt, wave = synth.clsvof_step_fields(np.random.default_rng(33), n, n)
        T = lambda x: torch.from_numpy(np.ascontiguousarray(x.ravel(order="F"))).to(dev)
        tf = {k: T(v) for k, v in f.items()}
        out = {k: torch.zeros(n * n, dtype=torch.float64, device=dev)
               for k in ("nxv", "nyv", "dis")}
        tv, tp = T(vof), T(phi)
        CL.clsvof_step(n, n, tf, dt, tv, tp, wave=wave, out=out, device_ptrs=True)  # warm-up
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("kernels")
        t0 = time.perf_counter()
        for _ in range(args.reps):
            CL.clsvof_step(n, n, tf, dt, tv, tp, wave=wave, out=out, device_ptrs=True)
        torch.cuda.synchronize()
        dt_ms = (time.perf_counter() - t0) / args.reps * 1e3
        torch.cuda.nvtx.range_pop()
        print(json.dumps({"kernel": "clsvof", "nx": n, "ny": n, "ms_step": dt_ms}))
        return
    c = synth.make_case(args.config, **({"n": args.n} if args.n else {}))
    t = {k: torch.from_numpy(np.ascontiguousarray(v.ravel(order="F"))).to(dev)
         for k, v in c.arrays.items() if isinstance(v, np.ndarray)}
    if args.kernel == "geometry":
        keys = ("vof", "phi", "vofS_in", "phiS", "nxS_in", "nyS_in", "vofS_u_in", "vofS_v_in")
        gs = P.ProjectionSolver(c.nx, c.ny, device_ptrs=True)
        gs.set_grid(t["dx"], t["dy"], t["dxU"], t["dyV"])
        gs.set_solid(*[t[k] for k in keys])  # warm-up
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("kernels")
        t0 = time.perf_counter()
        for _ in range(args.reps):
            gs.set_solid(*[t[k] for k in keys])
        torch.cuda.synchronize()
        dt_ms = (time.perf_counter() - t0) / args.reps * 1e3
        torch.cuda.nvtx.range_pop()
        gs.close()
        print(json.dumps({"config": args.config, "kernel": "geometry", "nx": c.nx, "ny": c.ny,
                          "ms_set_solid": dt_ms}))
        return
    if args.kernel == "cutcell":
        from . import cutcell as CU
        grids, fams = synth.cutcell_inputs(c)
        T = lambda x: torch.from_numpy(np.ascontiguousarray(x.ravel(order="F"))).to(dev)
        tg = {f: {k: T(v) for k, v in g.items()} for f, g in grids.items()}
        tf = {f: {k: T(v) for k, v in g.items()} for f, g in fams.items()}
        CU.grid_preprocess(tg, tf, nx=c.nx, ny=c.ny)  # warm-up
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("kernels")
        t0 = time.perf_counter()
        for _ in range(args.reps):
            CU.grid_preprocess(tg, tf, nx=c.nx, ny=c.ny)
        torch.cuda.synchronize()
        dt_ms = (time.perf_counter() - t0) / args.reps * 1e3
        torch.cuda.nvtx.range_pop()
        print(json.dumps({"config": args.config, "kernel": "cutcell", "nx": c.nx, "ny": c.ny,
                          "ms_grid_preprocess": dt_ms}))
        return
    if args.kernel == "tecplot":
        from . import output as Out
        rng = np.random.default_rng(17)
        f = {"x": t["x"], "y": t["y"], "p": t["ustar"], "u": t["u0"], "v": t["v0"],
             "phi": t["phi"], "vof": t["vof"], "phiS": t["phiS"], "vofS": t["vofS"],
             "mres": t["x"], "flux": torch.from_numpy(rng.standard_normal(
                 2 * (c.nx + 2) * (c.ny + 2))).to(dev), "nxS": t["nxS"], "nyS": t["nyS"]}
        body = torch.empty(15 * c.nx * c.ny * 25, dtype=torch.uint8, device=dev)
        st = torch.cuda.current_stream()
        Out.format_device("p", c.nx, c.ny, f, body, st.cuda_stream)  # warm-up
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("kernels")
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(args.reps):
            Out.format_device("p", c.nx, c.ny, f, body, st.cuda_stream)
        e1.record(st)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        ms = e0.elapsed_time(e1) / args.reps
        print(json.dumps({"config": args.config, "kernel": "tecplot", "nx": c.nx, "ny": c.ny,
                          "ms_format": ms, "text_GBps": 15 * c.nx * c.ny * 25 / (ms * 1e-3) / 1e9}))
        return
    if args.kernel == "momentum":
        from . import momentum as M
        T = lambda x: torch.from_numpy(np.ascontiguousarray(x.ravel(order="F"))).to(dev)
        mis = {cp: synth.momentum_inputs(c, cp) for cp in ("u", "v")}
        tin = {cp: {k: (T(v) if isinstance(v, np.ndarray) else v) for k, v in mi.items()}
               for cp, mi in mis.items()}
        work = {cp: (T(mi["pred"]), T(mi["Dp"])) for cp, mi in mis.items()}
        ms = M.MomentumSolver(c.nx, c.ny, device_ptrs=True)
        for cp in ("u", "v"):  # warm-up
            ms.solve(cp, tin[cp], *work[cp])
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("kernels")
        t0 = time.perf_counter()
        for _ in range(args.reps):
            sts = [ms.solve(cp, tin[cp], *work[cp]) for cp in ("u", "v")]
        torch.cuda.synchronize()
        dt_ms = (time.perf_counter() - t0) / args.reps * 1e3
        torch.cuda.nvtx.range_pop()
        ms.close()
        print(json.dumps({"config": args.config, "kernel": "momentum", "nx": c.nx, "ny": c.ny,
                          "ms_u_plus_v": dt_ms, "iters": [s.iters for s in sts]}))
        return
    direct = args.kernel == "projection"
    s = P.ProjectionSolver(c.nx, c.ny, device_ptrs=True, precision=args.precision,
                           use_graph=not direct, omega=args.omega,
                           coarse_from=args.coarse[0], coarse_sweeps=args.coarse[1])
    s.set_grid(t["dx"], t["dy"], t["dxU"], t["dyV"])
    s.set_geometry(**{k: t[k] for k in P.GEOMETRY_ARGS})
    s.assemble(t["DpU"], t["DpV"], c.betaP, c.betaM, c.bc)
    Pp = torch.zeros_like(t["p0"])
    _, st = s.poisson_equation_solver(t["ustar"], t["vstar"], c.vb, Pp=Pp)
    kid, bpc = KERNELS[args.kernel]
    bpc = bpc[args.precision]
    cells = c.nx * c.ny
    out = {"config": args.config, "kernel": args.kernel, "precision": args.precision,
           "nx": c.nx, "ny": c.ny, "solve_iters": st.iters}
    if args.kernel == "projection":
        u, v, p = t["u0"].clone(), t["v0"].clone(), t["p0"].clone()
        m = torch.zeros(cells, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("kernels")
        t0 = time.perf_counter()
        for _ in range(args.reps):
            s.assemble(t["DpU"], t["DpV"], c.betaP, c.betaM, c.bc)
            st = s.update_puv(t["ustar"], t["vstar"], u, v, p, c.vb, Pp=Pp, mres=m)[2]
        torch.cuda.synchronize()
        out["ms_per_projection"] = (time.perf_counter() - t0) / args.reps * 1e3
        torch.cuda.nvtx.range_pop()
        out["iters"] = st.iters
        s.close()
    elif args.kernel == "unet":
        from . import learned as Lr
        op = s.get_operator()
        s.close()
        params, _ = Lr.load_weights()
        h, w = (c.ny + 7) // 8 * 8, (c.nx + 7) // 8 * 8
        net = Lr.UNet(1, h, w)
        net.set_params(params)
        net.set_engine(args.engine)
        f = lambda a: torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).to(dev)
        sig = torch.zeros(1, dtype=torch.float32, device=dev)
        net.features(0, c.nx, c.ny, f(op["rhs"]), f(op["cE"]), f(op["cN"]), f(op["diag"]), sig)
        z = torch.empty((1, h, w), dtype=torch.float32, device=dev)
        net.forward(z)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("kernels")
        t0 = time.perf_counter()
        for _ in range(args.reps):
            net.forward(z)
        torch.cuda.synchronize()
        ms = (time.perf_counter() - t0) / args.reps * 1e3
        torch.cuda.nvtx.range_pop()
        net.close()
        flop = 2 * 9 * sum(ci * co / 4 ** lvl for (ci, co), lvl in zip(
            Lr.LAYERS, (0, 0, 1, 1, 2, 2, 3, 3, 2, 2, 1, 1, 0, 0))) * h * w
        out.update({"ms_per_forward": ms, "tflops": flop / (ms * 1e-3) / 1e12})
    else:
        o = ctypes.c_double(0.0)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("kernels")
        rc = P.load().scf_proj_time_kernel(s._h, kid, args.reps, ctypes.byref(o))
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        s.close()
        if rc != 0:
            raise RuntimeError(f"scf_proj_time_kernel: {rc}")
        out.update({"ms_per_launch": o.value, "bytes_per_cell": bpc,
                    "GBps": (bpc * cells / (o.value * 1e-3) / 1e9) if bpc else None})
    print(json.dumps(out))


if __name__ == "__main__":
    main()
