"""Kernel micro-benchmark of the projection path.

Sets up one workload through the C-ABI (device-resident inputs), runs one
projection so that every work vector holds real data, then launches a single
kernel of the path back to back inside an NVTX range named "kernels" and
prints its time per launch and its bandwidth on compulsory bytes.  A profiler
can restrict itself to that range (ncu --nvtx --nvtx-include "kernels/").

    python -m simcoflow_gb300.profile_kernels --config c2 --kernel sweep --precision mixed
"""
from __future__ import annotations

import argparse
import ctypes
import json

import numpy as np

from . import projection as P
from . import synth

KERNELS = {"sweep": (0, {"fp64": 48, "mixed": 20}), "pupdate_spmv": (1, {"fp64": 56, "mixed": 52}),
           "update_xr": (2, {"fp64": 48, "mixed": 56}),
           "resid_restrict": (3, {"fp64": 58, "mixed": 25}),
           "prolong": (4, {"fp64": 50, "mixed": 21}), "assemble": (5, {"fp64": 200, "mixed": 200}),
           "vcycle": (6, {"fp64": 0, "mixed": 0}), "setup": (7, {"fp64": 0, "mixed": 0})}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="c2")
    ap.add_argument("--kernel", default="sweep", choices=sorted(KERNELS))
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    args = ap.parse_args()
    import torch
    dev = torch.device("cuda", 0)
    c = synth.make_case(args.config)
    t = {k: torch.from_numpy(np.ascontiguousarray(v.ravel(order="F"))).to(dev)
         for k, v in c.arrays.items() if isinstance(v, np.ndarray)}
    s = P.ProjectionSolver(c.nx, c.ny, device_ptrs=True, precision=args.precision)
    s.set_grid(t["dx"], t["dy"], t["dxU"], t["dyV"])
    s.set_geometry(**{k: t[k] for k in P.GEOMETRY_ARGS})
    s.assemble(t["DpU"], t["DpV"], c.betaP, c.betaM, c.bc)
    Pp = torch.zeros_like(t["p0"])
    _, st = s.poisson_equation_solver(t["ustar"], t["vstar"], c.vb, Pp=Pp)
    kid, bpc = KERNELS[args.kernel]
    bpc = bpc[args.precision]
    out = ctypes.c_double(0.0)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("kernels")
    rc = P.load().scf_proj_time_kernel(s._h, kid, args.reps, ctypes.byref(out))
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    s.close()
    if rc != 0:
        raise RuntimeError(f"scf_proj_time_kernel: {rc}")
    cells = c.nx * c.ny
    print(json.dumps({"config": args.config, "kernel": args.kernel, "precision": args.precision,
                      "nx": c.nx, "ny": c.ny,
                      "ms_per_launch": out.value, "bytes_per_cell": bpc,
                      "GBps": (bpc * cells / (out.value * 1e-3) / 1e9) if bpc else None,
                      "solve_iters": st.iters}))


if __name__ == "__main__":
    main()
