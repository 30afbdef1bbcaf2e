"""Build recipe of the oracle (test infrastructure only).

Compiles oracle/scf_oracle.c (projection), oracle/mom_oracle.c (momentum
predictor solves) and oracle/out_oracle.c (Tecplot result files) into
oracle/_build/liboracle.so with gcc, and a copy of the synthetic-input
generator (gen/geometry.cpp) into oracle/_build/libgeom.so, so that the
CPU arm of the benchmark builds its inputs without loading anything of the
product package.
-ffp-contract=off keeps every multiply and add separately rounded, as in
the reference's Fortran build (mpif77 without FMA flags), so that the
restatement gives the same bits on x86-64 and aarch64.
"""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build" / "liboracle.so"
GEOM = HERE / "_build" / "libgeom.so"


def build(force: bool = False) -> Path:
    srcs = [HERE / "scf_oracle.c", HERE / "mom_oracle.c", HERE / "out_oracle.c",
            HERE / "clsvof_oracle.c"]
    OUT.parent.mkdir(exist_ok=True)
    newest = max(p.stat().st_mtime for p in srcs)
    if force or not OUT.exists() or OUT.stat().st_mtime < newest:
        cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
               *map(str, srcs), "-o", str(OUT), "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    return OUT


def geom_lib(force: bool = False) -> Path:
    """The oracle's build of the synthetic-input generator."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("_gen_build", HERE.parent / "gen" / "build.py")
    gb = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gb)
    return gb.compile_to(GEOM, force)


if __name__ == "__main__":
    print(build(force=True))
    print(geom_lib(force=True))
