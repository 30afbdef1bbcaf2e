"""Build recipe of the synthetic-input generator: gen/geometry.cpp (the
cut-cell geometry of a seeded case, in the reference's layouts) into a
shared library with g++.  build() writes gen/_lib/libscf_gen.so; the oracle's
build writes a second copy of the same source under oracle/_build for the
CPU arm of the benchmark, which loads nothing of the product."""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "_lib" / "libscf_gen.so"
SRC = HERE / "geometry.cpp"
HDR = HERE / "scf_geom.h"


def compile_to(out: Path, force: bool = False) -> Path:
    out.parent.mkdir(exist_ok=True)
    newest = max(SRC.stat().st_mtime, HDR.stat().st_mtime)
    if force or not out.exists() or out.stat().st_mtime < newest:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
               "-I", str(HERE), str(SRC), "-o", str(out)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"generator build failed:\n{r.stderr}")
    return out


def build(force: bool = False) -> Path:
    return compile_to(LIB, force)


if __name__ == "__main__":
    print(build(force=True))
