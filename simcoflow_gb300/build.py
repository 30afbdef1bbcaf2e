"""Build the native libraries of simcoflow_gb300 in-tree.

libscf_proj.so  CUDA kernels + C-ABI (include/scf_proj.h), sm_103a only

Objects and libraries go to simcoflow_gb300/_lib/ (git-ignored).  Each CUDA
translation unit is compiled in its own nvcc process, in parallel.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIB = PKG / "_lib"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["scf_kernels.cu", "scf_mg.cu", "scf_line.cu", "scf_unet.cu", "scf_unet_tc.cu",
                "scf_proj.cu",
                "scf_noalloc.cu", "scf_mom.cu", "scf_geom.cu", "scf_out.cu", "scf_cutcell.cu",
                "scf_clsvof.cu"]
# per-file flags: the cut-cell geometry and the level-set sweeps restate the
# reference's expressions with every multiply and add rounded on its own (no
# FMA contraction)
EXTRA_FLAGS = {"scf_cutcell.cu": ["-fmad=false"], "scf_clsvof.cu": ["-fmad=false"]}


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libscf_proj.so")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_proj(force: bool = False, verbose: bool = False) -> Path:
    LIB.mkdir(exist_ok=True)
    out = LIB / "libscf_proj.so"
    headers = list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    objs, jobs = [], []
    for src in CUDA_SOURCES:
        s = CSRC / src
        o = LIB / (Path(src).stem + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   *EXTRA_FLAGS.get(src, []), "-I", str(INCLUDE), "-c", str(s), "-o", str(o)]
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(_run, jobs))
    if force or jobs or _stale(out, objs):
        _run([nvcc(), *ARCH, "-shared", "-o", str(out), *map(str, objs), "-lcudart"])
    return out


def build_all(force: bool = False) -> None:
    build_proj(force)


if __name__ == "__main__":
    import sys
    build_all(force="--force" in sys.argv)
    print("built", sorted(p.name for p in LIB.glob("*.so")))
