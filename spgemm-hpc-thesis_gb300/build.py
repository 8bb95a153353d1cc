"""Builds libspgemm_gb300.so (the CUDA engine and its C ABI) in place.

Every translation unit is compiled by nvcc for sm_103a only, in parallel, then
linked into one shared library next to this file.  The FP64 arithmetic of the
numeric phase uses __dmul_rn / __dadd_rn; -fmad=false additionally forbids any
contraction of a multiply and an add into an FMA anywhere in the library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import platform

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OBJ = HERE / "_build" / platform.machine()  # host objects differ per architecture
LIB = HERE / "libspgemm_gb300.so"
SOURCES = ["engine.cu", "k_rowwork.cu", "k_symbolic.cu", "k_numeric.cu", "k_numeric_warp.cu", "k_numeric_alt.cu",
           "k_validate.cu", "k_transpose.cu", "mtx.cu", "noalloc.cu", "server.cu"]
HEADERS = ["spg_common.cuh", "spg_enum.cuh", "k_numeric_row.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC,-O3",
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the engine")


def _stale(target: Path, deps: list[Path]) -> bool:
    return not target.exists() or any(d.stat().st_mtime > target.stat().st_mtime for d in deps)


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> Path:
    OBJ.mkdir(parents=True, exist_ok=True)
    include = HERE.parent / "include"
    headers = [CSRC / h for h in HEADERS] + [include / "spgemm_gb300.h"]
    flags = NVCC_FLAGS + (extra_flags or [])
    jobs = []
    for src in SOURCES:
        obj = OBJ / (src + ".o")
        if force or _stale(obj, [CSRC / src, *headers]):
            jobs.append([nvcc(), *ARCH, *flags, f"-I{include}", "-c", str(CSRC / src), "-o", str(obj)])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as pool:
        for log in pool.map(run, jobs):
            if verbose and log:
                print(log, file=sys.stderr)
    objs = [OBJ / (s + ".o") for s in SOURCES]
    stamp = OBJ / "linked"
    if force or jobs or _stale(LIB, objs) or not stamp.exists() or _stale(stamp, [LIB]):
        tmp = LIB.with_suffix(".so.tmp")
        subprocess.run([nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"], check=True)
        os.replace(tmp, LIB)
        stamp.touch()
    build_synth(force)
    return LIB


SYNTH_LIB = HERE / "libspg_synth.so"


def build_synth(force: bool = False) -> Path:
    """Host-only generator library for the synthetic workloads (g++ + OpenMP)."""
    src = CSRC / "synth.cpp"
    if force or _stale(SYNTH_LIB, [src]):
        tmp = SYNTH_LIB.with_suffix(".so.tmp")
        subprocess.run(["g++", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c++17", str(src), "-o", str(tmp)],
                       check=True)
        os.replace(tmp, SYNTH_LIB)
    return SYNTH_LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
