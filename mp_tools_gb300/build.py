"""Builds libmpsq.so in-tree for sm_103a with nvcc (no cmake, no torch extension machinery).

The translation units compile in parallel and link against cuFFT; the result lands in
``mp_tools_gb300/_build/libmpsq.so`` next to its object files.  Rebuilding is skipped when the
library is newer than every source.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libmpsq.so"
SOURCES = ["nufft.cu", "spread_mma.cu", "job.cu", "timeaxis.cu", "dropin.cu", "maps.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
         "--expt-relaxed-constexpr"]


def nvcc() -> str:
    cand = os.environ.get("NVCC") or "/usr/local/cuda/bin/nvcc"
    return cand if Path(cand).exists() else "nvcc"


def _inputs() -> list[Path]:
    return ([CSRC / s for s in SOURCES] + sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh"))
            + [ROOT / "include" / "mpsq.h", Path(__file__)])


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _inputs())


SYNTH = BUILD / "libsynth.so"


def build_synth(force: bool = False) -> Path:
    """Host-side synthetic-workload helper (gcc, portable C, no CUDA)."""
    src = CSRC / "rsa.c"
    if not force and SYNTH.exists() and SYNTH.stat().st_mtime >= src.stat().st_mtime:
        return SYNTH
    BUILD.mkdir(parents=True, exist_ok=True)
    tmp = SYNTH.with_suffix(".so.tmp")
    r = subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-o", str(tmp), str(src), "-lm"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"gcc failed for rsa.c:\n{r.stderr}")
    os.replace(tmp, SYNTH)
    return SYNTH


def build(force: bool = False, verbose: bool = False) -> Path:
    build_synth(force)
    if not force and up_to_date():
        return LIB
    BUILD.mkdir(parents=True, exist_ok=True)
    cc = nvcc()

    def compile_one(src: str) -> Path:
        obj = BUILD / (Path(src).stem + ".o")
        cmd = [cc, *ARCH, *FLAGS, "-I", str(ROOT / "include"), "-c", str(CSRC / src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            sys.stdout.write(r.stdout + r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcufft", "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
