"""Build the engine's CUDA library (libgbsdf.so) in-tree for sm_103a.

Each translation unit compiles in its own nvcc process (in parallel), then one
link step produces ``rhizome_v24.15_gb300/gbsdf/libgbsdf.so``. Every unit is
compiled with ``-fmad=false``: the engine's bit-for-bit parity with the oracle
relies on products and sums rounding separately; kernels that want fused
multiply-adds write them explicitly.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = ROOT / "csrc"
INCLUDE = ROOT.parent / "include"
BUILD = ROOT / "_build"
LIB = PKG / "libgbsdf.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["engine.cu", "k_splat.cu", "k_parity.cu", "k_gwn.cu", "k_eikonal.cu", "k_misc.cu", "noalloc.cu", "k_learn.cu", "batch.cu", "tune.cu", "k_io.cu", "k_orient.cu", "k_iso.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgbsdf.so")


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC",
                   "-I", str(INCLUDE), "-I", str(CSRC), "--expt-relaxed-constexpr"]


def _stale(out: Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [INCLUDE / "gbsdf.h"]
    nv = nvcc()
    jobs = []
    for src in SOURCES:
        obj = BUILD / (Path(src).stem + ".o")
        if force or _stale(obj, [CSRC / src] + headers):
            jobs.append([nv, *_flags(), "-c", str(CSRC / src), "-o", str(obj)])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        list(ex.map(run, jobs))
    objs = [BUILD / (Path(s).stem + ".o") for s in SOURCES]
    if force or jobs or _stale(LIB, objs):
        run([nv, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
