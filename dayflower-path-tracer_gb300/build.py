"""Builds libdfpt.so, the renderer core, in-tree for sm_103a.

The kernels are compiled twice from one source: dfpt_kernels_fast.cu (FMA contraction allowed,
the path tracer's default) and dfpt_kernels_strict.cu (-fmad=false: one rounding per float
operation, the reference kernel's arithmetic). Host code is compiled with -ffp-contract=off so
the scene compiler gives the same arrays on x86-64 and aarch64. Translation units compile in
parallel; the library lands in dfpt/libdfpt.so next to its Python binding.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
INCLUDE = HERE.parent / "include"
OUT_DIR = HERE / "dfpt"
BUILD_DIR = HERE / "_build"
LIB = OUT_DIR / "libdfpt.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
               "--expt-relaxed-constexpr", f"-I{INCLUDE}", f"-I{CSRC}"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the renderer core needs the CUDA toolkit to build")


def _units():
    nvcc = _nvcc()
    gxx = shutil.which("g++") or "g++"
    return [
        ([nvcc, *ARCH, *NVCC_COMMON, "-c", str(CSRC / "dfpt_kernels_fast.cu")], BUILD_DIR / "dfpt_kernels_fast.o"),
        ([nvcc, *ARCH, *NVCC_COMMON, "-c", str(CSRC / "dfpt_kernels_wide.cu")], BUILD_DIR / "dfpt_kernels_wide.o"),
        ([nvcc, *ARCH, *NVCC_COMMON, "-fmad=false", "-c", str(CSRC / "dfpt_kernels_strict.cu")], BUILD_DIR / "dfpt_kernels_strict.o"),
        ([nvcc, *ARCH, *NVCC_COMMON, "-c", str(CSRC / "dfpt_api.cu")], BUILD_DIR / "dfpt_api.o"),
        ([nvcc, *ARCH, *NVCC_COMMON, "-c", str(CSRC / "dfpt_noalloc.cu")], BUILD_DIR / "dfpt_noalloc.o"),
        ([nvcc, *ARCH, *NVCC_COMMON, "-c", str(CSRC / "dfpt_probe.cu")], BUILD_DIR / "dfpt_probe.o"),
        ([nvcc, *ARCH, *NVCC_COMMON, "-c", str(CSRC / "dfpt_batch.cu")], BUILD_DIR / "dfpt_batch.o"),
        ([gxx, "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", f"-I{INCLUDE}", f"-I{CSRC}", "-c",
          str(CSRC / "dfpt_scene.cpp")], BUILD_DIR / "dfpt_scene.o"),
    ]


def _sources():
    return sorted(CSRC.glob("*")) + sorted(INCLUDE.glob("*.h"))


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _sources())


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and up_to_date():
        return LIB
    BUILD_DIR.mkdir(exist_ok=True)
    procs = []
    for cmd, obj in _units():
        full = cmd + ["-o", str(obj)]
        if verbose:
            print(" ".join(full), flush=True)
        procs.append((full, subprocess.Popen(full, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    failed = []
    for full, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((full, out))
        elif verbose and out.strip():
            print(out)
    if failed:
        msg = "\n\n".join(" ".join(c) + "\n" + o for c, o in failed)
        raise RuntimeError("libdfpt build failed:\n" + msg)
    link = [_nvcc(), *ARCH, "-shared", "-o", str(LIB) + ".tmp", *[str(o) for _, o in _units()]]
    if verbose:
        print(" ".join(link), flush=True)
    res = subprocess.run(link, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("libdfpt link failed:\n" + res.stdout + res.stderr)
    os.replace(str(LIB) + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
