"""Builds libdrv_gb300.so (the C-ABI library of include/drv.h) in-tree.

Every CUDA translation unit is compiled for sm_103a only, in parallel, then
linked with the static CUDA runtime into a position-independent shared
library next to this file. `-ffp-contract=off` keeps the host-side float
parameter math independent of the host's fused multiply-add.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libdrv_gb300.so"
CLI = PKG / "drv_frame_cli"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libdrv_gb300.so")
    return cand


def sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _compile(src: Path) -> Path:
    obj = BUILD / (src.name + ".o")
    deps = [src] + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "drv.h"]
    if obj.exists() and obj.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return obj
    cmd = [nvcc(), "-c", str(src), "-o", str(obj), "-O3", "-std=c++17", "-lineinfo", *ARCH,
           "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", str(PKG.parent / "include")]
    if src.suffix == ".cu":
        cmd += ["-Xptxas", "-warn-spills"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    srcs = sources()
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, srcs))
    if LIB.exists() and LIB.stat().st_mtime >= max(o.stat().st_mtime for o in objs):
        build_cli()
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), "-shared", "-o", str(tmp), *map(str, objs), *ARCH, "-cudart", "static",
           "-Xcompiler", "-fPIC"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    build_cli()
    if verbose:
        print(f"built {LIB}")
    return LIB


def build_cli() -> Path:
    """drv_frame_cli: the C++ caller of the C ABI (cpp/drv_frame_cli.cpp),
    linked against libdrv_gb300.so next to it."""
    src = PKG / "cpp" / "drv_frame_cli.cpp"
    if CLI.exists() and CLI.stat().st_mtime >= max(src.stat().st_mtime, LIB.stat().st_mtime):
        return CLI
    tmp = CLI.with_suffix(".tmp")
    cmd = [nvcc(), "-O2", "-std=c++17", str(src), "-o", str(tmp), "-I", str(PKG.parent / "include"), "-L", str(PKG),
           "-ldrv_gb300", "-Xlinker", "-rpath,$ORIGIN", "-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"drv_frame_cli build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, CLI)
    return CLI


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
