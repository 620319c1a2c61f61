"""Builds ``libmacsav.so`` (the CUDA library behind include/macsav.h) in tree.

Every translation unit is compiled for sm_103a only, in parallel, then linked
into one shared library next to this file.  Objects go to ``_build/``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess

PKG = pathlib.Path(__file__).resolve().parent
ROOT = PKG.parent
SRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = PKG / "libmacsav.so"
UNITS = ["plan", "stokes", "ops", "step", "capi", "static_reduce", "unet", "channel", "tgemm"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--diag-suppress=177",
         f"-I{ROOT / 'include'}"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and pathlib.Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmacsav.so")


def _sources_newer(target: pathlib.Path) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    deps = list(SRC.glob("*.cu")) + list(SRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h"))
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> pathlib.Path:
    if not force and not _sources_newer(LIB):
        return LIB
    OUT.mkdir(exist_ok=True)
    cc = nvcc()

    def compile_unit(name: str) -> pathlib.Path:
        obj = OUT / f"{name}.o"
        cmd = [cc, *ARCH, *FLAGS, "-c", str(SRC / f"{name}.cu"), "-o", str(obj)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}.cu:\n{res.stderr}")
        if verbose and res.stderr.strip():
            print(res.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as pool:
        objs = list(pool.map(compile_unit, UNITS))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
