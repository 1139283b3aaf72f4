"""Compile the CUDA step library (lbm_gb300/_lib/liblbm_gb300.so) for sm_103a with nvcc.

Translation units compile in parallel; a unit is rebuilt only when one of the sources is newer
than its object file. The FP64 unit is compiled with -fmad=false so that no multiply-add is
fused there (the FP64 path reproduces the reference's rounding exactly).
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "_lib"
OBJDIR = LIBDIR / "obj"
LIB = LIBDIR / "liblbm_gb300.so"
DRIVER_SRC = PKG / "driver" / "lbm_gb300_run.cpp"
DRIVER = LIBDIR / "lbm_gb300_run"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
          "-Xcompiler", "-O2"]
UNITS = {
    "capi": [],
    "step_fp64": ["-fmad=false"],
    "step_fp32": [],
    "step_fp16": [],
    "step_bf16": [],
}


def nvcc() -> str:
    path = shutil.which("nvcc")
    if path:
        return path
    cand = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc"
    if cand.exists():
        return str(cand)
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblbm_gb300.so")


def _deps() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + [INCLUDE / "lbm_gb300.h"]


def _compile(name: str, extra: list[str], verbose: bool, objdir: Path = OBJDIR) -> Path:
    src = CSRC / f"{name}.cu"
    obj = objdir / f"{name}.o"
    newest = max(p.stat().st_mtime for p in _deps() + [src])
    if obj.exists() and obj.stat().st_mtime >= newest:
        return obj
    cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", str(src), "-o", str(obj)]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stdout}\n{res.stderr}")
    if verbose and res.stderr:
        print(res.stderr)
    return obj


def build(verbose: bool = False, out_dir: Path | None = None, defines: tuple = ()) -> Path:
    """Compile every translation unit (in parallel) and link liblbm_gb300.so; returns its path.
    out_dir / defines build a separately configured copy (e.g. a different block size) elsewhere."""
    objdir = OBJDIR if out_dir is None else Path(out_dir) / "obj"
    lib = LIB if out_dir is None else Path(out_dir) / "liblbm_gb300.so"
    objdir.mkdir(parents=True, exist_ok=True)
    flags = [f"-D{d}" for d in defines]
    with ThreadPoolExecutor(max_workers=len(UNITS)) as pool:
        objs = list(pool.map(lambda kv: _compile(kv[0], kv[1] + flags, verbose, objdir), UNITS.items()))
    if not lib.exists() or lib.stat().st_mtime < max(o.stat().st_mtime for o in objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(lib), *map(str, objs)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    if out_dir is None:
        build_driver(lib)
    return lib


def build_driver(lib: Path = LIB) -> Path:
    """The C++ simulation driver (config file + XML scenario -> time loop -> VTS), linked against
    the library next to it."""
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        raise RuntimeError("a C++17 compiler (g++) is required for the driver")
    deps = [DRIVER_SRC, INCLUDE / "lbm_gb300.hpp", INCLUDE / "lbm_gb300_io.hpp", INCLUDE / "lbm_gb300.h", lib]
    if DRIVER.exists() and DRIVER.stat().st_mtime >= max(p.stat().st_mtime for p in deps):
        return DRIVER
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-Wextra", "-I", str(INCLUDE), str(DRIVER_SRC), "-o", str(DRIVER),
           "-L", str(lib.parent), "-llbm_gb300", "-Wl,-rpath,$ORIGIN", "-pthread"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"driver build failed:\n{res.stdout}\n{res.stderr}")
    return DRIVER


if __name__ == "__main__":
    import sys

    print(build(verbose="-v" in sys.argv))
