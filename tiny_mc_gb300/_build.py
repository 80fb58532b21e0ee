"""In-tree build of the native parts (no cmake, no pip):

* ``tiny_mc_gb300/libtmc_gb300.so`` — the CUDA library behind ``include/tmc.h``,
  compiled for sm_103a only (``-gencode arch=compute_103a,code=sm_103a``);
* ``tiny_mc_gb300/bin/tiny_mc`` — the drop-in headless driver (C);

Translation units compile in parallel; an object is rebuilt only when a
source or header is newer than it.
"""
from __future__ import annotations

import concurrent.futures as _cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libtmc_gb300.so")
DRIVER = os.path.join(PKG, "bin", "tiny_mc")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-v",
              "-I" + INCLUDE, "-I" + CSRC]
CC_FLAGS = ["-std=c11", "-O2", "-ffp-contract=off", "-fPIC", "-Wall", "-Wextra", "-I" + INCLUDE]


def _nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str], log: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    log.append(" ".join(cmd) + "\n" + r.stdout + r.stderr)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build_library(verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    cc = sorted(glob.glob(os.path.join(CSRC, "*.c")))
    jobs = []
    objs = []
    for src in cu:
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append([_nvcc(), *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj])
    for src in cc:
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append(["gcc", *CC_FLAGS, "-c", src, "-o", obj])
    log: list[str] = []
    with _cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for f in [ex.submit(_run, j, log) for j in jobs]:
            f.result()
    if _stale(LIB, objs):
        _run([_nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lm"], log)
    os.makedirs(os.path.dirname(DRIVER), exist_ok=True)
    drv_src = os.path.join(PKG, "host", "tiny_mc.c")
    if _stale(DRIVER, [drv_src, LIB]):
        _run(["gcc", *CC_FLAGS, "-o", DRIVER, drv_src, "-L" + PKG, "-ltmc_gb300",
              "-Wl,-rpath,$ORIGIN/.."], log)
    if verbose:
        print("\n".join(log))
    return LIB


if __name__ == "__main__":
    build_library(verbose=True)
