"""Builds librsx.so (CUDA kernels + C ABI) and the calc_saxs CLI in-tree.

Every CUDA translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, with nvcc; host
C++ files go through nvcc as well so they see the CUDA runtime headers.
Outputs: ``resaxs_gb300/librsx.so`` and ``resaxs_gb300/bin/calc_saxs``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
CLI = os.path.join(PKG, "cli")
OUT_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "librsx.so")
BIN_DIR = os.path.join(PKG, "bin")
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"

CUDA_SOURCES = ["debye_kernels.cu", "chain_kernels.cu", "adjoint_kernels.cu", "grid_kernels.cu", "sasa_kernels.cu", "batch_kernels.cu", "calib_kernels.cu",
                "noalloc_kernels.cu"]
HOST_SOURCES = ["rsx_common.cpp", "rsx_debye.cpp", "rsx_sasa.cpp", "rsx_batch.cpp",
                "rsx_ff.cpp", "rsx_autotune.cpp",
                "rsx_pdb.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: librsx needs the CUDA 13 toolkit to build")


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
    cmd = [nvcc(), GENCODE, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
           "-I", os.path.join(ROOT, "include"), "-I", CSRC, *extra, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def existing(names, folder):
    return [os.path.join(folder, n) for n in names if os.path.exists(os.path.join(folder, n))]


def build_library(verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    jobs = [(s, ["-Xptxas", "-warn-spills"]) for s in existing(CUDA_SOURCES, CSRC)]
    jobs += [(s, ["-x", "cu"]) for s in existing(HOST_SOURCES, CSRC)]
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(lambda j: _compile(*j), jobs))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), GENCODE, "-shared", "-Xcompiler", "-fPIC", *objs, "-o", tmp,
           "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


def build_cli(verbose: bool = False) -> str | None:
    src = os.path.join(CLI, "calc_saxs.cpp")
    if not os.path.exists(src):
        return None
    os.makedirs(BIN_DIR, exist_ok=True)
    exe = os.path.join(BIN_DIR, "calc_saxs")
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), src,
           "-o", exe, f"-L{PKG}", "-lrsx", "-Wl,-rpath,$ORIGIN/..", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"CLI build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print("built", exe)
    return exe


def build_all(verbose: bool = False) -> None:
    build_library(verbose)
    build_cli(verbose)


if __name__ == "__main__":
    build_all(verbose=True)
    sys.exit(0)
