"""Builds libgbglioma.so in-tree with nvcc for sm_103a (no torch, no cmake).

Each translation unit compiles in parallel; rd_exact.cu and likelihood.cu get
-fmad=false so their arithmetic rounds operation by operation as the
reference's does.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libgbglioma.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
          "--expt-relaxed-constexpr"]
NOFMA = {"rd_exact.cu", "likelihood.cu", "amr.cu", "propagation.cu", "affine_chain.cu", "synthetic.cu"}
SOURCES = ["abi.cu", "rd_exact.cu", "rd_fast.cu", "likelihood.cu", "amr.cu", "amr_plan.cu", "adjoint.cu",
           "surrogate.cu", "affine.cu", "affine_chain.cu", "propagation.cu", "synthetic.cu"]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return p


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(BUILD, src.replace(".cu", ".o"))
    cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    if src in NOFMA:
        cmd.insert(1, "-fmad=false")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


CLI = os.path.join(PKG, "cli")
BIN = os.path.join(PKG, "bin")
CLI_PROGRAMS = ["gbg_brain", "gbg_likelihood"]


def build_cli() -> list[str]:
    """The file-compatible brain/likelihood programs, linked to libgbglioma.so."""
    os.makedirs(BIN, exist_ok=True)
    cxx = shutil.which("g++") or "g++"
    out = []

    def one(name):
        exe = os.path.join(BIN, name)
        # -ffp-contract=off: no fused multiply-add (GCC contracts by default on
        # Arm), so the restated initial state rounds as the reference does
        cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off",
               "-I" + os.path.join(os.path.dirname(PKG), "include"),
               os.path.join(CLI, name + ".cpp"), "-o", exe, "-L" + PKG, "-lgbglioma",
               "-Wl,-rpath,$ORIGIN/.."]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"{name} failed to build:\n{r.stderr}")
        return exe

    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        out = list(ex.map(one, CLI_PROGRAMS))
    return out


def build(verbose: bool = False, extra: list[str] | None = None) -> str:
    """Compile every kernel source and link libgbglioma.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    extra = list(extra or [])
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    build_cli()
    if verbose:
        print(f"built {LIB} and {', '.join(CLI_PROGRAMS)}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
