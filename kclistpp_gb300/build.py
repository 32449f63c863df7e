"""Builds libkclpp.so (CUDA kernels for sm_103a + the C ABI) in-tree.

    python kclistpp_gb300/build.py            # library + drop-in programs
    python kclistpp_gb300/build.py --force    # rebuild everything

Translation units compile in parallel; objects go to kclistpp_gb300/_build/,
the library to kclistpp_gb300/libkclpp.so and the drop-in command-line
programs to kclistpp_gb300/bin/.  Host code is compiled with
-ffp-contract=off so that no floating-point multiply-add is fused (the
reference's FP64 results are reproduced operation by operation).
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
BIN = os.path.join(PKG, "bin")
LIB = os.path.join(PKG, "libkclpp.so")
INCLUDE = os.path.join(ROOT, "include")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CXXFLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function"]
NVCCFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                    "-Xcompiler", "-fPIC,-ffp-contract=off", "-I" + INCLUDE]

CU_SOURCES = ["kclpp_api.cu", "kclpp_k_count.cu", "kclpp_k_order.cu", "kclpp_k_seq.cu", "kclpp_warm.cu", "kclpp_sample.cu", "kclpp_peel.cu"]
CPP_SOURCES = ["kclpp_gen.cpp", "kclpp_order.cpp", "kclpp_trim.cpp", "kclpp_state.cpp", "kclpp_exact.cpp",
               "kclpp_certify.cpp"]
PROGRAMS = ["kCDensestNoAtom", "kCDensestCmpSync", "kClistCoreTrim", "NormalGraphCoreTrim", "kCDensestSamplingKclistpp"]


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _headers() -> list[str]:
    hs = [os.path.join(INCLUDE, "kclpp.h")]
    for f in os.listdir(CSRC):
        if f.endswith((".h", ".cuh")):
            hs.append(os.path.join(CSRC, f))
    return hs


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _compile(src: str, force: bool) -> str:
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src + ".o")
    if force or _newer(obj, [path] + _headers()):
        if src.endswith(".cu"):
            _run([NVCC] + NVCCFLAGS + ["-c", path, "-o", obj])
        else:
            _run(["g++"] + CXXFLAGS + ["-I" + INCLUDE, "-c", path, "-o", obj])
    return obj


def build(force: bool = False, jobs: int | None = None, programs: bool = True) -> str:
    """Compile the library (and the drop-in programs); returns the library path."""
    if not os.path.exists(NVCC):
        raise RuntimeError(f"nvcc not found at {NVCC}")
    os.makedirs(BUILD, exist_ok=True)
    srcs = CU_SOURCES + CPP_SOURCES
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, force), srcs))
    if force or _newer(LIB, objs):
        tmp = LIB + ".tmp"
        _run([NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"])
        os.replace(tmp, LIB)
    if programs:
        os.makedirs(BIN, exist_ok=True)
        for p in PROGRAMS:
            src = os.path.join(CSRC, "cli", p + ".c")
            out = os.path.join(BIN, p)
            if os.path.exists(src) and (force or _newer(out, [src, LIB, os.path.join(INCLUDE, "kclpp.h")])):
                _run(["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-I" + INCLUDE, src, "-o", out,
                      "-L" + PKG, "-lkclpp", "-Wl,-rpath," + PKG, "-lm"])
    return LIB


def clean() -> None:
    for p in (BUILD, BIN):
        shutil.rmtree(p, ignore_errors=True)
    if os.path.exists(LIB):
        os.remove(LIB)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--clean", action="store_true")
    ap.add_argument("-j", type=int, default=None)
    a = ap.parse_args()
    if a.clean:
        clean()
        sys.exit(0)
    print(build(force=a.force, jobs=a.j))
