"""Builds the native library (and the CPU oracle used by the tests).

    libtreelet_rt.so   <- csrc/*.cpp (g++) + csrc/capi.cu (nvcc, sm_103a)
    oracle/liboracle_rt.so  <- oracle/oracle_rt.cpp (g++), test infrastructure
    oracle/sample_gen  <- the CPU-baseline sample writer (g++), test infrastructure

Everything is compiled in place; object files go to the package's _build/
folder.  Host code is compiled with -ffp-contract=off and device code with
--fmad=false so that no multiply-add is fused: the traversal keeps the
reference's FP32 operation order.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)            # treelet-prefetching-for-rt_gb300/
REPO = os.path.dirname(ROOT)
CSRC = os.path.join(ROOT, "csrc")
BUILD = os.path.join(ROOT, "_build")
INCLUDE = os.path.join(REPO, "include")
ORACLE_DIR = os.path.join(REPO, "oracle")
LIB_PATH = os.path.join(PKG_DIR, "libtreelet_rt.so")
ORACLE_LIB = os.path.join(ORACLE_DIR, "liboracle_rt.so")
SAMPLE_GEN = os.path.join(ORACLE_DIR, "sample_gen")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_FLAGS = ["-std=c++17", "-O3", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function"]
NVCC_FLAGS = ["-std=c++17", "-O3", "--fmad=false", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off"] + ARCH

HOST_SOURCES = ["builder.cpp", "scenes.cpp", "treelets.cpp", "partition_capi.cpp"]
CUDA_SOURCES = ["capi.cu", "noalloc.cu", "mlp.cu"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps() -> list[str]:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(INCLUDE, "treelet_rt.h"))
    return files


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}")
    if verbose and r.stdout.strip():
        print(r.stdout)


def build_library(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    deps = _deps()
    jobs = []
    objs = []
    for src in HOST_SOURCES:
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if force or _stale(obj, deps):
            jobs.append(["g++", *HOST_FLAGS, f"-I{INCLUDE}", "-c", os.path.join(CSRC, src), "-o", obj])
    for src in CUDA_SOURCES:
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if force or _stale(obj, deps):
            jobs.append([_nvcc(), *NVCC_FLAGS, f"-I{INCLUDE}", "-c", os.path.join(CSRC, src), "-o", obj])
    with ThreadPoolExecutor(max_workers=max(1, min(8, len(jobs)))) as ex:
        for f in [ex.submit(_run, j, verbose) for j in jobs]:
            f.result()
    if force or jobs or _stale(LIB_PATH, objs):
        _run([_nvcc(), "-shared", *ARCH, "-o", LIB_PATH, *objs, "-lpthread"], verbose)
    return LIB_PATH


def build_oracle(verbose: bool = False, force: bool = False) -> str:
    src = os.path.join(ORACLE_DIR, "oracle_rt.cpp")
    deps = [src, os.path.join(ORACLE_DIR, "oracle_rt.h"), os.path.join(INCLUDE, "treelet_rt.h")]
    if force or _stale(ORACLE_LIB, deps):
        _run(["g++", *HOST_FLAGS, f"-I{INCLUDE}", "-shared", "-o", ORACLE_LIB, src, "-lpthread"], verbose)
    return ORACLE_LIB


def build_sample_gen(verbose: bool = False, force: bool = False) -> str:
    """oracle/sample_gen: writes the CPU-baseline sample (scene blob and rays)
    to files for the reference's walk, without loading any shared object of
    the library (the scene and ray generators are compiled in)."""
    srcs = [os.path.join(ORACLE_DIR, "sample_gen.cpp"), os.path.join(ORACLE_DIR, "oracle_rt.cpp"),
            os.path.join(CSRC, "scenes.cpp"), os.path.join(CSRC, "builder.cpp")]
    deps = srcs + [os.path.join(ORACLE_DIR, "oracle_rt.h")] + _deps()
    if force or _stale(SAMPLE_GEN, deps):
        _run(["g++", *HOST_FLAGS, f"-I{INCLUDE}", f"-I{CSRC}", "-o", SAMPLE_GEN, *srcs, "-lpthread"], verbose)
    return SAMPLE_GEN


def build_reference_pin(verbose: bool = False) -> None:
    """Builds the checker harnesses of oracle/ref_pin (the reference's own
    decoders, geometry, treelet formation and walks, compiled in place) into
    oracle/_ref/ when the reference tree is present.  Elsewhere, when the
    extracted reference files came along in oracle/_ref/extract/, rebuilds
    the walk harness from them (the CPU baseline times it); otherwise there is
    nothing to build."""
    ref = os.environ.get("TREELET_RT_REFERENCE", "/root/reference")
    pin = os.path.join(ORACLE_DIR, "ref_pin")
    if os.path.isdir(os.path.join(ref, "src", "cuda-sim")):
        _run(["make", "-s", "-C", pin, f"REFERENCE={ref}"], verbose)
    elif os.path.exists(os.path.join(ORACLE_DIR, "_ref", "extract", "tr_walks.inc")):
        _run(["make", "-s", "-C", pin, "extracted"], verbose)


def build_all(verbose: bool = False, force: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=4) as ex:
        jobs = [ex.submit(build_library, verbose, force), ex.submit(build_oracle, verbose, force),
                ex.submit(build_sample_gen, verbose, force), ex.submit(build_reference_pin, verbose)]
        for j in jobs:
            j.result()


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB_PATH)
