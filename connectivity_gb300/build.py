"""In-tree build of libgbconn.so, the scc/cc executables and the CPU oracle.

CUDA sources are compiled for sm_103a only (GB300); translation units are
compiled in parallel.  Outputs:
    connectivity_gb300/libgbconn.so
    connectivity_gb300/bin/scc, connectivity_gb300/bin/cc
    oracle/liboracle.so                (test infrastructure)
    oracle/_ref/ref_scc, ref_cc        (only where the reference sources are installed)
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
BIN = os.path.join(PKG, "bin")
LIB = os.path.join(PKG, "libgbconn.so")
ORACLE = os.path.join(ROOT, "oracle")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-Wall", "-Xcompiler", "-Wno-unused-function"]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-fopenmp", "-Wall", "-ffp-contract=off"]

CU_SOURCES = ["kernels.cu", "kernels_options.cu", "csr_build.cu", "api.cu", "batch.cu", "noalloc.cu", "serve.cu",
              "ingest.cu", "tune.cu", "small.cu", "afforest.cu"]
CPP_SOURCES = ["host_util.cpp"]
HEADERS = ["gb_internal.cuh", "run_device.cuh", "gen_common.h", "host_internal.h", "api_internal.h"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build_library(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(BIN, exist_ok=True)
    nvcc = _nvcc()
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "gbconn.h")]
    jobs, objs = [], []
    for s in CU_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if force or _newer(obj, [src] + hdrs):
            jobs.append([nvcc] + NVCC_FLAGS + ["-c", src, "-o", obj])
    for s in CPP_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if force or _newer(obj, [src] + hdrs):
            jobs.append(["g++"] + CXX_FLAGS + ["-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for f in [ex.submit(_run, j, verbose) for j in jobs]:
            f.result()
    if force or jobs or _newer(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lgomp"], verbose)
    for tool in ("scc", "cc"):
        src = os.path.join(CSRC, f"{tool}_main.cpp")
        exe = os.path.join(BIN, tool)
        if force or _newer(exe, [src, LIB, os.path.join(ROOT, "include", "gbconn.h")]):
            _run(["g++", "-O2", "-std=c++17", "-Wall", src, "-o", exe, "-L" + PKG, "-lgbconn",
                  "-Wl,-rpath,$ORIGIN/.."], verbose)
    return LIB


def build_oracle(verbose: bool = False, force: bool = False) -> str:
    """Test infrastructure: the C restatement and its generator, and the
    reference harness when the reference sources are installed
    (oracle/install_ref.sh into baseline/_ref/multistep, or REF_DIR)."""
    srcs = [os.path.join(ORACLE, "multistep.c"), os.path.join(ORACLE, "gen.c")]
    out = os.path.join(ORACLE, "liboracle.so")
    if force or _newer(out, srcs):
        _run(["gcc", "-O3", "-std=c11", "-fPIC", "-fopenmp", "-shared", "-Wall"] + srcs +
             ["-o", out], verbose)
    ref = os.path.join(ORACLE, "build_ref.sh")
    ref_out = os.path.join(ORACLE, "_ref", "ref_scc")
    ref_dir = os.environ.get("REF_DIR", os.path.join(ROOT, "baseline", "_ref", "multistep"))
    if os.path.isfile(os.path.join(ref_dir, "scc_main.cpp")) and (
            force or _newer(ref_out, [os.path.join(ORACLE, "ref_harness.cpp"), ref,
                                      os.path.join(ref_dir, "scc_main.cpp")])):
        _run(["sh", ref], verbose)
    return out


def build(verbose: bool = False, force: bool = False) -> None:
    build_library(verbose, force)
    build_oracle(verbose, force)


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
