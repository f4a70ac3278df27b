"""Build the native library and command-line tool in-tree.

Compiles ccf_gb300/csrc/*.cu and *.cpp for sm_103a with nvcc (translation
units in parallel), links ``ccf_gb300/lib/libccf_gb300.so`` (the C ABI of
include/ccf_gb300.h) and ``ccf_gb300/lib/ccf_gpu`` (the main_ccf-compatible
command line).  Objects go to ``ccf_gb300/_build``.  No cmake.
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
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libccf_gb300.so")
CLI = os.path.join(LIBDIR, "ccf_gpu")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++20", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "-Xcompiler", "-ffp-contract=off", "-I", os.path.join(ROOT, "include")]
LIB_SOURCES = ["stars.cu", "tree.cu", "fmm.cu", "fmm_check.cu", "solver.cu", "polish.cu", "engine.cu", "batch.cu", "stream.cu",
               "capi.cu",
               "noalloc.cu", "autotune.cpp", "params.cpp", "server.cpp"]


def nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _compile(src: str, verbose_ptxas: bool) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "ccf_gb300.h")]
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps) and not verbose_ptxas:
        return obj
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc(), "-x", "cu", *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj]
    if verbose_ptxas and src.endswith(".cu"):
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose_ptxas:
        sys.stderr.write(r.stderr)
    return obj


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    if force:
        for f in os.listdir(BUILD):
            os.remove(os.path.join(BUILD, f))
    srcs = [os.path.join(CSRC, s) for s in LIB_SOURCES]
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose_ptxas), srcs))
    newest = max(os.path.getmtime(o) for o in objs)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        tmp = LIB + ".tmp"
        cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    peaks_src = os.path.join(CSRC, "peaks.cu")
    peaks = os.path.join(LIBDIR, "ccf_peaks")
    if force or not os.path.exists(peaks) or os.path.getmtime(peaks) < os.path.getmtime(peaks_src):
        r = subprocess.run([nvcc(), *ARCH, "-O3", "-std=c++20", peaks_src, "-o", peaks], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"peaks build failed:\n{r.stdout}\n{r.stderr}")
    cli_src = os.path.join(CSRC, "cli.cpp")
    if os.path.exists(cli_src) and (force or not os.path.exists(CLI) or os.path.getmtime(CLI) < max(
            os.path.getmtime(LIB), os.path.getmtime(cli_src))):
        cmd = ["g++", "-std=c++20", "-O2", "-I", os.path.join(ROOT, "include"), cli_src, "-o", CLI,
               "-L", LIBDIR, "-lccf_gb300", f"-Wl,-rpath,{LIBDIR}", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"cli build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
