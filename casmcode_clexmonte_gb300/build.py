"""Build the in-tree CUDA library ``_build/libcem_gb300.so`` for sm_103a.

The translation units of ``csrc/`` (SOURCES) are compiled in parallel with
nvcc and linked with ``nvcc -shared``; then the C++ calculator plugin is
compiled with g++ against it. No cmake. Run as
``python -m casmcode_clexmonte_gb300.build``.
"""

from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libcem_gb300.so")
SOURCES = ["cem_api.cu", "cem_launch.cu", "cem_k2.cu", "cem_k3.cu", "cem_kfcc.cu", "cem_kfcc_b.cu", "cem_learned.cu", "cem_lgroup.cu", "cem_stream.cu",
           "cem_enforce.cu", "cem_nfold.cu",
           "cem_k256a.cu", "cem_k256b.cu", "cem_kbig.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
         "-I", os.path.join(ROOT, "include")]


def _stale(target: str, deps: list) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "cem.h"))
    nvcc = os.environ.get("NVCC", "nvcc")

    def compile_one(src):
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        if force or _stale(o, [s] + headers):
            cmd = [nvcc, *ARCH, *FLAGS, "-c", s, "-o", o]
            if verbose:
                print(" ".join(cmd))
            subprocess.run(cmd, check=True)
        return o

    with ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    if force or _stale(LIB, objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)
    build_plugin(force, verbose)
    return LIB


PLUGIN_DIR = os.path.join(HERE, "plugin")
PLUGIN = os.path.join(BUILD, "libcem_plugin.so")
PLUGIN_SOURCES = ["GpuMonteCalculator.cc", "plugin_capi.cc"]


def build_plugin(force: bool = False, verbose: bool = False) -> str:
    """The C++ calculator plugin (BaseMonteCalculator adaptors and their C
    entry points) over the C ABI of ``libcem_gb300.so``, with g++."""
    srcs = [os.path.join(PLUGIN_DIR, f) for f in PLUGIN_SOURCES]
    deps = srcs + [os.path.join(ROOT, "include", "cem.h"), LIB]
    for d, _, files in os.walk(os.path.join(PLUGIN_DIR, "shim")):
        deps += [os.path.join(d, f) for f in files]
    if force or _stale(PLUGIN, deps):
        cxx = os.environ.get("CXX", "g++")
        cmd = [cxx, "-std=c++17", "-O2", "-fPIC", "-shared", "-I", os.path.join(ROOT, "include"),
               "-I", os.path.join(PLUGIN_DIR, "shim"), *srcs, "-o", PLUGIN, "-L", BUILD,
               "-lcem_gb300", "-Wl,-rpath,$ORIGIN"]
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)
    return PLUGIN


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
