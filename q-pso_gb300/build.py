"""Build the sm_103a shared library ``_build/libqpso_gb300.so`` in-tree.

nvcc compiles the translation units in parallel with -gencode
arch=compute_103a,code=sm_103a only, --fmad=false (the arithmetic contract
of the fused kernels: one IEEE rounding per operation, fma only where the
source writes one) and -lineinfo for the profiler.  The command-line
drop-in ``_build/qpso_main`` (cli/qpso_main.cpp) links the library through
its C ABI only.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIB = os.path.join(BUILD, "libqpso_gb300.so")
CLI_SRC = os.path.join(HERE, "cli", "qpso_main.cpp")
CLI = os.path.join(BUILD, "qpso_main")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "--fmad=false", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
         "-I", INCLUDE, "-I", CSRC]
UNITS = ["qpso_kernels.cu", "qpso_api.cu", "qpso_noalloc.cu", "qpso_segment.cu", "qpso_seg_front.cu",
         "ingest.cpp"]
# the host code of these units computes float expressions that must round
# like the oracle's (or the reference's) on every host: no fused
# multiply-add on Arm either
UNIT_FLAGS = {"qpso_segment.cu": ["-Xcompiler", "-ffp-contract=off"],
              "qpso_api.cu": ["-Xcompiler", "-ffp-contract=off"],
              "qpso_seg_front.cu": ["-Xcompiler", "-ffp-contract=off"]}
HEADERS = ["qpso_device.cuh", "qpso_internal.cuh", "qpso_checks.h", "meshlets.h"]


def _sources():
    return [os.path.join(CSRC, u) for u in UNITS] + [os.path.join(CSRC, h) for h in HEADERS] + [
        os.path.join(INCLUDE, "qpso.h")]


def up_to_date() -> bool:
    if not os.path.exists(LIB) or not os.path.exists(CLI):
        return False
    t = min(os.path.getmtime(LIB), os.path.getmtime(CLI))
    return all(os.path.getmtime(s) <= t for s in _sources() + [CLI_SRC])


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)

    def compile_unit(u):
        obj = os.path.join(BUILD, os.path.splitext(u)[0] + ".o")
        cmd = [NVCC, *ARCH, *FLAGS, *UNIT_FLAGS.get(u, []), "-c", os.path.join(CSRC, u), "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s" % (u, r.stderr))
        if verbose:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-lpthread", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s" % r.stderr)
    os.replace(tmp, LIB)
    tmp = CLI + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O2", "-std=c++17", "-I", INCLUDE, CLI_SRC, "-o", tmp, "-L", BUILD, "-lqpso_gb300",
           "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("cli build failed:\n%s" % r.stderr)
    os.replace(tmp, CLI)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
