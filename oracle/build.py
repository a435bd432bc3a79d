"""Build recipe for the test-side checkers under oracle/.

TEST INFRASTRUCTURE ONLY.  Two shared libraries:

* ``oracle/_build/libqpso_oracle.so`` -- the scalar C restatement
  (qpso_oracle.c), built everywhere (here and on the GPU host).
* ``oracle/_ref/libqpso_refpin.so`` -- the reference's own main.h helpers
  compiled for the host CPU (ref_pin/ref_pin.cpp).  Built only where the
  reference sources are present; its outputs are frozen into
  tests/golden/ by tests/golden/make_golden.py.

and the reference's own CUDA kernels rebuilt for the GB300:

* ``oracle/_ref/ref_kernels_{ieee,fast}.cubin`` -- main.h plus the kernel
  section of main.cu (InitQPSO up to main(), main.cu:72-1195) compiled for
  sm_103a, once with IEEE arithmetic (--fmad=false, the parity build) and
  once with the reference Makefile's -use_fast_math -O3 (the timing build).
  Built only where the reference sources are present; the cubins are
  device code and travel to the GPU host, where
* ``oracle/_build/libqpso_refgpu.so`` (ref_gpu/ref_gpu.cu, this project's
  host harness, built everywhere nvcc is) loads them with the driver API.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
REFERENCE_SRC = os.environ.get("QPSO_REFERENCE_SRC", "/root/reference")
CUDA_INC = "/usr/local/cuda/include"

ORACLE_SO = os.path.join(BUILD, "libqpso_oracle.so")
REFPIN_SO = os.path.join(REF_OUT, "libqpso_refpin.so")


def _newer(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build_oracle(force: bool = False) -> str:
    src = [os.path.join(HERE, "qpso_oracle.c"), os.path.join(HERE, "qpso_oracle.h")]
    if not force and _newer(ORACLE_SO, src):
        return ORACLE_SO
    os.makedirs(BUILD, exist_ok=True)
    tmp = ORACLE_SO + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off",
           "-fno-fast-math", "-fopenmp", src[0], "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_ref_pin(force: bool = False) -> str | None:
    main_h = os.path.join(REFERENCE_SRC, "main.h")
    if not os.path.exists(main_h):
        return None
    src = [os.path.join(HERE, "ref_pin", "ref_pin.cpp"), main_h]
    if not force and _newer(REFPIN_SO, src):
        return REFPIN_SO
    os.makedirs(REF_OUT, exist_ok=True)
    tmp = REFPIN_SO + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O1", "-std=c++14", "-fPIC", "-shared", "-ffp-contract=off", "-w",
           "-I", os.path.join(HERE, "ref_pin", "stubs"), "-I", REFERENCE_SRC,
           "-I", CUDA_INC, "-DdeviceOverlap=asyncEngineCount", src[0], "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, REFPIN_SO)
    return REFPIN_SO


REF_CUBINS = {"ieee": os.path.join(REF_OUT, "ref_kernels_ieee.cubin"),
              "fast": os.path.join(REF_OUT, "ref_kernels_fast.cubin")}
REFGPU_SO = os.path.join(BUILD, "libqpso_refgpu.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _kernel_section(main_cu: str) -> str:
    """main.cu from the InitQPSO kernel up to (not including) main():
    every kernel of the path and nothing of the OpenCV host program."""
    lines = open(main_cu).read().splitlines(keepends=True)
    start = next(i for i, l in enumerate(lines) if l.startswith("__global__ void InitQPSO("))
    end = next(i for i, l in enumerate(lines) if l.startswith("int main("))
    return "".join(lines[start:end])


def _kernel_first_line(main_cu: str) -> int:
    lines = open(main_cu).read().splitlines()
    return 1 + next(i for i, l in enumerate(lines) if l.startswith("__global__ void InitQPSO("))


def build_ref_cubins(force: bool = False) -> dict | None:
    main_cu = os.path.join(REFERENCE_SRC, "main.cu")
    main_h = os.path.join(REFERENCE_SRC, "main.h")
    if not (os.path.exists(main_cu) and os.path.exists(main_h)):
        return None
    prelude = os.path.join(HERE, "ref_gpu", "prelude.cuh")
    deps = [main_cu, main_h, prelude, os.path.abspath(__file__)]
    if not force and all(_newer(c, deps) for c in REF_CUBINS.values()):
        return REF_CUBINS
    os.makedirs(REF_OUT, exist_ok=True)
    # the translation unit exists only while nvcc runs; kernels get C
    # linkage so that the harness finds them by their plain names
    gen = os.path.join(REF_OUT, "ref_kernels_gen%d.cu" % os.getpid())
    with open(gen, "w") as fp:
        fp.write('#include "prelude.cuh"\n#include "handle_error.h"\n#include "main.h"\n'
                 'extern "C" {\n#line %d "main.cu"\n' % _kernel_first_line(main_cu))
        fp.write(_kernel_section(main_cu))
        fp.write("\n}\n")
    flags = {"ieee": ["-O3", "--fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"],
             "fast": ["-O3", "-use_fast_math"]}
    try:
        for kind, out in REF_CUBINS.items():
            tmp = out + ".tmp%d" % os.getpid()
            cmd = [NVCC, "-cubin", *ARCH, "-std=c++14", "-w", "-lineinfo", *flags[kind],
                   "-DdeviceOverlap=asyncEngineCount", "-I", os.path.join(HERE, "ref_gpu"),
                   "-I", os.path.join(HERE, "ref_pin", "stubs"), "-I", REFERENCE_SRC, gen, "-o", tmp]
            subprocess.run(cmd, check=True)
            os.replace(tmp, out)
    finally:
        os.remove(gen)
    return REF_CUBINS


def build_refgpu(force: bool = False) -> str:
    """This project's harness for the reference kernels (no reference code)."""
    src = [os.path.join(HERE, "ref_gpu", "ref_gpu.cu"), os.path.join(HERE, "ref_gpu", "ref_gpu.h")]
    if not force and _newer(REFGPU_SO, src):
        return REFGPU_SO
    os.makedirs(BUILD, exist_ok=True)
    tmp = REFGPU_SO + ".tmp%d" % os.getpid()
    cmd = [NVCC, *ARCH, "-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", src[0], "-o", tmp, "-lcuda"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, REFGPU_SO)
    return REFGPU_SO


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref_pin(force="--force" in sys.argv))
    print(build_ref_cubins(force="--force" in sys.argv))
