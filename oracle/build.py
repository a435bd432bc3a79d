"""Build recipe for the test-side checkers under oracle/.

TEST INFRASTRUCTURE ONLY.  Two shared libraries:

* ``oracle/_build/libqpso_oracle.so`` -- the scalar C restatement
  (qpso_oracle.c), built everywhere (here and on the GPU host).
* ``oracle/_ref/libqpso_refpin.so`` -- the reference's own main.h helpers
  compiled for the host CPU (ref_pin/ref_pin.cpp).  Built only where the
  reference sources are present; its outputs are frozen into
  tests/golden/ by tests/golden/make_golden.py.
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


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref_pin(force="--force" in sys.argv))
