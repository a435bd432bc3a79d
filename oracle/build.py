"""Build recipe for the test-side checkers under oracle/.

TEST INFRASTRUCTURE ONLY.  Host libraries:

* ``oracle/_build/libqpso_oracle.so`` -- the scalar C restatement
  (qpso_oracle.c), built everywhere (here and on the GPU host).
* ``oracle/_ref/libqpso_refpin.so`` -- the reference's own main.h helpers
  compiled for the host CPU (ref_pin/ref_pin.cpp).  Built only where the
  reference sources are present; its outputs are frozen into
  tests/golden/ by tests/golden/make_golden.py.
* ``oracle/_ref/libqpso_segpin.so`` -- the reference's segmentation core
  (GraphCannySeg's disjoint-set forest, segment_graph, small-component
  merge, collectSets) compiled for the host between the stand-ins of
  ref_pin/seg_*.h.  Same conditions; frozen into tests/golden/ref_seg.npz.

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


SEGPIN_SO = os.path.join(REF_OUT, "libqpso_segpin.so")


def _code_braces(line: str) -> int:
    code = line.split("//", 1)[0]
    return code.count("{") - code.count("}")


def _block(lines: list[str], start: int) -> tuple[int, int]:
    """[start, end) of the brace-balanced block that opens on or after
    line `start` (// comments ignored)."""
    depth, opened = 0, False
    for i in range(start, len(lines)):
        d = _code_braces(lines[i])
        opened = opened or "{" in lines[i].split("//", 1)[0]
        depth += d
        if opened and depth == 0:
            return start, i + 1
    raise ValueError("unbalanced block at line %d" % (start + 1))


def _find(lines: list[str], text: str, after: int = 0) -> int:
    return next(i for i in range(after, len(lines)) if text in lines[i])


def _segmentation_pieces(src: str) -> str:
    """The reference's disjoint-set forest and graph segmentation, read
    from GraphCannySeg.h/.cpp where they lie, each piece under a #line of
    its own: THRESHOLD, edge, uni_elt, universe (header); edge's
    constructors and operator<, universe's methods, segment_graph and the
    small-component merge loop (source)."""
    h = open(os.path.join(src, "GraphCannySeg.h")).read().splitlines(keepends=True)
    c = open(os.path.join(src, "GraphCannySeg.cpp")).read().splitlines(keepends=True)

    def piece(lines, name, a, b):
        return '#line %d "%s"\n%s' % (a + 1, name, "".join(lines[a:b]))

    out = []
    i = _find(h, "#define THRESHOLD(size, c)")
    out.append(piece(h, "GraphCannySeg.h", i, i + 1))
    out.append("namespace GraphCanny {\n")
    out.append(piece(h, "GraphCannySeg.h", *_block(h, _find(h, "struct edge{"))))
    end = _find(h, "} uni_elt;")
    start = max(i for i in range(end) if h[i].strip() == "typedef struct {")
    out.append(piece(h, "GraphCannySeg.h", start, end + 1))
    out.append(piece(h, "GraphCannySeg.h", *_block(h, _find(h, "class universe {"))))
    out.append("}\n#include \"seg_class.h\"\nnamespace GraphCanny {\n")
    for sig in ("edge::edge()", "edge::edge(int a_, int b_, float w_)", "bool operator<(const edge &a, const edge &b)",
                "universe::universe(int elements)", "universe::~universe()", "int universe::find(int x)",
                "void universe::join(int x, int y)", "bool universe::printSet(", "void universe::collectSets("):
        out.append(piece(c, "GraphCannySeg.cpp", *_block(c, _find(c, sig))))
    seg = _find(c, "GraphCannySeg<T>::segment_graph(int num_vertices")
    assert c[seg - 1].strip() == "template <class T>"
    out.append(piece(c, "GraphCannySeg.cpp", seg - 1, _block(c, seg)[1]))
    loop = _find(c, "for (int i = 0; i < num; i++) {", _find(c, "// post process small components"))
    out.append("template <class T>\nvoid GraphCannySeg<T>::merge_small(universe *u, edge *edges, int num) {\n")
    out.append(piece(c, "GraphCannySeg.cpp", *_block(c, loop)))
    out.append("}\n}\n")
    return "".join(out)


def build_seg_pin(force: bool = False) -> str | None:
    """oracle/_ref/libqpso_segpin.so: the reference's segmentation core
    (union-find forest, segment_graph, small-component merge, collectSets)
    compiled for the host between the stand-ins of ref_pin/seg_*.h."""
    hdr = os.path.join(REFERENCE_SRC, "GraphCannySeg.h")
    cpp = os.path.join(REFERENCE_SRC, "GraphCannySeg.cpp")
    if not (os.path.exists(hdr) and os.path.exists(cpp)):
        return None
    mine = [os.path.join(HERE, "ref_pin", f) for f in ("seg_prelude.h", "seg_class.h", "seg_api.h")]
    if not force and _newer(SEGPIN_SO, [hdr, cpp, os.path.abspath(__file__), *mine]):
        return SEGPIN_SO
    os.makedirs(REF_OUT, exist_ok=True)
    gen = os.path.join(REF_OUT, "seg_pin_gen%d.cpp" % os.getpid())
    with open(gen, "w") as fp:
        fp.write('#include "seg_prelude.h"\n')
        fp.write(_segmentation_pieces(REFERENCE_SRC))
        fp.write('#include "seg_api.h"\n')
    tmp = SEGPIN_SO + ".tmp%d" % os.getpid()
    try:
        subprocess.run(["g++", "-O1", "-std=c++14", "-fPIC", "-shared", "-ffp-contract=off", "-w",
                        "-I", os.path.join(HERE, "ref_pin"), gen, "-o", tmp], check=True)
        os.replace(tmp, SEGPIN_SO)
    finally:
        os.remove(gen)
    return SEGPIN_SO


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
    print(build_seg_pin(force="--force" in sys.argv))
    print(build_ref_cubins(force="--force" in sys.argv))
