"""Build recipe for the test infrastructure under oracle/.

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
# Directory holding the reference's sources (main.cu, main.h,
# GraphCannySeg.{h,cpp}), given by the environment: QPSO_REFERENCE_SRC.  The
# reference builds below are skipped when it is unset or lacks the files.
REFERENCE_SRC = os.environ.get("QPSO_REFERENCE_SRC", "")


def _ref_path(name: str) -> str:
    """A reference source file, or a path that never exists when the
    reference directory is not given."""
    if not REFERENCE_SRC:
        return os.path.join(HERE, "_no_reference_given", name)
    return os.path.join(REFERENCE_SRC, name)


CUDA_INC = "/usr/local/cuda/include"

ORACLE_SO = os.path.join(BUILD, "libqpso_oracle.so")
REFPIN_SO = os.path.join(REF_OUT, "libqpso_refpin.so")


def _newer(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build_oracle(force: bool = False) -> str:
    src = [os.path.join(HERE, "qpso_oracle.c"), os.path.join(HERE, "qpso_seg_front.c"),
           os.path.join(HERE, "qpso_oracle.h")]
    if not force and _newer(ORACLE_SO, src):
        return ORACLE_SO
    os.makedirs(BUILD, exist_ok=True)
    tmp = ORACLE_SO + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off",
           "-fno-fast-math", "-fopenmp", src[0], src[1], "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_ref_pin(force: bool = False) -> str | None:
    main_h = _ref_path("main.h")
    if not os.path.exists(main_h):
        # without the sources, a library built earlier from them still serves
        return REFPIN_SO if os.path.exists(REFPIN_SO) else None
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
    main_cu = _ref_path("main.cu")
    main_h = _ref_path("main.h")
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


def _code_only(lines: list[str]) -> list[str]:
    """The lines with comments, string and character literals blanked out
    (line structure kept), for counting braces."""
    out, block = [], False
    for line in lines:
        res, i, n = [], 0, len(line)
        while i < n:
            if block:
                j = line.find("*/", i)
                if j < 0:
                    i = n
                else:
                    block, i = False, j + 2
                continue
            ch = line[i]
            if line.startswith("//", i):
                break
            if line.startswith("/*", i):
                block, i = True, i + 2
                continue
            if ch in "\"'":
                j = i + 1
                while j < n and line[j] != ch:
                    j += 2 if line[j] == "\\" else 1
                i = j + 1
                continue
            res.append(ch)
            i += 1
        out.append("".join(res))
    return out


def _block(lines: list[str], start: int) -> tuple[int, int]:
    """[start, end) of the brace-balanced block that opens on or after
    line `start` (comments and literals ignored)."""
    code = _code_only(lines[start:])
    depth, opened = 0, False
    for k, text in enumerate(code):
        opened = opened or "{" in text
        depth += text.count("{") - text.count("}")
        if opened and depth == 0:
            return start, start + k + 1
    raise ValueError("unbalanced block at line %d" % (start + 1))


def _find(lines: list[str], text: str, after: int = 0) -> int:
    return next(i for i in range(after, len(lines)) if text in lines[i])


def _segmentation_pieces(src: str) -> str:
    """The reference's graph segmentation from its pixel planes to its
    cluster lists, read from GraphCannySeg.h/.cpp where they lie, each piece
    under a #line of its own.  Header: deg2rad, THRESHOLD, the pixel types,
    square, the image template, mapminmax, the Gaussian smoothing (mask,
    normalisation, separable convolution), edge, uni_elt, universe, and the
    edge weight diff() inside a stand-in of the GraphCannySeg class (members
    in ref_pin/seg_class.h).  Source: the image constructor and destructor,
    edge's constructors and operator<, universe's methods, segment_graph,
    and three fragments of segment_image: the depth normalisation, the
    pixel-graph loop and the small-component merge loop."""
    h = open(os.path.join(src, "GraphCannySeg.h")).read().splitlines(keepends=True)
    c = open(os.path.join(src, "GraphCannySeg.cpp")).read().splitlines(keepends=True)

    def piece(lines, name, a, b):
        return '#line %d "%s"\n%s' % (a + 1, name, "".join(lines[a:b]))

    def hdr(a, b):
        return piece(h, "GraphCannySeg.h", a, b)

    def cpp(a, b):
        return piece(c, "GraphCannySeg.cpp", a, b)

    def templated(lines, sig):
        i = _find(lines, sig)
        assert lines[i - 1].strip() == "template <class T>", sig
        return i - 1, _block(lines, i)[1]

    out = []
    i = _find(h, "#ifndef deg2rad")
    out.append(hdr(i, i + 3))
    i = _find(h, "#define THRESHOLD(size, c)")
    out.append(hdr(i, i + 1))
    out.append("namespace GraphCanny {\n")
    for sig in ("struct edge{", "struct rgb{", "struct hsv{", "struct CIELab{"):
        out.append(hdr(*_block(h, _find(h, sig))))
    i = _find(h, "inline T square(const T &x)")
    out.append(hdr(i - 1, i + 1))
    out.append(hdr(*templated(h, "class image {")))
    for macro in ("#define imRef(im, x, y)", "#define imPtr(im, x, y)"):
        i = _find(h, macro)
        out.append(hdr(i, i + 1))
    out.append(hdr(*templated(h, "inline T mapminmax(const T& x")))
    out.append(hdr(*_block(h, _find(h, "static inline void convolve_even(image<float> *src"))))
    i = _find(h, "#define WIDTH 4.0")
    out.append(hdr(i, i + 1))
    out.append(hdr(*_block(h, _find(h, "static inline void normalize(std::vector<float> &mask)"))))
    i = _find(h, "#define MAKE_FILTER(name, fun)")
    j = i
    while h[j].rstrip().endswith("\\"):
        j += 1
    out.append(hdr(i, j + 1))
    i = _find(h, "MAKE_FILTER(fgauss,")
    out.append(hdr(i, i + 1))
    out.append(hdr(*_block(h, _find(h, "static inline image<float> *smooth(image<float> *src, float sigma)"))))
    end = _find(h, "} uni_elt;")
    start = max(i for i in range(end) if h[i].strip() == "typedef struct {")
    out.append(hdr(start, end + 1))
    out.append(hdr(*_block(h, _find(h, "class universe {"))))
    out.append("template <class T>\nclass GraphCannySeg {\npublic:\n#include \"seg_class.h\"\n")
    out.append(hdr(*_block(h, _find(h, "inline float diff(image<float> *r, image<float> *g, image<float> *b,"))))
    out.append("};\n")
    out.append(cpp(*templated(c, "image<T>::image(const int width, const int height, const bool init)")))
    out.append(cpp(*templated(c, "image<T>::~image()")))
    for sig in ("edge::edge()", "edge::edge(int a_, int b_, float w_)", "bool operator<(const edge &a, const edge &b)",
                "universe::universe(int elements)", "universe::~universe()", "int universe::find(int x)",
                "void universe::join(int x, int y)", "bool universe::printSet(", "void universe::collectSets("):
        out.append(cpp(*_block(c, _find(c, sig))))
    out.append(cpp(*templated(c, "GraphCannySeg<T>::segment_graph(int num_vertices")))
    # segment_image fragments, each wrapped in a member of the stand-in
    seg_img = _find(c, "GraphCannySeg<T>::segment_image()")
    a = _find(c, "uint16_t max_depth_val =", seg_img)
    b = _block(c, _find(c, "for(size_t idx=0;idx<depth_mm_norm->WxH();++idx)", a))[1]
    out.append("template <class T>\nimage<float> *GraphCannySeg<T>::depth_norm() {\n")
    out.append(cpp(a, b))
    out.append("return depth_mm_norm;\n}\n")
    a = _find(c, "int num = 0;", _find(c, "// 8-connectivity", seg_img))
    b = _block(c, a + 1)[1]
    out.append("template <class T>\nint GraphCannySeg<T>::build_edges(image<float> *smooth_h, image<float> *smooth_s,\n"
               "    image<float> *smooth_v, image<float> *depth_mm_norm, edge *edges) {\n"
               "std::vector<float> w_planes(4 * (size_t)mWidth * mHeight);\n"
               "float *pW1 = w_planes.data(), *pW2 = pW1 + (size_t)mWidth * mHeight;\n"
               "float *pW3 = pW2 + (size_t)mWidth * mHeight, *pW4 = pW3 + (size_t)mWidth * mHeight;\n")
    out.append(cpp(a, b))
    out.append("return num;\n}\n")
    loop = _find(c, "for (int i = 0; i < num; i++) {", _find(c, "// post process small components"))
    out.append("template <class T>\nvoid GraphCannySeg<T>::merge_small(universe *u, edge *edges, int num) {\n")
    out.append(cpp(*_block(c, loop)))
    out.append("}\n}\n")
    return "".join(out)


def build_seg_pin(force: bool = False) -> str | None:
    """oracle/_ref/libqpso_segpin.so: the reference's segmentation core
    (union-find forest, segment_graph, small-component merge, collectSets)
    compiled for the host between the stand-ins of ref_pin/seg_*.h."""
    hdr = _ref_path("GraphCannySeg.h")
    cpp = _ref_path("GraphCannySeg.cpp")
    if not (os.path.exists(hdr) and os.path.exists(cpp)):
        return SEGPIN_SO if os.path.exists(SEGPIN_SO) else None
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
