"""The C-ABI library builds for sm_103a, loads, exports every function that
include/qpso.h declares, and its structs have the header's layout.  No
compute call is made here (no GPU on the CPU runner)."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HDR = os.path.join(ROOT, "include", "qpso.h")


@pytest.fixture(scope="module")
def lib():
    import build as pkg_build
    import qpso

    pkg_build.build()
    return qpso.load_library()


def declared_functions():
    txt = open(HDR).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(qpso_[a-z0-9_]+)\s*\(", txt)))


def test_header_and_binding_agree():
    import qpso

    assert declared_functions() == sorted(qpso.EXPORTS)


def test_every_binding_declares_its_argument_types(lib):
    """Without argtypes ctypes passes a Python int as a C int, masking a
    64-bit array address to its low 32 bits."""
    import qpso

    missing = [f for f in qpso.EXPORTS if getattr(lib, f).argtypes is None]
    assert not missing, missing


def test_every_declared_symbol_is_exported(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", os.path.abspath(lib._name)],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r" T (qpso_\w+)", out))
    missing = [f for f in declared_functions() if f not in exported]
    assert not missing, missing


def test_struct_layout_matches_header(tmp_path):
    import qpso

    src = tmp_path / "layout.c"
    src.write_text(r'''
#include <stdio.h>
#include <stddef.h>
#include "qpso.h"
int main(void) {
  printf("%zu %zu %zu %zu\n", sizeof(qpso_camera), sizeof(qpso_solve_desc), sizeof(qpso_result),
         sizeof(qpso_launch_config));
  printf("%zu %zu %zu %zu %zu %zu\n", offsetof(qpso_solve_desc, num_points),
         offsetof(qpso_solve_desc, t_hi), offsetof(qpso_solve_desc, w), offsetof(qpso_solve_desc, qinit),
         offsetof(qpso_solve_desc, seed), offsetof(qpso_solve_desc, stream));
  printf("%zu %zu\n", offsetof(qpso_result, raster_writes), offsetof(qpso_result, tile_passes));
  printf("%zu %zu %zu\n", sizeof(qpso_cluster), offsetof(qpso_cluster, depth_points),
         offsetof(qpso_cluster, centroid_mm));
  printf("%zu %zu %zu %zu\n", sizeof(qpso_seg_params), offsetof(qpso_seg_params, kx),
         offsetof(qpso_seg_params, ks), offsetof(qpso_seg_params, kdc));
  return 0;
}
''')
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [list(map(int, l.split())) for l in subprocess.run([str(exe)], capture_output=True,
                                                             text=True, check=True).stdout.splitlines()]
    D = qpso.SolveDesc
    assert got[0] == [C.sizeof(qpso.Camera), C.sizeof(D), C.sizeof(qpso.Result),
                      C.sizeof(qpso.LaunchConfig)]
    assert got[1] == [D.num_points.offset, D.t_hi.offset, D.w.offset, D.qinit.offset,
                      D.seed.offset, D.stream.offset]
    assert got[2] == [qpso.Result.raster_writes.offset, qpso.Result.tile_passes.offset]
    K = qpso.Cluster
    assert got[3] == [C.sizeof(K), K.depth_points.offset, K.centroid_mm.offset]
    G = qpso.SegParams
    assert got[4] == [C.sizeof(G), G.kx.offset, G.ks.offset, G.kdc.offset]


def test_host_only_entry_points(lib):
    import qpso

    d = qpso.solve_desc()
    assert (d.num_particles, d.iterations, d.c1, d.c2, d.w, d.vdot) == (1024, 20, 1.0, 1.0, 0.3, 3.0)
    assert (d.ang_lo, d.ang_hi, d.cluster_label) == (-10.0, 10.0, -1)
    assert np.allclose(list(d.qinit), [0.7071, 0.7071, 0, 0])
    lo, hi = qpso.box_from_centroid([20.0, -140.0, 650.0], 0.3, 0.3)
    c = np.float32([20.0, -140.0, 650.0]) * np.float32(0.001)
    assert lo == list((c - np.float32(0.3)).astype(np.float32))
    assert hi == list((c + np.float32(0.3)).astype(np.float32))
    assert lib.qpso_version().startswith(b"qpso-gb300")


def test_no_gpu_fails_loudly(lib):
    """Without a usable GPU the context cannot be created: there is no CPU
    fallback."""
    import qpso

    if os.path.exists("/dev/nvidia0"):
        pytest.skip("a GPU is present")
    with pytest.raises(qpso.QpsoError):
        qpso.Context(0)
