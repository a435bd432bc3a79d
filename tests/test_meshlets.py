"""The meshlet partition built at mesh upload keeps every face exactly once,
respects its caps (64 faces and vertices for meshes up to 16384 faces, 128
above), shares vertices (the fused kernels transform each meshlet vertex once
per pose) and stores each meshlet's exact object-space box and the group
boxes."""
import os
import subprocess

import numpy as np
import pytest

import scene

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def meshlet_check(tmp_path_factory):
    exe = tmp_path_factory.mktemp("mlet") / "meshlet_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "q-pso_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "meshlet_check.cpp"), "-o", str(exe)], check=True)
    return str(exe)


@pytest.mark.parametrize("kind,n", [("icosphere", 1280), ("icosphere", 20480), ("box", 5000),
                                    ("cylinder", 5000), ("ellipsoid", 12000), ("ellipsoid", 30)])
def test_partition(meshlet_check, tmp_path, kind, n):
    soa, F = scene.make_mesh(kind, n, 100.0, seed=3)
    path = tmp_path / "mesh.bin"
    soa.astype(np.float32).tofile(path)
    out = subprocess.run([meshlet_check, str(path)], capture_output=True, text=True)
    assert out.returncode == 0, out.returncode
    faces, mlets, slots, cap = map(int, out.stdout.split())
    assert faces == F
    assert cap == (64 if F <= 16384 else 128)
    assert mlets >= (F + cap - 1) // cap
    # vertex sharing: well below 3 transforms per face on closed meshes
    if F >= 1000:
        assert slots / F < 0.8, slots / F


def test_partition_of_unshared_triangles(meshlet_check, tmp_path):
    """A soup of disjoint triangles has no sharing; caps still hold."""
    rng = np.random.default_rng(0)
    F = 700
    soa = rng.normal(size=9 * F).astype(np.float32)
    path = tmp_path / "soup.bin"
    soa.tofile(path)
    out = subprocess.run([meshlet_check, str(path)], capture_output=True, text=True)
    assert out.returncode == 0
    faces, mlets, slots, cap = map(int, out.stdout.split())
    assert faces == F and slots == 3 * F and mlets >= (3 * F + cap - 1) // cap
