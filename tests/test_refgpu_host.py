"""Host side of the harness for the reference's rebuilt CUDA kernels (no
GPU): the uniform table equals the oracle's Philox draws, and the in-frame
check that guards every render launch bounds every vertex projection of an
accepted pose."""
import numpy as np

import scene
from oracle import pyoracle as po
from oracle import refgpu


def test_uniform_table_is_the_oracles_draws():
    L = po.lib()
    for seed, stream in [(11, 2), ((7 << 32) + 3, 0)]:
        t = refgpu.uniform_table(seed, stream)
        assert t.shape == (refgpu.RAND_STRIDE, refgpu.NPARTICLE) and t.dtype == np.float32
        rng = np.random.default_rng(seed & 0xFFFF)
        for _ in range(500):
            j, p = int(rng.integers(refgpu.RAND_STRIDE)), int(rng.integers(refgpu.NPARTICLE))
            assert t[j, p] == np.float32(L.qo_uniform(seed, stream, p, j))
        assert t.min() >= 0.0 and t.max() < 1.0


def test_in_frame_bounds_every_vertex():
    """Accepted poses keep every projected vertex 8 px inside the image (the
    margin the raster rectangles and the fitness window need); poses off to
    the side, behind or at the camera are refused."""
    w = scene.workload_c1()
    soa, F = w["meshes"][0]
    cam = po.camera_ref_accv()
    rng = np.random.default_rng(3)
    V = np.stack([np.asarray(soa[j * F:(j + 1) * F]) for j in range(9)])  # 9 x F
    accepted = refused = 0
    for _ in range(120):
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        z = rng.uniform(0.2, 1.2)
        s = np.array([rng.uniform(-0.5, 0.5) * z, rng.uniform(-0.4, 0.4) * z, z, *q], np.float32)
        ok = refgpu.in_frame(soa, F, s[None])[0]
        if not ok:
            refused += 1
            continue
        accepted += 1
        for f in range(0, F, 7):
            for j in range(3):
                u, v, zz = po.project(s, V[[j, 3 + j, 6 + j], f], cam)
                assert 8.0 - 1e-3 <= u <= 632.0 + 1e-3 and 8.0 - 1e-3 <= v <= 472.0 + 1e-3
                assert zz > 50.0
    assert accepted > 10 and refused > 10
    behind = np.array([0, 0, -0.5, 1, 0, 0, 0], np.float32)
    near = np.array([0, 0, 0.03, 1, 0, 0, 0], np.float32)
    assert not refgpu.in_frame(soa, F, np.stack([behind, near])).any()


def test_reference_shape_box_keeps_every_pose_in_frame():
    """bench.py's reference-shaped solve: any translation in its box, at
    any rotation, passes the harness's in-frame check, so the reference's
    loop never stops on a pose; meshes beyond the kernels' reach get none."""
    import bench

    rng = np.random.default_rng(9)
    for wl in ("c1", "c2", "c3"):
        w, _ = bench.load_workload(wl)
        sh = bench.reference_shape(w)
        soa, F = w["meshes"][sh["mesh"]]
        lo, hi = np.array(sh["t_lo"]), np.array(sh["t_hi"])
        corners = np.array([[hi[0] if k & 1 else lo[0], hi[1] if k & 2 else lo[1], hi[2] if k & 4 else lo[2]]
                            for k in range(8)])
        ts = np.concatenate([corners, rng.uniform(lo, hi, (40, 3))])
        q = rng.normal(size=(len(ts), 4))
        q /= np.linalg.norm(q, axis=1, keepdims=True)
        poses = np.concatenate([ts, q], axis=1).astype(np.float32)
        assert refgpu.in_frame(soa, F, poses).all(), wl
        x0, x1, y0, y1 = sh["aabb"]
        assert 0 <= x0 <= x1 <= 639 and 0 <= y0 <= y1 <= 479
    w, _ = bench.load_workload("c5")
    assert bench.reference_shape(w) is None
