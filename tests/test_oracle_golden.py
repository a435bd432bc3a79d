"""The oracle against the reference's own code (tests/golden/ref_pin.npz,
generated from the reference's main.h by tests/golden/make_golden.py) and
against published known answers."""
import math
import os

import numpy as np
import pytest

from oracle import pyoracle as po

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def ref():
    return dict(np.load(os.path.join(G, "ref_pin.npz")))


def test_philox_known_answers():
    # Random123 kat_vectors for philox4x32_10
    assert po.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert po.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6,
                                                             0x6D5451FD]
    assert po.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == [
        0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_uniform_range_and_streams():
    u = [po.uniform(7, 3, p, k) for p in range(8) for k in range(24)]
    assert all(0.0 <= x < 1.0 for x in u)
    assert abs(np.mean(u) - 0.5) < 0.1
    assert po.uniform(7, 3, 1, 5) != po.uniform(7, 4, 1, 5)
    assert po.uniform(7, 3, 1, 5) != po.uniform(8, 3, 1, 5)
    assert po.uniform(7, 3, 1, 5) == po.uniform(7, 3, 1, 5)


def test_series_math_accuracy():
    for x in np.linspace(-25, 25, 2001):
        assert abs(po.sin(x) - math.sin(x)) <= 2e-16 * max(1.0, abs(x))
        assert abs(po.cos(x) - math.cos(x)) <= 2e-16 * max(1.0, abs(x))
    for x in np.linspace(-1, 1, 4001):
        assert abs(po.acos(x) - math.acos(x)) <= 1e-15
    assert po.acos(1.0000001) == 0.0 and abs(po.acos(-1.5) - math.pi) < 1e-15


def test_fp32_series_accuracy():
    """The fp32 sin/cos/acos of the PSO step stay within a few float ulps of
    the true functions (both sides of the arithmetic contract use them)."""
    xs = np.float32(np.linspace(-30, 30, 6001))
    assert max(abs(po.sinf(float(x)) - math.sin(float(x))) for x in xs) < 4e-7
    assert max(abs(po.cosf(float(x)) - math.cos(float(x))) for x in xs) < 4e-7
    for x in np.float32(np.linspace(-1, 1, 6001)):
        assert abs(po.acosf(float(x)) - math.acos(float(x))) <= 1e-6 * max(1.0, math.acos(float(x)))
    assert po.acosf(1.0000001) == 0.0
    assert abs(po.sinf(5000.0) - math.sin(5000.0)) < 1e-6


def test_raster_matches_reference_render(ref):
    """renderFixedPointAABB (main.h:1306-1491) compiled from the reference:
    every depth of every face's rectangle and the AABB are bit-exact."""
    cam = po.camera()
    tris, boxes, depth, off = ref["tris"], ref["boxes"], ref["raster_depth"], ref["raster_off"]
    for i, v in enumerate(tris):
        zb = po.zbuf_new(cam)
        _, box = po.raster_face(v[0], v[1], v[2], cam, zb)
        x0, x1, y0, y1 = boxes[i]
        assert list(box) == [min(50000, x0), max(-1, x1), min(50000, y0), max(-1, y1)]
        img = zb[po.GUARD:po.GUARD + 480, po.GUARD:po.GUARD + 640]
        want = depth[off[i]:off[i + 1]].reshape(y1 - y0, x1 - x0)
        np.testing.assert_array_equal(img[y0:y1, x0:x1], want, err_msg="triangle %d" % i)
        rest = img.copy()
        rest[y0:y1, x0:x1] = po.DEPTH_BG
        assert (rest == po.DEPTH_BG).all()


def test_raster_fixture_covers_edge_cases(ref):
    """The fixture holds culled faces (back-facing / empty rectangle) and
    written ones, and bbox-fill quirk cases (writes outside the triangle)."""
    off = ref["raster_off"]
    sizes = np.diff(off)
    assert (sizes == 0).sum() >= 5
    assert (sizes > 100).sum() >= 20


def test_host_render_raster_matches_reference(ref):
    """CPUfixedPointRender (main.h:1857-1991), the rasteriser of the
    reference's best-pose CSV, compiled from the reference: iround snapping
    and float depth differ from the kernel rasteriser; every written pixel
    and value is bit-exact."""
    g = np.load(os.path.join(G, "ref_pin_cpu_render.npz"))
    cam = po.camera()
    tris, sel, idx, val, off = ref["tris"], g["tri_sel"], g["tri_idx"], g["tri_val"], g["tri_off"]
    assert len(sel) >= 250
    assert (val != np.round(val)).mean() > 0.5  # depth is kept as a float
    for j, i in enumerate(sel):
        buf = np.full((480, 640), 60000.0, np.float32)
        po.raster_face_cpu(tris[i][0], tris[i][1], tris[i][2], cam, buf)
        want = np.full(480 * 640, 60000.0, np.float32)
        want[idx[off[j]:off[j + 1]]] = val[off[j]:off[j + 1]]
        np.testing.assert_array_equal(buf.ravel(), want, err_msg="triangle %d" % i)


def test_host_render_of_mesh_matches_reference():
    """RenderCPU (main.h:2012-2043) of the C1 mesh at four poses through the
    reference's own projection and rasteriser: bit-exact."""
    import scene
    g = np.load(os.path.join(G, "ref_pin_cpu_render.npz"))
    w = scene.workload_c1()
    soa, F = w["meshes"][0]
    K = np.load(os.path.join(G, "ref_pin.npz"))["intrinsics"]  # the reference's compiled-in camera
    cam = po.camera(fx=float(np.float32(K[0])), fy=float(np.float32(K[1])), cx=float(np.float32(K[2])),
                    cy=float(np.float32(K[3])))
    idx, val, off = g["render_idx"], g["render_val"], g["render_off"]
    for j, pose in enumerate(g["poses"]):
        want = np.full(480 * 640, 60000.0, np.float32)
        want[idx[off[j]:off[j + 1]]] = val[off[j]:off[j + 1]]
        assert off[j + 1] - off[j] > 500
        # with the intrinsics rounded to float (an fp32 fma; equal here)
        got = po.render_cpu(soa, F, pose, cam)
        np.testing.assert_array_equal(got.ravel(), want, err_msg="pose %d" % j)
        # and with the reference's own double projection (equal by construction)
        got = po.render_cpu(soa, F, pose, po.camera_ref_accv())
        np.testing.assert_array_equal(got.ravel(), want, err_msg="pose %d, reference projection" % j)


def _f(a):
    return np.ascontiguousarray(a, np.float32)


def test_quaternion_helpers_match_reference(ref):
    import ctypes as C

    L = po.lib()
    fp = C.POINTER(C.c_float)
    for i in range(len(ref["S"])):
        s, q, v = _f(ref["S"][i]), _f(ref["Q"][i]), _f(ref["V"][i])
        o3, o4 = np.zeros(3, np.float32), np.zeros(4, np.float32)
        L.qo_rotate(po.ptr(s, fp), po.ptr(v, fp), po.ptr(o3, fp))
        np.testing.assert_array_equal(o3, ref["rot"][i])
        L.qo_quat_prod(po.ptr(s, fp), po.ptr(q, fp), po.ptr(o4, fp))
        np.testing.assert_array_equal(o4, ref["prod"][i])
        L.qo_quat_prod_conj(po.ptr(s, fp), po.ptr(q, fp), po.ptr(o4, fp))
        np.testing.assert_array_equal(o4, ref["prodc"][i])
        n = s.copy()
        L.qo_normalize_quat(po.ptr(n, fp))
        np.testing.assert_array_equal(n, ref["norm"][i])
        c = _f(ref["Q"][i][3:7])
        L.qo_cast_top_half(po.ptr(c, fp))
        np.testing.assert_array_equal(c, ref["cast"][i])


def test_kinematics_match_reference_within_series_tolerance(ref):
    """QuatKinematicsPSOStateVect(WithInit) (main.h:266-307, 373-413): the
    reference calls libm cos/sin here, the oracle its own series; they agree
    to float rounding."""
    import ctypes as C

    L = po.lib()
    fp = C.POINTER(C.c_float)
    for i in range(len(ref["S"])):
        s = _f(ref["S"][i])
        s[3:] /= np.linalg.norm(s[3:])
        w = _f(ref["W"][i])
        k = s.copy()
        L.qo_quat_kinematics(po.ptr(k, fp), po.ptr(w, fp))
        np.testing.assert_allclose(k, ref["kin"][i], atol=2e-6)
        qi = _f([0, 0, 0, 0.7071, 0.7071, 0, 0])
        ki = np.zeros(7, np.float32)
        L.qo_quat_kinematics_init(po.ptr(qi, fp), po.ptr(ki, fp), po.ptr(w, fp))
        np.testing.assert_allclose(ki[3:], ref["kin_init"][i][3:], atol=2e-6)


def test_projection_matches_reference_double_path(ref):
    """projectModelPointsToPixels (main.h:513-545) evaluates cx + fx*(x/z) in
    double with the ACCV macros; the oracle's fp32 fma with the intrinsics
    rounded to float agrees within a few float ulps of u, v (the difference
    is the rounding of fx, cx to float), and z exactly."""
    K = ref["intrinsics"]
    cam = po.camera(fx=K[0], fy=K[1], cx=K[2], cy=K[3])
    for i in range(len(ref["proj"])):
        o = po.project(ref["proj_pose"][i], ref["proj_pt"][i], cam)
        want = ref["proj"][i]
        assert o[2] == want[2]
        assert abs(o[0] - want[0]) <= 4 * np.spacing(np.float32(abs(want[0]))) + 1e-4
        assert abs(o[1] - want[1]) <= 4 * np.spacing(np.float32(abs(want[1]))) + 1e-4


def test_reference_camera_projection_bit_exact(ref):
    """With the reference's own ACCV camera (projected in double, as its
    kernels rebuilt for the GPU do) the oracle's projection equals the
    reference's projectModelPointsToPixels bit for bit."""
    cam = po.camera_ref_accv()
    for i in range(len(ref["proj"])):
        o = po.project(ref["proj_pose"][i], ref["proj_pt"][i], cam)
        np.testing.assert_array_equal(np.asarray(o, np.float32), np.asarray(ref["proj"][i][:3], np.float32))


def test_oracle_c1_solve_is_frozen():
    """The oracle's own C1 solve reproduces its committed trace bit for bit."""
    import scene
    from tests.helpers import oracle_params

    g = np.load(os.path.join(G, "oracle_c1.npz"))
    w = scene.workload_c1()
    soa, F = w["meshes"][0]
    depth, labels, _ = w["frames"][0]
    out = po.solve(soa, F, scene.masked_depth(depth, labels, 0), po.camera(),
                   oracle_params(w["solves"][0]), trace=True)
    np.testing.assert_array_equal(out["trace_gbest"], g["trace_gbest"])
    np.testing.assert_array_equal(out["pos"], g["pos"])
