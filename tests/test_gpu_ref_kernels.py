"""The reference's own CUDA kernels, rebuilt for sm_103a from main.h and
main.cu:72-1195 (IEEE build), against the oracle on the GB300.

This pins the parts of the oracle that the host build of main.h cannot
reach: the fitness kernel (main.cu:550-764), the best update
(main.cu:768-855), the particle update (main.cu:858-1060) and InitQPSO
(main.cu:72-198), as well as the raster through the real kernel.  Inputs are
identical on both sides: the same poses, and the reference's uniform table
filled with the oracle's Philox draws.  The kernels' ACCV camera is the
oracle's PROJ_REF_ACCV projection.

Bars: depth buffers and render boxes bit-exact; fitness within 1e-5
relative of the FP64 recomputation (spec tolerance); translations and
velocities of init and update bit-exact where no transcendental is
involved, quaternions within 4e-6 (CUDA's sinf/cosf/acosf against the
oracle's own series).  Every pose is checked in frame before it is rendered
(the reference's raster does not clip).
"""
import numpy as np
import pytest

import scene
from oracle import pyoracle as po
from oracle import refgpu

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not refgpu.available("ieee"),
                                 reason="reference kernels not built (reference sources absent)")]

N = 1024
# translation box of the solves here: keeps every particle of the
# 60x40x30 mm ellipsoid inside the ACCV image at any rotation
T_LO = (-0.08, -0.06, 0.70)
T_HI = (0.08, 0.06, 0.90)
SEED, STREAM = 11, 2


@pytest.fixture(scope="module")
def c1_scene():
    w = scene.workload_c1()
    soa, F = w["meshes"][0]
    depth, labels, _ = w["frames"][0]
    obs = scene.masked_depth(depth, labels, 0)
    info = scene.cluster_info(depth, labels, 0)
    return soa, F, obs, info


@pytest.fixture(scope="module")
def rk(c1_scene):
    soa, F, obs, info = c1_scene
    k = refgpu.RefKernels("ieee")
    k.set_scene(soa, F, obs.astype(np.int32), T_LO, T_HI, info["num_points"], info["aabb"])
    yield k
    k.close()


def _poses(soa, F, n, seed):
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < n:
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        z = rng.uniform(0.6, 1.0)
        s = np.array([rng.uniform(-0.2, 0.2) * z, rng.uniform(-0.15, 0.15) * z, z, *q], np.float32)
        if refgpu.in_frame(soa, F, s[None])[0]:
            out.append(s)
    return np.stack(out)


def _oracle_params(info, P=N, iterations=1):
    prm = po.default_params()
    prm.t_lo[:] = T_LO
    prm.t_hi[:] = T_HI
    x0, x1, y0, y1 = info["aabb"]
    prm.cl_min_x, prm.cl_max_x, prm.cl_min_y, prm.cl_max_y = x0, x1, y0, y1
    prm.num_points = info["num_points"]
    prm.num_particles = P
    prm.iterations = iterations
    prm.seed = SEED
    prm.stream = STREAM
    return prm


def _rows_exact(win):
    """The reference's fitness loop finds a pixel's row with a float
    reciprocal (main.cu:628); True when that gives the exact row for every
    index the loop visits, so that every window pixel is visited once."""
    x0, x1, y0, y1 = win
    W, H = x1 - x0, y1 - y0
    T = -(-(W * H) // 1024) * 1024
    t = np.arange(T, dtype=np.int64)
    yf = np.floor(t.astype(np.float32) * (np.float32(1.0) / np.float32(W))).astype(np.int64)
    return bool((yf == t // W).all())


def test_render_and_aabb_bit_exact(rk, c1_scene):
    """RenderFixedPointKernelAABB + ComputeAABBFinalReductionKernel: every
    depth buffer and render box equals the oracle's raster with the
    reference's camera."""
    soa, F, obs, info = c1_scene
    poses = _poses(soa, F, 48, 1)
    pos = np.zeros((7, N), np.float32)
    pos[:, :len(poses)] = poses.T
    rk.set_state(pos=pos)
    depth, aabb, _ = rk.render_score(len(poses), want_depth=True)
    cam = po.camera_ref_accv()
    G = po.GUARD
    zb = po.zbuf_new(cam)
    written = 0
    for i, s in enumerate(poses):
        zb.fill(po.DEPTH_BG)
        zbuf, box, n = po.render(soa, F, s, cam, zb)
        np.testing.assert_array_equal(depth[i], zbuf[G:G + 480, G:G + 640], err_msg="pose %d" % i)
        assert tuple(aabb[i]) == tuple(box), i
        written += int((depth[i] < po.DEPTH_BG).sum())
    assert written > 48 * 200


def test_fitness_matches_fp64(rk, c1_scene):
    """ComputeFitnessKernel: the fitness of each pose is within 1e-5
    relative of the oracle's counts recomputed in FP64, wherever the
    reference's float row index visits every window pixel once."""
    soa, F, obs, info = c1_scene
    poses = _poses(soa, F, 64, 2)
    pos = np.zeros((7, N), np.float32)
    pos[:, :len(poses)] = poses.T
    rk.set_state(pos=pos)
    _, _, fit = rk.render_score(len(poses))
    cam = po.camera_ref_accv()
    prm = _oracle_params(info)
    zb = po.zbuf_new(cam)
    checked = 0
    x0, x1, y0, y1 = info["aabb"]
    for i, s in enumerate(poses):
        zb.fill(po.DEPTH_BG)
        zbuf, box, _ = po.render(soa, F, s, cam, zb)
        win = (min(box[0], x0), max(box[1], x1), min(box[2], y0), max(box[3], y1))
        if not _rows_exact(win):
            continue
        sc = po.score(zbuf, box, obs, cam, prm)
        want = po.fitness_fp64(sc, info["num_points"])
        assert abs(float(fit[i]) - want) <= 1e-5 * abs(want), (i, float(fit[i]), want)
        checked += 1
    assert checked >= 32


def test_init_matches_oracle(rk, c1_scene):
    """InitQPSO over 1024 particles from the oracle's draws."""
    _, _, _, info = c1_scene
    rk.set_rand_table(refgpu.uniform_table(SEED, STREAM))
    rk.init()
    st = rk.get_state()
    prm = _oracle_params(info)
    pos = np.zeros((7, N), np.float32)
    vel = np.zeros((7, N), np.float32)
    pb = np.zeros((7, N), np.float32)
    for p in range(N):
        po.init_particle(prm, p, pos, vel, pb)
    np.testing.assert_array_equal(st["pos"][:3], pos[:3])
    np.testing.assert_array_equal(st["vel"], vel)
    np.testing.assert_allclose(st["pos"][3:], pos[3:], rtol=0, atol=4e-6)
    np.testing.assert_array_equal(st["pbest"], st["pos"])
    assert (st["cursor"] == 12).all()


def test_best_and_update_match_oracle(rk, c1_scene):
    """UpdatePersonalAndGlobalBest after thrust::min_element, then
    UpdateParticlesEquationKernel, from one shared state and fitness."""
    _, _, _, info = c1_scene
    prm = _oracle_params(info, iterations=2)
    pos = np.zeros((7, N), np.float32)
    vel = np.zeros((7, N), np.float32)
    pb = np.zeros((7, N), np.float32)
    for p in range(N):
        po.init_particle(prm, p, pos, vel, pb)
    pb[:3] += np.float32(0.01)  # personal bests that differ from the poses
    rng = np.random.default_rng(5)
    fit = rng.uniform(0.01, 2.0, N).astype(np.float32)
    pbf = np.full(N, 1e10, np.float32)
    pbf[::3] = rng.uniform(0.01, 2.0, (N + 2) // 3).astype(np.float32)  # some personal bests hold
    rk.set_rand_table(refgpu.uniform_table(SEED, STREAM))
    rk.set_state(pos=pos, vel=vel, pbest=pb, fit=fit, pbest_fit=pbf, best_fit=np.float32([1e10]),
                 best_pose=np.zeros(7, np.float32), cursor=np.full(N, 12, np.uint32))
    rk.best_and_update()
    st = rk.get_state()
    # the best update (main.cu:768-855), first minimum as thrust finds it
    better = fit < pbf
    pbf2 = np.where(better, fit, pbf)
    pb2 = np.where(better[None, :], pos, pb)
    b = int(np.argmin(fit))
    gb = pos[:, b].copy()
    np.testing.assert_array_equal(st["pbest_fit"], pbf2)
    np.testing.assert_array_equal(st["pbest"], pb2)
    assert st["best_fit"][0] == fit[b]
    np.testing.assert_array_equal(st["best_pose"], gb)
    for p in range(N):
        po.update_particle(prm, p, 1, pos, vel, pb2, gb)
    np.testing.assert_array_equal(st["pos"][:3], pos[:3])
    np.testing.assert_array_equal(st["vel"][:3], vel[:3])
    np.testing.assert_allclose(st["vel"][3:], vel[3:], rtol=0, atol=1e-5)
    np.testing.assert_allclose(st["pos"][3:], pos[3:], rtol=0, atol=4e-6)
    assert (st["cursor"] == 24).all()


def test_reference_solve_loop(rk, c1_scene):
    """The reference's loop (init, then render, score, best update and
    update over 1024 particles) for three iterations: the first iteration's
    best fitness equals the oracle's within 1e-3, and the best fitness never
    rises.  Not closer: the initial quaternions differ by float ulps (CUDA's
    sinf/cosf against the oracle's series), which moves a few raster pixels,
    and the reference's float row index double-visits pixels of some window
    widths (a race the oracle does not copy)."""
    soa, F, obs, info = c1_scene
    rk.set_rand_table(refgpu.uniform_table(SEED, STREAM))
    out = rk.solve(3)
    assert out["status"] == refgpu.OK, out["error"]
    assert out["done"] == 3 and out["ms"] > 0
    tr = out["trace"]
    assert (np.diff(tr) <= 0).all()
    o = po.solve(soa, F, obs, po.camera_ref_accv(), _oracle_params(info, iterations=1), trace=True, threads=8)
    want = float(o["trace_gbest"][0][0])
    assert abs(float(tr[0]) - want) <= 1e-3 * abs(want), (float(tr[0]), want)


@pytest.mark.skipif(not refgpu.available("fast"), reason="reference kernels not built")
def test_library_solve_agrees_with_reference_kernels(c1_scene):
    """The drop-in end to end: this library's qpso_solve and the reference's
    own kernels (its -use_fast_math build and host loop) on the same mesh,
    observed depth, cluster, translation box, camera (the ACCV intrinsics,
    rounded to float for the library) and uniform draws, 1024 particles x
    5 iterations.  The first iteration's best fitness agrees within 1e-3.
    Later iterations are not compared: the swarm is chaotic, and the two
    differ by float ulps from the first update on (CUDA's sinf/cosf/acosf
    against this project's series, double against float intrinsics).  Both
    best fitnesses can only fall."""
    import qpso

    soa, F, obs, info = c1_scene
    w = scene.workload_c1()
    depth, labels, _ = w["frames"][0]
    with refgpu.RefKernels("fast") as rk:
        rk.set_scene(soa, F, obs.astype(np.int32), T_LO, T_HI, info["num_points"], info["aabb"])
        rk.set_rand_table(refgpu.uniform_table(SEED, STREAM))
        ref = rk.solve(5)
    assert ref["status"] == refgpu.OK and ref["done"] == 5
    with qpso.Context(0) as ctx:
        mid = ctx.mesh_upload(soa, F)
        fid = ctx.frame_upload(depth, qpso.Camera(572.41140, 573.57043, 325.26110, 242.04899, 640, 480),
                               labels=labels)
        x0, x1, y0, y1 = info["aabb"]
        d = qpso.solve_desc(mesh_id=mid, frame_id=fid, cluster_label=0, cl_min_x=x0, cl_max_x=x1, cl_min_y=y0,
                            cl_max_y=y1, num_points=info["num_points"], t_lo=T_LO, t_hi=T_HI, num_particles=N,
                            iterations=5, seed=SEED, stream=STREAM)
        r, st = ctx.solve_traced(d)
    ours = st["trace_gbest"][:, 0]
    assert r.flags == 0
    assert abs(float(ours[0]) - float(ref["trace"][0])) <= 1e-3 * float(ref["trace"][0]), (ours[0], ref["trace"][0])
    assert (np.diff(ours) <= 0).all() and (np.diff(ref["trace"]) <= 0).all()


@pytest.mark.skipif(not refgpu.available("fast"), reason="reference kernels not built")
def test_fast_math_build_render_close_to_oracle(c1_scene):
    """The reference's kernels as its Makefile builds them (-use_fast_math,
    multiply-add contraction): on the same 48 poses the depth buffers may
    differ from the oracle's raster only in rare pixels (measured on the
    GB300: none of 167,315), by at most 1 mm where both wrote (a contracted
    depth can round the other way at a .5), the render boxes by at most 1 px
    (a vertex snapped to the neighbouring 1/16 px), and the fitness stays
    within 1e-3 of the FP64 recomputation."""
    soa, F, obs, info = c1_scene
    poses = _poses(soa, F, 48, 1)
    with refgpu.RefKernels("fast") as rk:
        rk.set_scene(soa, F, obs.astype(np.int32), T_LO, T_HI, info["num_points"], info["aabb"])
        pos = np.zeros((7, N), np.float32)
        pos[:, :len(poses)] = poses.T
        rk.set_state(pos=pos)
        depth, aabb, fit = rk.render_score(len(poses), want_depth=True)
    cam = po.camera_ref_accv()
    G = po.GUARD
    zb = po.zbuf_new(cam)
    prm = _oracle_params(info)
    x0, x1, y0, y1 = info["aabb"]
    diff = written = 0
    for i, s in enumerate(poses):
        zb.fill(po.DEPTH_BG)
        zbuf, box, _ = po.render(soa, F, s, cam, zb)
        want = zbuf[G:G + 480, G:G + 640]
        d = depth[i] != want
        diff += int(d.sum())
        written += int((want < po.DEPTH_BG).sum())
        both = d & (depth[i] < po.DEPTH_BG) & (want < po.DEPTH_BG)
        if both.any():
            assert np.abs(depth[i][both].astype(np.int64) - want[both]).max() <= 1
        assert np.abs(aabb[i] - box).max() <= 1
        win = (min(box[0], x0), max(box[1], x1), min(box[2], y0), max(box[3], y1))
        if _rows_exact(win):
            sc = po.score(zbuf, box, obs, cam, prm)
            ref = po.fitness_fp64(sc, info["num_points"])
            assert abs(float(fit[i]) - ref) <= 1e-3 * abs(ref), (i, float(fit[i]), ref)
    assert written > 48 * 200
    print("fast-math build: %d of %d rendered pixels differ" % (diff, written))
    assert diff <= written // 1000, (diff, written)


@pytest.mark.skipif(not refgpu.available("fast"), reason="reference kernels not built")
def test_library_reference_projection_equals_reference_kernels(c1_scene):
    """This library with QPSO_PROJ_REF_ACCV (the reference's projection,
    its ACCV intrinsics in double) against the reference's own kernels as
    its Makefile builds them, on the same 48 poses: every rendered window
    and render box is bit-identical, and the fitness of the library's
    exact counts is within 1e-5 of the reference kernel's float sums
    wherever the reference's float row index visits every window pixel
    once (elsewhere it double-visits or skips a pixel, a documented
    deviation of the reference)."""
    import qpso

    soa, F, obs, info = c1_scene
    w = scene.workload_c1()
    depth_frame, labels, _ = w["frames"][0]
    poses = _poses(soa, F, 48, 1)
    with refgpu.RefKernels("fast") as rk:
        rk.set_scene(soa, F, obs.astype(np.int32), T_LO, T_HI, info["num_points"], info["aabb"])
        pos = np.zeros((7, N), np.float32)
        pos[:, :len(poses)] = poses.T
        rk.set_state(pos=pos)
        ref_depth, ref_aabb, ref_fit = rk.render_score(len(poses), want_depth=True)
    cam = qpso.Camera(0, 0, 0, 0, 640, 480, qpso.PROJ_REF_ACCV)
    with qpso.Context(0) as ctx:
        mid = ctx.mesh_upload(soa, F)
        fid = ctx.frame_upload(depth_frame, cam, labels=labels)
        x0, x1, y0, y1 = info["aabb"]
        d = qpso.solve_desc(mesh_id=mid, frame_id=fid, cluster_label=0, cl_min_x=x0, cl_max_x=x1,
                            cl_min_y=y0, cl_max_y=y1, num_points=info["num_points"], t_lo=T_LO, t_hi=T_HI)
        fit = ctx.score_poses(d, poses)
        for i, s in enumerate(poses):
            bx0, bx1, by0, by1 = (int(v) for v in ref_aabb[i])
            wx0 = bx0 & ~3
            ww = (bx1 - wx0 + 3) // 4 * 4
            hh = by1 - by0
            assert ww * hh * 4 < 200 * 1024, (ww, hh)
            got, box = ctx.render(mid, cam, s, wx0, by0, ww, hh)
            assert tuple(box) == tuple(ref_aabb[i]), i
            want = ref_depth[i][by0:by0 + hh, wx0:wx0 + ww]
            np.testing.assert_array_equal(got, want, err_msg="pose %d" % i)
    checked = 0
    for i in range(len(poses)):
        b = ref_aabb[i]
        win = (min(b[0], x0), max(b[1], x1), min(b[2], y0), max(b[3], y1))
        if _rows_exact(win):
            assert abs(float(fit[i]) - float(ref_fit[i])) <= 1e-5 * abs(float(ref_fit[i])), i
            checked += 1
    assert checked >= 32
