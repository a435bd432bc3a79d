"""Parity of the sm_103a path (through the C ABI) with the oracle.

Bar: depth tiles, render AABBs and integer fitness counts bit-exact; the
fitness and the whole PSO trajectory bit-exact as well (both sides follow
the same arithmetic contract), which is stricter than the 0.5 deg / 1 mm
pose tolerance; float fitness within 1e-5 relative of an FP64
recomputation from the integer counts.
"""
import numpy as np
import pytest

import scene
from oracle import pyoracle as po
from tests.helpers import gpu_camera, gpu_desc, oracle_obs, oracle_params, rot_err_deg, upload_workload

pytestmark = pytest.mark.gpu

FIT_RTOL_FP64 = 1e-5
POSE_TOL_DEG = 0.5
POSE_TOL_M = 1e-3


@pytest.fixture(scope="module")
def c1_gpu(gpu_ctx, c1):
    mids, fids = upload_workload(gpu_ctx, c1)
    return c1, mids, fids


def random_poses(rng, s, n, spread=1.0):
    f = scene.solve_fields(s)
    lo, hi = np.array(f["t_lo"]), np.array(f["t_hi"])
    c = (lo + hi) / 2
    t = c + (rng.uniform(-1, 1, (n, 3)) * (hi - lo) / 2 * spread)
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    q[q[:, 0] < 0] *= -1
    return np.concatenate([t, q], 1).astype(np.float32)


def test_render_tiles_bit_exact(gpu_ctx, c1_gpu):
    w, mids, _ = c1_gpu
    soa, F = w["meshes"][0]
    s = w["solves"][0]
    rng = np.random.default_rng(1)
    poses = np.concatenate([s["gt_pose"][None], random_poses(rng, s, 24, 0.4)])
    cam_o, cam_g = po.camera(), gpu_camera()
    for pose in poses:
        zb, box, _ = po.render(soa, F, pose, cam_o)
        x0, x1, y0, y1 = box
        x0 = max(int(x0), -po.GUARD) & ~3
        y0 = max(int(y0), -po.GUARD)
        ww = min(((min(int(x1), 640 + po.GUARD) - x0 + 3) & ~3), 200)
        hh = min(min(int(y1), 480 + po.GUARD) - y0, 200)
        if ww <= 0 or hh <= 0:
            continue
        tile, gbox = gpu_ctx.render(mids[0], cam_g, pose, x0, y0, ww, hh)
        np.testing.assert_array_equal(gbox, box)
        want = zb[y0 + po.GUARD:y0 + po.GUARD + hh, x0 + po.GUARD:x0 + po.GUARD + ww]
        np.testing.assert_array_equal(tile, want)


def test_best_pose_depth_image_bit_exact(gpu_ctx, c1_gpu):
    """The best-pose depth image (RenderCPU arithmetic: iround snapping,
    float depth) equals the oracle's restatement, pinned against the
    reference's own host render, for in-view, partly off-image and
    near-camera poses of the C1 mesh and of a 12-face box."""
    w, mids, _ = c1_gpu
    soa, F = w["meshes"][0]
    s = w["solves"][0]
    rng = np.random.default_rng(12)
    cam_o, cam_g = po.camera(), gpu_camera()
    poses = [s["gt_pose"]] + list(random_poses(rng, s, 6, 0.6))
    edge = np.array(s["gt_pose"], np.float32).copy()
    edge[0] += 0.2  # partly right of the image
    near = np.array(s["gt_pose"], np.float32).copy()
    near[:3] = [0.0, 0.0, 0.1]  # object filling most of the frame
    poses += [edge, near]
    box_soa, box_F = scene.make_mesh("box", 12, 80.0, seed=1)
    box_id = gpu_ctx.mesh_upload(box_soa, box_F)
    for mesh, nf, mid in [(soa, F, mids[0]), (box_soa, box_F, box_id)]:
        for pose in poses:
            want = po.render_cpu(mesh, nf, pose, cam_o)
            got = gpu_ctx.render_depth_f32(mid, cam_g, pose)
            np.testing.assert_array_equal(got, want)
    assert (po.render_cpu(soa, F, near, cam_o) < 60000).mean() > 0.2


def _oracle_scores(w, s, poses, **over):
    soa, F = w["meshes"][s["mesh"]]
    prm = oracle_params(s, **over)
    obs = oracle_obs(w, s)
    cam = po.camera()
    out = []
    for pose in poses:
        zb, box, _ = po.render(soa, F, pose, cam, mode=prm.raster_mode)
        out.append(po.score(zb, box, obs, cam, prm))
    return out, prm


def test_edge_mode_fitness_trace_and_batch_bit_exact(gpu_ctx, c1_gpu):
    """QPSO_RASTER_EDGE (the reference's inside mask applied): fitness of
    given poses, a solve's per-iteration global best and final swarm, the
    raster write count, and batched == plain with REF and EDGE solves mixed
    in one launch, all equal to the oracle's EDGE mode."""
    import qpso

    w, mids, fids = c1_gpu
    s = dict(w["solves"][0], particles=48, iterations=10, seed=11, stream=3)
    soa, F = w["meshes"][0]
    rng = np.random.default_rng(21)
    poses = np.concatenate([s["gt_pose"][None], random_poses(rng, s, 15, 0.4)])
    d_edge = gpu_desc(s, mids[0], fids[0], raster_mode=qpso.RASTER_EDGE)
    d_ref = gpu_desc(s, mids[0], fids[0])
    scores, _ = _oracle_scores(w, s, poses, raster_mode=po.RASTER_EDGE)
    got = gpu_ctx.score_poses(d_edge, poses)
    np.testing.assert_array_equal(got, np.array([sc.fit for sc in scores], np.float32))
    assert not np.array_equal(got, gpu_ctx.score_poses(d_ref, poses))  # the modes do differ
    want = po.solve(soa, F, oracle_obs(w, s), po.camera(), oracle_params(s, raster_mode=po.RASTER_EDGE),
                    trace=True)
    r, st = gpu_ctx.solve_traced(d_edge)
    assert r.flags == 0
    np.testing.assert_array_equal(st["trace_gbest"], want["trace_gbest"])
    np.testing.assert_array_equal(st["pos"], want["pos"])
    np.testing.assert_array_equal(st["pbest_fit"], want["pbest_fit"])
    assert r.raster_writes == want["raster_writes"]
    rb = gpu_ctx.solve_batch([d_ref, d_edge, d_ref])
    ra = gpu_ctx.solve(d_ref)
    for x, y in [(rb[0], ra), (rb[1], r), (rb[2], ra)]:
        assert x.fit == y.fit and list(x.pose) == list(y.pose) and x.raster_writes == y.raster_writes
    old = gpu_ctx.get_launch_config()
    try:  # several tile passes per render
        gpu_ctx.set_launch_config(plain=(128, 1024, 2))
        np.testing.assert_array_equal(gpu_ctx.score_poses(d_edge, poses), got)
    finally:
        gpu_ctx.set_launch_config(plain=old[0], batch=old[1])
    with pytest.raises(qpso.QpsoError) as e:
        gpu_ctx.solve(gpu_desc(s, mids[0], fids[0], raster_mode=7))
    assert e.value.status == qpso.ERR_ARG


def test_ref_mode_raster_writes_match_oracle(gpu_ctx, c1_gpu):
    """The write count of a REF solve is the oracle's (rectangle pixels
    inside the raster domain), at one and at many tile passes."""
    w, mids, fids = c1_gpu
    s = dict(w["solves"][0], particles=32, iterations=6, seed=2, stream=5)
    soa, F = w["meshes"][0]
    want = po.solve(soa, F, oracle_obs(w, s), po.camera(), oracle_params(s), trace=True)
    old = gpu_ctx.get_launch_config()
    try:
        for cfg in [(256, 16384, 1), (128, 1024, 2)]:
            gpu_ctx.set_launch_config(plain=cfg)
            assert gpu_ctx.solve(gpu_desc(s, mids[0], fids[0])).raster_writes == want["raster_writes"]
    finally:
        gpu_ctx.set_launch_config(plain=old[0], batch=old[1])


def test_fitness_bit_exact_and_fp64(gpu_ctx, c1_gpu):
    w, mids, fids = c1_gpu
    s = w["solves"][0]
    rng = np.random.default_rng(2)
    poses = np.concatenate([s["gt_pose"][None], random_poses(rng, s, 200, 1.0)])
    got = gpu_ctx.score_poses(gpu_desc(s, mids[0], fids[0]), poses)
    scores, prm = _oracle_scores(w, s, poses)
    want = np.array([sc.fit for sc in scores], np.float32)
    np.testing.assert_array_equal(got, want)
    for sc in scores:
        if sc.n_rendered:
            ref = po.fitness_fp64(sc, prm.num_points)
            assert abs(sc.fit - ref) <= FIT_RTOL_FP64 * abs(ref)


def test_fitness_full_frame_window_and_partial_row(gpu_ctx, c1_gpu):
    """Cluster AABB = the whole frame (the stress configuration's window)
    and odd windows whose area leaves a partial last row."""
    w, mids, fids = c1_gpu
    s = w["solves"][0]
    rng = np.random.default_rng(3)
    poses = random_poses(rng, s, 40, 0.8)
    for aabb in [(0, 640, 0, 480), (300, 371, 90, 153), (310, 313, 100, 400)]:
        over = dict(cl_min_x=aabb[0], cl_max_x=aabb[1], cl_min_y=aabb[2], cl_max_y=aabb[3])
        got = gpu_ctx.score_poses(gpu_desc(s, mids[0], fids[0], **over), poses)
        scores, _ = _oracle_scores(w, s, poses, **over)
        np.testing.assert_array_equal(got, np.array([sc.fit for sc in scores], np.float32))
        assert any(sc.partial_len > 0 for sc in scores) or aabb == (0, 640, 0, 480)


def test_fitness_off_screen_and_behind_camera(gpu_ctx, c1_gpu):
    """Poses whose render leaves the image, leaves the raster domain, or
    puts vertices behind the camera (no conservative bound: banded passes)."""
    w, mids, fids = c1_gpu
    s = w["solves"][0]
    gt = s["gt_pose"].copy()
    poses = []
    for dx, dy, dz in [(0.25, 0, 0), (-0.3, 0.1, 0), (0, 0.25, -0.2), (0.9, 0, -0.5), (0, 0, -0.66),
                       (0, 0, -0.69), (0, 0, -0.75), (3.0, 0, 0), (0, 0, 0.5)]:
        p = gt.copy()
        p[:3] += np.float32([dx, dy, dz])
        poses.append(p)
    poses = np.array(poses, np.float32)
    got = gpu_ctx.score_poses(gpu_desc(s, mids[0], fids[0]), poses)
    scores, _ = _oracle_scores(w, s, poses)
    np.testing.assert_array_equal(got, np.array([sc.fit for sc in scores], np.float32))


@pytest.mark.parametrize("kind,n,extent", [("box", 12, 150.0), ("icosphere", 80, 220.0),
                                           ("cylinder", 40, 180.0)])
def test_low_poly_meshes_large_faces(gpu_ctx, c1_gpu, kind, n, extent):
    """Few large faces (rectangles of hundreds of pixels): the warp-wide
    raster path must match the oracle as exactly as the per-lane path."""
    w, _, fids = c1_gpu
    s = w["solves"][0]
    soa, F = scene.make_mesh(kind, n, extent, seed=4, bump_mm=0.0)
    mid = gpu_ctx.mesh_upload(soa, F)
    rng = np.random.default_rng(6)
    poses = random_poses(rng, s, 48, 0.7)
    got = gpu_ctx.score_poses(gpu_desc(s, mid, fids[0]), poses)
    prm = oracle_params(s)
    obs = oracle_obs(w, s)
    cam = po.camera()
    want = []
    for pose in poses:
        zb, box, _ = po.render(soa, F, pose, cam)
        want.append(po.score(zb, box, obs, cam, prm).fit)
    np.testing.assert_array_equal(got, np.array(want, np.float32))
    # a short solve with this mesh, batched and plain
    s2 = dict(s, particles=24, iterations=6, seed=9, stream=3)
    want = po.solve(soa, F, obs, cam, oracle_params(s2), trace=True)
    r, st = gpu_ctx.solve_traced(gpu_desc(s2, mid, fids[0]))
    np.testing.assert_array_equal(st["trace_gbest"], want["trace_gbest"])
    rb = gpu_ctx.solve_batch([gpu_desc(s2, mid, fids[0])])[0]
    assert rb.fit == want["fit"]
    gpu_ctx.mesh_release(mid)


def test_stress_mesh_full_frame_window(gpu_ctx):
    """The stress configuration's sizes: the 327,680-face level-7 icosphere
    (2,560+ meshlets, so passes after the first cull meshlets by their
    projected object-space boxes) and a full 640x480 fitness window.  Fitness
    of several poses (near the ground truth and spread over the box) and a
    short solve's trace equal the oracle's, with one pass per render and with
    many tile passes.  (512, 49152, 1) fits a CTA only with 64-vertex
    meshlet caches: for this mesh's 128-vertex meshlets the library halves
    its tile, and the results stay the same."""
    w = scene.workload_c5(particles=8, iterations=3)
    mids, fids = upload_workload(gpu_ctx, w)
    s = w["solves"][0]
    soa, F = w["meshes"][0]
    d = gpu_desc(s, mids[0], fids[0])
    rng = np.random.default_rng(8)
    poses = np.concatenate([s["gt_pose"][None], random_poses(rng, s, 5, 0.5)])
    scores, _ = _oracle_scores(w, s, poses)
    want = np.array([sc.fit for sc in scores], np.float32)
    assert scores[0].n_rendered > 0
    trace = po.solve(soa, F, oracle_obs(w, s), po.camera(), oracle_params(s), trace=True)
    old = gpu_ctx.get_launch_config()
    try:
        for cfg in [(256, 49152, 1), (256, 2048, 1), (128, 4096, 2), (512, 49152, 1)]:
            gpu_ctx.set_launch_config(plain=cfg, batch=cfg)
            np.testing.assert_array_equal(gpu_ctx.score_poses(d, poses), want)
            r, st = gpu_ctx.solve_traced(d)
            assert r.flags == 0
            np.testing.assert_array_equal(st["trace_gbest"], trace["trace_gbest"])
            rb = gpu_ctx.solve_batch([d])[0]
            assert rb.flags == 0 and rb.fit == r.fit and list(rb.pose) == list(r.pose)
            if cfg[1] == 2048:
                assert r.tile_passes > 4 * s["particles"] * s["iterations"]
    finally:
        gpu_ctx.set_launch_config(plain=old[0], batch=old[1])
    # the reported best fitness is the fitness of the reported pose
    again = gpu_ctx.score_poses(d, np.array(r.pose[:], np.float32)[None])
    assert again[0] == r.fit


def test_small_tiles_force_multipass(gpu_ctx, c1_gpu):
    """A tile capacity far below the render bound makes every particle-render
    take several row/column passes; the fitness must not change."""
    w, mids, fids = c1_gpu
    s = w["solves"][0]
    rng = np.random.default_rng(4)
    poses = random_poses(rng, s, 32, 0.5)
    base = gpu_ctx.score_poses(gpu_desc(s, mids[0], fids[0]), poses)
    old = gpu_ctx.get_launch_config()
    try:
        gpu_ctx.set_launch_config(plain=(128, 256, 1))
        small = gpu_ctx.score_poses(gpu_desc(s, mids[0], fids[0]), poses)
    finally:
        gpu_ctx.set_launch_config(plain=old[0], batch=old[1])
    np.testing.assert_array_equal(small, base)


def test_plain_solve_trace_bit_exact(gpu_ctx, c1_gpu):
    """C1 (64 particles x 50 iterations, Philox seed 0): the global-best
    trace of every iteration and the final swarm equal the oracle's."""
    w, mids, fids = c1_gpu
    s = w["solves"][0]
    soa, F = w["meshes"][0]
    want = po.solve(soa, F, oracle_obs(w, s), po.camera(), oracle_params(s), trace=True)
    r, st = gpu_ctx.solve_traced(gpu_desc(s, mids[0], fids[0]))
    assert r.flags == 0
    np.testing.assert_array_equal(st["trace_gbest"], want["trace_gbest"])
    np.testing.assert_array_equal(st["pos"], want["pos"])
    np.testing.assert_array_equal(st["vel"], want["vel"])
    np.testing.assert_array_equal(st["pbest"], want["pbest"])
    np.testing.assert_array_equal(st["pbest_fit"], want["pbest_fit"])
    pose = np.array(r.pose[:], np.float32)
    assert np.abs(pose[:3] - want["pose"][:3]).max() <= POSE_TOL_M
    assert rot_err_deg(pose[3:], want["pose"][3:]) <= POSE_TOL_DEG
    g = np.load("tests/golden/oracle_c1.npz")
    np.testing.assert_array_equal(st["trace_gbest"], g["trace_gbest"])


@pytest.mark.parametrize("cfg", [(256, 16384, 1), (128, 4096, 4), (512, 8192, 3), (256, 512, 5), (256, 1024, 10)])
def test_plain_launch_shapes_agree(gpu_ctx, c1_gpu, cfg):
    w, mids, fids = c1_gpu
    s = dict(w["solves"][0], particles=40, iterations=12, seed=5, stream=9)
    soa, F = w["meshes"][0]
    want = po.solve(soa, F, oracle_obs(w, s), po.camera(), oracle_params(s), trace=True)
    old = gpu_ctx.get_launch_config()
    try:
        gpu_ctx.set_launch_config(plain=cfg)
        r, st = gpu_ctx.solve_traced(gpu_desc(s, mids[0], fids[0]))
    finally:
        gpu_ctx.set_launch_config(plain=old[0], batch=old[1])
    np.testing.assert_array_equal(st["trace_gbest"], want["trace_gbest"])


def test_batch_equals_plain_and_oracle(gpu_ctx, c1_gpu):
    """Uneven instances (particle counts, iteration counts, seeds, cluster
    windows) in one persistent launch give the same results as their own
    plain solves and as the oracle."""
    w, mids, fids = c1_gpu
    base = w["solves"][0]
    soa, F = w["meshes"][0]
    variants = [dict(particles=64, iterations=20, seed=0, stream=0),
                dict(particles=37, iterations=9, seed=1, stream=1),
                dict(particles=128, iterations=15, seed=2, stream=2),
                dict(particles=5, iterations=25, seed=3, stream=3),
                dict(particles=96, iterations=1, seed=4, stream=4)]
    solves = [dict(base, **v) for v in variants]
    descs = [gpu_desc(s, mids[0], fids[0]) for s in solves]
    wants = [po.solve(soa, F, oracle_obs(w, s), po.camera(), oracle_params(s)) for s in solves]
    plains = [gpu_ctx.solve(d) for d in descs]
    for cfg in [(256, 16384, 1), (256, 8192, 2)]:
        old = gpu_ctx.get_launch_config()
        try:
            gpu_ctx.set_launch_config(batch=cfg)
            res = gpu_ctx.solve_batch(descs)
            res2 = gpu_ctx.solve_batch(descs)  # graph replay
        finally:
            gpu_ctx.set_launch_config(plain=old[0], batch=old[1])
        for r, r2, plain, want in zip(res, res2, plains, wants):
            assert r.flags == 0
            assert r.fit == plain.fit == want["fit"] == r2.fit
            np.testing.assert_array_equal(np.array(r.pose[:], np.float32), want["pose"])
            np.testing.assert_array_equal(np.array(r2.pose[:], np.float32), want["pose"])


def test_autotune_keeps_results(gpu_ctx, c1_gpu):
    """The autotuner only changes speed: after tuning either path, solves
    still equal the oracle bit for bit."""
    w, mids, fids = c1_gpu
    soa, F = w["meshes"][0]
    solves = [dict(w["solves"][0], particles=48, iterations=6, seed=21, stream=s) for s in range(3)]
    descs = [gpu_desc(s, mids[0], fids[0]) for s in solves]
    old = gpu_ctx.get_launch_config()
    try:
        cfg_p, ms_p = gpu_ctx.autotune(descs, batched=False, tune_iters=2)
        cfg_b, ms_b = gpu_ctx.autotune(descs, batched=True, tune_iters=2)
        assert gpu_ctx.get_launch_config() == (cfg_p, cfg_b)
        assert ms_p > 0 and ms_b > 0
        res = gpu_ctx.solve_batch(descs)
        for s, d, r in zip(solves, descs, res):
            want = po.solve(soa, F, oracle_obs(w, s), po.camera(), oracle_params(s))
            assert r.fit == want["fit"] and gpu_ctx.solve(d).fit == want["fit"]
            np.testing.assert_array_equal(np.array(r.pose[:], np.float32), want["pose"])
    finally:
        gpu_ctx.set_launch_config(plain=old[0], batch=old[1])


def test_solution_near_ground_truth(gpu_ctx, c1_gpu):
    """Sanity of the whole solve: the best fitness is at most a little above
    the fitness of the ground-truth pose (the ellipsoid is nearly symmetric,
    so the pose itself may be a symmetric twin)."""
    w, mids, fids = c1_gpu
    s = w["solves"][0]
    r = gpu_ctx.solve(gpu_desc(s, mids[0], fids[0]))
    gt_fit = gpu_ctx.score_poses(gpu_desc(s, mids[0], fids[0]), s["gt_pose"][None])[0]
    assert r.fit <= 2.0 * gt_fit
    assert np.abs(np.array(r.pose[:3]) - s["gt_pose"][:3]).max() < 0.03


def test_bounded_wait_expires(gpu_ctx):
    import qpso

    st, bits = gpu_ctx.barrier_selftest(50_000_000)
    assert st == qpso.ERR_TIMEOUT and bits & qpso.ERR_BIT_TIMEOUT
    # the context is still usable afterwards
    st2, _ = gpu_ctx.barrier_selftest(10_000_000)
    assert st2 == qpso.ERR_TIMEOUT


def test_argument_errors(gpu_ctx, c1_gpu):
    import qpso

    w, mids, fids = c1_gpu
    s = w["solves"][0]
    with pytest.raises(qpso.QpsoError) as e:
        gpu_ctx.solve(gpu_desc(s, 9999, fids[0]))
    assert e.value.status == qpso.ERR_NOT_FOUND
    with pytest.raises(qpso.QpsoError) as e:
        gpu_ctx.solve(gpu_desc(s, mids[0], fids[0], num_particles=0))
    assert e.value.status == qpso.ERR_ARG
    with pytest.raises(qpso.QpsoError) as e:
        gpu_ctx.solve(gpu_desc(s, mids[0], fids[0], cl_min_x=10, cl_max_x=10))
    assert e.value.status == qpso.ERR_ARG
    with pytest.raises(qpso.QpsoError) as e:
        gpu_ctx.solve(gpu_desc(s, mids[0], fids[0], num_points=0))
    assert e.value.status == qpso.ERR_ARG
    with pytest.raises(qpso.QpsoError) as e:
        gpu_ctx.set_launch_config(plain=(100, 16384, 1))
    assert e.value.status == qpso.ERR_ARG
    with pytest.raises(qpso.QpsoError):
        gpu_ctx.mesh_upload(np.full(9, np.nan, np.float32), 1)
    depth, labels, _ = w["frames"][0]
    with pytest.raises(qpso.QpsoError) as e:  # unknown projection
        gpu_ctx.frame_upload(depth, qpso.Camera(525, 525, 319.5, 239.5, 640, 480, 7), labels=labels)
    assert e.value.status == qpso.ERR_ARG
