"""qpso_score_poses_noalloc: scoring for callers that cannot let a library
call cudaMalloc (their device memory belongs to their own pool or caching
allocator, or they run a real-time loop where an allocation's implicit
synchronisation is not acceptable).  The caller owns every input and output
buffer on the device; the entry point keeps its intermediates in a fixed
4 MiB device array.  Its fitness must equal the allocating entry point's
(qpso_score_poses) bit for bit, on two calls in a row that share the array.

Kept in a file of its own, collected after the other test files.
"""
import ctypes as C

import numpy as np
import pytest

import scene
from tests.helpers import gpu_camera, gpu_desc, upload_workload

pytestmark = pytest.mark.gpu


def _poses(rng, s, n):
    f = scene.solve_fields(s)
    lo, hi = np.array(f["t_lo"]), np.array(f["t_hi"])
    t = (lo + hi) / 2 + rng.uniform(-0.5, 0.5, (n, 3)) * (hi - lo) / 2
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    q[q[:, 0] < 0] *= -1
    p = np.concatenate([t, q], 1).astype(np.float32)
    p[0] = s["gt_pose"]
    return p


@pytest.mark.parametrize("masked", [False, True], ids=["label", "premasked"])
@pytest.mark.parametrize("projection", [0, 1], ids=["fp32", "ref_accv"])
@pytest.mark.parametrize("raster_mode", [0, 1], ids=["ref", "edge"])
def test_noalloc_scoring_equals_allocating_scoring(gpu_ctx, c1, raster_mode, projection, masked):
    """Both raster modes, both camera projections, and a cluster selected
    from the label map (cluster_label >= 0) or given as depth already masked
    to it (cluster_label = -1)."""
    torch = pytest.importorskip("torch")
    import qpso

    L = qpso.load_library()
    w = c1
    s = w["solves"][0]
    soa, F = w["meshes"][0]
    depth, labels, _ = w["frames"][0]
    label = s["cluster"]["label"]
    if masked:
        depth = scene.masked_depth(depth, labels, label)
    cam = qpso.Camera(*scene.camera_tuple(), projection)
    mid = gpu_ctx.mesh_upload(soa, F)
    fid = gpu_ctx.frame_upload(depth, cam, labels=None if masked else labels)
    over = dict(raster_mode=raster_mode)
    if masked:
        over["cluster_label"] = -1
    desc = gpu_desc(s, mid, fid, **over)
    rng = np.random.default_rng(11 + 4 * raster_mode + 2 * projection + int(masked))
    poses_a, poses_b = _poses(rng, s, 97), _poses(rng, s, 64)
    want_a = gpu_ctx.score_poses(desc, poses_a)
    want_b = gpu_ctx.score_poses(desc, poses_b)
    assert np.isfinite(want_a[0]) and np.isfinite(want_b[0])

    dev = torch.device("cuda", 0)
    d_mesh = torch.from_numpy(np.ascontiguousarray(soa, np.float32)).to(dev)
    d_depth = torch.from_numpy(np.ascontiguousarray(depth).view(np.int16)).to(dev)
    d_labels = torch.from_numpy(np.ascontiguousarray(labels, np.int32)).to(dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    try:
        for poses, want in ((poses_a, want_a), (poses_b, want_b)):
            d_poses = torch.from_numpy(poses).to(dev)
            d_fit = torch.full((len(poses),), -1.0, dtype=torch.float32, device=dev)
            d_flags = torch.full((1,), 7, dtype=torch.int32, device=dev)
            torch.cuda.synchronize(dev)
            st = L.qpso_score_poses_noalloc(d_mesh.data_ptr(), F, d_depth.data_ptr(),
                                            None if masked else d_labels.data_ptr(), C.byref(cam),
                                            C.byref(desc), d_poses.data_ptr(), len(poses),
                                            d_fit.data_ptr(), d_flags.data_ptr(), C.c_void_p(stream))
            assert st == qpso.OK
            torch.cuda.synchronize(dev)
            got = d_fit.cpu().numpy()
            np.testing.assert_array_equal(got, want)
            assert int(d_flags.cpu().item()) == 0
    finally:
        gpu_ctx.frame_release(fid)
        gpu_ctx.mesh_release(mid)


def test_noalloc_refuses_what_the_allocating_path_refuses(gpu_ctx, c1):
    """Cluster boxes outside the raster domain, labels below -1, unknown
    raster modes and non-finite intrinsics are argument errors here as in
    qpso_score_poses and qpso_frame_upload.  Every check comes before any
    pointer is dereferenced, so the dummy pointers are never read."""
    import qpso

    L = qpso.load_library()
    s = c1["solves"][0]
    dummy = C.c_void_p(16)
    cam = qpso.Camera(*scene.camera_tuple())
    bad_descs = [gpu_desc(s, 0, 0, cl_min_x=-2000), gpu_desc(s, 0, 0, cl_max_y=480 + 1025),
                 gpu_desc(s, 0, 0, cluster_label=-2), gpu_desc(s, 0, 0, raster_mode=2),
                 gpu_desc(s, 0, 0, num_points=0)]
    for d in bad_descs:
        st = L.qpso_score_poses_noalloc(dummy, 1, dummy, dummy, C.byref(cam), C.byref(d), dummy, 1,
                                        dummy, None, None)
        assert st == qpso.ERR_ARG
    good = gpu_desc(s, 0, 0)
    for bad_cam in [qpso.Camera(float("nan"), 525.0, 319.5, 239.5, 640, 480),
                    qpso.Camera(525.0, 525.0, float("inf"), 239.5, 640, 480),
                    qpso.Camera(525.0, 525.0, 319.5, 239.5, 640, 480, 5)]:
        st = L.qpso_score_poses_noalloc(dummy, 1, dummy, dummy, C.byref(bad_cam), C.byref(good),
                                        dummy, 1, dummy, None, None)
        assert st == qpso.ERR_ARG


def test_noalloc_rejects_frames_beyond_the_scratch(gpu_ctx, c1):
    import qpso

    L = qpso.load_library()
    s = c1["solves"][0]
    desc = gpu_desc(s, 0, 0)
    big = qpso.Camera(525.0, 525.0, 1023.5, 1023.5, 2048, 2048)
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    st = L.qpso_score_poses_noalloc(dummy, 1, dummy, dummy, C.byref(big), C.byref(desc), dummy, 1,
                                    dummy, None, None)
    assert st == qpso.ERR_ARG
