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


def test_noalloc_scoring_equals_allocating_scoring(gpu_ctx, c1):
    torch = pytest.importorskip("torch")
    import qpso

    L = qpso.load_library()
    w = c1
    s = w["solves"][0]
    soa, F = w["meshes"][0]
    depth, labels, _ = w["frames"][0]
    mids, fids = upload_workload(gpu_ctx, w)
    desc = gpu_desc(s, mids[0], fids[0])
    rng = np.random.default_rng(11)
    poses_a, poses_b = _poses(rng, s, 97), _poses(rng, s, 64)
    want_a = gpu_ctx.score_poses(desc, poses_a)
    want_b = gpu_ctx.score_poses(desc, poses_b)

    dev = torch.device("cuda", 0)
    d_mesh = torch.from_numpy(np.ascontiguousarray(soa, np.float32)).to(dev)
    d_depth = torch.from_numpy(np.ascontiguousarray(depth).view(np.int16)).to(dev)
    d_labels = torch.from_numpy(np.ascontiguousarray(labels, np.int32)).to(dev)
    cam = gpu_camera()
    stream = torch.cuda.current_stream(dev).cuda_stream
    for poses, want in ((poses_a, want_a), (poses_b, want_b)):
        d_poses = torch.from_numpy(poses).to(dev)
        d_fit = torch.full((len(poses),), -1.0, dtype=torch.float32, device=dev)
        d_flags = torch.full((1,), 7, dtype=torch.int32, device=dev)
        torch.cuda.synchronize(dev)
        st = L.qpso_score_poses_noalloc(d_mesh.data_ptr(), F, d_depth.data_ptr(),
                                        d_labels.data_ptr(), C.byref(cam), C.byref(desc),
                                        d_poses.data_ptr(), len(poses), d_fit.data_ptr(),
                                        d_flags.data_ptr(), C.c_void_p(stream))
        assert st == qpso.OK
        torch.cuda.synchronize(dev)
        got = d_fit.cpu().numpy()
        np.testing.assert_array_equal(got, want)
        assert int(d_flags.cpu().item()) == 0


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
