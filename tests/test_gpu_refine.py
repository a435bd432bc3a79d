"""qpso_refine: the local refinement of a solved pose, on the GPU, against
the oracle's replay of the same search (oracle/pyoracle.py refine): the
same candidates scored by the oracle's render and fitness.  Bar: the
refined pose and its fitness bit-equal, in both raster modes; the fitness
never above the starting pose's; the search deterministic; and, from
ground-truth poses of the C2 meshes moved by a few millimetres and
degrees, the translation error reduced."""
import numpy as np
import pytest

import qpso
import scene
from oracle import pyoracle as po
from tests.helpers import gpu_desc, oracle_obs, oracle_params, upload_workload

pytestmark = pytest.mark.gpu


def _perturbed(rng, gt, dt=0.006, dr=0.08):
    p = np.array(gt, np.float64)
    p[:3] += rng.normal(0, dt, 3)
    q = np.array(p[3:], np.float64)
    h = rng.normal(0, dr, 3) * 0.5
    dq = np.array([1.0, *h])
    w0, x0, y0, z0 = dq
    w1, x1, y1, z1 = q
    r = np.array([w0 * w1 - x0 * x1 - y0 * y1 - z0 * z1, w0 * x1 + x0 * w1 + y0 * z1 - z0 * y1,
                  w0 * y1 - x0 * z1 + y0 * w1 + z0 * x1, w0 * z1 + x0 * y1 - y0 * x1 + z0 * w1])
    p[3:] = r / np.linalg.norm(r)
    return p.astype(np.float32)


@pytest.mark.parametrize("mode", [qpso.RASTER_EDGE, qpso.RASTER_REF], ids=["edge", "ref"])
def test_refine_equals_the_oracle_replay(gpu_ctx, c1, mode):
    w = c1
    s = w["solves"][0]
    soa, F = w["meshes"][0]
    mids, fids = upload_workload(gpu_ctx, w)
    desc = gpu_desc(s, mids[0], fids[0], seed=3, stream=1)
    p0 = _perturbed(np.random.default_rng(5), s["gt_pose"])
    prm = qpso.refine_params(rounds=8, candidates=24, raster_mode=mode)
    pose, fit = gpu_ctx.refine(desc, p0, prm)
    want_pose, want_fit = po.refine(soa, F, oracle_obs(w, s), po.camera(), oracle_params(s), p0, 3, 1,
                                    rounds=8, candidates=24, step_t=prm.step_t, step_rot=prm.step_rot, mode=mode)
    np.testing.assert_array_equal(pose, want_pose)
    assert np.float32(fit) == want_fit
    # never worse than the start (the normalised input pose), and deterministic
    start_pose, start = po.refine(soa, F, oracle_obs(w, s), po.camera(), oracle_params(s), p0, 3, 1,
                                  rounds=0, candidates=24, step_t=prm.step_t, step_rot=prm.step_rot, mode=mode)
    assert fit <= start
    pose2, fit2 = gpu_ctx.refine(desc, p0, prm)
    np.testing.assert_array_equal(pose2, pose)
    assert fit2 == fit


def test_refine_reduces_translation_error_near_the_truth(gpu_ctx):
    """The fitness optimum is not exactly the true pose (depth noise, 5%
    dropout, nearly symmetric shapes), so not every pose improves; over the
    frame's eight solves the search (default parameters) is deterministic
    and, as the oracle's replay of it shows, six of eight move closer and
    the median error does not rise (9.9 to 9.8 mm; one solve's first steps
    of 3 cm carry it to a worse optimum of the fitness, 7.7 to 37 mm)."""
    w = scene.workload_c2(particles=64, iterations=10)
    mids, fids = upload_workload(gpu_ctx, w)
    rng = np.random.default_rng(3)
    before, after = [], []
    for s in w["solves"]:
        gt = np.asarray(s["gt_pose"], np.float64)
        p0 = _perturbed(rng, gt)
        pose, _ = gpu_ctx.refine(gpu_desc(s, mids[s["mesh"]], fids[s["frame"]]), p0)
        before.append(np.linalg.norm(p0[:3] - gt[:3]))
        after.append(np.linalg.norm(pose[:3] - gt[:3]))
    before, after = np.array(before), np.array(after)
    assert (after < before).sum() >= 6, (before, after)
    assert np.median(after) <= np.median(before), (before, after)


def test_refine_argument_errors(gpu_ctx, c1):
    w = c1
    s = w["solves"][0]
    mids, fids = upload_workload(gpu_ctx, w)
    desc = gpu_desc(s, mids[0], fids[0])
    for bad in (qpso.refine_params(candidates=11), qpso.refine_params(raster_mode=7),
                qpso.refine_params(step_t=float("nan"))):
        with pytest.raises(qpso.QpsoError) as e:
            gpu_ctx.refine(desc, s["gt_pose"], bad)
        assert e.value.status == qpso.ERR_ARG
    p = np.array(s["gt_pose"], np.float32)
    p[0] = np.inf
    with pytest.raises(qpso.QpsoError) as e:
        gpu_ctx.refine(desc, p)
    assert e.value.status == qpso.ERR_ARG
