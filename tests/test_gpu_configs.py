"""Parity with the oracle at the shapes of the benchmark configurations.

* C3 (batching): one persistent launch over clusters of meshes of uneven
  size, 1k to 34k faces, so that meshes cut into 64-face meshlets (up to
  16,384 faces) and into 128-face meshlets share a launch; 128, 512 and
  1024 particles; cluster windows from about 40 to 300 px a side.  The
  iterations are cut to 6 so that the oracle finishes in seconds.
* C4 (serving): requests over the serving pool's meshes (up to 93k faces),
  256 and 1024 particles, admitted while others run, each result compared
  with the oracle directly.
* C2 (production size): 256 particles x 100 iterations, every cluster of a
  frame, the plain trace and the batched results against the oracle.

The loop being matched is the reference's host loop (main.cu:1625-1727).
Bar: bit-exact fitness, pose and raster write counts (which implies the
0.5 deg / 1 mm pose tolerance, also asserted).
"""
import os
import time

import numpy as np
import pytest

import scene
from oracle import pyoracle as po
from tests.helpers import gpu_desc, oracle_obs, oracle_params, rot_err_deg, upload_workload

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1
POSE_TOL_DEG = 0.5
POSE_TOL_M = 1e-3


def oracle_solve(w, s, trace=False):
    soa, F = w["meshes"][s["mesh"]]
    return po.solve(soa, F, oracle_obs(w, s), po.camera(), oracle_params(s), trace=trace,
                    threads=THREADS)


def assert_matches_oracle(r, want):
    assert r.flags == 0
    assert r.fit == want["fit"]
    pose = np.array(r.pose[:], np.float32)
    np.testing.assert_array_equal(pose, want["pose"])
    assert r.raster_writes == want["raster_writes"]
    assert np.abs(pose[:3] - want["pose"][:3]).max() <= POSE_TOL_M
    assert rot_err_deg(pose[3:], want["pose"][3:]) <= POSE_TOL_DEG


@pytest.fixture(scope="module")
def c3_mix(gpu_ctx):
    w = scene.workload_c3(n_frames=3, iterations=6)
    order = sorted(range(len(w["solves"])), key=lambda i: w["meshes"][w["solves"][i]["mesh"]][1])
    n = len(order)
    pick = [order[0], order[n // 5], order[2 * n // 5], order[3 * n // 5], order[4 * n // 5],
            order[n - 2], order[n - 1]]
    counts = (128, 512, 1024)
    solves = [dict(w["solves"][i], particles=counts[j % 3]) for j, i in enumerate(pick)]
    mids, fids = upload_workload(gpu_ctx, w)
    descs = [gpu_desc(s, mids[s["mesh"]], fids[s["frame"]]) for s in solves]
    wants = [oracle_solve(w, s, trace=True) for s in solves]
    return w, solves, descs, wants


def test_c3_mix_covers_the_config(c3_mix):
    w, solves, _, _ = c3_mix
    faces = [w["meshes"][s["mesh"]][1] for s in solves]
    sides = [max(s["cluster"]["aabb"][1] - s["cluster"]["aabb"][0],
                 s["cluster"]["aabb"][3] - s["cluster"]["aabb"][2]) for s in solves]
    assert len({s["mesh"] for s in solves}) >= 4
    assert min(faces) < 1500 and max(faces) > 16384  # 64- and 128-face meshlets in one launch
    assert {s["particles"] for s in solves} == {128, 512, 1024}
    assert min(sides) < 100 and max(sides) > 150


@pytest.mark.parametrize("cfg", [None, (256, 4096, 2)], ids=["default", "small_tiles"])
def test_c3_batch_equals_oracle(gpu_ctx, c3_mix, cfg):
    _, _, descs, wants = c3_mix
    old = gpu_ctx.get_launch_config()
    try:
        if cfg is not None:
            gpu_ctx.set_launch_config(batch=cfg)
        res = gpu_ctx.solve_batch(descs)
    finally:
        gpu_ctx.set_launch_config(plain=old[0], batch=old[1])
    for r, want in zip(res, wants):
        assert_matches_oracle(r, want)


def test_c3_plain_traces_equal_oracle(gpu_ctx, c3_mix):
    _, _, descs, wants = c3_mix
    for d, want in zip(descs, wants):
        r, st = gpu_ctx.solve_traced(d)
        assert_matches_oracle(r, want)
        np.testing.assert_array_equal(st["trace_gbest"], want["trace_gbest"])
        np.testing.assert_array_equal(st["pbest_fit"], want["pbest_fit"])


def test_c4_served_requests_equal_oracle(gpu_ctx):
    import qpso

    w = scene.workload_c4(n_frames=4, iterations=4)
    mids, fids = upload_workload(gpu_ctx, w)
    order = sorted(range(len(w["solves"])), key=lambda i: -w["meshes"][w["solves"][i]["mesh"]][1])
    pick = order[:2] + order[len(order) // 2:len(order) // 2 + 3] + order[-3:]
    solves = [dict(w["solves"][i], particles=(256, 1024)[j % 2], stream=100 + j)
              for j, i in enumerate(pick)]
    assert max(w["meshes"][s["mesh"]][1] for s in solves) > 90000
    descs = [gpu_desc(s, mids[s["mesh"]], fids[s["frame"]]) for s in solves]
    wants = [oracle_solve(w, s) for s in solves]
    with qpso.Server(gpu_ctx, max_slots=4, iters_per_epoch=2) as srv:
        ids = []
        for i, d in enumerate(descs):
            ids.append(srv.submit(d))
            if i % 3 == 2:
                time.sleep(0.003)  # later requests arrive while earlier ones run
        got = [srv.wait(rid) for rid in ids]
        st = srv.stats()
    assert st["completed"] == len(descs) and st["failed"] == 0
    assert st["peak_active"] >= 2
    for (r, lat), want in zip(got, wants):
        assert lat > 0
        assert_matches_oracle(r, want)


def test_c2_full_size_equals_oracle(gpu_ctx):
    w = scene.workload_c2()
    mids, fids = upload_workload(gpu_ctx, w)
    solves = w["solves"]
    assert all(s["particles"] == 256 and s["iterations"] == 100 for s in solves)
    descs = [gpu_desc(s, mids[s["mesh"]], fids[s["frame"]]) for s in solves]
    want0 = oracle_solve(w, solves[0], trace=True)
    r, st = gpu_ctx.solve_traced(descs[0])
    assert_matches_oracle(r, want0)
    np.testing.assert_array_equal(st["trace_gbest"], want0["trace_gbest"])
    np.testing.assert_array_equal(st["pos"], want0["pos"])
    np.testing.assert_array_equal(st["pbest"], want0["pbest"])
    wants = [want0] + [oracle_solve(w, s) for s in solves[1:]]
    for r, want in zip(gpu_ctx.solve_batch(descs), wants):
        assert_matches_oracle(r, want)
