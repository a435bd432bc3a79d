"""Serving loop: continuous batching of solve requests (qpso_server_*).

Each request's result must equal the same descriptor solved alone
(qpso_solve) bit for bit, whatever else shares the GPU; requests that
arrive while others run are admitted as slots and memory free up.
"""
import time

import numpy as np
import pytest

import scene
from tests.helpers import gpu_desc, upload_workload

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mix(gpu_ctx, c1):
    """Requests over two workloads (the C1 ellipsoid and a C2 frame with
    several meshes) with uneven particle counts, iterations and seeds."""
    w2 = scene.workload_c2(frames=1, particles=64, iterations=10)
    m1, f1 = upload_workload(gpu_ctx, c1)
    m2, f2 = upload_workload(gpu_ctx, w2)
    rng = np.random.default_rng(5)
    descs = []
    for i in range(14):
        if i % 2 == 0:
            s = dict(c1["solves"][0], particles=int(rng.choice([16, 40, 96])),
                     iterations=int(rng.integers(3, 12)), seed=100 + i, stream=i)
            descs.append(gpu_desc(s, m1[0], f1[0]))
        else:
            s = w2["solves"][int(rng.integers(0, len(w2["solves"])))]
            s = dict(s, particles=int(rng.choice([32, 64])), iterations=int(rng.integers(2, 9)),
                     seed=200 + i, stream=i)
            descs.append(gpu_desc(s, m2[s["mesh"]], f2[0]))
    return descs


def test_results_equal_alone_under_continuous_batching(gpu_ctx, mix):
    import qpso

    alone = [gpu_ctx.solve(d) for d in mix]
    with qpso.Server(gpu_ctx, max_slots=5, iters_per_epoch=2) as srv:
        ids = []
        for i, d in enumerate(mix):
            ids.append(srv.submit(d))
            if i % 4 == 3:
                time.sleep(0.002)  # later requests arrive while earlier ones run
        got = [srv.wait(rid) for rid in ids]
        st = srv.stats()
    assert st["completed"] == len(mix) and st["failed"] == 0
    assert st["peak_active"] >= 2  # requests overlapped on the device
    assert st["peak_active"] <= 5
    assert st["bytes_in_use"] == 0
    for (r, lat), a in zip(got, alone):
        assert r.flags == 0 and lat > 0
        assert r.fit == a.fit
        assert list(r.pose) == list(a.pose)


def test_admission_by_slots_and_budget(gpu_ctx, mix):
    import qpso

    # one slot: strictly one request at a time
    with qpso.Server(gpu_ctx, max_slots=1, iters_per_epoch=3) as srv:
        ids = [srv.submit(d) for d in mix[:4]]
        for rid in ids:
            srv.wait(rid)
        assert srv.stats()["peak_active"] == 1
    # a budget that fits only one request at a time
    with qpso.Server(gpu_ctx, max_slots=8, hbm_budget_bytes=2_200_000, iters_per_epoch=3) as srv:
        ids = [srv.submit(d) for d in mix[:4]]
        res = [srv.wait(rid) for rid in ids]
        st = srv.stats()
        assert st["peak_active"] == 1 and st["peak_bytes"] <= 2_200_000
        for (r, _), d in zip(res, mix[:4]):
            assert r.fit == gpu_ctx.solve(d).fit
    # a request that can never fit is refused at submission
    with qpso.Server(gpu_ctx, max_slots=2, hbm_budget_bytes=100_000) as srv:
        with pytest.raises(qpso.QpsoError) as e:
            srv.submit(mix[0])
        assert e.value.status == qpso.ERR_BUSY


def test_poll_and_unknown_ids(gpu_ctx, mix):
    import qpso

    with qpso.Server(gpu_ctx, max_slots=2) as srv:
        rid = srv.submit(mix[0])
        deadline = time.time() + 60
        out = None
        while out is None and time.time() < deadline:
            out = srv.poll(rid)
            time.sleep(0.001)
        assert out is not None and out[0].fit == gpu_ctx.solve(mix[0]).fit
        with pytest.raises(qpso.QpsoError) as e:
            srv.poll(rid)  # a result is handed out once
        assert e.value.status == qpso.ERR_NOT_FOUND
