"""Several GPUs run independent replicas of the solve (there is no exchange
step): bench.py's ranks meet only at a barrier and take the maximum time over
ranks.  These run two ranks on the CPU with the gloo backend."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    d = bench.Dist(2)
    d.barrier()
    got = d.max(1.5 + rank)  # each rank's own "time"
    d.barrier()
    d.close()
    with open(os.path.join(out_dir, "rank%d.json" % rank), "w") as fp:
        json.dump({"max": got}, fp)


def test_two_ranks_barrier_and_max_over_ranks(tmp_path):
    import torch.multiprocessing as mp

    port = _free_port()
    mp.start_processes(_rank, args=(port, str(tmp_path)), nprocs=2, start_method="spawn", join=True)
    for r in range(2):
        assert json.load(open(tmp_path / ("rank%d.json" % r)))["max"] == 2.5


@pytest.mark.timeout(300)
def test_reference_arm_under_torchrun_prints_on_rank0_only():
    """The reference arm launched as an N>1 run is (torchrun, one rank per GPU): rank 0
    times the CPU implementation and prints one line; rank 1 exits 0."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py", "--impl",
           "reference", "--workload", "c1", "--steps", "1", "--warmup", "0", "--gpus", "2"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=280)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    j = json.loads(lines[0])
    assert j["impl"] == "reference" and j["value"] > 0 and j["n_gpus"] == 2
    assert j["e2e"]["h2d_bytes_per_step"] == 0
