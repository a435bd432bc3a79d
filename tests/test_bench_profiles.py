"""bench.py reads per-launch figures of the dominant kernels from the
committed ncu summaries (profiles/<kernel>_kernel_<workload>.md): the
roofline's traffic and the issue roofline's instruction count.  These
checks keep the summaries and the reader in step (no GPU)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402

# (workload, kernel): the default kernel each bench workload reports on
DOMINANT = [("c2", "step"), ("c2", "batch"), ("c3", "batch"), ("c5", "step")]


@pytest.mark.parametrize("workload,kernel", DOMINANT)
def test_summaries_carry_the_figures_bench_reads(workload, kernel):
    inst = bench.profile_figure(workload, kernel, "inst_per_launch")
    assert inst is not None and inst > 1e6, (workload, kernel)
    path = os.path.join(ROOT, "profiles", "%s_kernel_%s.md" % (kernel, workload))
    text = open(path).read()
    assert "ncu" in text and "--clock-control none" in text, "summary without its command"
    dram = bench.profile_figure(workload, kernel, "dram_bytes_per_launch")
    if dram is not None:
        assert dram > 0


def test_missing_figures_read_as_none():
    assert bench.profile_figure("c2", "step", "no_such_key") is None
    assert bench.profile_figure("c9", "step", "inst_per_launch") is None


@pytest.mark.timeout(120)
def test_segmentation_reference_arm_line():
    """bench.py --workload seg --impl reference: the oracle's segmentation
    timed on the host, one JSON line with the contract's keys."""
    import json
    import subprocess

    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "seg", "--steps", "1",
                        "--warmup", "0"], cwd=ROOT, capture_output=True, text=True, timeout=100)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    j = json.loads(lines[0])
    assert j["impl"] == "reference" and j["unit"] == "frames/s" and j["value"] > 0
    assert j["cpu_baseline"]["kind"] == "port" and j["e2e"]["h2d_bytes_per_step"] == 0


def test_segmentation_frame_has_clusters():
    """The seg workload's frame splits into a dozen sets with the reference
    main's constants (min_size 500), on the oracle."""
    from oracle import pyoracle as po

    lists, ns = po.segment_planes(*bench.segmentation_frame(), po.seg_params())
    assert 5 <= ns <= 40 and all(len(L) - 1 >= 500 for L in lists)
