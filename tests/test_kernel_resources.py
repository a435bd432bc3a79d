"""Resource guard for the fused kernels (no GPU): compile qpso_kernels.cu
for sm_103a with ptxas's resource report and check that the default
variant (REF raster, fp32 projection) of every fused kernel keeps its
launch-bound register budget and at most a few bytes of spills.  More
spills in these kernels have meant measurably slower solves, so a change
that adds them should be timed before it goes in."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "q-pso_gb300", "csrc")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")

# kernel (mangled-name stem) -> most spill-store bytes allowed in variant 0
LIMITS = {"qpso_step_kernel": 16, "qpso_batch_kernel": 32, "qpso_epoch_kernel": 32,
          "score_poses_mlet_kernel": 8}


@pytest.mark.timeout(300)
def test_default_variants_keep_registers_and_spills(tmp_path):
    if not (os.path.exists(NVCC) or shutil.which("nvcc")):
        pytest.skip("nvcc not available")
    nvcc = NVCC if os.path.exists(NVCC) else shutil.which("nvcc")
    out = subprocess.run([nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--fmad=false",
                          "-std=c++17", "-Xptxas", "-v", "-I", os.path.join(ROOT, "include"), "-I", CSRC,
                          os.path.join(CSRC, "qpso_kernels.cu"), "-o", str(tmp_path / "k.cubin")],
                         capture_output=True, text=True, timeout=280)
    assert out.returncode == 0, out.stderr[-2000:]
    found = {}
    current = None
    for line in out.stderr.splitlines():
        m = re.search(r"Compiling entry function '(\S+)'", line)
        if m:
            current = m.group(1)
            continue
        if current is None:
            continue
        m = re.search(r"(\d+) bytes spill stores", line)
        if m:
            found.setdefault(current, {})["spill"] = int(m.group(1))
        m = re.search(r"Used (\d+) registers", line)
        if m:
            found.setdefault(current, {})["regs"] = int(m.group(1))
    for stem, limit in LIMITS.items():
        # variant 0 of the template: ...<stem>ILi0EE...
        names = [n for n in found if stem in n and "ILi0E" in n]
        assert names, "no default variant of %s in the ptxas report" % stem
        for n in names:
            assert found[n]["regs"] <= 64, (n, found[n])
            assert found[n].get("spill", 0) <= limit, (n, found[n])
