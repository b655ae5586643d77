"""The bounded mbarrier wait of the tcgen05 kernels gives up instead of hanging: a
kernel that waits on a barrier nothing arrives on returns (and frees its TMEM), one whose
barrier completes sees it, and the context stays usable (tests/tc_wait_timeout.cu, built
here with nvcc for sm_103a)."""
import os
import subprocess
import tempfile

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")


def test_bounded_mbarrier_wait_gives_up_and_completes():
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "tc_wait_timeout")
        subprocess.run([NVCC, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "-o", exe,
                        os.path.join(HERE, "tc_wait_timeout.cu")], check=True)
        r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "timeout=1 completed=1 after=1" in r.stdout
