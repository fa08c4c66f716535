"""Bounded waits of the tensor-core kernels: tests/cuda/wait_timeout.cu, built with nvcc against
the library's own wait helper, waits on an mbarrier phase that nothing completes (the wait must give
up and report it) and on one that completes, then runs another kernel: the context stays usable."""
import json
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.gpu
def test_bounded_mbarrier_wait_times_out_and_context_survives(tmp_path):
    from akuaengine_gb300 import build

    exe = str(tmp_path / "wait_timeout")
    cmd = [build.nvcc_path(), *build.ARCH_FLAGS, "-O2", "-std=c++17",
           "-I", os.path.join(ROOT, "akuaengine_gb300", "csrc"),
           os.path.join(ROOT, "tests", "cuda", "wait_timeout.cu"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    res = json.loads(out.stdout.strip().splitlines()[-1])
    print(res)
    assert res["sync"] == "cudaSuccess"
    assert res["timeout_result"] == 0 and res["arrived_result"] == 1
    assert res["after"] == 4 * 32
    assert res["timeout_cycles"] > res["arrived_cycles"]


def test_wait_helper_compiles(tmp_path):
    """The wait test program compiles for sm_103a here (no GPU needed)."""
    from akuaengine_gb300 import build

    if shutil.which(build.nvcc_path()) is None and not os.path.exists(build.nvcc_path()):
        pytest.skip("nvcc not available")
    cmd = [build.nvcc_path(), *build.ARCH_FLAGS, "-O2", "-std=c++17", "-c",
           "-I", os.path.join(ROOT, "akuaengine_gb300", "csrc"),
           os.path.join(ROOT, "tests", "cuda", "wait_timeout.cu"), "-o", str(tmp_path / "w.o")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
