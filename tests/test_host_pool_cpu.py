"""The context's host worker pool (the threads that validate and pack the
regions of a batch), built from the library's own header and run on CPU."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _cuda_include():
    for d in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        if d and os.path.isfile(os.path.join(d, "include", "cuda_runtime.h")):
            return os.path.join(d, "include")
    return None


@pytest.mark.skipif(shutil.which("g++") is None or _cuda_include() is None,
                    reason="needs g++ and the CUDA headers")
def test_host_pool(tmp_path):
    exe = str(tmp_path / "host_pool_check")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-pthread",
                        f"-I{ROOT}/include", f"-I{ROOT}/pmmc_gb300/csrc", f"-I{_cuda_include()}",
                        os.path.join(HERE, "host_pool_check.cpp"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
