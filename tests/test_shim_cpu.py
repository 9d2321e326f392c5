"""The drop-in shim compiles against the reference's own headers (where the
reference tree exists): every GPU entry point the reference declares is
defined with the same signature on top of the C ABI."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = "/root/reference/src"

pytestmark = pytest.mark.skipif(not os.path.isdir(REF) or shutil.which("g++") is None,
                                reason="reference headers not present")


def test_shim_compiles_against_reference_headers(tmp_path):
    obj = tmp_path / "shim.o"
    r = subprocess.run(["g++", "-std=c++17", "-c", "-w", f"-I{REF}/include", f"-I{REF}/thirdparty",
                        f"-I{ROOT}/include", os.path.join(ROOT, "pmmc_gb300", "shim",
                                                          "looper_solver_gpu.cpp"),
                        "-o", str(obj)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    syms = subprocess.run(["nm", "-C", str(obj)], capture_output=True, text=True).stdout
    for name in ("LooperSolver::parallelMonteCarloArcs(float)",
                 "LooperSolver::ParallelMonteCarloSmooth(float, unsigned long long)",
                 "LooperSolver::ParallelMonteCarloHeatmap(float)",
                 "InteractionArcs::parallelMarkArcs(bool)", "setGpuSeed(unsigned int)",
                 "GpuResourceCache::init()", "GpuResourceCache::cleanup()"):
        assert f" T {name}" in syms, name
