"""The drop-in shim compiles against the reference's own headers (where the
reference tree exists): every GPU entry point the reference declares is
defined with the same signature on top of the C ABI."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# the reference tree, as oracle/Makefile takes it (REF_ROOT, same default)
REF = os.path.join(os.environ.get("REF_ROOT", "/root/reference"), "src")

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


def test_reference_program_links_with_the_shim(tmp_path):
    """The reference's own pMMC-reconstruct program, built from its sources
    where they lie with the shim in place of its four GPU .cu files
    (ParallelMonteCarlo{Arcs,Heatmap,Smooth}.cu, ParallelMarkArcs.cu), links
    against libpmmc_gb300.so with no symbol left undefined, and starts.
    (Its sources do not travel to GPU hosts, so the pipeline itself is not
    run there.)"""
    import concurrent.futures as cf
    nvcc = "/usr/local/cuda/bin/nvcc"
    lib = os.path.join(ROOT, "pmmc_gb300", "libpmmc_gb300.so")
    if not os.path.exists(nvcc) or not os.path.exists(lib):
        pytest.skip("nvcc or the built library missing")
    inc = [f"-I{REF}/include", f"-I{REF}/thirdparty", f"-I{ROOT}/include"]
    jobs = [["g++", "-std=c++17", "-O1", "-fopenmp", "-w", *inc, "-c",
             f"{REF}/apps/pMMC-reconstruct/main_reconstruct.cpp", "-o", "main.o"],
            ["g++", "-std=c++17", "-O1", "-w", *inc, "-c",
             os.path.join(ROOT, "pmmc_gb300", "shim", "looper_solver_gpu.cpp"), "-o", "shim.o"],
            ["gcc", "-O1", "-w", "-c", f"{REF}/thirdparty/ini.c", "-o", "ini.o"],
            [nvcc, "-std=c++17", "-O1", "-w", "-gencode", "arch=compute_103a,code=sm_103a", *inc,
             "-c", f"{REF}/HierarchicalChromosome.cu", "-o", "hc.o"]]
    jobs += [["g++", "-std=c++17", "-O1", "-w", *inc, "-c", f"{REF}/thirdparty/{f}.cpp", "-o",
              f"{f}.o"] for f in ("common", "mtxlib", "INIReader", "rmsd")]
    with cf.ThreadPoolExecutor(8) as ex:
        res = list(ex.map(lambda c: subprocess.run(c, cwd=tmp_path, capture_output=True,
                                                   text=True), jobs))
    for r in res:
        assert r.returncode == 0, r.stderr[-2000:]
    objs = ["main.o", "common.o", "mtxlib.o", "INIReader.o", "rmsd.o", "ini.o", "hc.o", "shim.o"]
    r = subprocess.run(["g++", "-fopenmp", "-o", "pMMC-reconstruct", *objs,
                        f"-L{os.path.dirname(lib)}", "-lpmmc_gb300", "-L/usr/local/cuda/lib64",
                        "-lcudart", f"-Wl,-rpath,{os.path.dirname(lib)}"],
                       cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    out = subprocess.run([str(tmp_path / "pMMC-reconstruct")], capture_output=True, text=True,
                         timeout=60)
    assert "Usage: pMMC-reconstruct" in out.stdout + out.stderr


def test_drop_in_fails_loudly_without_a_device(tmp_path):
    """The drop-in parallelMonteCarloArcs, called from the reference's own
    LooperSolver on a host without a CUDA device, ends the program with the
    library's status (PMMC_ERR_NO_DEVICE = 2) and message, as the reference's
    gpuErrchk does on a CUDA error: no CPU annealer runs in its place."""
    import concurrent.futures as cf
    import torch
    lib = os.path.join(ROOT, "pmmc_gb300", "libpmmc_gb300.so")
    if not os.path.exists(lib):
        pytest.skip("the built library missing")
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    inc = [f"-I{REF}/include", f"-I{REF}/thirdparty", f"-I{ROOT}/include"]
    jobs = [["g++", "-std=c++17", "-O1", "-w", *inc, "-c",
             os.path.join(ROOT, "tests", "shim_no_device.cpp"), "-o", "drv.o"],
            ["g++", "-std=c++17", "-O1", "-w", *inc, "-c",
             os.path.join(ROOT, "pmmc_gb300", "shim", "looper_solver_gpu.cpp"), "-o", "shim.o"],
            ["gcc", "-O1", "-w", "-c", f"{REF}/thirdparty/ini.c", "-o", "ini.o"]]
    jobs += [["g++", "-std=c++17", "-O1", "-w", *inc, "-c", f"{REF}/thirdparty/{f}.cpp", "-o",
              f"{f}.o"] for f in ("common", "mtxlib", "INIReader", "rmsd")]
    with cf.ThreadPoolExecutor(8) as ex:
        res = list(ex.map(lambda c: subprocess.run(c, cwd=tmp_path, capture_output=True,
                                                   text=True), jobs))
    for r in res:
        assert r.returncode == 0, r.stderr[-2000:]
    objs = ["drv.o", "shim.o", "common.o", "mtxlib.o", "INIReader.o", "rmsd.o", "ini.o"]
    r = subprocess.run(["g++", "-fopenmp", "-o", "drv", *objs, f"-L{os.path.dirname(lib)}",
                        "-lpmmc_gb300", "-L/usr/local/cuda/lib64", "-lcudart",
                        f"-Wl,-rpath,{os.path.dirname(lib)}"],
                       cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    (tmp_path / "seg.bed").write_text("chr1\t0\t1000000\n")
    out = subprocess.run([str(tmp_path / "drv"), str(tmp_path / "seg.bed")], cwd=tmp_path,
                         capture_output=True, text=True, timeout=120)
    assert out.returncode == 2, (out.returncode, out.stdout[-500:], out.stderr[-500:])
    assert "GPUassert (pmmc_gb300): context: no usable CUDA device" in out.stderr
    assert "returned" not in out.stdout


def test_shim_reads_every_setting_the_reference_gpu_files_read():
    """Every Settings:: parameter the reference's four replaced GPU files read
    is read by the shim, except the heatmap kernel's launch geometry
    ([cuda] num_threads, blocks_multiplier), which this library chooses
    itself."""
    import re
    pat = re.compile(r"Settings::(\w+)")
    ref = set()
    for f in ("ParallelMonteCarloArcs.cu", "ParallelMonteCarloHeatmap.cu",
              "ParallelMonteCarloSmooth.cu", "ParallelMarkArcs.cu"):
        ref |= set(pat.findall(open(os.path.join(REF, f)).read()))
    shim = set(pat.findall(open(os.path.join(ROOT, "pmmc_gb300", "shim",
                                             "looper_solver_gpu.cpp")).read()))
    assert ref - shim == {"cudaThreadsPerBlock", "cudaBlocksMultiplier"}
