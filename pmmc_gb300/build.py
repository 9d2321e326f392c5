"""Build the CUDA library in-tree: pmmc_gb300/libpmmc_gb300.so (sm_103a).

Each .cu under csrc/ is compiled in parallel with nvcc
(-gencode arch=compute_103a,code=sm_103a -lineinfo -O3) and the objects are
linked into one shared library whose C ABI is include/pmmc_gb300.h.  No
PyTorch extension machinery is involved; Python reaches the library through
ctypes (pmmc_gb300/capi.py).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpmmc_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers_mtime() -> float:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return max(os.path.getmtime(h) for h in hs)


def build(force: bool = False, verbose: bool = False, ptxas_v: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    hm = _headers_mtime()
    # -ffp-contract=off: host arithmetic that restates the reference's
    # (freqToDistance, energies) rounds alike on x86-64 and aarch64
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                    "-I", INCLUDE, "-I", CSRC, "--expt-relaxed-constexpr"]
    if ptxas_v:
        flags += ["-Xptxas", "-v"]

    def one(src: str) -> tuple[str, str]:
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        if (not force and not ptxas_v and os.path.exists(obj)
                and os.path.getmtime(obj) >= max(os.path.getmtime(src), hm)):
            return obj, ""
        cmd = [cc, *flags, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        return obj, r.stderr

    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(one, srcs))
    objs = [o for o, _ in results]
    if verbose or ptxas_v:
        for _, log in results:
            if log:
                sys.stderr.write(log)
    if (force or not os.path.exists(LIB)
            or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs)):
        cmd = [cc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_v="--ptxas-v" in sys.argv)
    print(LIB)
