"""Build libsolveit_gpu.so in-tree (solveit-code_gb300/_build/).

Every .cu file under csrc/ is compiled for sm_103a only
(-gencode arch=compute_103a,code=sm_103a), in parallel, then linked into one
shared library exporting the C ABI of include/solveit_gpu.h.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libsolveit_gpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no contraction into fused multiply-adds (gcc contracts by default
# on aarch64), so FP32 clocks and level tables match the reference's x86 build
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
           "-Xcompiler", "-ffp-contract=off",
           "--expt-relaxed-constexpr", "-diag-suppress", "1444"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _compile(src, extra):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    cmd = [nvcc()] + ARCH + NVFLAGS + extra + ["-I", os.path.join(ROOT, "include"), "-I", CSRC, "-c", src,
                                               "-o", obj]
    if os.path.exists(obj) and os.path.getmtime(obj) > max(
            [os.path.getmtime(src)] + [os.path.getmtime(os.path.join(CSRC, h)) for h in os.listdir(CSRC)
                                       if h.endswith((".cuh", ".h"))] +
            [os.path.getmtime(os.path.join(ROOT, "include", "solveit_gpu.h"))]):
        return obj, ""
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    return obj, r.stderr


def build(verbose=False, extra=()):
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: _compile(s, list(extra)), srcs))
    objs = [o for o, _ in results]
    if verbose:
        for _, err in results:
            if err:
                sys.stderr.write(err)
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
