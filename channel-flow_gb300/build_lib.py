"""Builds libchannel_gpu.so (CUDA for sm_103a + the C++ host parts) in-tree.

Every translation unit is compiled in parallel with one -gencode
(compute_103a / sm_103a), then linked into channel-flow_gb300/libchannel_gpu.so.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libchannel_gpu.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
            "-I", os.path.join(ROOT, "include"), "-I", CSRC]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-I", os.path.join(ROOT, "include")]

CU_SOURCES = ["cf_api.cu", "k_core.cu", "k_dsm.cu", "k_dsm_fused.cu", "k_poisson.cu", "k_eqwm.cu", "k_stats.cu",
              "k_noalloc.cu", "k_amd.cu", "k_wmlp.cu"]
CXX_SOURCES = ["io.cpp"]


def _newer(src: str, dst: str, deps: list[str]) -> bool:
    if not os.path.exists(dst):
        return True
    t = os.path.getmtime(dst)
    return any(os.path.getmtime(p) > t for p in [src] + deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(verbose: bool = False, extra: list[str] | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    hdrs.append(os.path.join(ROOT, "include", "channel_gpu.h"))
    jobs, objs = [], []
    for s in CU_SOURCES:
        src, obj = os.path.join(CSRC, s), os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if _newer(src, obj, hdrs):
            jobs.append([NVCC] + ARCH + CU_FLAGS + (extra or []) + ["-c", src, "-o", obj])
    for s in CXX_SOURCES:
        src, obj = os.path.join(CSRC, s), os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if _newer(src, obj, hdrs):
            jobs.append(["g++"] + CXX_FLAGS + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    if jobs or not os.path.exists(LIB):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    if verbose:
        print("built", LIB, file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
