"""Builds the CUDA engine library libdsf_gb300.so in-tree for sm_103a.

Each .cu translation unit is compiled in parallel with nvcc, then linked
into one shared library exporting the C ABI of include/dsf_gb300.h.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libdsf_gb300.so")
PEAK_LIB = os.path.join(HERE, "libdsf_peak_probe.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["dsf_kernels.cu", "dsf_k3_f32_hc.cu", "dsf_k3_f32_hc_mp.cu", "dsf_k3_f32_other.cu", "dsf_k3b_f32.cu", "dsf_k3_f64.cu", "dsf_prep_kernels.cu", "dsf_engine.cu", "dsf_noalloc.cu", "dsf_tsc.cu", "dsf_k3f_hc.cu", "dsf_k3f_other.cu"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.exists(cand) or cand == "nvcc"):
            return cand
    return "nvcc"


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra_flags=()):
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(REPO, "include", "dsf_gb300.h"))
    nvcc = _nvcc()
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-O3",
                     "-I", os.path.join(REPO, "include")] + list(extra_flags)
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc] + common + ["-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            futs = [ex.submit(subprocess.run, j, capture_output=True, text=True) for j in jobs]
            for j, f in zip(jobs, futs):
                r = f.result()
                if verbose or r.returncode != 0:
                    sys.stderr.write(" ".join(j) + "\n" + r.stdout + r.stderr)
                if r.returncode != 0:
                    raise RuntimeError(f"nvcc failed for {j[-3]}")
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc] + ARCH + ["-shared", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            raise RuntimeError("link failed")
    src = os.path.join(CSRC, "peak_probe.cu")
    if force or _stale(PEAK_LIB, [src]):
        cmd = [nvcc] + ARCH + ["-O3", "-Xcompiler", "-fPIC", "-shared", "-o", PEAK_LIB, src]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            raise RuntimeError("peak probe build failed")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
