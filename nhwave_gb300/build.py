"""Build ``libnhw_gpu.so`` (the C-ABI library) in-tree for sm_103a.

Plain nvcc / g++ invocations, compiled in parallel, no build system:
  setup_host.cpp   g++ -O2 -ffp-contract=off            (host set-up)
  nhw_fp64.cu      nvcc --fmad=false                     (plain FP64 form)
  nhw_fp32.cu      nvcc --fmad=true                      (FP32+IR form)
  capi.cu          nvcc                                  (C-ABI)
  noalloc.cu       nvcc --fmad=false                     (allocation-free entry point)
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libnhw_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libnhw_gpu.so")


def _sources():
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC))
            if f.endswith((".cu", ".cuh", ".cpp", ".h"))] + [
        os.path.join(os.path.dirname(HERE), "include", "nhwave_gb300.h")]


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    if not force and os.path.exists(LIB):
        newest = max(os.path.getmtime(s) for s in _sources())
        if os.path.getmtime(LIB) >= newest:
            return LIB
    nvcc = _nvcc()
    common = ["-std=c++17", "-O3", "-lineinfo", "--extended-lambda", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", *ARCH]
    jobs = [
        (["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-c",
          os.path.join(CSRC, "setup_host.cpp"), "-o", os.path.join(OUT, "setup_host.o")]),
        ([nvcc, *common, "--fmad=false", "-c", os.path.join(CSRC, "nhw_fp64.cu"),
          "-o", os.path.join(OUT, "nhw_fp64.o")]),
        ([nvcc, *common, "--fmad=true", "-c", os.path.join(CSRC, "nhw_fp32.cu"),
          "-o", os.path.join(OUT, "nhw_fp32.o")]),
        ([nvcc, *common, "-c", os.path.join(CSRC, "capi.cu"), "-o", os.path.join(OUT, "capi.o")]),
        ([nvcc, *common, "--fmad=false", "-c", os.path.join(CSRC, "noalloc.cu"),
          "-o", os.path.join(OUT, "noalloc.o")]),
    ]
    if verbose:
        jobs[1][1:1] = ["-Xptxas", "-v"]
        jobs[2][1:1] = ["-Xptxas", "-v"]
    procs = [subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT) for j in jobs]
    errs = []
    for j, p in zip(jobs, procs):
        out, _ = p.communicate()
        text = out.decode(errors="replace")
        if p.returncode != 0:
            errs.append(" ".join(j) + "\n" + text)
        elif verbose and text.strip():
            print(text, file=sys.stderr)
    if errs:
        raise RuntimeError("libnhw_gpu build failed:\n" + "\n".join(errs))
    tmp = LIB + f".tmp{os.getpid()}"
    subprocess.check_call([nvcc, *ARCH, "-shared", "-o", tmp,
                           *[os.path.join(OUT, o) for o in ("setup_host.o", "nhw_fp64.o", "nhw_fp32.o", "capi.o", "noalloc.o")]])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
