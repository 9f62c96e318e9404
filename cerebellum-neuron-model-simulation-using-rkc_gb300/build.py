"""Build the native library in-tree: libgbrkc.so (CUDA kernels for sm_103a +
host runtime + C ABI) and the gbrkc_main CLI.

Kernel translation units use -fmad=false (the FP64 path reproduces the
oracle bit for bit; wanted fused multiply-adds are written explicitly).  The
mixed-precision unit (FP32 gating) also takes approximate FP32 division
(-prec-div=false, within 2 ulp): it is checked against FP64 by tolerance, and
FP64 arithmetic is unaffected by the flag;
host code uses -ffp-contract=off so setup arithmetic is identical on x86 and
aarch64 hosts.  Objects go to _build/ next to this file.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgbrkc.so")
CLI = os.path.join(HERE, "gbrkc_main")
ROOT = os.path.dirname(HERE)

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc") if os.path.exists(os.path.join(CUDA_HOME, "bin", "nvcc")) else "nvcc"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
           "-diag-suppress", "177,550"] + ARCH
CXX = os.environ.get("CXX", "g++")
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
            f"-I{CUDA_HOME}/include", f"-I{os.path.join(ROOT, 'include')}"]

KERNEL_TUS = ["kernels_fp64.cu", "kernels_fp32.cu", "compat.cu", "noalloc.cu", "synapse.cu"]
TU_FLAGS = {"kernels_fp32.cu": ["-prec-div=false"]}
HOST_TUS = ["engine.cpp", "host_init.cpp", "server.cpp"]


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh", ".cu"))]
    headers.append(os.path.join(ROOT, "include", "gbrkc.h"))
    procs, objs = [], []
    for tu in KERNEL_TUS + HOST_TUS:
        src = os.path.join(CSRC, tu)
        if not os.path.exists(src):
            continue
        obj = os.path.join(BUILD, tu + ".o")
        objs.append(obj)
        if not _newer(obj, [src, os.path.abspath(__file__)] + headers):
            continue
        if tu.endswith(".cu"):
            cmd = [NVCC] + NVFLAGS + TU_FLAGS.get(tu, []) + ["-c", src, "-o", obj]
        else:
            cmd = [CXX] + CXXFLAGS + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        procs.append((tu, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for tu, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((tu, out.decode(errors="replace")))
    if failed:
        for tu, out in failed:
            sys.stderr.write(f"--- {tu}\n{out}\n")
        raise RuntimeError("native build failed: " + ", ".join(t for t, _ in failed))
    if _newer(LIB, objs):
        cmd = [NVCC, "-shared", "-o", LIB] + objs + ARCH
        subprocess.run(cmd, check=True)
    cli_src = os.path.join(CSRC, "cli.cpp")
    if os.path.exists(cli_src) and _newer(CLI, [cli_src, LIB]):
        cmd = [CXX] + CXXFLAGS + [cli_src, "-o", CLI, f"-L{HERE}", "-lgbrkc", f"-Wl,-rpath,{HERE}",
                                  f"-L{CUDA_HOME}/lib64", "-lcudart", "-pthread"]
        subprocess.run(cmd, check=True)
    return LIB


def clean() -> None:
    shutil.rmtree(BUILD, ignore_errors=True)
    for f in (LIB, CLI):
        if os.path.exists(f):
            os.remove(f)


if __name__ == "__main__":
    build(verbose=True)
    print(LIB)
