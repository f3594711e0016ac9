"""Builds libxyce_gb300.so in-tree for sm_103a (nvcc for the kernels, g++ for
the host C++), compiling the translation units in parallel."""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libxyce_gb300.so")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU = ["xg_kernels.cu", "xg_lu.cu", "xg_bsim4.cu", "xg_mlp.cu"]
CPP = ["xg_api.cpp", "xg_symbolic.cpp", "xg_params.cpp", "xg_bsim4_params.cpp"]


def _needs(obj: str, srcs: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(s) > t for s in srcs)


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(HERE, "..", "include", "xyce_gb300.h"))
    return hs


def build(verbose: bool = False, ptxas_verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    hdrs = _headers()
    jobs = []
    for f in CU:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT, f + ".o")
        cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
               "-c", src, "-o", obj]
        if ptxas_verbose:
            cmd.insert(1, "-Xptxas=-v")
        if ptxas_verbose or _needs(obj, [src, *hdrs]):
            jobs.append(cmd)
    for f in CPP:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT, f + ".o")
        cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-pthread", "-Wall", "-Wno-unused-function",
               f"-I{CUDA}/include", "-c", src, "-o", obj]
        if _needs(obj, [src, *hdrs]):
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or ptxas_verbose:
                sys.stdout.write(r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    objs = [os.path.join(OUT, f + ".o") for f in CU + CPP]
    if _needs(LIB, objs):
        cmd = [NVCC, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: " + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, ptxas_verbose="-v" in sys.argv))
