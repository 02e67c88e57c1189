"""Builds libplk.so in-tree: nvcc for the sm_103a kernels, g++ for the host
code, compiled in parallel and linked into ``phylommand_gb300/lib/libplk.so``.

    python -m phylommand_gb300.build
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB_DIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIB_DIR, "libplk.so")
REPLAY = os.path.join(LIB_DIR, "plk_replay")
ROOT = os.path.dirname(HERE)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["plk_kernels.cu", "plk_prune4s.cu", "plk_prune4p.cu", "plk_prune4w.cu", "plk_prune20.cu", "plk_prune20u.cu", "plk_batch.cu", "plk_nni.cu", "plk_features.cu",
              "plk_mlp.cu", "plk_noalloc.cu", "plk_peak.cu"]
CPP_SOURCES = ["plk_api.cpp", "plk_host.cpp", "plk_fit.cpp", "plk_batch_api.cpp", "plk_sim.cpp", "plk_io.cpp"]


def _cuda_home() -> str:
    home = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if home:
        return home
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return "/usr/local/cuda"


def _nvcc() -> str:
    return os.path.join(_cuda_home(), "bin", "nvcc")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)


def _stale(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    cuda = _cuda_home()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "plk.h"))
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17",
                         "-Xcompiler", "-fPIC", "-Xptxas", "-warn-spills", "-c", s, "-o", o])
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra",
                         "-I" + os.path.join(cuda, "include"), "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for cmd in jobs:
            if verbose:
                print(" ".join(cmd), flush=True)
        list(ex.map(_run, jobs))
    if force or jobs or not os.path.exists(LIB):
        cmd = [_nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart_static", "-lpthread", "-ldl", "-lrt"]
        if verbose:
            print(" ".join(cmd), flush=True)
        _run(cmd)
    # a plain C caller of the ABI, linked against libplk.so only (found next to it)
    src = os.path.join(HERE, "capi", "plk_replay.c")
    if force or _stale(REPLAY, [src, LIB, os.path.join(ROOT, "include", "plk.h")]):
        cmd = ["gcc", "-O2", "-std=c99", "-Wall", "-Wextra", "-I" + os.path.join(ROOT, "include"), src,
               "-L" + LIB_DIR, "-lplk", "-Wl,-rpath,$ORIGIN", "-o", REPLAY]
        if verbose:
            print(" ".join(cmd), flush=True)
        _run(cmd)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
