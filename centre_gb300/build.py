"""Build the CUDA library libcentre_gpu.so in-tree for sm_103a, and the
command-line tool centre_gpu on top of it.

Each translation unit under csrc/ is compiled in parallel with nvcc and the
objects are linked into centre_gb300/libcentre_gpu.so (no torch involved; the
C ABI is declared in include/centre_gpu.h).  The host sources under host/
(input file, NetCDF files, the three pipeline stages, the command-line main) are
compiled with the host C++ compiler and linked into centre_gb300/centre_gpu,
which finds the library next to itself.

    python -m centre_gb300.build [--verbose-ptxas]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcentre_gpu.so")
HOST = os.path.join(HERE, "host")
TOOL = os.path.join(HERE, "centre_gpu")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _compile(src: str, ptxas_verbose: bool) -> tuple[str, str]:
    obj = os.path.join(OBJ, src[:-3] + ".o")
    deps = [os.path.join(CSRC, src)] + [
        os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))
    ] + [os.path.join(ROOT, "include", "centre_gpu.h")]
    if (not ptxas_verbose and os.path.exists(obj)
            and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps)):
        return obj, ""
    # host code without FMA contraction: the host-side double arithmetic that
    # must match the reference bit for bit (KDE bandwidth, bin thresholds)
    # then rounds the same on x86-64 and aarch64
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-ffp-contract=off",
           "-I", os.path.join(ROOT, "include"), "-I", CSRC, "-c", os.path.join(CSRC, src),
           "-o", obj]
    if ptxas_verbose:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def cxx() -> str:
    for cand in (os.environ.get("CXX"), shutil.which("g++"), shutil.which("c++")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("no host C++ compiler (g++) found")


def _compile_host(src: str) -> str:
    obj = os.path.join(OBJ, "host_" + src[:-4] + ".o")
    deps = [os.path.join(HOST, src)] + [
        os.path.join(HOST, h) for h in os.listdir(HOST) if h.endswith(".hpp")
    ] + [os.path.join(ROOT, "include", "centre_gpu.h")]
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    cmd = [cxx(), "-O2", "-std=c++17", "-Wall", "-I", os.path.join(ROOT, "include"), "-I", HOST,
           "-c", os.path.join(HOST, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"host compile failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build_tool(jobs: int | None = None) -> str:
    """centre_gpu: the input-file tool (host/), linked against the library."""
    srcs = sorted(f for f in os.listdir(HOST) if f.endswith(".cpp"))
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, len(srcs))) as ex:
        objs = list(ex.map(_compile_host, srcs))
    if (not os.path.exists(TOOL)
            or os.path.getmtime(TOOL) < max(os.path.getmtime(o) for o in objs + [LIB])):
        tmp = TOOL + ".tmp"
        cmd = [cxx(), "-o", tmp, *objs, "-L", HERE, "-lcentre_gpu", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"tool link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, TOOL)
    return TOOL


def build(ptxas_verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(OBJ, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, ptxas_verbose), srcs))
    if ptxas_verbose:
        for (_, log), s in zip(results, srcs):
            if log:
                print(f"== {s}\n{log}")
    objs = [o for o, _ in results]
    if (not os.path.exists(LIB)
            or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs)):
        tmp = LIB + ".tmp"
        cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    build_tool(jobs)
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--verbose-ptxas", action="store_true")
    a = ap.parse_args()
    print(build(a.verbose_ptxas))
    sys.exit(0)
