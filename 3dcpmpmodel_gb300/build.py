"""Build recipe for libcpmp.so (the C-ABI library), in-tree.

Every translation unit is compiled with nvcc for sm_103a only, in parallel,
into ``_build/``; the shared library links the CUDA runtime statically so it
depends on nothing but the CUDA driver library.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcpmp.so")
RUNNER = os.path.join(HERE, "cpmp_run")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC]
# (source, extra flags)
# the library's units; cpmp_run.cpp is the separate driver executable
UNITS = [
    ("api.cpp", []),
    ("eos.cpp", []),
    ("tecplot.cpp", []),
    ("k_plain_f32.cu", []),
    ("k_plain_f64.cu", ["--fmad=false"]),
    ("k_fused.cu", ["--fmad=false"]),
    ("k_pair_f16.cu", ["--fmad=false"]),
    ("k_pair_bf16.cu", ["--fmad=false"]),
    ("k_pair_f32.cu", ["--fmad=false"]),
    ("k_split_force.cu", ["--fmad=false"]),
    ("k_split_f16.cu", ["--fmad=false"]),
    ("k_split_bf16.cu", ["--fmad=false"]),
    ("k_split_f32.cu", ["--fmad=false"]),
    ("k_batch_f16.cu", ["--fmad=false"]),
    ("k_batch_bf16.cu", ["--fmad=false"]),
    ("k_batch_f32.cu", ["--fmad=false"]),
    # no FMA contraction: the reductions give the same bits whether a single
    # box's kernel or the batched one runs them
    ("k_diag.cu", ["--fmad=false"]),
    ("k_adjoint_f32.cu", []),
    ("k_adjoint_f64.cu", ["--fmad=false"]),
]


def nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise FileNotFoundError("nvcc not found")


def _sources_mtime() -> float:
    t = 0.0
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            t = max(t, os.path.getmtime(os.path.join(d, f)))
    return max(t, os.path.getmtime(__file__))


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build_runner() -> str:
    """The cpmp_run command-line driver, linked against libcpmp.so with an
    $ORIGIN run path (host code only)."""
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-I", INCLUDE, os.path.join(CSRC, "cpmp_run.cpp"),
           "-L", HERE, "-lcpmp", "-Wl,-rpath,$ORIGIN", "-o", RUNNER + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"cpmp_run failed to build:\n{r.stdout}\n{r.stderr}")
    os.replace(RUNNER + ".tmp", RUNNER)
    return RUNNER


def build(force: bool = False, jobs: int | None = None) -> str:
    """Compile and link libcpmp.so (and the cpmp_run driver) unless they are
    newer than every source."""
    fresh = lambda f: os.path.exists(f) and os.path.getmtime(f) >= _sources_mtime()  # noqa: E731
    if not force and fresh(LIB) and fresh(RUNNER):
        return LIB
    if not force and fresh(LIB):
        build_runner()
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    jobs = jobs or min(len(UNITS), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(lambda u: _compile(*u), UNITS))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    build_runner()
    return LIB


if __name__ == "__main__":
    print(build(force=True))
