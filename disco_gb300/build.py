"""Build the in-tree native library libdisco_gb300.so for sm_103a.

Host C set-up (gcc) and CUDA kernels (nvcc, -gencode arch=compute_103a,
code=sm_103a) are compiled in parallel and linked into one shared library in
disco_gb300/_lib/.  No cmake; a rebuild happens only when a source is newer
than the library.
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
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libdisco_gb300.so")
INCLUDE = os.path.join(ROOT, "include")

GENCODE = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = ["-std=c++17", "-O3", GENCODE, "-lineinfo", "-Xcompiler", "-fPIC",
              "--expt-relaxed-constexpr"]
CC_FLAGS = ["-std=gnu11", "-O2", "-fPIC", "-Wall", "-ffp-contract=off"]

HOST_SOURCES = ["host/disco_host.c", "host/h5lite.c", "host/checkpoint.c"]
# (source, extra nvcc flags): the plain-FP64 instances are compiled without
# FMA contraction so their FP64 arithmetic rounds like the reference's C build.
# FP64 path: no FMA contraction (it must round like the reference build).
# Mixed path: FP32 division and square root need not be correctly rounded
# (they only touch FP32 values; FP64 arithmetic is unaffected).
F32_FLAGS = ["-prec-div=false", "-prec-sqrt=false"]
CUDA_SOURCES = [("cuda/disco_gpu.cu", []),
                ("cuda/inst_euler_f64.cu", ["--fmad=false"]),
                ("cuda/inst_euler_f32.cu", F32_FLAGS),
                ("cuda/inst_mhd_f64.cu", ["--fmad=false"]),
                ("cuda/inst_mhd_f32.cu", F32_FLAGS),
                ("cuda/inst_grmhd_f64.cu", ["--fmad=false"])]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources_mtime() -> float:
    newest = 0.0
    for base in (CSRC, INCLUDE):
        for dp, _, fns in os.walk(base):
            for fn in fns:
                if fn.endswith((".c", ".h", ".cu", ".cuh")):
                    newest = max(newest, os.path.getmtime(os.path.join(dp, fn)))
    return max(newest, os.path.getmtime(__file__))


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile libdisco_gb300.so (if stale) and return its path."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _sources_mtime():
        return LIB
    os.makedirs(os.path.join(LIBDIR, "obj"), exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    objs = []
    for src in HOST_SOURCES:
        obj = os.path.join(LIBDIR, "obj", os.path.basename(src) + ".o")
        jobs.append(["gcc", *CC_FLAGS, f"-I{INCLUDE}", "-c", os.path.join(CSRC, src), "-o", obj])
        objs.append(obj)
    for src, extra in CUDA_SOURCES:
        obj = os.path.join(LIBDIR, "obj", os.path.basename(src) + ".o")
        jobs.append([nvcc, *NVCC_FLAGS, *extra, f"-I{INCLUDE}", "-c", os.path.join(CSRC, src), "-o", obj])
        objs.append(obj)
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        for cmd, fut in [(c, ex.submit(_run, c)) for c in jobs]:
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
            fut.result()
    tmp = LIB + ".tmp"
    _run([nvcc, "-shared", GENCODE, "-o", tmp, *objs, "-lcudart"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
