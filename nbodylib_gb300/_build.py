"""Compile libnbkdt.so (the sm_103a CUDA kernels and the C ABI) in-tree with nvcc.

Translation units compile in parallel; the library lands in nbodylib_gb300/_lib/.
Nothing else is built here: the CPU checkers live in oracle/ and build separately.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libnbkdt.so")
SOURCES = ["capi.cu", "build.cu", "knn.cu", "smooth.cu", "phase.cu", "fof.cu", "ball.cu", "adjoint.cu",
           "batch.cu", "noalloc.cu", "probe.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code is compiled without floating-point contraction: the kernel table is built on
# the host and must round exactly as the reference's (GCC on aarch64 would fuse a*b+c).
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler",
         "-ffp-contract=off", "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libnbkdt")
    return exe


def _obj(src: str) -> str:
    return os.path.join(OUT_DIR, "obj", os.path.splitext(src)[0] + ".o")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> str:
    os.makedirs(os.path.join(OUT_DIR, "obj"), exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "nbkdt.h"))
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    exe = nvcc()

    def compile_one(src):
        obj = _obj(src)
        path = os.path.join(CSRC, src)
        if not force and not _stale(obj, [path] + headers):
            return obj, ""
        cmd = [exe, *ARCH, *FLAGS, *(extra or []), "-c", path, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(compile_one, srcs))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            if log:
                print(log)
    if force or _stale(LIB, objs):
        cmd = [exe, *ARCH, "-shared", "-o", LIB, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
