"""Build the sm_103a library and the `faces` executable in-tree.

    python -m faces_gb300.build        (or faces_gb300.build.build())

Outputs (git-ignored):
    faces_gb300/lib/libfaces_gb300.so  C ABI of include/faces_gb300.h
    faces_gb300/bin/faces              drop-in for the reference's gpu/main.cc

Translation units compile in parallel with one -gencode (sm_103a).  Host code
is built with -ffp-contract=off so FP64 host arithmetic rounds the same way on
x86_64 and aarch64.
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
OBJ = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
BINDIR = os.path.join(HERE, "bin")
LIB = os.path.join(LIBDIR, "libfaces_gb300.so")
EXE = os.path.join(BINDIR, "faces")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include")] + ARCH

# (source, object); the row kernel's instantiations are split over several
# units so they compile in parallel
UNITS = (["faces_api.cu", "kernels.cu", "tiles.cu", "seams.cu", "static_share.cu", "batch.cu", "serve.cu"]
         + [f"tiles_n{n}.cu" for n in range(2, 13)]
         + [f"batch_k{f}.cu" for f in ("00", "20", "10", "11", "12")])


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build faces_gb300")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _deps() -> list[str]:
    out = [os.path.join(ROOT, "include", "faces_gb300.h"), os.path.abspath(__file__)]
    for f in os.listdir(CSRC):
        if f.endswith((".cuh", ".h")):
            out.append(os.path.join(CSRC, f))
    return out


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile everything that is out of date; returns the library path."""
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(BINDIR, exist_ok=True)
    cc = nvcc()
    deps = _deps()
    jobs = []
    objs = []
    for u in UNITS:
        src = os.path.join(CSRC, u)
        obj = os.path.join(OBJ, u.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [src] + deps):
            jobs.append([cc, *NVCC_FLAGS, "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    if force or jobs or _stale(LIB, objs):
        _run([cc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    main_src = os.path.join(CSRC, "faces_main.cc")
    if force or _stale(EXE, [main_src, LIB] + deps):
        _run([cc, "-O2", "-std=c++17", "-Xcompiler", "-ffp-contract=off", "-x", "cu", *ARCH,
              "-I" + os.path.join(ROOT, "include"), main_src, "-o", EXE,
              "-L" + LIBDIR, "-lfaces_gb300", "-Xlinker", "-rpath,$ORIGIN/../lib"])
    if verbose:
        print(LIB)
        print(EXE)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
