"""Build tests/native/_build/librows_emu.so (CPU replay of the row and general
tile kernels, g++) and libptile_emu.so (CPU replay of the periodic tile step,
nvcc as host code)."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "_build", "librows_emu.so")


def build() -> str:
    src = os.path.join(HERE, "rows_emu.cc")
    csrc = os.path.join(ROOT, "faces_gb300", "csrc")
    deps = [src] + [os.path.join(csrc, f) for f in ("geom.cuh", "rows_setup.cuh", "tables.h", "tile_ops.cuh")]
    if os.path.exists(OUT) and all(os.path.getmtime(d) <= os.path.getmtime(OUT) for d in deps):
        return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-x", "c++",
                    "-I" + csrc, src, "-o", OUT], check=True)
    return OUT


PTILE_OUT = os.path.join(HERE, "_build", "libptile_emu.so")


def build_ptile() -> str:
    src = os.path.join(HERE, "ptile_emu.cu")
    csrc = os.path.join(ROOT, "faces_gb300", "csrc")
    deps = [src] + [os.path.join(csrc, f) for f in ("geom.cuh", "rows_setup.cuh", "tables.h", "tile_ops.cuh",
                                                     "tile_steps.cuh", "ptile_steps.cuh",
                                                     "xtile_steps.cuh", "v6_steps.cuh", "seam_steps.cuh")]
    if os.path.exists(PTILE_OUT) and all(os.path.getmtime(d) <= os.path.getmtime(PTILE_OUT) for d in deps):
        return PTILE_OUT
    os.makedirs(os.path.dirname(PTILE_OUT), exist_ok=True)
    import shutil
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "-shared",
                    "-Xcompiler", "-fPIC,-ffp-contract=off", "-I" + csrc, src, "-o", PTILE_OUT], check=True)
    return PTILE_OUT
