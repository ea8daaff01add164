"""Build tests/native/_build/librows_emu.so (CPU replay of the row kernel)."""
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
