"""Run the reference's own CUDA executables and this repository's `faces`
executable on the same stdin, on one GPU, and print one JSON line per run.

    python baseline/run_gpu.py [--quick] [--out FILE] [--argset NAME] [--variant V --threads T]
                               [--faces-only] [--faces-options OPT]

The reference's executables come from `make -C baseline gpu` (built here from
the staged, unmodified sources in baseline/_ref/src if they are missing).
Each is one MPI task (1x1x1) in the reference's own open, non-periodic mode:
the reference's init (gpu/main.cc:10-19), nk*(nj+1)*ni shares of which nk*nj*ni
are timed, its CPU Mugs oracle and its compare (gpu/main.cc:39-105).  The
`faces` executable gets the same ten numbers with the same meaning and checks
its result on the device against the closed form.

GB/s counts 16 bytes per field point per timed share (each point read and
written once), the same algorithmic bytes for every implementation.

Argument sets: the reference's own (gpu/frontier-run-all-1.sh:15,17), the
48^3 n=8 roofline field, and a 40^3 n=12 field (885 MB: above L2, small
enough for a full ncu capture of one launch).  --argset, --variant, --threads
and --faces-options select one run each (for profiling under ncu).
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BIN = os.path.join(HERE, "_ref", "bin")
SRC = os.path.join(HERE, "_ref", "src", "gpu", "main.cc")
FACES = os.path.join(ROOT, "faces_gb300", "bin", "faces")

ARGSETS = {
    "15x14x13_n12": "1 1 1 15 14 13 12 10 10 100",
    "95x94x93_n12": "1 1 1 95 94 93 12 3 1 10",
    "48cubed_n8": "1 1 1 48 48 48 8 1 1 100",
    "40cubed_n12": "1 1 1 40 40 40 12 1 1 3",
}
VARIANTS = ["v26-inner", "v26-all", "v6-basic"]
THREADS = [32, 256, 1024]

TIME_RE = re.compile(r"^time (\S+) avg (\S+) min (\S+) max", re.M)
PASS_RE = re.compile(r"^(\d+) tasks passed correctness check", re.M)


def points(args: str) -> tuple[int, int]:
    v = [int(x) for x in args.split()]
    lx, ly, lz, mx, my, mz, n, nk, nj, ni = v
    return lx * ly * lz * mx * my * mz * n ** 3, nk * nj * abs(ni)


def run_one(cmd: list[str], stdin: str, timeout: float) -> dict:
    t0 = time.perf_counter()
    try:
        p = subprocess.run(cmd, input=stdin, capture_output=True, text=True, timeout=timeout)
    except subprocess.TimeoutExpired:
        return {"ok": False, "error": f"timeout after {timeout:.0f} s"}
    wall = time.perf_counter() - t0
    m, q = TIME_RE.search(p.stdout), PASS_RE.search(p.stdout)
    out = {"rc": p.returncode, "wall_s": round(wall, 2)}
    if p.returncode != 0 or not m:
        out.update(ok=False, error=(p.stdout + p.stderr)[-400:])
        return out
    pts, timed = points(stdin)
    t = float(m.group(1))
    out.update(ok=True, time_s=t, tasks_passed=int(q.group(1)) if q else None,
               ms_per_share=round(1e3 * t / timed, 4), gbs=round(16 * pts * timed / t / 1e9, 1))
    return out


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--quick", action="store_true", help="MAXTHREADS=256 builds only")
    ap.add_argument("--out", default="")
    ap.add_argument("--timeout", type=float, default=300.0)
    ap.add_argument("--faces-only", action="store_true", help="run only this repository's executable")
    ap.add_argument("--argset", choices=list(ARGSETS), help="run this argument set only")
    ap.add_argument("--variant", choices=VARIANTS, help="run this reference build only")
    ap.add_argument("--threads", type=int, choices=THREADS, help="run this MAXTHREADS only")
    ap.add_argument("--faces-options", choices=["default", "--autotune", "--messages", "--v6", "--v6f", "--rows", "none"],
                    help="run the faces executable with these options only (none: not at all)")
    args = ap.parse_args()
    if args.argset:
        for k in [k for k in ARGSETS if k != args.argset]:
            del ARGSETS[k]
    if args.variant:
        VARIANTS[:] = [args.variant]
    if args.faces_only:
        VARIANTS.clear()
    elif not os.path.isfile(SRC):
        print(json.dumps({"unavailable": "the reference sources are not staged in baseline/_ref/src "
                                         "(make -C baseline stage, where the reference is present)"}))
        return
    threads = [args.threads] if args.threads else [256] if args.quick else THREADS
    # build what runs: every reference build, or the one selected
    targets = ([os.path.join(BIN, f"faces-{v}-t{t}") for v in VARIANTS for t in threads]
               if args.variant or args.threads else ["gpu"])
    r = subprocess.run(["make", "-C", HERE, "-s", f"-j{os.cpu_count() or 4}", *targets], capture_output=True,
                       text=True) if VARIANTS else None
    if VARIANTS and r.returncode != 0:
        print(json.dumps({"unavailable": "reference build failed: " + (r.stdout + r.stderr)[-400:]}))
        return
    lines = []
    faces_opts = ([], ["--autotune"], ["--messages"], ["--v6"])
    if args.faces_options:
        faces_opts = () if args.faces_options == "none" else \
            ([],) if args.faces_options == "default" else ([args.faces_options],)
    for name, stdin in ARGSETS.items():
        for v in VARIANTS:
            for t in threads:
                exe = os.path.join(BIN, f"faces-{v}-t{t}")
                rec = {"impl": "reference", "variant": v, "maxthreads": t, "args": name, "stdin": stdin}
                rec.update(run_one([exe], stdin + "\n", args.timeout))
                lines.append(rec)
                print(json.dumps(rec), flush=True)
        for opts in faces_opts:
            rec = {"impl": "faces_gb300", "options": " ".join(opts) or "(default)", "args": name, "stdin": stdin}
            rec.update(run_one([FACES, *opts], stdin + "\n", args.timeout))
            lines.append(rec)
            print(json.dumps(rec), flush=True)
    if args.out:
        with open(args.out, "w") as fh:
            for rec in lines:
                fh.write(json.dumps(rec) + "\n")


if __name__ == "__main__":
    sys.exit(main())
