"""Benchmark of the Faces halo-sum step on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl faces|reference]

Workload (one step = one share): a single field, 1x1x1 virtual rank grid
with periodic self-neighbours, mx=my=mz=48 elements of n=8 (56,623,104 FP64
points, 452,984,832 bytes), integer-valued doubles uniform in [0,2^20),
summed by the fused direct kernel.  The field is larger than the 126 MB L2,
so no flush is needed between steps.

value     = whole-job HBM GB/s: algorithmic bytes (each field point read and
            written once per share: 16 B/point) * steps / time, device time
            from CUDA events on the launching stream, max over ranks
e2e       = the same metric through the C ABI from pinned host memory: each
            e2e step is the configuration's job -- upload the field, 100 shares
            (ni = 100), download the result -- via faces_run_host
roofline  = the row kernel against MEASURED_PEAKS.json's copy bandwidth
cpu_baseline = the reference's v-26 pack/inner/unpack loops transcribed to
            host C with OpenMP (the oracle), timed on this host's cores

--impl reference times that CPU implementation alone (the reference's own
Mugs/Faces code cannot run on this machine: see the design doc).

With N > 1 (torchrun) every rank advances its own copy of the field on its
GPU: independent fields, no collective on the data path (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "halo-sum HBM GB/s (% of peak); batched steps/s and p50/p99 latency vs plain"
SHAPE = dict(lx=1, ly=1, lz=1, mx=48, my=48, mz=48, n=8)
PERIODIC = True
SEED = 1
E2E_SHARES = 100  # ni of the configuration (nk=1 nj=1 ni=100)
# Every share multiplies a point shared by c copies by c, so integer inputs
# below 2^20 overflow to +inf after ~330 shares.  As in the reference's own
# loop (gpu/main.cc:176-184) the field is re-initialized every ni = 100
# shares; here the re-init runs INSIDE the timed region and counts against
# the result.
RESEED_EVERY = 100
KERNEL_NAME = "faces::tile_kernel<8,4,3>"
L2_BYTES = 126 * 2 ** 20


def workload_config(points: int, field_bytes: int) -> dict:
    return {
        "workload": "single field, 1x1x1 periodic virtual rank grid, mx=my=mz=48 elements, n=8 "
                    f"({points:,} FP64 points, {field_bytes:,} B), fused direct kernel, one share per step",
        "lx_ly_lz": [1, 1, 1], "m": [48, 48, 48], "n": 8, "periodic": True,
        "bytes_per_step": 16 * points,
        "l2": f"inputs larger than L2 ({field_bytes / 1e6:.0f} MB field > {L2_BYTES / 1e6:.0f} MB L2), no flush",
        "parallelism": "independent field per GPU",
    }


# ---------------------------------------------------------------------------
# distributed helpers (also exercised with gloo on CPU by the tests)
# ---------------------------------------------------------------------------

def dist_env() -> tuple[int, int, int]:
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def max_over_ranks(x: float) -> float:
    """Max of a host float over all ranks (identity without a process group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return x
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier() -> None:
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------

class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "100", "-f", self.path], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.15)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        rows = []
        try:
            with open(self.path) as fh:
                for line in fh:
                    p = [x.strip() for x in line.split(",")]
                    if len(p) >= 9 and p[1].isdigit():
                        rows.append(p)
        except OSError:
            pass
        finally:
            if self.path and os.path.exists(self.path):
                os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        sm = [int(r[1]) for r in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": int(rows[0][2]), "reasons": reasons,
                "samples": len(rows), "power_w_max": max(float(r[3]) for r in rows if r[3] not in ("", "[N/A]"))}


# ---------------------------------------------------------------------------
# measured peaks and profile summaries
# ---------------------------------------------------------------------------

def hbm_peak() -> tuple[float, str]:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled_traffic() -> float | None:
    """dram bytes per launch of the row kernel on this workload, from the
    committed ncu summary (profiles/tile_kernel_n8_48cubed.txt)."""
    path = os.path.join(ROOT, "profiles", "tile_kernel_n8_48cubed.txt")
    try:
        with open(path) as fh:
            for line in fh:
                if line.startswith("traffic_bytes_per_launch:"):
                    return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


# ---------------------------------------------------------------------------
# CPU baseline: the oracle's v-26 loops on the host cores
# ---------------------------------------------------------------------------

def cpu_baseline(budget_s: float = 12.0, min_steps: int = 2) -> dict:
    import numpy as np  # noqa: F401
    from oracle import oracle as O
    O.build()
    s = O.Shape(**SHAPE, periodic=PERIODIC)
    u = O.init_int(s, SEED)
    threads = O.max_threads()
    O.v26_share(s, u, True, 1, threads)  # warm-up
    done, t0 = 0, time.perf_counter()
    while done < min_steps or time.perf_counter() - t0 < budget_s:
        O.v26_share(s, u, True, 1, threads)
        done += 1
        if done >= 1000:
            break
    el = time.perf_counter() - t0
    gbs = 16.0 * s.points * done / el / 1e9
    return {"value": round(gbs, 3), "unit": "GB/s", "cores": threads, "kind": "port",
            "sample": f"{done} shares of the full 48^3 n=8 periodic field (1 warm-up), {el:.1f} s, "
                      f"v-26 pack/inner/swap/unpack loops in C + OpenMP ({threads} threads)",
            "ms_per_step": round(el / done * 1e3, 3)}


# ---------------------------------------------------------------------------
# the GPU arm
# ---------------------------------------------------------------------------

def run_faces(args) -> dict | None:
    import numpy as np
    import torch
    import torch.distributed as dist

    import faces_gb300 as F

    rank, world, local = dist_env()
    if world > 1 and not dist.is_initialized():
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    f = F.Faces(**SHAPE, periodic=PERIODIC)
    points = f.points
    bytes_step = 16 * points
    field_bytes = 8 * f.total_doubles
    u = f.field(dev)
    stream = torch.cuda.current_stream(dev)
    f.init_int(u, SEED, stream)
    for _ in range(args.warmup):
        f.share(u, True, stream)
    torch.cuda.synchronize(dev)
    launches = f.launches_per_share(True)

    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    nseg = (args.steps + RESEED_EVERY - 1) // RESEED_EVERY
    seg = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nseg)]
    f.init_int(u, SEED, stream)
    with ClockSampler(local) as clk:
        barrier()
        torch.cuda.synchronize(dev)
        e0.record(stream)
        done = 0
        for k in range(nseg):
            if k:
                f.init_int(u, SEED, stream)
            todo = min(RESEED_EVERY, args.steps - done)
            seg[k][0].record(stream)
            for _ in range(todo):
                f.share(u, True, stream)
            seg[k][1].record(stream)
            done += todo
        e1.record(stream)
        torch.cuda.synchronize(dev)
        barrier()
    ms = e0.elapsed_time(e1)
    share_ms = sum(a.elapsed_time(b) for a, b in seg)
    t_max = max_over_ranks(ms * 1e-3)
    clocks = clk.summary()

    # correctness of what was timed: closed form of the last segment's shares
    last = args.steps - (nseg - 1) * RESEED_EVERY
    chk = f.check(u, init="int", seed=SEED, nshares=last)

    # end to end through the C ABI from pinned host memory
    e2e = None
    if not args.no_e2e and (rank == 0 or world > 1):
        host_in = torch.empty(f.total_doubles, dtype=torch.float64, pin_memory=True)
        host_out = torch.empty(f.total_doubles, dtype=torch.float64, pin_memory=True)
        f.init_int(u, SEED, stream)
        torch.cuda.synchronize(dev)
        host_in.copy_(u.cpu())
        hi, ho = host_in.numpy(), host_out.numpy()
        f.run_host(hi, ho, E2E_SHARES, True, stream)  # warm-up (allocates the device copy)
        nrep = 3
        t0 = time.perf_counter()
        for _ in range(nrep):
            f.run_host(hi, ho, E2E_SHARES, True, stream)
        el = max_over_ranks(time.perf_counter() - t0)
        e2e = {"value": round(world * bytes_step * E2E_SHARES * nrep / el / 1e9, 3), "unit": "GB/s",
               "h2d_bytes_per_step": field_bytes, "d2h_bytes_per_step": field_bytes,
               "steps": nrep, "shares_per_step": E2E_SHARES,
               "ms_per_step": round(el / nrep * 1e3, 3),
               "call": "faces_run_host (C ABI): pinned host field -> device, 100 shares, -> host"}
        del host_in, host_out

    if rank != 0:
        return None
    peak, peak_kind = hbm_peak()
    avg_launch_s = share_ms * 1e-3 / (args.steps * launches)
    achieved = bytes_step / avg_launch_s / 1e9
    value = world * bytes_step * args.steps / t_max / 1e9
    out = {
        "metric": METRIC,
        "value": round(value, 3),
        "unit": "GB/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(t_max * 1e3 / args.steps, 6),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic: integer-valued FP64 uniform in [0,2^20) (splitmix64 seed 1)",
        "config": workload_config(points, field_bytes),
        "pct_of_peak": round(100 * achieved / peak, 2),
        "points_per_s": round(world * points * args.steps / t_max, 1),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": profiled_traffic(),
                     "kernel": KERNEL_NAME,
                     "algorithmic_bytes_per_launch": bytes_step,
                     "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({peak_kind})"},
        "clocks": clocks,
        "e2e": e2e,
        "gpu_launches": args.steps * launches + (nseg - 1),
        "reinit": f"field re-initialized every {RESEED_EVERY} shares inside the timed region "
                  f"({nseg - 1} init launches counted in value; excluded from roofline.achieved)",
        "check": {"maxrel": chk.maxrel, "passed": chk.passed,
                  "what": f"device closed form of the last {last} shares, gpu/main.cc:39-105 rule"},
    }
    if world == 1 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline()
    return out


def run_reference(args) -> dict | None:
    rank, world, _ = dist_env()
    if rank != 0:
        return None
    cb = cpu_baseline(budget_s=min(60.0, 2.0 + 0.05 * max(args.steps, 1)), min_steps=max(1, min(args.steps, 3)))
    done = int(cb["sample"].split()[0])
    from oracle import oracle as O
    s = O.Shape(**SHAPE, periodic=PERIODIC)
    return {
        "metric": METRIC, "value": cb["value"], "unit": "GB/s", "n_gpus": world, "steps": done,
        "warmup": args.warmup, "ms_per_step": cb["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: integer-valued FP64 uniform in [0,2^20) (splitmix64 seed 1)",
        "config": workload_config(s.points, 8 * s.total_doubles),
        "impl": "reference",
        "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": cb["value"], "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's own code cannot run here (its GPU build needs its sources and MPI; "
                "binaries built in the development container are x86): its v-26 loops, transcribed to C "
                "with OpenMP, are timed instead",
    }


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["faces", "reference"], default="faces")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end host-buffer leg")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    out = run_reference(args) if args.impl == "reference" else run_faces(args)
    if out is not None:
        print(json.dumps(out), flush=True)
    try:
        import torch.distributed as dist
        if dist.is_initialized():
            dist.destroy_process_group()
    except Exception:
        pass


if __name__ == "__main__":
    main()
