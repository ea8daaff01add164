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
            (ni = 100), download the result -- 8 jobs per faces_run_host_many
            call, whose copies overlap the neighbouring jobs' shares (one job
            per faces_run_host call is reported beside it)
roofline  = the periodic tile kernel against MEASURED_PEAKS.json's copy bandwidth
cpu_baseline = the reference's v-26 pack/inner/unpack loops transcribed to
            host C with OpenMP (the oracle), timed on this host's cores

--impl reference times that CPU implementation alone.

c3       = 3x3x3 periodic virtual ranks of 16^3 elements, n=6: 26 messages
            per rank packed, swapped by buffer and unpack-added (v-26), with
            direct mode, v-6 and fused v-6 beside it; GB/s over field and
            message bytes
reference_gpu = the reference's own CUDA build (gpu/main.cc + v-26 Faces.cc,
            one-rank MPI stand-in, built by baseline/Makefile where its
            sources are staged) against this repository's `faces` executable
            on the same stdin, open mode (the reference has no periodic mode)
batched  = 512 fields of mixed shape advanced by one persistent launch per
            share, against one launch per field (steps/s of each)
served   = a 400-job Poisson trace through the job server, batched and
            plain: steps/s and p50/p99 latency (rank 0 only)

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
E2E_JOBS = 8      # independent jobs per faces_run_host_many call in the e2e leg
E2E_CALLS = 4     # timed calls (the copies' overlap varies a little from call to call)
# Every share multiplies a point shared by c copies by c, so integer inputs
# below 2^20 overflow to +inf after ~330 shares.  As in the reference's own
# loop (gpu/main.cc:176-184) the field is re-initialized every ni = 100
# shares; here the re-init runs INSIDE the timed region and counts against
# the result.
RESEED_EVERY = 100
def kernel_name(t: dict) -> str:
    """The step's kernel for n = 8 on this field from faces_get_tuning."""
    k = 1 << max(0, (t["chunk"] - 1).bit_length())
    if t["kernel"] == 3:
        return "faces::seam_kernel<8>"
    if t["kernel"] == 2:
        return "faces::rows_kernel<8>"
    if t["kernel"] == 1:
        return f"faces::tile_kernel<8,{k},3>"
    if t["order"] == 3:
        return "faces::wtile_kernel<8,1,3,4>"
    return f"faces::ptile_kernel<8,{k},3>"
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
    """dram bytes per launch of the periodic tile kernel on this workload,
    from the committed ncu summary (profiles/ptile_kernel_n8_48cubed.txt)."""
    path = os.path.join(ROOT, "profiles", "ptile_kernel_n8_48cubed.txt")
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
    # tile settings for this field, timed on the device (outside the timed
    # region), or given (--tune chunk,order,width: for profiling runs)
    f.init_int(u, SEED, stream)
    if args.tune:
        chunk, order, width = (int(x) for x in args.tune.split(","))
        f.set_tuning(chunk=chunk, width=width, order=order)
        how = f"given: --tune {args.tune}"
    else:
        f.autotune(u, True, 5, stream)
        how = "faces_autotune before timing"
    tuned = f.tuning()
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

    # end to end through the C ABI from pinned host memory: E2E_JOBS jobs per
    # faces_run_host_many call (each job: upload, 100 shares, download; the
    # copies of neighbouring jobs overlap the shares), and one job per
    # faces_run_host call for comparison
    e2e = None
    if not args.no_e2e and (rank == 0 or world > 1):
        f.init_int(u, SEED, stream)
        torch.cuda.synchronize(dev)
        src = u.cpu()
        host_in = [torch.empty(f.total_doubles, dtype=torch.float64, pin_memory=True) for _ in range(2)]
        host_out = [torch.empty(f.total_doubles, dtype=torch.float64, pin_memory=True) for _ in range(4)]
        for h in host_in:
            h.copy_(src)
        hi = [h.numpy() for h in host_in]
        ho = [h.numpy() for h in host_out]
        # inputs alternate between two buffers, outputs cycle over four (downloads run in job order)
        ins = [hi[j % 2] for j in range(E2E_JOBS)]
        outs = [ho[j % 4] for j in range(E2E_JOBS)]
        f.run_host_many(ins[:2], outs[:2], E2E_SHARES, True, stream)  # warm-up (allocates the device fields)
        nrep = E2E_CALLS
        t0 = time.perf_counter()
        for _ in range(nrep):
            f.run_host_many(ins, outs, E2E_SHARES, True, stream)
        el = max_over_ranks(time.perf_counter() - t0)
        # the downloaded results are the closed form of 100 shares
        probe = torch.from_numpy(outs[-1]).to(u.device)
        e2e_chk = f.check(probe, init="int", seed=SEED, nshares=E2E_SHARES)
        del probe
        f.run_host(hi[0], ho[0], E2E_SHARES, True, stream)  # warm-up
        t1 = time.perf_counter()
        for _ in range(nrep):
            f.run_host(hi[0], ho[0], E2E_SHARES, True, stream)
        el1 = max_over_ranks(time.perf_counter() - t1)
        jobs = nrep * E2E_JOBS
        e2e = {"value": round(world * bytes_step * E2E_SHARES * jobs / el / 1e9, 3), "unit": "GB/s",
               "h2d_bytes_per_step": field_bytes, "d2h_bytes_per_step": field_bytes,
               "steps": jobs, "shares_per_step": E2E_SHARES,
               "ms_per_step": round(el / jobs * 1e3, 3),
               "call": f"faces_run_host_many (C ABI), {E2E_JOBS} jobs per call: each job uploads a pinned host "
                       "field, runs 100 shares and downloads the result; uploads and downloads run on two copy "
                       "streams while the neighbouring jobs' shares run",
               "results_checked": bool(e2e_chk.passed and e2e_chk.maxrel == 0.0),
               "one_job_per_call": {"value": round(world * bytes_step * E2E_SHARES * nrep / el1 / 1e9, 3),
                                    "ms_per_step": round(el1 / nrep * 1e3, 3),
                                    "call": "faces_run_host: upload, 100 shares, download, synchronous"}}
        del host_in, host_out, hi, ho, ins, outs

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
        "config": dict(workload_config(points, field_bytes), tuning=dict(tuned, how=how)),
        "pct_of_peak": round(100 * achieved / peak, 2),
        "points_per_s": round(world * points * args.steps / t_max, 1),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": profiled_traffic(),
                     "kernel": kernel_name(tuned),
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
    if not args.no_c3:
        out["c3"] = c3_leg(F, dev)
    if world == 1 and not args.no_refgpu:
        out["reference_gpu"] = reference_gpu_leg()
    if not args.no_mixed:
        del u
        f.close()
        torch.cuda.empty_cache()
        out["batched"] = batched_leg(F, dev)
        out["served"] = served_leg(F)
    return out


# ---------------------------------------------------------------------------
# C3: virtual ranks exchanging messages
# ---------------------------------------------------------------------------

C3_SHAPE, C3_STEPS = (3, 3, 3, 16, 16, 16, 6), 50


def c3_message_doubles(shape, v6: bool) -> int:
    """Message doubles of one share: v-26 -- every rank's 26 messages (faces
    n^2 m_a m_b, edges n m_a, corners 1; gpu/v-26-messages/Faces.cc:16-27);
    v-6 -- six face messages per rank (gpu/v-6-messages-basic/Faces.cc)."""
    lx, ly, lz, mx, my, mz, n = shape
    faces = n * n * (my * mz + mx * mz + mx * my)
    edges = n * (mx + my + mz)
    per_rank = 2 * faces if v6 else 2 * faces + 4 * edges + 8
    return lx * ly * lz * per_rank


def c3_leg(F, dev) -> dict:
    """C3 at full size: 50 shares per mode, timed with CUDA events after
    autotuning (outside the timing); each run checked against the closed
    form of its 50 shares."""
    import torch
    stream = torch.cuda.current_stream(dev)
    peak, peak_kind = hbm_peak()
    modes = {}
    for mode in ("messages", "messages-fused", "direct", "v6", "v6f"):
        f = F.Faces(*C3_SHAPE, periodic=True, messages=mode.startswith("messages"), v6=mode == "v6", v6f=mode == "v6f",
                    pack_fused=mode == "messages-fused")
        u = f.field(dev)
        f.init_int(u, SEED, stream)
        if not mode.startswith("v6"):
            f.autotune(u, True, 3, stream)
        status = f.status() if mode == "messages-fused" else 0
        f.init_int(u, SEED, stream)
        for _ in range(3):
            f.share(u, True, stream)
        f.init_int(u, SEED, stream)
        ms = _events_ms(lambda: f.share_n(u, C3_STEPS, True, stream), stream, 1) / C3_STEPS
        chk = f.check(u, init="int", seed=SEED, nshares=C3_STEPS)
        msg = 0 if mode == "direct" else c3_message_doubles(C3_SHAPE, mode.startswith("v6"))
        b = 16 * (f.points + msg)
        modes[mode] = {"ms_per_share": round(ms, 5), "gbs": round(b / (ms * 1e-3) / 1e9, 1),
                       "field_gbs": round(16 * f.points / (ms * 1e-3) / 1e9, 1),
                       "frac": round(b / (ms * 1e-3) / 1e9 / peak, 4), "bytes_per_share": b,
                       "message_doubles": msg, "launches_per_share": f.launches_per_share(True),
                       "tuning": f.tuning(),
                       "check_passed": bool(chk.passed and chk.maxrel == 0.0 and status == 0 and
                                            (mode != "messages-fused" or f.status() == 0))}
        del u
        f.close()
    torch.cuda.empty_cache()
    m = modes["messages"]
    return {"workload": "3x3x3 periodic virtual ranks (27 subdomains in one HBM), 16^3 elements of n=6 each "
                        f"({27 * 16 ** 3 * 216:,} points), integer-valued, {C3_STEPS} shares per mode",
            "value": m["gbs"], "unit": "GB/s", "mode": "v-26 messages (pack, buffer swap, unpack-add)",
            "roofline": {"bound": "hbm", "achieved": m["gbs"], "peak": peak, "frac": m["frac"],
                         "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({peak_kind})"},
            "bytes": "16 B per field point + 16 B per message double (pack write + unpack read)",
            "modes": modes}


# ---------------------------------------------------------------------------
# the reference's own CUDA build beside this repository's executable
# ---------------------------------------------------------------------------

def reference_gpu_leg(timeout: float = 240.0) -> dict:
    """The reference's gpu/main.cc with v-26 Faces.cc (FUSE_SEND, FUSE_INNER,
    FUSE_RECV; MAXTHREADS 256), unmodified, built for sm_103a against a
    one-rank MPI stand-in, on `1 1 1 48 48 48 8 1 1 100` -- the roofline
    field in the reference's open mode -- and on the reference's own two
    argument sets (gpu/frontier-run-all-1.sh:15,17), and this repository's
    `faces` executable on the same stdin.  Each prints the reference's `time`
    and `tasks passed` lines; GB/s = 16 B per point per timed share."""
    sys.path.insert(0, os.path.join(ROOT, "baseline"))
    import run_gpu as RG
    stdin = RG.ARGSETS["48cubed_n8"] + "\n"
    exe = os.path.join(RG.BIN, "faces-v26-all-t256")
    if not os.path.isfile(exe):
        if not os.path.isfile(RG.SRC):
            return {"unavailable": "the reference's sources are not staged in baseline/_ref/src"}
        r = subprocess.run(["make", "-C", os.path.join(ROOT, "baseline"), "-s", exe], capture_output=True, text=True)
        if r.returncode != 0:
            return {"unavailable": "reference build failed: " + (r.stdout + r.stderr)[-300:]}
    ref = RG.run_one([exe], stdin, timeout)
    ours = RG.run_one([RG.FACES], stdin, timeout)
    out = {"stdin": stdin.strip(), "mode": "open (non-periodic), reference init, nk=1 nj=1 ni=100",
           "reference": dict(ref, build="v-26-messages -DFUSE_SEND -DFUSE_INNER -DFUSE_RECV -DMAXTHREADS=256, "
                                        "nvcc sm_103a (baseline/Makefile)"),
           "faces_gb300": dict(ours, build="faces executable, default settings")}
    if ref.get("ok") and ours.get("ok"):
        out["speedup"] = round(ref["time_s"] / ours["time_s"], 2)
    # the reference's own argument sets, same two executables
    shapes = {}
    for name in ("15x14x13_n12", "95x94x93_n12"):
        stdin = RG.ARGSETS[name] + "\n"
        r, o = RG.run_one([exe], stdin, timeout), RG.run_one([RG.FACES], stdin, timeout)
        rec = {"stdin": stdin.strip(), "reference_gbs": r.get("gbs"), "faces_gb300_gbs": o.get("gbs"),
               "reference_ok": bool(r.get("ok") and r.get("tasks_passed") == 1),
               "faces_gb300_ok": bool(o.get("ok") and o.get("tasks_passed") == 1)}
        if r.get("ok") and o.get("ok"):
            rec["speedup"] = round(r["time_s"] / o["time_s"], 2)
        shapes[name] = rec
    out["reference_shapes"] = shapes
    return out


# ---------------------------------------------------------------------------
# batched and served workloads (reported beside the headline, rank 0 only)
# ---------------------------------------------------------------------------

C4_FIELDS, C4_STEPS = 512, 20
C5_JOBS, C5_BUDGET = 400, 150 << 30


def c4_mix(seed: int = 4, nfields: int = C4_FIELDS) -> list[tuple]:
    """512 periodic single-rank fields, mx,my,mz uniform in [2,24], n uniform in {3..10}."""
    import numpy as np
    rng = np.random.default_rng(seed)
    mix = []
    for _ in range(nfields):
        m = tuple(int(x) for x in rng.integers(2, 25, size=3))
        mix.append((1, 1, 1) + m + (int(rng.integers(3, 11)),))
    return mix


def c5_jobs(F, count: int = C5_JOBS, seed: int = 5) -> list:
    """Jobs of rank grid {1,2}^3, m per dimension log-uniform in [2,32], n uniform
    in {4..8}, 10..200 shares, periodic, integer-valued fields seeded per job."""
    import numpy as np
    rng = np.random.default_rng(seed)
    jobs = []
    for i in range(count):
        L = [int(x) for x in rng.integers(1, 3, size=3)]
        m = [int(np.floor(np.exp(rng.uniform(np.log(2), np.log(33))))) for _ in range(3)]
        n = int(rng.integers(4, 9))
        jobs.append(F.job(*L, *m, n, nshares=int(rng.integers(10, 201)), periodic=True, init="int", seed=i))
    return jobs


def _events_ms(fn, stream, reps: int) -> float:
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def batched_leg(F, dev) -> dict:
    """C4: one persistent launch per share of all 512 fields (a CUDA graph of
    20 shares), against one launch of the single-field kernel per field."""
    import torch
    mix = c4_mix()
    fields = []
    for i, sh in enumerate(mix):
        f = F.Faces(*sh, periodic=True)
        fields.append((f, f.field(dev)))
    points = sum(f.points for f, _ in fields)
    stream = torch.cuda.current_stream(dev)

    def reinit():
        for i, (f, u) in enumerate(fields):
            f.init_int(u, 100 + i, stream)

    b = F.Batch()
    for f, u in fields:
        b.add(f, u)
    b.commit()
    reinit()
    b.autotune(3, stream)
    info = b.info()
    reinit()
    b.share_n(C4_STEPS, True, stream)  # warm-up (captures the graph)
    reinit()
    ms_batched = _events_ms(lambda: b.share_n(C4_STEPS, True, stream), stream, 1) / C4_STEPS
    sample = list(range(0, len(fields), 37))
    checks = [fields[i][0].check(fields[i][1], init="int", seed=100 + i, nshares=C4_STEPS) for i in sample]
    reinit()
    b.share_each(True, stream)  # warm-up
    reinit()
    ms_plain = _events_ms(lambda: b.share_each(True, stream), stream, C4_STEPS)
    b.close()
    for f, _ in fields:
        f.close()
    del fields
    torch.cuda.empty_cache()
    return {
        "workload": f"{len(mix)} periodic single-rank fields, mx,my,mz uniform in [2,24], n uniform in {{3..10}} "
                    f"({points:,} points, seeded per field), {C4_STEPS} shares",
        "steps_per_s": round(1e3 / ms_batched, 2),
        "plain_steps_per_s": round(1e3 / ms_plain, 2),
        "speedup_vs_plain": round(ms_plain / ms_batched, 3),
        "gbs": round(16 * points / (ms_batched * 1e-3) / 1e9, 1),
        "plain_gbs": round(16 * points / (ms_plain * 1e-3) / 1e9, 1),
        "launches_per_step": 1, "plain_launches_per_step": len(mix),
        "autotuned": info,
        "batched": "CUDA graph of 20 launches of the batched tile kernel (faces_batch_share_n)",
        "plain": "one faces_share per field per share (faces_batch_share_each)",
        "check": {"fields_checked": len(sample), "max_maxrel": max(c.maxrel for c in checks),
                  "passed": all(c.passed for c in checks)},
    }


def served_leg(F) -> dict:
    """C5: a 400-job Poisson trace through the job server, batched and plain."""
    import numpy as np
    jobs = c5_jobs(F)
    shares = sum(j.nshares for j in jobs)
    pts = sum(j.lx * j.ly * j.lz * j.mx * j.my * j.mz * j.n ** 3 * j.nshares for j in jobs)
    runs = []
    for plain, rates in ((False, (float("inf"), 2000.0, 1000.0, 500.0, 250.0)),
                         (True, (float("inf"), 2000.0, 1000.0, 500.0, 250.0))):
        for rate in rates:
            rng = np.random.default_rng(7)
            arr = (np.zeros(len(jobs)) if rate == float("inf")
                   else np.cumsum(rng.exponential(1.0 / rate, size=len(jobs))))
            with F.Server(C5_BUDGET, plain=plain, release_done=True) as srv:
                srv.run_trace(jobs[:8], np.zeros(8))  # warm-up
                _, lat, mk = srv.run_trace(jobs, arr)
                st = srv.stats()
            runs.append({"form": "plain" if plain else "batched",
                         "rate_jobs_per_s": None if rate == float("inf") else rate,
                         "steps_per_s": round(shares / mk, 1), "gbs": round(16 * pts / mk / 1e9, 1),
                         "p50_ms": round(float(np.percentile(lat, 50)) * 1e3, 3),
                         "p99_ms": round(float(np.percentile(lat, 99)) * 1e3, 3),
                         "makespan_s": round(mk, 4), "ticks": st["ticks"], "launches": st["launches"],
                         "peak_resident_gb": round(st["peak_resident_bytes"] / 1e9, 3)})
    sat = {r["form"]: r["steps_per_s"] for r in runs if r["rate_jobs_per_s"] is None}
    curve = {form: [(r["rate_jobs_per_s"] or "inf", r["steps_per_s"], r["p50_ms"], r["p99_ms"]) for r in runs
                    if r["form"] == form] for form in ("batched", "plain")}
    return {
        "workload": f"{len(jobs)} jobs: rank grid in {{1,2}}^3, m per dimension log-uniform in [2,32], n uniform in "
                    "{4..8}, 10..200 shares, periodic, integer fields; Poisson arrivals (rate inf = all at t=0)",
        "budget_gb": C5_BUDGET / 2 ** 30,
        "steps": "job shares (one share of one job)",
        "runs": runs,
        "speedup_vs_plain_saturated": round(sat["batched"] / sat["plain"], 3),
        "curve": {"columns": ["rate jobs/s", "job-steps/s", "p50 ms", "p99 ms"], **curve},
        "latency": "arrival to GPU completion of the job's last share",
    }


def profile_c4(F, shares: int) -> dict:
    """The 512-field batch with default settings, `shares` batched shares
    (no autotune, no graph): the case the batched kernel is profiled on."""
    import torch
    fields = []
    for i, sh in enumerate(c4_mix()):
        f = F.Faces(*sh, periodic=True)
        u = f.field()
        f.init_int(u, 100 + i)
        fields.append((f, u))
    b = F.Batch()
    for f, u in fields:
        b.add(f, u)
    b.commit()
    b.tune(1, 0, 0, 1)  # whole-column units, full tiles, one unit per run: faces_batch_autotune's pick
    for _ in range(shares):
        b.share()
    torch.cuda.synchronize()
    return {"case": "c4", "shares": shares, "batch": b.info()}


def profile_c3(F, mode: str, shares: int) -> dict:
    """The C3 grid (3x3x3 periodic ranks of 16^3 elements, n=6) in one mode,
    default settings, `shares` shares one call at a time: the case the C3
    kernels are profiled on."""
    import torch
    f = F.Faces(*C3_SHAPE, periodic=True, messages=mode == "messages", v6=mode == "v6", v6f=mode == "v6f")
    u = f.field()
    f.init_int(u, SEED)
    for _ in range(shares):
        f.share(u)
    torch.cuda.synchronize()
    chk = f.check(u, init="int", seed=SEED, nshares=shares)
    return {"case": "c3", "mode": mode, "shares": shares, "tuning": f.tuning(), "check_passed": bool(chk.passed)}


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
        "note": "the reference's CPU code for this operation is its Mugs checker (gpu/Mugs.cc), which has no "
                "periodic neighbours, and this configuration is periodic: the reference's v-26 loops, transcribed "
                "to C with OpenMP, are timed on it instead; the reference's own CUDA build runs beside this "
                "repository's executable in the GPU arm's reference_gpu object",
    }


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["faces", "reference"], default="faces")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end host-buffer leg")
    ap.add_argument("--no-mixed", action="store_true", help="skip the batched and served legs")
    ap.add_argument("--no-c3", action="store_true", help="skip the C3 virtual-rank leg")
    ap.add_argument("--no-refgpu", action="store_true", help="skip the reference's own CUDA build")
    ap.add_argument("--tune", default="", metavar="CHUNK,ORDER,WIDTH",
                    help="set the tile settings instead of autotuning (profiling runs)")
    ap.add_argument("--profile-c4", type=int, default=0, metavar="N",
                    help="only build the 512-field batch and run N batched shares (for ncu)")
    ap.add_argument("--profile-c3", default="", metavar="MODE,N",
                    help="only run N shares of the C3 grid in MODE (messages, direct, v6, v6f) (for ncu)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.profile_c4:
        import faces_gb300 as F
        print(json.dumps(profile_c4(F, args.profile_c4)), flush=True)
        return
    if args.profile_c3:
        import faces_gb300 as F
        mode, n = args.profile_c3.split(",")
        print(json.dumps(profile_c3(F, mode, int(n))), flush=True)
        return
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
