"""bench.py's rank path (run_faces) on two gloo ranks, on CPU.

Each rank runs the whole GPU arm -- its own field, warm-up, the timed shares
with the re-initialisation inside the timed region, the barrier and the max
of the per-rank times, the device check and the end-to-end leg -- with a
stand-in library: the Faces object below runs the oracle's shares on a CPU
tensor, and torch.cuda's events, streams and synchronisation are replaced by
host-clock equivalents.  Rank 1 is made slower than rank 0, so the line rank 0
prints must carry rank 1's time; rank 1 prints nothing."""
import datetime
import os
import socket
import sys
import time
import traceback
from types import SimpleNamespace

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHAPE = dict(lx=1, ly=1, lz=1, mx=3, my=2, mz=2, n=3)
STEPS, WARMUP, RESEED, E2E_SHARES, E2E_JOBS = 6, 3, 4, 3, 3
SLOW_S = 0.004  # rank 1's extra time per share


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


class FakeEvent:
    def __init__(self, enable_timing=False):
        self.t = None

    def record(self, stream=None):
        self.t = time.perf_counter()

    def elapsed_time(self, other):
        return (other.t - self.t) * 1e3


def fake_library(rank: int):
    """a faces_gb300 stand-in: the same calls bench.run_faces makes, computed
    by the oracle on CPU tensors"""
    from oracle import oracle as O

    class Faces:
        def __init__(self, lx, ly, lz, mx, my, mz, n, periodic=False):
            self.s = O.Shape(lx, ly, lz, mx, my, mz, n, periodic)
            self.points = self.s.points
            self.total_doubles = self.s.total_doubles
            self.calls = 0
            self._tuning = {"kernel": 0, "chunk": 2, "order": 0, "width": 1}

        def field(self, dev):
            return torch.zeros(self.total_doubles, dtype=torch.float64)

        def init_int(self, u, seed, stream=None):
            u.copy_(torch.from_numpy(O.init_int(self.s, seed)))

        def autotune(self, u, compute, reps, stream=None):
            pass

        def set_tuning(self, **kw):
            self._tuning.update(kw)

        def tuning(self):
            return dict(self._tuning)

        def launches_per_share(self, compute):
            return 1

        def share(self, u, compute=True, stream=None):
            O.groups_share(self.s, u.numpy(), compute, 1)
            self.calls += 1
            if rank == 1:
                time.sleep(SLOW_S)

        def check(self, u, init="int", seed=1, nshares=1):
            want = O.groups_share(self.s, O.init_int(self.s, seed), True, nshares)
            got = u.cpu().numpy().copy()
            maxrel, npass, _ = O.compare(self.s, got, want)
            return SimpleNamespace(maxrel=maxrel, passed=npass == self.s.nranks)

        def run_host(self, hin, hout, shares, compute=True, stream=None):
            hout[:] = hin
            O.groups_share(self.s, hout, compute, shares)
            if rank == 1:
                time.sleep(SLOW_S * shares)

        def run_host_many(self, ins, outs, shares, compute=True, stream=None):
            for a, b in zip(ins, outs):
                self.run_host(a, b, shares, compute, stream)

        def close(self):
            pass

    return SimpleNamespace(Faces=Faces)


def worker(rank: int, world: int, port: int, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    # a short timeout: a rank that fails must not leave the other waiting long
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=60))
    try:
        out.put(run_rank(rank))
    except BaseException:
        out.put((rank, "error", traceback.format_exc()))
        raise
    dist.barrier()
    dist.destroy_process_group()


def run_rank(rank: int):
    sys.modules["faces_gb300"] = fake_library(rank)
    empty = torch.empty
    torch.empty = lambda *a, pin_memory=False, **k: empty(*a, **k)
    torch.cuda.set_device = lambda d: None
    torch.cuda.current_stream = lambda d=None: None
    torch.cuda.synchronize = lambda d=None: None
    torch.cuda.empty_cache = lambda: None
    torch.cuda.Event = FakeEvent
    import bench
    bench.SHAPE = dict(SHAPE)
    bench.RESEED_EVERY = RESEED
    bench.E2E_SHARES = E2E_SHARES
    bench.E2E_JOBS = E2E_JOBS
    args = SimpleNamespace(steps=STEPS, warmup=WARMUP, tune="", no_e2e=False, no_cpu=True, no_c3=True,
                           no_refgpu=True, no_mixed=True)
    return rank, bench.run_faces(args), None


def test_rank_path_on_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        got = {}
        for _ in procs:
            r, line, tb = q.get(timeout=180)
            assert line != "error", f"rank {r}:\n{tb}"
            got[r] = (line, tb)
        for p in procs:
            p.join(timeout=120)
            assert p.exitcode == 0
    finally:
        for p in procs:
            if p.is_alive():
                p.terminate()
    assert got[1][0] is None  # only rank 0 prints
    line = got[0][0]
    from oracle import oracle as O
    s = O.Shape(**SHAPE, periodic=True)
    bytes_step = 16 * s.points
    assert line["n_gpus"] == 2 and line["steps"] == STEPS and line["warmup"] == WARMUP
    # the max over ranks: rank 1 sleeps SLOW_S per share, rank 0 does not
    assert line["ms_per_step"] >= SLOW_S * 1e3
    t_max = line["ms_per_step"] * STEPS * 1e-3
    # whole-job rate: both ranks' points over the slower rank's time
    assert line["points_per_s"] == pytest.approx(2 * s.points * STEPS / t_max, rel=1e-3)
    assert line["config"]["bytes_per_step"] == bytes_step
    # the timed region re-initialises every RESEED shares; the check covers the last segment
    nseg = -(-STEPS // RESEED)
    assert line["gpu_launches"] == STEPS + nseg - 1
    assert line["check"]["passed"] and line["check"]["maxrel"] == 0.0
    e2e = line["e2e"]
    assert e2e["results_checked"]
    assert e2e["h2d_bytes_per_step"] == e2e["d2h_bytes_per_step"] == 8 * s.total_doubles
    sys.path.insert(0, ROOT)
    import bench
    assert e2e["steps"] == bench.E2E_CALLS * E2E_JOBS
    # the end-to-end time is also the max over ranks (rank 1: SLOW_S per share)
    assert e2e["ms_per_step"] >= E2E_SHARES * SLOW_S * 1e3 * 0.99
    assert line["config"]["parallelism"] == "independent field per GPU"
