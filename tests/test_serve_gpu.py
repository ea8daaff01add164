"""The job server: jobs that arrive while others run, admitted against an
HBM budget and advanced together one share per tick, must each end exactly
as the same job run alone with faces_share_n."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

GB = 1 << 30


def random_jobs(F, count, seed, max_m=6, ns=range(2, 11), max_shares=7):
    rng = np.random.default_rng(seed)
    jobs = []
    for i in range(count):
        L = [int(x) for x in rng.integers(1, 3, size=3)]
        m = [int(x) for x in rng.integers(1, max_m + 1, size=3)]
        n = int(rng.choice(list(ns)))
        jobs.append(F.job(*L, *m, n, nshares=int(rng.integers(1, max_shares + 1)),
                          periodic=bool(rng.integers(0, 2)), init="int", seed=1000 + seed * 100 + i))
    return jobs


def field_bytes(F, *shape):
    f = F.Faces(*shape)
    b = 8 * f.total_doubles
    f.close()
    return b


def alone(F, j):
    f = F.Faces(j.lx, j.ly, j.lz, j.mx, j.my, j.mz, j.n, periodic=bool(j.flags & F.PERIODIC))
    u = f.field()
    if j.init == 0:
        f.init_ref(u)
    elif j.init == 1:
        f.init_int(u, j.seed)
    else:
        u.copy_(torch.from_numpy(j._keep))
    f.share_n(u, j.nshares)
    torch.cuda.synchronize()
    out = u.cpu().numpy()
    f.close()
    return out


@pytest.mark.parametrize("form", ["batched", "plain", "chunk_units_runs8", "long_tiles", "half_tiles"])
def test_results_equal_alone(faces_lib, form):
    """A mix of periodic and open jobs: ticks switch between the periodic-only
    kernel form (where the tile form applies) and the mixed one."""
    F = faces_lib
    jobs = random_jobs(F, 24, seed=1)
    tune = {"chunk_units_runs8": (64, 8, 0), "long_tiles": (1, 8, 2), "half_tiles": (2, 1, 1)}.get(form)
    with F.Server(4 * GB, plain=form == "plain") as srv:
        if tune:
            srv.tune(*tune)
        ids = [srv.submit(j) for j in jobs]
        srv.drain()
        st = srv.stats()
        assert st["completed"] == len(jobs)
        assert st["job_shares"] == sum(j.nshares for j in jobs)
        for j, jid in zip(jobs, ids):
            s = srv.status(jid)
            assert s["state"] == "done" and s["shares_done"] == j.nshares and s["latency_s"] > 0
            assert np.array_equal(srv.fetch(jid), alone(F, j)), (j.lx, j.ly, j.lz, j.mx, j.my, j.mz, j.n)


def test_arrivals_while_running(faces_lib):
    """Jobs submitted between ticks join the running set (continuous batching)."""
    F = faces_lib
    jobs = random_jobs(F, 30, seed=2, max_shares=12)
    with F.Server(4 * GB) as srv:
        ids = []
        joined_while_running = 0
        for k, j in enumerate(jobs):
            ids.append(srv.submit(j))
            for _ in range(k % 3):
                srv.poll(wait=True)
            if srv.stats()["running"] > 1:
                joined_while_running += 1
        srv.drain()
        assert joined_while_running > 5
        for j, jid in zip(jobs, ids):
            assert np.array_equal(srv.fetch(jid), alone(F, j))


def test_budget_admission(faces_lib):
    """A small budget admits jobs a few at a time; resident bytes never exceed it."""
    F = faces_lib
    jobs = [F.job(1, 1, 1, 6, 6, 6, 8, nshares=3, periodic=True, seed=50 + i) for i in range(8)]
    fb = field_bytes(F, 1, 1, 1, 6, 6, 6, 8)
    budget = 3 * fb + 100
    with F.Server(budget, release_done=True) as srv:
        for j in jobs:
            srv.submit(j)
        srv.drain()
        st = srv.stats()
        assert st["completed"] == 8
        assert fb < st["peak_resident_bytes"] <= budget
        assert st["resident_bytes"] == 0
        with pytest.raises(F.FacesError):
            srv.submit(F.job(1, 1, 1, 20, 20, 20, 8, nshares=1))  # larger than the budget
        with pytest.raises(F.FacesError):
            srv.submit(F.job(1, 1, 1, 2, 2, 2, 12, nshares=1))  # n outside 2..10


def test_unreleased_results_hold_budget(faces_lib):
    F = faces_lib
    fb = field_bytes(F, 1, 1, 1, 4, 4, 4, 6)
    with F.Server(fb) as srv:
        a = srv.submit(F.job(1, 1, 1, 4, 4, 4, 6, nshares=2, seed=1))
        b = srv.submit(F.job(1, 1, 1, 4, 4, 4, 6, nshares=2, seed=2))
        with pytest.raises(F.FacesError):
            srv.drain()
        assert srv.status(a)["state"] == "done" and srv.status(b)["state"] == "queued"
        ra = srv.fetch(a)
        srv.release(a)
        srv.drain()
        assert srv.status(b)["state"] == "done"
        assert np.array_equal(ra, alone(F, F.job(1, 1, 1, 4, 4, 4, 6, nshares=2, seed=1)))


def test_host_and_reference_inits(faces_lib):
    F = faces_lib
    rng = np.random.default_rng(3)
    shape = (2, 1, 1, 3, 2, 4, 5)
    host = rng.integers(0, 1 << 20, size=field_bytes(F, *shape) // 8).astype(np.float64)
    jobs = [F.job(*shape, nshares=3, init="host", host_in=host),
            F.job(1, 1, 1, 3, 3, 3, 7, nshares=2, init="ref", periodic=True)]
    with F.Server(GB) as srv:
        ids = [srv.submit(j) for j in jobs]
        srv.drain()
        for j, jid in zip(jobs, ids):
            assert np.array_equal(srv.fetch(jid), alone(F, j))


def test_run_trace(faces_lib):
    """A Poisson trace replayed in real time: every job completes, latencies
    are positive, results are exact."""
    F = faces_lib
    jobs = random_jobs(F, 40, seed=4, max_shares=20)
    rng = np.random.default_rng(9)
    arrivals = np.cumsum(rng.exponential(1e-3, size=len(jobs)))
    with F.Server(4 * GB) as srv:
        ids, lat, makespan = srv.run_trace(jobs, arrivals)
        assert np.all(lat > 0) and makespan >= arrivals[-1]
        assert srv.stats()["completed"] == len(jobs)
        for j, jid in list(zip(jobs, ids))[::5]:
            assert np.array_equal(srv.fetch(jid), alone(F, j))
