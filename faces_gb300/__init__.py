"""faces_gb300 -- GB300 (sm_103a) Faces halo-sum step behind the reference's
Faces interface.

The reference's in-process API is ``class Faces { Faces(rank, lx, ly, lz, mx,
my, mz, n); void share(Double6D &u, bool compute = true); }``
(gpu/v-26-messages/Faces.h:6-39) with the field a DArray<double,6>
(gpu/DArray.h).  :class:`Faces` here is that object for all lx*ly*lz virtual
ranks of one GPU; the field is a CUDA float64 tensor (or raw device pointer)
in the DArray layout, ranks stored rank-major.  Every call goes through the C
ABI of include/faces_gb300.h in ``lib/libfaces_gb300.so``; there is no CPU
fallback -- importing this package without the built library raises.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

__all__ = ["Faces", "FacesError", "lib", "library_path", "PERIODIC", "MESSAGES", "GATHER", "ROWS"]

HERE = os.path.dirname(os.path.abspath(__file__))
library_path = os.path.join(HERE, "lib", "libfaces_gb300.so")
exe_path = os.path.join(HERE, "bin", "faces")

PERIODIC = 0x1
MESSAGES = 0x2
GATHER = 0x4
ROWS = 0x8
GENERAL = 0x10
V6 = 0x20
V6F = 0x40
SEAMS = 0x80
PACK_FUSED = 0x100

_ERRNAMES = {-1: "EINVAL", -2: "ECUDA", -3: "ENOMEM", -4: "EALIGN", -5: "EUNSUPPORTED"}


class FacesError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"faces_gb300 error {code} ({_ERRNAMES.get(code, '?')}): {msg}")
        self.code = code


_lib = None


def lib() -> ctypes.CDLL:
    """The loaded C-ABI library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.isfile(library_path):
        raise ImportError(
            f"{library_path} is missing: build it with `python -m faces_gb300.build` "
            "(faces_gb300 has no CPU fallback)")
    L = ctypes.CDLL(library_path)
    c_int, c_long, c_uint, c_ull, vp = ctypes.c_int, ctypes.c_long, ctypes.c_uint, ctypes.c_ulonglong, ctypes.c_void_p
    dp = ctypes.c_void_p
    L.faces_create.argtypes = [ctypes.POINTER(vp)] + [c_int] * 7 + [c_uint]
    L.faces_destroy.argtypes = [vp]
    L.faces_layout.argtypes = [vp, ctypes.POINTER(c_long), ctypes.POINTER(c_long), ctypes.POINTER(c_long)]
    L.faces_field_alloc.argtypes = [vp, ctypes.POINTER(vp)]
    L.faces_field_free.argtypes = [vp]
    L.faces_share.argtypes = [vp, dp, c_int, vp]
    L.faces_share_n.argtypes = [vp, dp, c_int, c_int, vp]
    L.faces_init_ref.argtypes = [vp, dp, vp]
    L.faces_init_int.argtypes = [vp, dp, c_ull, vp]
    L.faces_check.argtypes = [vp, dp, c_int, c_ull, c_int, c_int, ctypes.POINTER(ctypes.c_double),
                              ctypes.POINTER(ctypes.c_double), ctypes.POINTER(c_int), ctypes.POINTER(c_int),
                              ctypes.POINTER(ctypes.c_double), vp]
    L.faces_run_host.argtypes = [vp, dp, dp, c_int, c_int, vp]
    L.faces_run_host_many.argtypes = [vp, c_int, ctypes.POINTER(vp), ctypes.POINTER(vp), c_int, c_int, vp]
    L.faces_run_host_many.restype = c_int
    L.faces_set_tuning.argtypes = [vp, c_int, c_int, c_int]
    L.faces_launches_per_share.argtypes = [vp, c_int]
    L.faces_status.argtypes = [vp, ctypes.POINTER(c_int)]
    L.faces_test_pack_wait.argtypes = [vp, c_int, c_long]
    L.faces_autotune.argtypes = [vp, dp, c_int, c_int, vp]
    L.faces_autotune.restype = c_int
    L.faces_get_tuning.argtypes = [vp] + [ctypes.POINTER(c_int)] * 5
    L.faces_get_tuning.restype = c_int
    L.faces_last_error.restype = ctypes.c_char_p
    ip = ctypes.POINTER(c_int)
    L.faces_batch_create.argtypes = [ctypes.POINTER(vp)]
    L.faces_batch_add.argtypes = [vp, dp] + [c_int] * 7 + [c_uint, ip]
    L.faces_batch_commit.argtypes = [vp]
    L.faces_batch_share.argtypes = [vp, c_int, vp]
    L.faces_batch_share_n.argtypes = [vp, c_int, c_int, vp]
    L.faces_batch_share_each.argtypes = [vp, c_int, vp]
    L.faces_batch_tune.argtypes = [vp, c_int, c_int, c_int, c_int]
    L.faces_batch_autotune.argtypes = [vp, c_int, vp]
    L.faces_batch_info.argtypes = [vp, ip, ip, ip, ip, ip, ip, ip]
    L.faces_batch_tune_warp.argtypes = [vp, c_int, c_int]
    L.faces_server_tune_warp.argtypes = [vp, c_int, c_int]
    L.faces_batch_warp_info.argtypes = [vp, ip, ip, ip, ip]
    L.faces_batch_destroy.argtypes = [vp]
    jp, sp = ctypes.POINTER(FacesJob), ctypes.POINTER(ServeStats)
    llp, dblp = ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_double)
    L.faces_server_create.argtypes = [ctypes.POINTER(vp), ctypes.c_size_t, c_int, c_uint]
    L.faces_server_submit.argtypes = [vp, jp, llp]
    L.faces_server_poll.argtypes = [vp, c_int]
    L.faces_server_drain.argtypes = [vp]
    L.faces_server_job_status.argtypes = [vp, ctypes.c_longlong, ip, ip, dblp, dblp]
    L.faces_server_field.argtypes = [vp, ctypes.c_longlong, ctypes.POINTER(vp), ctypes.POINTER(c_long)]
    L.faces_server_fetch.argtypes = [vp, ctypes.c_longlong, dp]
    L.faces_server_release.argtypes = [vp, ctypes.c_longlong]
    L.faces_server_stats.argtypes = [vp, sp]
    L.faces_server_run_trace.argtypes = [vp, c_int, jp, dblp, llp, dblp, dblp]
    L.faces_server_destroy.argtypes = [vp]
    L.faces_server_tune.argtypes = [vp, c_int, c_int, c_int]
    for name in ("faces_server_create", "faces_server_submit", "faces_server_poll", "faces_server_drain",
                 "faces_server_job_status", "faces_server_field", "faces_server_fetch", "faces_server_release",
                 "faces_server_stats", "faces_server_run_trace", "faces_server_destroy", "faces_server_tune",
                 "faces_server_tune_warp"):
        getattr(L, name).restype = c_int
    for name in ("faces_create", "faces_destroy", "faces_layout", "faces_field_alloc", "faces_field_free",
                 "faces_share", "faces_share_n", "faces_init_ref", "faces_init_int", "faces_check",
                 "faces_run_host", "faces_set_tuning", "faces_launches_per_share", "faces_batch_create",
                 "faces_batch_add", "faces_batch_commit", "faces_batch_share", "faces_batch_share_n",
                 "faces_batch_share_each", "faces_batch_tune", "faces_batch_autotune", "faces_batch_info",
                 "faces_batch_tune_warp", "faces_batch_warp_info",
                 "faces_batch_destroy"):
        getattr(L, name).restype = c_int
    _lib = L
    return L


class FacesJob(ctypes.Structure):
    """struct faces_job of include/faces_gb300.h."""
    _fields_ = [("lx", ctypes.c_int), ("ly", ctypes.c_int), ("lz", ctypes.c_int), ("mx", ctypes.c_int),
                ("my", ctypes.c_int), ("mz", ctypes.c_int), ("n", ctypes.c_int), ("flags", ctypes.c_uint),
                ("nshares", ctypes.c_int), ("init", ctypes.c_int), ("seed", ctypes.c_ulonglong),
                ("host_in", ctypes.c_void_p)]


class ServeStats(ctypes.Structure):
    """struct faces_serve_stats of include/faces_gb300.h."""
    _fields_ = [("submitted", ctypes.c_longlong), ("admitted", ctypes.c_longlong),
                ("completed", ctypes.c_longlong), ("ticks", ctypes.c_longlong), ("launches", ctypes.c_longlong),
                ("job_shares", ctypes.c_longlong), ("point_shares", ctypes.c_double),
                ("resident_bytes", ctypes.c_size_t), ("peak_resident_bytes", ctypes.c_size_t),
                ("budget_bytes", ctypes.c_size_t), ("queued", ctypes.c_int), ("running", ctypes.c_int)]


def job(lx: int, ly: int, lz: int, mx: int, my: int, mz: int, n: int, *, nshares: int, periodic: bool = False,
        init: str = "int", seed: int = 0, host_in=None) -> FacesJob:
    """A job for Server: a field of this shape, nshares shares.  init: "ref"
    (gpu/main.cc:10-19), "int" (integer values from seed) or "host" (host_in,
    a float64 numpy array of the field size, read when the job is admitted)."""
    j = FacesJob(lx, ly, lz, mx, my, mz, n, PERIODIC if periodic else 0, nshares,
                 {"ref": 0, "int": 1, "host": 2}[init], seed, None)
    j._keep = None
    if init == "host":
        j.host_in = host_in.ctypes.data
        j._keep = host_in
    return j


def _check(rc: int) -> int:
    if rc < 0:
        raise FacesError(rc, lib().faces_last_error().decode(errors="replace"))
    return rc


def _ptr(u) -> int:
    """Device address of a CUDA tensor (float64, contiguous) or an int."""
    if isinstance(u, int):
        return u
    import torch
    if not isinstance(u, torch.Tensor):
        raise TypeError("field must be a torch CUDA tensor or a device address")
    if not u.is_cuda or u.dtype != torch.float64 or not u.is_contiguous():
        raise ValueError("field must be a contiguous float64 CUDA tensor")
    return u.data_ptr()


def _stream(stream) -> int | None:
    if stream is None:
        try:
            import torch
            if torch.cuda.is_available() and torch.cuda.is_initialized():
                return torch.cuda.current_stream().cuda_stream
        except Exception:
            pass
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


@dataclass(frozen=True)
class CheckResult:
    maxrel: float
    npass: int
    rank_maxrel: list
    where: tuple  # rank, ix, iy, iz, jx, jy, jz of the largest error
    values: tuple  # (u, expected) there

    @property
    def passed(self) -> bool:
        return self.maxrel < 1e-15


class Faces:
    """All lx*ly*lz ranks' Faces objects (gpu/v-26-messages/Faces.cc:10-82).

    periodic -- wrap the rank grid (the reference never wraps, K1)
    messages -- v-26 strategy: 26 messages per rank packed, swapped by buffer
                direction and unpack-added (else one owner per shared point)
    gather   -- force the generic one-thread-per-point kernel
    rows     -- use the register row kernel instead of the shared-memory tiles
    general  -- periodic fields: the general tile step instead of the periodic one
    v6       -- v-6 strategy: six face messages per rank, sweeps z, y, x
                (gpu/v-6-messages-basic/Faces.cc:65-173)
    v6f      -- v-6 in the fused form of gpu/v-6-messages-overlap-fusable/
                Faces.cc: four launches per share, the same results as v6
    seams    -- the seam kernel: one thread per shared point of each
                element's lower seam planes, no shared memory (direct mode)
    pack_fused -- message mode: the pack in the message-mode tile kernel's
                prologue, one cooperative launch per share (by default the
                pack is its own launch)
    """

    def __init__(self, lx: int, ly: int, lz: int, mx: int, my: int, mz: int, n: int, *,
                 periodic: bool = False, messages: bool = False, gather: bool = False, rows: bool = False,
                 general: bool = False, v6: bool = False, v6f: bool = False, seams: bool = False,
                 pack_fused: bool = False):
        flags = ((PERIODIC if periodic else 0) | (MESSAGES if messages else 0) | (GATHER if gather else 0)
                 | (ROWS if rows else 0) | (GENERAL if general else 0) | (V6 if v6 else 0) | (V6F if v6f else 0)
                 | (SEAMS if seams else 0) | (PACK_FUSED if pack_fused else 0))
        h = ctypes.c_void_p()
        _check(lib().faces_create(ctypes.byref(h), lx, ly, lz, mx, my, mz, n, flags))
        self._h = h
        self.shape = (lx, ly, lz, mx, my, mz, n)
        self.periodic, self.messages, self.gather, self.rows = periodic, messages, gather, rows
        self.general, self.v6, self.v6f, self.seams = general, v6, v6f, seams
        self.pack_fused = pack_fused
        s = (ctypes.c_long * 6)()
        rd, tot = ctypes.c_long(), ctypes.c_long()
        _check(lib().faces_layout(h, s, ctypes.byref(rd), ctypes.byref(tot)))
        self.strides = tuple(s)
        self.rank_doubles = rd.value
        self.total_doubles = tot.value
        self.nranks = lx * ly * lz

    # -- lifetime -------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().faces_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- geometry ---------------------------------------------------------
    @property
    def points(self) -> int:
        lx, ly, lz, mx, my, mz, n = self.shape
        return n ** 3 * mx * my * mz * lx * ly * lz

    def index(self, ix, iy, iz, jx, jy, jz, rank: int = 0) -> int:
        """DArray index (gpu/DArray.h:34-38) of a point of one rank."""
        s = self.strides
        return rank * self.rank_doubles + ix + iy * s[1] + iz * s[2] + jx * s[3] + jy * s[4] + jz * s[5]

    def field(self, device=None):
        """A zero-filled CUDA float64 tensor of the field size (DArray alloc)."""
        import torch
        return torch.zeros(self.total_doubles, dtype=torch.float64, device=device or "cuda")

    # -- the step ---------------------------------------------------------
    def share(self, u, compute: bool = True, stream=None) -> None:
        """Faces::share(u, compute) on every rank (stream-ordered)."""
        _check(lib().faces_share(self._h, _ptr(u), int(compute), _stream(stream)))

    def share_n(self, u, nshares: int, compute: bool = True, stream=None) -> None:
        _check(lib().faces_share_n(self._h, _ptr(u), int(compute), nshares, _stream(stream)))

    def init_ref(self, u, stream=None) -> None:
        """gpu/main.cc:10-19 initial values on every rank."""
        _check(lib().faces_init_ref(self._h, _ptr(u), _stream(stream)))

    def init_int(self, u, seed: int, stream=None) -> None:
        """Integer-valued doubles uniform in [0,2^20)."""
        _check(lib().faces_init_int(self._h, _ptr(u), ctypes.c_ulonglong(seed), _stream(stream)))

    def check(self, u, *, init: str = "ref", seed: int = 0, nshares: int = 1, compute: bool = True,
              stream=None) -> CheckResult:
        """gpu/main.cc:39-105 on the device against the closed form of nshares shares."""
        rm = (ctypes.c_double * self.nranks)()
        mx = ctypes.c_double()
        npass = ctypes.c_int()
        where = (ctypes.c_int * 7)()
        vals = (ctypes.c_double * 2)()
        _check(lib().faces_check(self._h, _ptr(u), 0 if init == "ref" else 1, ctypes.c_ulonglong(seed), nshares,
                                 int(compute), rm, ctypes.byref(mx), ctypes.byref(npass), where, vals,
                                 _stream(stream)))
        return CheckResult(mx.value, npass.value, list(rm), tuple(where), tuple(vals))

    def run_host(self, u_in, u_out, nshares: int, compute: bool = True, stream=None) -> None:
        """End to end from host memory: upload, nshares shares, download."""
        import numpy as np
        for a in (u_in, u_out):
            if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous
                    and a.size == self.total_doubles):
                raise ValueError("host buffers must be contiguous float64 arrays of the field size")
        _check(lib().faces_run_host(self._h, u_in.ctypes.data, u_out.ctypes.data, int(compute), nshares,
                                    _stream(stream)))

    def run_host_many(self, u_in: list, u_out: list, nshares: int, compute: bool = True, stream=None) -> None:
        """Independent jobs from host memory: job j uploads u_in[j], runs
        nshares shares and downloads to u_out[j]; uploads and downloads of
        neighbouring jobs overlap the shares (faces_run_host_many)."""
        import numpy as np
        if len(u_in) != len(u_out):
            raise ValueError("one output buffer per input buffer")
        for a in list(u_in) + list(u_out):
            if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous
                    and a.size == self.total_doubles):
                raise ValueError("host buffers must be contiguous float64 arrays of the field size")
        nj = len(u_in)
        ins = (ctypes.c_void_p * max(nj, 1))(*[a.ctypes.data for a in u_in])
        outs = (ctypes.c_void_p * max(nj, 1))(*[a.ctypes.data for a in u_out])
        _check(lib().faces_run_host_many(self._h, nj, ins, outs, int(compute), nshares, _stream(stream)))

    def set_tuning(self, chunk: int = 0, width: int = 0, order: int = -1) -> None:
        """Elements per x-chunk, width (row kernel: tiles per block; tile
        kernel: resident blocks per SM) and tile order (0 strided, 1
        contiguous; seam kernel: 0 chunked, 1 lean); 0 / -1 keep the
        defaults (and the default kernel)."""
        _check(lib().faces_set_tuning(self._h, chunk, width, order))

    def autotune(self, u, compute: bool = True, trials: int = 3, stream=None) -> int:
        """Keeps the fastest tile settings for this field; returns the shares
        its timed launches applied to u (re-initialise u afterwards)."""
        return _check(lib().faces_autotune(self._h, _ptr(u), int(compute), trials, _stream(stream)))

    def tuning(self) -> dict:
        """The step's settings: elements per tile, chunks per unit, blocks, the
        kernel (0 tile step, 1 general tile step, 2 row kernel, 3 seam kernel)
        and the order (seam kernel: 0 chunked, 1 lean)."""
        v = [ctypes.c_int() for _ in range(5)]
        _check(lib().faces_get_tuning(self._h, *[ctypes.byref(x) for x in v]))
        return dict(zip(("chunk", "unit_chunks", "blocks", "kernel", "order"), (x.value for x in v)))

    def launches_per_share(self, compute: bool = True) -> int:
        return _check(lib().faces_launches_per_share(self._h, int(compute)))

    def test_pack_wait(self, extra: int, polls: int = 1 << 22) -> None:
        """Test hook: the fused step's waits expect `extra` (0 or 1) more
        arrivals than exist, so that they run out after `polls` polls."""
        _check(lib().faces_test_pack_wait(self._h, extra, polls))

    def status(self) -> int:
        """Device status bits, read and cleared (synchronous): bit 0 = the
        fused message-mode step's wait for the pack ran out."""
        b = ctypes.c_int()
        _check(lib().faces_status(self._h, ctypes.byref(b)))
        return b.value


class Batch:
    """Many independent fields advanced together (no counterpart in the
    reference, which runs one field per process: gpu/main.cc:169-180).

    add() the fields (each a Faces shape and a device field of that shape),
    commit(), then share() advances every field by one share with one
    persistent launch; share_n() replays n shares as one CUDA graph;
    share_each() is one faces_share per field.  The fields stay owned by
    the caller and must outlive the batch.
    """

    def __init__(self):
        h = ctypes.c_void_p()
        _check(lib().faces_batch_create(ctypes.byref(h)))
        self._h = h
        self._fields = []

    def add(self, faces: Faces, u) -> int:
        lx, ly, lz, mx, my, mz, n = faces.shape
        flags = ((PERIODIC if faces.periodic else 0) | (MESSAGES if faces.messages else 0)
                 | (GATHER if faces.gather else 0) | (ROWS if faces.rows else 0)
                 | (GENERAL if faces.general else 0) | (V6 if faces.v6 else 0) | (V6F if faces.v6f else 0)
                 | (SEAMS if faces.seams else 0) | (PACK_FUSED if faces.pack_fused else 0))
        fid = ctypes.c_int()
        _check(lib().faces_batch_add(self._h, _ptr(u), lx, ly, lz, mx, my, mz, n, flags, ctypes.byref(fid)))
        self._fields.append(u)
        return fid.value

    def commit(self) -> None:
        _check(lib().faces_batch_commit(self._h))

    def share(self, compute: bool = True, stream=None) -> None:
        _check(lib().faces_batch_share(self._h, int(compute), _stream(stream)))

    def share_n(self, nshares: int, compute: bool = True, stream=None) -> None:
        _check(lib().faces_batch_share_n(self._h, int(compute), nshares, _stream(stream)))

    def share_each(self, compute: bool = True, stream=None) -> None:
        _check(lib().faces_batch_share_each(self._h, int(compute), _stream(stream)))

    def tune(self, unit_div: int = 0, blocks_per_sm: int = 0, half: int = -1, run: int = 0) -> None:
        _check(lib().faces_batch_tune(self._h, unit_div, blocks_per_sm, half, run))

    def tune_warp(self, max_n: int = -1, boost: int = 0) -> None:
        """The warp form for small n (faces_batch_tune_warp)."""
        _check(lib().faces_batch_tune_warp(self._h, max_n, boost))

    def autotune(self, trials: int = 3, stream=None) -> int:
        """Keeps the fastest work split; returns the shares it applied to
        each field of the batched launch (each timed launch is a share)."""
        return _check(lib().faces_batch_autotune(self._h, trials, _stream(stream)))

    def info(self) -> dict:
        v = [ctypes.c_int() for _ in range(7)]
        _check(lib().faces_batch_info(self._h, *[ctypes.byref(x) for x in v]))
        out = dict(zip(("fields", "fused_fields", "units", "unit_div", "blocks", "half", "run"),
                       (x.value for x in v)))
        w = [ctypes.c_int() for _ in range(4)]
        _check(lib().faces_batch_warp_info(self._h, *[ctypes.byref(x) for x in w]))
        out.update(zip(("warp_max_n", "warp_boost", "warp_units", "warp_blocks"), (x.value for x in w)))
        return out

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().faces_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


SERVE_PLAIN = 0x1
SERVE_RELEASE_DONE = 0x2
JOB_STATES = ("queued", "running", "done", "released")


class Server:
    """Halo-sum jobs arriving over time on one GPU (no counterpart in the
    reference, which runs one job per process: gpu/main.cc:134-197).

    Jobs are admitted in arrival order against an HBM budget (bytes) and run
    together: every tick is one share of every running job in one persistent
    launch.  plain=True launches the single-field kernel once per job per
    tick instead (the one-field-per-launch form).  release_done frees a
    job's field as soon as it is done (its result can then not be fetched).
    """

    def __init__(self, budget_bytes: int, max_jobs: int = 0, *, plain: bool = False, release_done: bool = False):
        h = ctypes.c_void_p()
        flags = (SERVE_PLAIN if plain else 0) | (SERVE_RELEASE_DONE if release_done else 0)
        _check(lib().faces_server_create(ctypes.byref(h), int(budget_bytes), max_jobs, flags))
        self._h = h
        self._inputs = {}

    def submit(self, j: FacesJob) -> int:
        jid = ctypes.c_longlong()
        _check(lib().faces_server_submit(self._h, ctypes.byref(j), ctypes.byref(jid)))
        if getattr(j, "_keep", None) is not None:
            self._inputs[jid.value] = j._keep  # read at admission
        return jid.value

    def poll(self, wait: bool = False) -> int:
        return _check(lib().faces_server_poll(self._h, int(wait)))

    def drain(self) -> int:
        return _check(lib().faces_server_drain(self._h))

    def status(self, jid: int) -> dict:
        st, sd = ctypes.c_int(), ctypes.c_int()
        w, lat = ctypes.c_double(), ctypes.c_double()
        _check(lib().faces_server_job_status(self._h, jid, ctypes.byref(st), ctypes.byref(sd), ctypes.byref(w),
                                             ctypes.byref(lat)))
        return {"state": JOB_STATES[st.value], "shares_done": sd.value, "wait_s": w.value, "latency_s": lat.value}

    def field_ptr(self, jid: int) -> tuple[int, int]:
        p, tot = ctypes.c_void_p(), ctypes.c_long()
        _check(lib().faces_server_field(self._h, jid, ctypes.byref(p), ctypes.byref(tot)))
        return p.value, tot.value

    def fetch(self, jid: int):
        import numpy as np
        _, tot = self.field_ptr(jid)
        out = np.empty(tot, dtype=np.float64)
        _check(lib().faces_server_fetch(self._h, jid, out.ctypes.data))
        return out

    def release(self, jid: int) -> None:
        _check(lib().faces_server_release(self._h, jid))
        self._inputs.pop(jid, None)

    def tune(self, unit_div: int = 0, run: int = 0, half: int = -1) -> None:
        """Work list settings of the batched launch (faces_server_tune)."""
        _check(lib().faces_server_tune(self._h, unit_div, run, half))

    def tune_warp(self, max_n: int = -1, boost: int = 0) -> None:
        """The warp form for small n (faces_server_tune_warp)."""
        _check(lib().faces_server_tune_warp(self._h, max_n, boost))

    def stats(self) -> dict:
        st = ServeStats()
        _check(lib().faces_server_stats(self._h, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in ServeStats._fields_}

    def run_trace(self, jobs, arrivals):
        """Replays arrivals (seconds, non-decreasing) in real time; returns
        (job ids, latencies in seconds, makespan in seconds)."""
        import numpy as np
        nj = len(jobs)
        arr = (FacesJob * nj)(*jobs)
        t = np.ascontiguousarray(arrivals, dtype=np.float64)
        ids = (ctypes.c_longlong * nj)()
        lat = np.empty(nj, dtype=np.float64)
        mk = ctypes.c_double()
        _check(lib().faces_server_run_trace(self._h, nj, arr, t.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                            ids, lat.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                            ctypes.byref(mk)))
        return list(ids), lat, mk.value

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().faces_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
