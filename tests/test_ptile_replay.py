"""CPU replay of the periodic tile step (tests/native/ptile_emu.cu): the
step's own pstage / pxpass / pyzpass, run thread by thread on the host for
every tile, with the stage at the kernel's exact size between guard cells,
under a model where tiles read the share's starting field and the threads
of a phase read the cells as they were before it.  The result must equal
the oracle bit for bit, for block (256) and warp (32) teams and for the
tile lengths both kernels use: the single-field powers of 2 and the
batched kernel's stage-filling lengths."""
import ctypes
import os
import shutil
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "native"))
import build_emu  # noqa: E402

if not (shutil.which("nvcc") or os.path.exists("/usr/local/cuda/bin/nvcc")):
    pytest.skip("nvcc is needed to build the replay", allow_module_level=True)

_emu = None


def emu():
    global _emu
    if _emu is None:
        L = ctypes.CDLL(build_emu.build_ptile())
        L.ptile_emulate.argtypes = [ctypes.c_int] * 9 + [ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                                                         ctypes.c_char_p, ctypes.c_int]
        L.ptile_emulate.restype = ctypes.c_int
        _emu = L
    return _emu


def row_stride(n):
    """smem_row_stride: the smallest even stride >= n that is 2 mod 4"""
    e = (n + 1) // 2 * 2
    return e if e % 4 == 2 else e + 2


def tile_kmax(n):
    v = 20480 // (n * n * row_stride(n) * 8)
    return next((k for k in (32, 16, 8, 4, 2) if v >= k), 1)


def batch_tile(n, stage=2688):
    """the batched kernel's periodic-step tile length at the default stage
    (sized by n = 8's 4-element tile: 2688 doubles)"""
    return min(32, (stage - 2 * n * n) // (n * n * row_stride(n)))


def batch_warp_tile(n, stage=2688):
    """the batched kernel's warp form: one eighth of three default stages"""
    w = (3 * stage // 8) & ~1
    return min(32, (w - 2 * n * n) // (n * n * row_stride(n)))


def form_default_k(n, form):
    """the default tile length of the periodic ("p") and message-mode ("x")
    steps on a large field: the longest power of 2 (up to max(tile_kmax, 8))
    whose three stages and tile records stay within 110 KB (PMeta 80 B +
    int4 per stage; XMeta 240 B per record, one more record than stages)"""
    rec = 3 * 96 if form == "p" else 4 * 240
    k = 1
    while k * 2 <= max(tile_kmax(n), 8) and 8 * 3 * (2 * k * n * n * row_stride(n) + 2 * n * n) + rec <= 110 * 1024:
        k *= 2
    return k


def test_form_default_lengths():
    assert [form_default_k(n, "p") for n in range(3, 13)] == [32, 16, 16, 8, 8, 4, 4, 4, 2, 2]
    assert [form_default_k(n, "x") for n in range(3, 13)] == [32, 16, 16, 8, 8, 4, 4, 4, 2, 2]


def tile_kwarp(n):
    """the warp form's tile length (about 6 KB of stage)"""
    v = 6144 // (n * n * row_stride(n) * 8)
    return next((k for k in (32, 16, 8, 4, 2) if v >= k), 1)


def cases():
    out = []
    for n in range(2, 13):
        ks = sorted({1, 2, tile_kmax(n), form_default_k(n, "p")} | ({batch_tile(n)} if n <= 10 else set()))
        for K in ks:
            out.append((n, K, 256))
        for K in sorted({tile_kmax(n), tile_kwarp(n)} | ({batch_warp_tile(n)} if n <= 5 else set())):
            out.append((n, K, 32))
    return out


@pytest.mark.parametrize("n,K,T", cases(), ids=lambda v: str(v))
@pytest.mark.parametrize("grid", [(1, 1, 1), (2, 1, 2)], ids=["1rank", "2x1x2"])
def test_ptile_replay_matches_oracle(oracle, n, K, T, grid):
    O = oracle
    mx = min(K, 32) + 3 if K > 2 else 5
    s = O.Shape(*grid, mx, 3, 2, n, periodic=True)
    rng = np.random.default_rng(n * 100 + K)
    u0 = O.init_int(s, 3)
    m = u0 != 0
    u0[m] = rng.standard_normal(m.sum())
    u = u0.copy()
    err = ctypes.create_string_buffer(256)
    rc = emu().ptile_emulate(*grid, mx, 3, 2, n, K, T, u.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 2, err,
                             256)
    assert rc == 0, err.value.decode()
    exp = O.groups_share(s, u0.copy(), True, 2)
    assert np.array_equal(u, exp), f"{np.count_nonzero(u != exp)} points differ"


def test_batch_warp_tile_lengths():
    """the warp form's lengths replayed above (n = 2: 32, 3: 18, 4: 10, 5: 6)"""
    assert [batch_warp_tile(n) for n in range(2, 6)] == [32, 18, 10, 6]


def test_batch_tile_lengths():
    """the lengths replayed above are the batched kernel's (n = 4: 27, 5: 17,
    6: 12, 7: 5, 8: 4, 9: 3, 10: 2)"""
    assert [batch_tile(n) for n in range(4, 11)] == [27, 17, 12, 5, 4, 3, 2]


_xemu = None


def xemu():
    global _xemu
    if _xemu is None:
        L = ctypes.CDLL(build_emu.build_ptile())
        L.xtile_emulate.argtypes = [ctypes.c_int] * 11 + [ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                                                          ctypes.c_char_p, ctypes.c_int]
        L.xtile_emulate.restype = ctypes.c_int
        _xemu = L
    return _xemu


def xcases():
    out = []
    for n in range(2, 13):
        for K in sorted({1, 2, tile_kmax(n), form_default_k(n, "x")}):
            out.append((n, K, 256))
        out.append((n, tile_kmax(n), 32))
    return out


XGRIDS = [
    # (grid, periodic, messages)
    ((1, 1, 1), True, True),
    ((2, 1, 2), True, True),
    ((2, 2, 1), False, True),
    ((1, 1, 1), False, True),
    ((1, 1, 1), False, False),
]


@pytest.mark.parametrize("n,K,T", xcases(), ids=lambda v: str(v))
@pytest.mark.parametrize("grid,periodic,messages", XGRIDS,
                         ids=["1rank-p-msg", "2x1x2-p-msg", "2x2x1-open-msg", "1rank-open-msg", "1rank-open-direct"])
def test_xtile_replay_matches_oracle(oracle, n, K, T, grid, periodic, messages):
    """The message-mode step (and the open one-rank direct step), replayed
    thread by thread, equals the oracle on random normal inputs, 2 shares;
    the chunk leaves a partial last tile where it can."""
    O = oracle
    mx = K + 2 if K > 1 else 3
    s = O.Shape(*grid, mx, 3, 2, n, periodic=periodic)
    rng = np.random.default_rng(n * 1000 + K * 10 + T)
    u0 = O.init_int(s, 3)
    m = u0 != 0
    u0[m] = rng.standard_normal(m.sum())
    u = u0.copy()
    err = ctypes.create_string_buffer(256)
    rc = xemu().xtile_emulate(*grid, mx, 3, 2, n, K, T, int(periodic), int(messages),
                              u.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 2, err, 256)
    assert rc == 0, err.value.decode()
    exp = O.groups_share(s, u0.copy(), True, 2)
    assert np.array_equal(u, exp), f"{np.count_nonzero(u != exp)} points differ"


_v6emu = None


def v6emu():
    global _v6emu
    if _v6emu is None:
        L = ctypes.CDLL(build_emu.build_ptile())
        L.v6_emulate.argtypes = [ctypes.c_int] * 10 + [ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                                                       ctypes.c_char_p, ctypes.c_int]
        L.v6_emulate.restype = ctypes.c_int
        _v6emu = L
    return _v6emu


V6CASES = [
    # lx ly lz mx my mz n periodic
    (1, 1, 1, 3, 2, 4, 5, True),
    (2, 1, 2, 2, 3, 2, 4, True),
    (2, 2, 1, 3, 1, 2, 6, False),
    (1, 1, 1, 2, 2, 2, 2, False),
    (3, 1, 1, 1, 2, 3, 3, True),
    (1, 2, 2, 2, 2, 1, 8, False),
    (2, 2, 2, 1, 1, 1, 7, True),
]


@pytest.mark.parametrize("case", V6CASES, ids=lambda c: "x".join(map(str, c[:7])) + ("p" if c[7] else "o"))
@pytest.mark.parametrize("fused", [False, True], ids=["basic", "fused"])
@pytest.mark.parametrize("compute", [True, False])
def test_v6_replay_matches_oracle(oracle, case, fused, compute):
    """v-6 in both forms, every launch's threads in order and in reverse,
    NaN-filled messages: equals the oracle's v-6 restatement bit for bit."""
    O = oracle
    *shape, periodic = case
    s = O.Shape(*shape, periodic=periodic)
    rng = np.random.default_rng(sum(shape))
    u0 = O.init_int(s, 3)
    m = u0 != 0
    u0[m] = rng.standard_normal(m.sum())
    u = u0.copy()
    err = ctypes.create_string_buffer(256)
    rc = v6emu().v6_emulate(*shape, int(periodic), int(fused), int(compute),
                            u.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 2, err, 256)
    assert rc == 0, err.value.decode()
    exp = O.v6_share(s, u0.copy(), compute, 2)
    assert np.array_equal(u, exp), f"{np.count_nonzero(u != exp)} points differ"


_semu = None


def semu():
    global _semu
    if _semu is None:
        L = ctypes.CDLL(build_emu.build_ptile())
        L.seam_emulate.argtypes = [ctypes.c_int] * 10 + [ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                                                         ctypes.c_char_p, ctypes.c_int]
        L.seam_emulate.restype = ctypes.c_int
        _semu = L
    return _semu


def seam_default_chunk(n):
    """the seam kernel's default chunk: about eight slots per thread of a
    256-thread block"""
    return max(1, 8 * 256 // (n - 1) ** 2)


SEAMGRIDS = [
    # lx ly lz mx my mz periodic
    (1, 1, 1, 4, 3, 2, True),
    (1, 1, 1, 4, 3, 2, False),
    (2, 1, 2, 3, 2, 2, True),
    (2, 2, 1, 3, 2, 1, False),
    (3, 2, 2, 2, 1, 2, False),
    (2, 2, 2, 1, 1, 1, True),
]


@pytest.mark.parametrize("n", list(range(2, 13)) + [16])
@pytest.mark.parametrize("grid", SEAMGRIDS, ids=lambda g: "x".join(map(str, g[:6])) + ("p" if g[6] else "o"))
@pytest.mark.parametrize("E", [1, 3, 0], ids=["E1", "E3", "Ewhole"])
@pytest.mark.parametrize("mode", [0, 1, 2, 3], ids=["fwd", "rev", "lean", "lean-rev"])
def test_seam_replay_matches_oracle(oracle, n, grid, E, mode):
    """The seam step in both forms (chunked; lean, with the boundary planes'
    launch), every thread run one by one, in order or in reverse: no point is
    touched by two threads of a share, no address leaves the field, and 2
    shares equal the oracle bit for bit (random normal inputs)."""
    O = oracle
    *shape, periodic = grid
    s = O.Shape(*shape, n, periodic=periodic)
    rng = np.random.default_rng(n * 100 + sum(shape))
    u0 = O.init_int(s, 3)
    m = u0 != 0
    u0[m] = rng.standard_normal(m.sum())
    u = u0.copy()
    err = ctypes.create_string_buffer(256)
    rc = semu().seam_emulate(*shape, n, int(periodic), E, mode,
                             u.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 2, err, 256)
    assert rc == 0, err.value.decode()
    exp = O.groups_share(s, u0.copy(), True, 2)
    assert np.array_equal(u, exp), f"{np.count_nonzero(u != exp)} points differ"


def test_seam_default_chunk():
    assert [seam_default_chunk(n) for n in (2, 4, 8, 12, 16)] == [2048, 227, 41, 16, 9]
