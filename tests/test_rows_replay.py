"""CPU replay of the row kernel's own addressing code (rows_setup.cuh).

tests/native/rows_emu.cc runs the kernel's tile/slot setup for every tile and
slot, emulates one share in lockstep, checks every pointer against the field
and message buffers and that no point is written twice, and the result must
equal the oracle bit for bit.  This is the write-set disjointness check and
the bounds check of every launch shape, done before any GPU run.
"""
import ctypes
import itertools
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "native"))
import build_emu  # noqa: E402

_emu = None


def emu():
    global _emu
    if _emu is None:
        L = ctypes.CDLL(build_emu.build())
        L.rows_emulate.argtypes = [ctypes.c_int] * 11 + [ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                                                          ctypes.c_char_p, ctypes.c_int]
        L.rows_emulate.restype = ctypes.c_int
        L.tiles_emulate.argtypes = [ctypes.c_int] * 10 + [ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                                                           ctypes.c_char_p, ctypes.c_int,
                                                           ctypes.POINTER(ctypes.c_long)]
        L.tiles_emulate.restype = ctypes.c_int
        _emu = L
    return _emu


def replay(s, u, *, messages, chunk=0, tpb=0, nsteps=1):
    err = ctypes.create_string_buffer(256)
    rc = emu().rows_emulate(s.lx, s.ly, s.lz, s.mx, s.my, s.mz, s.n, int(s.periodic), int(messages), chunk, tpb,
                            u.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), nsteps, err, 256)
    assert rc == 0, err.value.decode()
    return u


SHAPES = [
    (1, 1, 1, 4, 4, 4, 5), (1, 1, 1, 3, 2, 5, 8), (1, 1, 1, 1, 1, 1, 3), (1, 1, 1, 2, 3, 1, 2),
    (2, 1, 1, 3, 2, 2, 4), (1, 2, 2, 2, 3, 2, 6), (3, 3, 3, 2, 2, 2, 6), (2, 2, 2, 1, 1, 1, 7),
    (1, 1, 1, 5, 2, 3, 10), (2, 1, 2, 2, 2, 1, 12), (1, 1, 1, 2, 2, 2, 16), (1, 3, 1, 3, 1, 2, 9),
    (2, 2, 1, 1, 2, 1, 2), (1, 1, 2, 1, 1, 3, 2),
]


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(map(str, s)))
@pytest.mark.parametrize("periodic", [False, True], ids=["open", "periodic"])
@pytest.mark.parametrize("messages", [False, True], ids=["direct", "messages"])
def test_replay_matches_oracle(oracle, shape, periodic, messages):
    O = oracle
    s = O.Shape(*shape, periodic=periodic)
    rng = np.random.default_rng(1)
    for init in ("int", "rand"):
        u0 = O.init_int(s, 9)
        if init == "rand":
            m = u0 != 0
            u0[m] = rng.standard_normal(m.sum())
        got = replay(s, u0.copy(), messages=messages, nsteps=2)
        exp = O.groups_share(s, u0.copy(), True, 2)
        assert np.array_equal(got, exp), f"{init}: {np.count_nonzero(got != exp)} points differ"


@pytest.mark.parametrize("chunk,tpb", [(1, 1), (2, 3), (3, 2), (4, 0)])
def test_replay_chunks(oracle, chunk, tpb):
    O = oracle
    for periodic, messages in itertools.product([False, True], [False, True]):
        s = O.Shape(2, 1, 2, 7, 2, 3, 5, periodic=periodic)
        u0 = O.init_ref(s)
        got = replay(s, u0.copy(), messages=messages, chunk=chunk, tpb=tpb, nsteps=2)
        assert np.array_equal(got, O.groups_share(s, u0.copy(), True, 2))


def replay_tiles(s, u, *, messages, K, nsteps=1, counts=None):
    err = ctypes.create_string_buffer(256)
    reg = (ctypes.c_long * 2)()
    rc = emu().tiles_emulate(s.lx, s.ly, s.lz, s.mx, s.my, s.mz, s.n, int(s.periodic), int(messages), K,
                             u.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), nsteps, err, 256, reg)
    assert rc == 0, err.value.decode()
    if counts is not None:
        counts[:] = [reg[0], reg[1]]
    return u


@pytest.mark.parametrize("shape", [sh for sh in SHAPES if sh[6] <= 12], ids=lambda s: "x".join(map(str, s)))
@pytest.mark.parametrize("periodic", [False, True], ids=["open", "periodic"])
@pytest.mark.parametrize("messages", [False, True], ids=["direct", "messages"])
@pytest.mark.parametrize("K", [1, 2, 4, 8])
def test_tile_replay_matches_oracle(oracle, shape, periodic, messages, K):
    """the shared-memory tile kernel's copy-in / groups / copy-out code"""
    O = oracle
    s = O.Shape(*shape, periodic=periodic)
    rng = np.random.default_rng(2)
    u0 = O.init_int(s, 4)
    m = u0 != 0
    u0[m] = rng.standard_normal(m.sum())
    got = replay_tiles(s, u0.copy(), messages=messages, K=K, nsteps=2)
    exp = O.groups_share(s, u0.copy(), True, 2)
    assert np.array_equal(got, exp), f"{np.count_nonzero(got != exp)} points differ"


def test_periodic_tiles_are_regular(oracle):
    """every tile of a periodic field takes the dense passes; non-periodic
    fields exercise both paths"""
    O = oracle
    s = O.Shape(1, 1, 1, 4, 3, 2, 6, periodic=True)
    counts = [0, 0]
    replay_tiles(s, O.init_int(s, 1), messages=False, K=2, counts=counts)
    assert counts[0] == counts[1] > 0
    s = O.Shape(2, 1, 1, 4, 3, 2, 6, periodic=False)
    replay_tiles(s, O.init_int(s, 1), messages=False, K=2, counts=counts)
    assert 0 < counts[0] < counts[1]
