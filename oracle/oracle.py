"""ctypes bindings for the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module; the product path (faces_gb300) never does.

Arrays are numpy float64 vectors in the padded DArray layout of
gpu/DArray.h:91-101, all virtual ranks rank-major (see faces_oracle.h).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libmugs_ref.so")
# The reference's sources, for compiling its own Mugs as the oracle's checker:
# FACES_REFERENCE_DIR, else the unmodified copy `make -C baseline stage` puts
# in baseline/_ref/src (git-ignored); absent, the checker is not built.
REFERENCE_DIR = os.environ.get("FACES_REFERENCE_DIR") or os.path.join(os.path.dirname(HERE), "baseline", "_ref", "src")


class Geom(ctypes.Structure):
    _fields_ = [(k, ctypes.c_int) for k in ("lx", "ly", "lz", "mx", "my", "mz", "n", "periodic")]


@dataclass(frozen=True)
class Shape:
    lx: int = 1
    ly: int = 1
    lz: int = 1
    mx: int = 1
    my: int = 1
    mz: int = 1
    n: int = 2
    periodic: bool = False

    def geom(self) -> Geom:
        return Geom(self.lx, self.ly, self.lz, self.mx, self.my, self.mz, self.n, int(self.periodic))

    @property
    def nranks(self) -> int:
        return self.lx * self.ly * self.lz

    @property
    def jz_stride(self) -> int:
        plane = self.n ** 3 * self.mx * self.my
        return ((plane - 1) // 512 + 1) * 512

    @property
    def rank_doubles(self) -> int:
        return self.jz_stride * self.mz

    @property
    def total_doubles(self) -> int:
        return self.rank_doubles * self.nranks

    @property
    def points(self) -> int:
        return self.n ** 3 * self.mx * self.my * self.mz * self.nranks

    def view6(self, u: np.ndarray, rank: int = 0) -> np.ndarray:
        """(jz, jy, jx, iz, iy, ix) view of one rank's elements (no padding)."""
        n = self.n
        r = u[rank * self.rank_doubles:(rank + 1) * self.rank_doubles].reshape(self.mz, self.jz_stride)
        return r[:, : n ** 3 * self.mx * self.my].reshape(self.mz, self.my, self.mx, n, n, n)


def build(quiet: bool = True) -> None:
    """Build liboracle.so (always) and the reference Mugs (when its sources exist)."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-C", HERE, "-s"], check=True, stdout=out)
    if os.path.isfile(os.path.join(REFERENCE_DIR, "gpu", "Mugs.cc")):
        subprocess.run(["make", "-C", HERE, "-s", "ref", f"REFERENCE_DIR={REFERENCE_DIR}"],
                       check=True, stdout=out)


_lib = None
_ref = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.isfile(LIB):
            build()
        L = ctypes.CDLL(LIB)
        dp = ctypes.POINTER(ctypes.c_double)
        gp = ctypes.POINTER(Geom)
        L.orc_init_ref.argtypes = [gp, dp]
        L.orc_init_int.argtypes = [gp, dp, ctypes.c_uint64]
        L.orc_int_value.argtypes = [ctypes.c_uint64, ctypes.c_long]
        L.orc_int_value.restype = ctypes.c_double
        L.orc_groups_share.argtypes = [gp, dp, ctypes.c_int, ctypes.c_int]
        L.orc_mugs_share.argtypes = [gp, dp, ctypes.c_int, ctypes.c_int]
        L.orc_v26_share.argtypes = [gp, dp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.orc_v6_share.argtypes = [gp, dp, ctypes.c_int, ctypes.c_int]
        L.orc_compare.argtypes = [gp, dp, dp, ctypes.POINTER(ctypes.c_int),
                                  ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
        L.orc_compare.restype = ctypes.c_double
        L.orc_max_threads.restype = ctypes.c_int
        L.orc_check.argtypes = [gp]
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.isfile(REF_LIB)


def ref_lib() -> ctypes.CDLL:
    global _ref
    if _ref is None:
        R = ctypes.CDLL(REF_LIB)
        R.mugs_ref_share.argtypes = [ctypes.c_int] * 9 + [ctypes.POINTER(ctypes.c_double), ctypes.c_int]
        R.mugs_ref_share.restype = ctypes.c_int
        _ref = R
    return _ref


def _dp(u: np.ndarray):
    assert u.dtype == np.float64 and u.flags.c_contiguous
    return u.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def alloc(s: Shape) -> np.ndarray:
    return np.zeros(s.total_doubles, dtype=np.float64)


def init_ref(s: Shape) -> np.ndarray:
    u = alloc(s)
    lib().orc_init_ref(ctypes.byref(s.geom()), _dp(u))
    return u


def init_int(s: Shape, seed: int) -> np.ndarray:
    u = alloc(s)
    lib().orc_init_int(ctypes.byref(s.geom()), _dp(u), ctypes.c_uint64(seed))
    return u


def groups_share(s: Shape, u: np.ndarray, compute: bool = True, nsteps: int = 1) -> np.ndarray:
    lib().orc_groups_share(ctypes.byref(s.geom()), _dp(u), int(compute), nsteps)
    return u


def mugs_share(s: Shape, u: np.ndarray, compute: bool = True, nsteps: int = 1) -> np.ndarray:
    lib().orc_mugs_share(ctypes.byref(s.geom()), _dp(u), int(compute), nsteps)
    return u


def v6_share(s: Shape, u: np.ndarray, compute: bool = True, nsteps: int = 1) -> np.ndarray:
    """v-6 (gpu/v-6-messages-basic/Faces.cc:65-173): z, y, x sweeps."""
    lib().orc_v6_share(ctypes.byref(s.geom()), _dp(u), int(compute), nsteps)
    return u


def v26_share(s: Shape, u: np.ndarray, compute: bool = True, nsteps: int = 1, nthreads: int = 0) -> np.ndarray:
    lib().orc_v26_share(ctypes.byref(s.geom()), _dp(u), int(compute), nsteps, nthreads)
    return u


def ref_mugs_share(s: Shape, u: np.ndarray, compute: bool = True, nsteps: int = 1, nthreads: int = 1) -> np.ndarray:
    """The reference's own gpu/Mugs.cc (non-periodic only)."""
    assert not s.periodic, "the reference's Mugs has no periodic neighbours"
    rc = ref_lib().mugs_ref_share(s.lx, s.ly, s.lz, s.mx, s.my, s.mz, s.n, int(compute), nsteps, _dp(u), nthreads)
    assert rc == 0
    return u


def compare(s: Shape, a: np.ndarray, b: np.ndarray):
    """gpu/main.cc:39-105: (max relative error, ranks passing < 1e-15, (rank, where))."""
    npass = ctypes.c_int(0)
    wr = ctypes.c_int(0)
    where = (ctypes.c_int * 6)()
    mv = lib().orc_compare(ctypes.byref(s.geom()), _dp(a), _dp(b), ctypes.byref(npass), ctypes.byref(wr), where)
    return mv, npass.value, (wr.value, tuple(where))


def max_threads() -> int:
    return lib().orc_max_threads()
