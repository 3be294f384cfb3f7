"""ctypes binding of the CPU oracle (oracle/fsibe_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg, never by the product package.  The oracle exports the same entry points as
include/fsibe.h with the prefix orc_ and the same argument meaning.
"""
import ctypes as C
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
if REPO not in sys.path:
    sys.path.insert(0, REPO)

from fsibe_2d_gb300._abi import FsibeParams  # noqa: E402
from fsibe_2d_gb300._binding import Run, declare  # noqa: E402

LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
SRC = os.path.join(HERE, "fsibe_oracle.cpp")


def build(force=False):
    """Compile the oracle with g++ (-O3, OpenMP, no FMA contraction, portable flags)."""
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= os.path.getmtime(SRC):
        return LIB_PATH
    cmd = ["g++", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c++17", "-ffp-contract=off",
           "-o", LIB_PATH, SRC]
    subprocess.check_call(cmd)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        declare(L, "orc_")
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_set_threads.restype = C.c_int
        L.orc_delta_phi4star.argtypes = [C.c_double]
        L.orc_delta_phi4star.restype = C.c_double
        dp = C.POINTER(C.c_double)
        L.orc_differentiate1d.argtypes = [dp, dp, C.c_int, C.c_double, C.c_int]
        L.orc_gttrf_solve.argtypes = [C.c_int, dp, dp, dp, dp]
        L.orc_getrf_solve.argtypes = [C.c_int, dp, dp]
        L.orc_newton_system.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_int] + [dp] * 10
        L.orc_time.argtypes = [C.c_void_p]
        L.orc_time.restype = C.c_double
        _lib = L
    return _lib


class OracleRun(Run):
    """The oracle's context with the same methods as fsibe_2d_gb300.Run."""

    def __init__(self, params: FsibeParams):
        super().__init__(lib(), "orc_", params)


def set_threads(n):
    return lib().orc_set_threads(int(n))
