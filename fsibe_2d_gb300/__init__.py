"""fsibe_2d_gb300 -- GB300-native (sm_103a) FSIBE_2D fluid step + flexible-beam coupling.

The compute path is the in-tree CUDA library fsibe_2d_gb300/_lib/libfsibe_gb300.so behind the
C ABI of include/fsibe.h.  This module only binds that ABI (ctypes); there is no CPU
fallback: if the library is missing, `Run(...)` raises.
"""
import ctypes as C
import os

import numpy as np

from ._abi import (FsibeParams, FsibeScalars, make_params, BEAM_DATA_COLUMNS, STATUS_NAMES,  # noqa: F401
                   FSIBE_FP64, FSIBE_FP32C, FSIBE_BDF2, FSIBE_CRANK_NICHOLSON, FSIBE_EULER_IMPLICIT)
from ._binding import FsibeError, declare, backup_time, Run as _Run  # noqa: F401

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libfsibe_gb300.so")

_lib = None


class AdjointInfo(C.Structure):
    _fields_ = [("forward_steps", C.c_int32), ("adjoint_steps", C.c_int32), ("snapshots", C.c_int32),
                ("ms_total", C.c_float)]


def library():
    """Load libfsibe_gb300.so (raises if it was not built: there is no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"CUDA library not built: {LIB_PATH} is missing "
                               "(run __graft_entry__.build() or python -m fsibe_2d_gb300.build)")
        L = C.CDLL(LIB_PATH)
        declare(L, "fsibe_")
        L.fsibe_set_stream.argtypes = [C.c_void_p, C.c_void_p]
        L.fsibe_strerror.argtypes = [C.c_int]
        L.fsibe_strerror.restype = C.c_char_p
        L.fsibe_time_steps.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_float)]
        L.fsibe_launches_per_step.argtypes = [C.c_void_p, C.POINTER(C.c_int)]
        L.fsibe_use_graph.argtypes = [C.c_void_p, C.c_int]
        L.fsibe_tiles.argtypes = [C.c_void_p, C.POINTER(C.c_int32)]
        L.fsibe_tile_config.argtypes = [C.c_void_p, C.POINTER(C.c_int32)]
        L.fsibe_beam_cluster.argtypes = [C.c_void_p, C.POINTER(C.c_int32)]
        L.fsibe_press_y_engine.argtypes = [C.c_void_p, C.POINTER(C.c_int32)]
        L.fsibe_ensemble_create.argtypes = [C.POINTER(FsibeParams), C.c_int, C.POINTER(C.c_void_p)]
        L.fsibe_ensemble_destroy.argtypes = [C.c_void_p]
        L.fsibe_ensemble_get.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_void_p)]
        L.fsibe_ensemble_step.argtypes = [C.c_void_p, C.c_int]
        L.fsibe_ensemble_time_steps.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_float)]
        L.fsibe_ensemble_last_error.argtypes = [C.c_void_p]
        L.fsibe_ensemble_last_error.restype = C.c_char_p
        _dp = C.POINTER(C.c_double)
        L.fsibe_drag_objective.argtypes = [C.c_void_p, _dp, C.c_double, C.c_int, C.c_int, _dp]
        L.fsibe_drag_gradient.argtypes = [C.c_void_p, _dp, C.c_double, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp,
                                          C.POINTER(AdjointInfo)]
        L.fsibe_force_objective.argtypes = [C.c_void_p, C.c_int, _dp, C.c_double, C.c_int, C.c_int, _dp]
        L.fsibe_force_gradient.argtypes = [C.c_void_p, C.c_int, _dp, C.c_double, C.c_int, C.c_int, C.c_int, _dp, _dp,
                                           _dp, _dp, C.POINTER(AdjointInfo)]
        L.fsibe_beam_phase_cycles.argtypes = [C.c_void_p, C.POINTER(C.c_longlong), C.c_int]
        L.fsibe_running_sums.argtypes = [_dp, C.c_int32, _dp, C.POINTER(C.c_int32)]
        _lib = L
    return _lib


def running_sums(terms):
    """The beam kernels' running sums of integrate_position on the GPU: terms (4, n) float64;
    returns (sums (4, n) with sums[q, k] = s_k of row q, rows that failed the step check)."""
    t = np.ascontiguousarray(terms, dtype=np.float64)
    if t.ndim != 2 or t.shape[0] != 4:
        raise ValueError("terms must have shape (4, n)")
    out = np.empty_like(t)
    ns = C.c_int32(0)
    L = library()
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    st = L.fsibe_running_sums(dp(t), C.c_int32(t.shape[1]), dp(out), C.byref(ns))
    if st != 0:
        raise RuntimeError(f"fsibe_running_sums: status {st}: {L.fsibe_last_error(None).decode()}")
    return out, ns.value


class Run(_Run):
    """One GPU simulation context: device-resident fields, reference-named entry points."""

    def __init__(self, params: FsibeParams):
        super().__init__(library(), "fsibe_", params)

    def set_stream(self, stream_handle):
        """Run this context's kernels on a cudaStream_t (an int handle, e.g. torch's)."""
        self._call("set_stream", C.c_void_p(stream_handle))

    def time_steps(self, nsteps):
        """Device milliseconds (CUDA events on the context's stream) for nsteps steps."""
        ms = C.c_float()
        self._call("time_steps", C.c_int(nsteps), C.byref(ms), soft=(10,))
        return ms.value

    def launches_per_step(self):
        n = C.c_int()
        self._call("launches_per_step", C.byref(n))
        return n.value

    def use_graph(self, enable=True):
        self._call("use_graph", C.c_int(1 if enable else 0))

    def tiles(self):
        """Rows per block the autotuner chose for (nl_x, press_x, press_fin)."""
        out = (C.c_int32 * 3)()
        self._call("tiles", out)
        return tuple(out)

    def tile_config(self):
        """(rows, blocks-per-SM bound) of the fused x kernels nl_x, press_x, press_fin as the
        autotuner chose them (bound 0: the kernel's default; 16: the paired FP32 press_x)."""
        out = (C.c_int32 * 6)()
        self._call("tile_config", out)
        return [(out[2 * q], out[2 * q + 1]) for q in range(3)]

    def press_y_engine(self):
        """k_press_y's transform engine: 0 paired (FP32), 1 one butterfly a thread."""
        out = C.c_int32(0)
        self._call("press_y_engine", C.byref(out))
        return out.value

    def beam_phase_cycles(self, reset=False):
        """The beam kernels' 32 phase counters (fsibe_beam_phase_cycles)."""
        out = (C.c_longlong * 32)()
        self._call("beam_phase_cycles", out, C.c_int(1 if reset else 0))
        return list(out)

    def beam_cluster(self):
        """CTAs of the cluster running the beam's Newton step (0: the single-CTA kernel)."""
        out = C.c_int32(0)
        self._call("beam_cluster", C.byref(out))
        return out.value

    # -- adjoint on a prescribed rigid mask (FP64 form, iFLUSI = 0) -----------------------
    def force_objective(self, component, vort0, nsteps, avg_from, nu=0.0):
        """Mean of Force(component + 1) -- 0 drag, 1 lift -- after steps avg_from..nsteps from the
        physical vorticity vort0 (ny, nx)."""
        v = np.ascontiguousarray(vort0, dtype=np.float64)
        J = C.c_double()
        self._call("force_objective", C.c_int(component), v.ctypes.data_as(C.POINTER(C.c_double)), C.c_double(nu),
                   C.c_int(nsteps), C.c_int(avg_from), C.byref(J))
        return J.value

    def force_gradient(self, component, vort0, nsteps, avg_from, nu=0.0, snapshots=40):
        """(J, dJ/dvort0, dJ/dmask, dJ/dnu, info) of force_objective by the discrete adjoint with
        checkpointing."""
        v = np.ascontiguousarray(vort0, dtype=np.float64)
        gv = np.empty((self.ny, self.nx))
        gm = np.empty((self.ny, self.nx))
        J, gnu, info = C.c_double(), C.c_double(), AdjointInfo()
        dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        self._call("force_gradient", C.c_int(component), dp(v), C.c_double(nu), C.c_int(nsteps), C.c_int(avg_from),
                   C.c_int(snapshots), C.byref(J), dp(gv), dp(gm), C.byref(gnu), C.byref(info))
        return J.value, gv, gm, gnu.value, info

    def lift_objective(self, vort0, nsteps, avg_from, nu=0.0):
        return self.force_objective(1, vort0, nsteps, avg_from, nu)

    def lift_gradient(self, vort0, nsteps, avg_from, nu=0.0, snapshots=40):
        return self.force_gradient(1, vort0, nsteps, avg_from, nu, snapshots)

    def drag_objective(self, vort0, nsteps, avg_from, nu=0.0):
        """Mean drag after steps avg_from..nsteps from the physical vorticity vort0 (ny, nx)."""
        v = np.ascontiguousarray(vort0, dtype=np.float64)
        J = C.c_double()
        self._call("drag_objective", v.ctypes.data_as(C.POINTER(C.c_double)), C.c_double(nu), C.c_int(nsteps),
                   C.c_int(avg_from), C.byref(J))
        return J.value

    def drag_gradient(self, vort0, nsteps, avg_from, nu=0.0, snapshots=40):
        """(J, dJ/dvort0, dJ/dmask, dJ/dnu, info) by the discrete adjoint with checkpointing."""
        v = np.ascontiguousarray(vort0, dtype=np.float64)
        gv = np.empty((self.ny, self.nx))
        gm = np.empty((self.ny, self.nx))
        J, gnu, info = C.c_double(), C.c_double(), AdjointInfo()
        dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        self._call("drag_gradient", dp(v), C.c_double(nu), C.c_int(nsteps), C.c_int(avg_from), C.c_int(snapshots),
                   C.byref(J), dp(gv), dp(gm), C.byref(gnu), C.byref(info))
        return J.value, gv, gm, gnu.value, info


class _EnsembleRun(Run):
    """One run of an Ensemble: the ensemble owns its context."""

    def __init__(self, ctx, params):
        self._lib = library()
        self._prefix = "fsibe_"
        self.params = params
        self.nx, self.ny, self.ns = params.nx, params.ny, params.ns
        self._ctx = ctx

    def close(self):
        self._ctx = C.c_void_p()


class Ensemble:
    """Independent runs of any sizes advanced together (fsibe_ensemble_*): after the start-up
    step, one CUDA graph launch per step carries every run's step on its own stream."""

    def __init__(self, params_list):
        L = library()
        arr = (FsibeParams * len(params_list))(*params_list)
        self._e = C.c_void_p()
        st = L.fsibe_ensemble_create(arr, len(params_list), C.byref(self._e))
        if st:
            raise FsibeError(st, "fsibe_ensemble_create", self._err())
        self.runs = []
        for i, p in enumerate(params_list):
            ctx = C.c_void_p()
            L.fsibe_ensemble_get(self._e, i, C.byref(ctx))
            self.runs.append(_EnsembleRun(ctx, p))

    def _err(self):
        m = library().fsibe_ensemble_last_error(self._e if getattr(self, "_e", None) else None)
        return m.decode() if m else ""

    def step(self, nsteps=1):
        st = library().fsibe_ensemble_step(self._e, nsteps)
        if st:
            raise FsibeError(st, "fsibe_ensemble_step", self._err())

    def time_steps(self, nsteps):
        """Device milliseconds for nsteps steps of the whole ensemble."""
        ms = C.c_float()
        st = library().fsibe_ensemble_time_steps(self._e, nsteps, C.byref(ms))
        if st:
            raise FsibeError(st, "fsibe_ensemble_time_steps", self._err())
        return ms.value

    def close(self):
        if getattr(self, "_e", None):
            for r in self.runs:
                r.close()
            library().fsibe_ensemble_destroy(self._e)
            self._e = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # pragma: no cover
            pass
