"""Host-side mirror of the reference's entry points over a C ABI context.

`Run` wraps one fsibe_ctx (one simulation).  Its methods carry the reference's routine
names and argument meaning (tommy-engels/FSIBE_2D, file:line in each docstring) so that
code written against the Fortran routines reads the same here.  Arrays are numpy float64
in the reference layout: physical fields (ny, nx) C-order == Fortran (0:nx-1,0:ny-1);
spectral fields in the packed Temperton layout of coftxy.

Errors follow the reference's "stop" semantics by raising FsibeError with the status code.
"""
import ctypes as C
import os
import struct

import numpy as np

from ._abi import FsibeParams, FsibeScalars, STATUS_NAMES, FSIBE_ERR_BRAKE, FSIBE_RECORD_COLS

_dp = C.POINTER(C.c_double)


class FsibeError(RuntimeError):
    def __init__(self, status, where, msg=""):
        self.status = status
        name = STATUS_NAMES.get(status, str(status))
        super().__init__(f"{where}: {name} ({status}) {msg}".rstrip())


def _ptr(a):
    return a.ctypes.data_as(_dp)


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None and a.shape != shape:
        a = a.reshape(shape)
    return a


def declare(lib, prefix, ctx_type=C.c_void_p):
    """Set argtypes/restype of every entry point of include/fsibe.h on lib (with prefix)."""
    def f(name, *args, res=C.c_int):
        fn = getattr(lib, prefix + name)
        fn.argtypes = list(args)
        fn.restype = res
        return fn
    P = ctx_type
    f("create", C.POINTER(FsibeParams), C.POINTER(C.c_void_p))
    f("destroy", P)
    for name in ("fft_forward", "fft_inverse", "cofdx", "cofdy", "cofdxdx", "cofdydy", "cofdxdy", "poisson"):
        f(name, P, _dp, _dp)
    f("vis", P, C.c_double, _dp)
    f("dealiase_mask", P, _dp)
    f("init_fields", P, _dp)
    f("create_mask", P, C.c_double)
    f("fluid_step", P, C.c_int)
    f("get_forces", P, C.c_double)
    f("solid_step", P, C.c_double)
    f("advance", P)
    f("step", P)
    f("run", P, C.c_int, _dp)
    f("run_records", P, C.c_int, _dp)
    f("upload_vortk", P, _dp)
    f("download_vortk", P, _dp)
    f("download_vort", P, _dp)
    f("upload_u", P, _dp)
    f("download_u", P, _dp)
    f("download_press", P, _dp)
    f("upload_press", P, _dp)
    f("download_vor_mean", P, _dp)
    f("upload_mask", P, _dp, _dp, _dp)
    f("download_mask", P, _dp, _dp, _dp)
    f("upload_beam", P, _dp, _dp, _dp, _dp, _dp)
    f("download_beam", P, _dp, _dp, _dp, _dp, _dp)
    f("get_scalars", P, C.POINTER(FsibeScalars))
    f("write_backup", P, C.c_char_p)
    f("surface_integral", P, C.c_double, _dp)
    f("pressure_snapshot", P, C.c_double, _dp)
    f("read_backup", P, C.c_char_p)
    f("last_error", P, res=C.c_char_p)


def backup_time(path):
    """The time in the first record of a runtime backup (a Fortran sequential record of one
    8-byte real), or None when the file is missing or its first record is not that."""
    try:
        with open(path, "rb") as f:
            head = f.read(16)
    except OSError:
        return None
    if len(head) < 16:
        return None
    n, t, m = struct.unpack("<id", head[:12]) + struct.unpack("<i", head[12:16])
    return t if n == 8 and m == 8 else None


class Run:
    """One simulation context (fsibe_create .. fsibe_destroy)."""

    def __init__(self, lib, prefix, params: FsibeParams):
        self._lib = lib
        self._prefix = prefix
        self.params = params
        self.nx, self.ny, self.ns = params.nx, params.ny, params.ns
        self._ctx = C.c_void_p()
        st = getattr(lib, prefix + "create")(C.byref(params), C.byref(self._ctx))
        if st:
            raise FsibeError(st, prefix + "create", self._err())

    # -- plumbing ---------------------------------------------------------------------
    def _err(self):
        try:
            m = getattr(self._lib, self._prefix + "last_error")(self._ctx)
            return m.decode() if m else ""
        except Exception:  # pragma: no cover
            return ""

    def _call(self, name, *args, soft=()):
        st = getattr(self._lib, self._prefix + name)(self._ctx, *args)
        if st and st not in soft:
            raise FsibeError(st, self._prefix + name, self._err())
        return st

    def close(self):
        if self._ctx:
            getattr(self._lib, self._prefix + "destroy")(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:  # pragma: no cover
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def shape(self):
        return (self.ny, self.nx)

    # -- spectral operators (packed layout) ----------------------------------------
    def _unary(self, name, a):
        a = _f64(a, self.shape)
        out = np.empty(self.shape)
        self._call(name, _ptr(a), _ptr(out))
        return out

    def coftxy(self, f):
        """Forward 2D real DFT, 1/(nx*ny), packed (cof_fftw33.f90:142-193)."""
        return self._unary("fft_forward", f)

    def cofitxy(self, fk):
        """Inverse of the packed layout, unnormalized c2r (cof_fftw33.f90:197-243)."""
        return self._unary("fft_inverse", fk)

    def cofdx(self, fk):
        """d/dx in the packed layout (cofdx.f90:1-29)."""
        return self._unary("cofdx", fk)

    def cofdy(self, fk):
        """d/dy in the packed layout (cofdy.f90:1-30)."""
        return self._unary("cofdy", fk)

    def cofdxdx(self, fk):
        return self._unary("cofdxdx", fk)

    def cofdydy(self, fk):
        return self._unary("cofdydy", fk)

    def cofdxdy(self, fk):
        """cofdxdy.f90:1-32 (returns minus the mixed derivative, as the reference does)."""
        return self._unary("cofdxdy", fk)

    def poisson(self, f):
        """ans = f / |k|^2, k=0 block zero (poisson.f90:1-30)."""
        return self._unary("poisson", f)

    def vis(self, dt):
        """workvis = exp(-nu dt |k|^2) in the packed layout (cal_vis.f90:1-36)."""
        out = np.empty(self.shape)
        self._call("vis", C.c_double(dt), _ptr(out))
        return out

    cal_vis = vis

    def dealiase_mask(self):
        out = np.empty(self.shape)
        self._call("dealiase_mask", _ptr(out))
        return out

    # -- time step -------------------------------------------------------------------
    def init_fields(self, vort):
        """inicond=111: vortk = coftxy(vort), u = cal_velocity(0) (init_fields.f90:110-130),
        plus init_beams / InitializeSolidSolver / the start-up create_mask (time_step.f90:60-84)."""
        v = _f64(vort, self.shape)
        self._call("init_fields", _ptr(v))

    def BeamSurfaceIntegral(self, time):
        """BeamForces.f90:306-509: returns the 11 columns of the 'surface' file (time, drag,
        lift, drag_surf, lift_surf, Ft(1), Fn(1), Fp(1), Ft(2), Fn(2), Fp(2))."""
        out = np.zeros(11)
        self._call("surface_integral", C.c_double(time), _ptr(out))
        return out

    def ComputePressureSnapshot(self, time):
        """NavierStokes.f90:598-665: the static pressure of the current vorticity with the
        velocity at `time` and the current mask, (ny, nx); the state is not changed."""
        out = np.empty(self.shape)
        self._call("pressure_snapshot", C.c_double(time), _ptr(out))
        return out

    pressure_snapshot = ComputePressureSnapshot

    def MakeRuntimeBackup(self, path):
        """Write the state between two steps as runtime_backup<n>.in (save_fields.f90:109-152):
        Fortran sequential unformatted records, reals 8 bytes, integers 4."""
        self._call("write_backup", os.fsencode(os.fspath(path)))

    def resume(self, path):
        """init_fields with inicond=2 (init_fields.f90:44-100) plus init_beams /
        InitializeSolidSolver / the start-up create_mask (time_step.f90:60-84); the next step
        is an AB2 step with a Crank-Nicolson solid step."""
        self._call("read_backup", os.fsencode(os.fspath(path)))

    def make_runtime_backup(self, directory, nbackup):
        """MakeRuntimeBackup's file naming (save_fields.f90:122-147): write
        <directory>/runtime_backup<nbackup>.in and return the next nbackup (1 - nbackup),
        so that successive backups alternate between two files."""
        if nbackup not in (0, 1):
            raise ValueError("nbackup is 0 or 1")
        self.MakeRuntimeBackup(os.path.join(os.fspath(directory), "runtime_backup%d.in" % nbackup))
        return 1 - nbackup

    def resume_latest(self, directory):
        """inicond = 2 (init_fields.f90:44-92): of runtime_backup0.in and runtime_backup1.in,
        resume from the one whose first record holds the later time (a time above zero);
        missing files are skipped.  Raises FileNotFoundError when neither holds one
        ("Unable to resume").  Returns the path used."""
        best, tbest = None, 0.0
        for i in (0, 1):
            path = os.path.join(os.fspath(directory), "runtime_backup%d.in" % i)
            t = backup_time(path)
            if t is not None and t > tbest:
                best, tbest = path, t
        if best is None:
            raise FileNotFoundError("unable to resume: no runtime backup with a time above zero in %s" % directory)
        self.resume(best)
        return best

    def create_mask(self, time):
        self._call("create_mask", C.c_double(time))

    def EvolveFluidExplicit(self):
        self._call("fluid_step", 1)

    def EvolveFluidAB2(self):
        self._call("fluid_step", 0)

    def GetForces(self, time):
        self._call("get_forces", C.c_double(time))

    def SolidSolverWrapper(self, time):
        """GravityImpulse + SolidSolverWrapper with dt = the current dt1."""
        return self._call("solid_step", C.c_double(time), soft=(FSIBE_ERR_BRAKE,))

    def advance(self):
        self._call("advance")

    def step(self):
        return self._call("step", soft=(FSIBE_ERR_BRAKE,))

    def time_step(self, nsteps):
        """nsteps iterations of time_step.f90's loop body; returns the beam_data rows."""
        rows = np.zeros((nsteps, 21))
        self._call("run", C.c_int(nsteps), _ptr(rows), soft=(FSIBE_ERR_BRAKE,))
        return rows

    def run_records(self, nsteps):
        """nsteps iterations of the time loop with its per-step output (time_step.f90:178-236):
        an (nsteps, FSIBE_RECORD_COLS) array of the beam_data, u_max, energies and IBES_iter
        rows; fsibe_2d_gb300.outputs.write_step_files writes them in the reference's files."""
        rec = np.zeros((nsteps, FSIBE_RECORD_COLS))
        self._call("run_records", C.c_int(nsteps), _ptr(rec), soft=(FSIBE_ERR_BRAKE,))
        return rec

    # -- state -----------------------------------------------------------------------
    def vortk(self):
        out = np.empty(self.shape)
        self._call("download_vortk", _ptr(out))
        return out

    def set_vortk(self, vk):
        v = _f64(vk, self.shape)
        self._call("upload_vortk", _ptr(v))

    def vort(self):
        out = np.empty(self.shape)
        self._call("download_vort", _ptr(out))
        return out

    def u(self):
        out = np.empty((2,) + self.shape)
        self._call("download_u", _ptr(out))
        return out

    def set_u(self, u):
        v = _f64(u, (2,) + self.shape)
        self._call("upload_u", _ptr(v))

    def press(self):
        out = np.empty(self.shape)
        self._call("download_press", _ptr(out))
        return out

    def set_press(self, p):
        v = _f64(p, self.shape)
        self._call("upload_press", _ptr(v))

    def vor_mean(self):
        out = np.empty(self.shape)
        self._call("download_vor_mean", _ptr(out))
        return out

    def mask(self):
        m, vx, vy = (np.empty(self.shape) for _ in range(3))
        self._call("download_mask", _ptr(m), _ptr(vx), _ptr(vy))
        return m, vx, vy

    def set_mask(self, m, vx, vy):
        m, vx, vy = (_f64(a, self.shape) for a in (m, vx, vy))
        self._call("upload_mask", _ptr(m), _ptr(vx), _ptr(vy))

    def beam(self):
        """(beam (6, ns) rows x,y,vx,vy,theta,theta_dot; p_old; p_new; tau_old; tau_new)"""
        ns = self.ns
        b = np.empty((6, ns))
        po, pn, to, tn = (np.empty(ns) for _ in range(4))
        self._call("download_beam", _ptr(b), _ptr(po), _ptr(pn), _ptr(to), _ptr(tn))
        return b, po, pn, to, tn

    def set_beam(self, beam, p_old, p_new, tau_old, tau_new):
        ns = self.ns
        arrs = [_f64(beam, (6, ns))] + [_f64(a, (ns,)) for a in (p_old, p_new, tau_old, tau_new)]
        self._call("upload_beam", *[_ptr(a) for a in arrs])

    def scalars(self):
        s = FsibeScalars()
        self._call("get_scalars", C.byref(s))
        return s
