"""ctypes mirror of include/fsibe.h: the parameter and scalar structs and the status codes.

The struct layouts must match the C header field for field; tests/test_abi.py checks the
sizes against the values the C library reports.
"""
import ctypes as C

FSIBE_OK = 0
FSIBE_ERR_PARAM = 1
FSIBE_ERR_CUDA = 2
FSIBE_ERR_NAN = 3
FSIBE_ERR_NEWTON_MAXIT = 4
FSIBE_ERR_SINGULAR = 5
FSIBE_ERR_INTERP_OOB = 6
FSIBE_ERR_TIMEOUT = 7
FSIBE_ERR_UNSUPPORTED = 8
FSIBE_ERR_MASK_OOB = 9
FSIBE_ERR_BRAKE = 10
FSIBE_ERR_STATE = 11

# values per step of fsibe_run_records (include/fsibe.h)
FSIBE_RECORD_COLS = 46

STATUS_NAMES = {
    0: "FSIBE_OK", 1: "FSIBE_ERR_PARAM", 2: "FSIBE_ERR_CUDA", 3: "FSIBE_ERR_NAN",
    4: "FSIBE_ERR_NEWTON_MAXIT", 5: "FSIBE_ERR_SINGULAR", 6: "FSIBE_ERR_INTERP_OOB",
    7: "FSIBE_ERR_TIMEOUT", 8: "FSIBE_ERR_UNSUPPORTED", 9: "FSIBE_ERR_MASK_OOB",
    10: "FSIBE_ERR_BRAKE", 11: "FSIBE_ERR_STATE",
}

FSIBE_FP64 = 0
FSIBE_FP32C = 1

FSIBE_EULER_IMPLICIT = 1
FSIBE_CRANK_NICHOLSON = 2
FSIBE_BDF2 = 5


class FsibeParams(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("ns", C.c_int32), ("precision", C.c_int32),
        ("xl", C.c_double), ("yl", C.c_double), ("nu", C.c_double), ("eps", C.c_double),
        ("cfl", C.c_double), ("dt_fixed", C.c_double), ("time_end", C.c_double),
        ("eta", C.c_double), ("mue", C.c_double), ("t_release", C.c_double), ("tau", C.c_double),
        ("angle_beam", C.c_double), ("grav", C.c_double), ("sigma", C.c_double),
        ("iImpulse", C.c_int32), ("time_method_solid", C.c_int32),
        ("iFLUSI", C.c_int32), ("iMotion", C.c_int32), ("iViscous", C.c_int32), ("iSaveBeam", C.c_int32),
        ("iBeam", C.c_int32), ("iSharpTrailing", C.c_int32), ("iMeanVelocity", C.c_int32), ("idealis", C.c_int32),
        ("T_fullspeed", C.c_double), ("theta_inf", C.c_double),
        ("x0", C.c_double), ("y0", C.c_double), ("length", C.c_double),
        ("t_beam", C.c_double), ("N_smooth", C.c_double),
        ("newton_tol", C.c_double), ("newton_maxit", C.c_int32), ("reserved", C.c_int32),
        ("iWalls", C.c_int32), ("iCylinder", C.c_int32), ("iSponge", C.c_int32), ("reserved2", C.c_int32),
        ("h_channel", C.c_double), ("R_cylinder", C.c_double), ("SpongeSize", C.c_double), ("eps_sponge", C.c_double),
    ]


class FsibeScalars(C.Structure):
    _fields_ = [
        ("time", C.c_double), ("dt0", C.c_double), ("dt1", C.c_double),
        ("u_max", C.c_double), ("mean_ux", C.c_double), ("mean_uy", C.c_double),
        ("vor_rms", C.c_double), ("kinetic", C.c_double), ("dissipation", C.c_double),
        ("porous_diss", C.c_double), ("inflow_solid", C.c_double), ("inflow_mean", C.c_double),
        ("force", C.c_double * 2), ("force_unst", C.c_double * 2), ("force_press", C.c_double * 2),
        ("inertial_force", C.c_double * 2),
        ("e_kinetic", C.c_double), ("e_elastic", C.c_double), ("e_pot", C.c_double),
        ("beam_data", C.c_double * 21),
        ("newton_iters", C.c_int32), ("status", C.c_int32), ("step", C.c_int32), ("reserved", C.c_int32),
    ]

    def as_dict(self):
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            if hasattr(v, "__len__"):
                v = list(v)
            out[name] = v
        return out


#: Columns of one beam_data row (BeamIO.f90:193-216).
BEAM_DATA_COLUMNS = (
    "time", "p_new[ns-1]", "p_new[3ns/4]", "p_new[ns/2]", "x[ns-1]", "y[ns-1]", "vx[ns-1]", "vy[ns-1]",
    "theta[ns-1]", "theta_dot[ns-1]", "drag", "lift", "drag_unst", "lift_unst", "force_press_x",
    "force_press_y", "inertial_x", "inertial_y", "E_kinetic", "E_elastic", "E_pot",
)


def make_params(nx=256, ny=256, ns=64, xl=4.0, yl=4.0, Re=100.0, eps=1.0e-3, dt=2.0e-4, cfl=0.1,
                time_end=1.0e9, EI=0.1, mu=1.0, x0=1.0, y0=2.0, length=1.0, thickness_cells=4.0,
                N_smooth=2.0, newton_tol=1.0e-10, newton_maxit=50, precision=FSIBE_FP64,
                angle_beam=0.0, iFLUSI=1, iViscous=1, iSaveBeam=3, iSharpTrailing=0,
                time_method_solid=FSIBE_BDF2, theta_inf=0.0, iMeanVelocity=3, idealis=1,
                t_release=0.0, tau=0.0, grav=0.0, sigma=0.0, iImpulse=0, iMotion=0, iBeam=1,
                iWalls=0, h_channel=0.0, iCylinder=0, R_cylinder=0.0, iSponge=0, SpongeSize=0.0, eps_sponge=1.0,
                T_fullspeed=0.0):
    """Parameters in the reference's units (params.f90): nu = 1/Re, t_beam is the HALF
    thickness = thickness_cells/2 * dx, eps is the penalization parameter, eta = EI,
    mue = density ratio."""
    p = FsibeParams()
    p.nx, p.ny, p.ns, p.precision = nx, ny, ns, precision
    p.xl, p.yl = xl, yl
    p.nu = 1.0 / Re
    p.eps = eps
    p.cfl, p.dt_fixed, p.time_end = cfl, dt, time_end
    p.eta, p.mue = EI, mu
    p.t_release, p.tau, p.angle_beam, p.grav, p.sigma = t_release, tau, angle_beam, grav, sigma
    p.iImpulse, p.time_method_solid = iImpulse, time_method_solid
    p.iFLUSI, p.iMotion, p.iViscous, p.iSaveBeam = iFLUSI, iMotion, iViscous, iSaveBeam
    p.iBeam, p.iSharpTrailing, p.iMeanVelocity, p.idealis = iBeam, iSharpTrailing, iMeanVelocity, idealis
    p.T_fullspeed, p.theta_inf = T_fullspeed, theta_inf
    p.x0, p.y0, p.length = x0, y0, length
    p.t_beam = 0.5 * thickness_cells * xl / nx
    p.N_smooth = N_smooth
    p.newton_tol, p.newton_maxit = newton_tol, newton_maxit
    p.iWalls, p.iCylinder, p.iSponge = iWalls, iCylinder, iSponge
    p.h_channel, p.R_cylinder, p.SpongeSize, p.eps_sponge = h_channel, R_cylinder, SpongeSize, eps_sponge
    return p
