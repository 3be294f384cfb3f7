"""Channel walls, the leading-edge cylinder and the sponges on the GPU against the oracle.

The reference's optional solid features (create_mask.f90:21-210 walls and cylinder, 223-470
the sponges; NavierStokes.f90:142-164 the vorticity-sponge term, :103-122 the sharp outflow
sponge's integral) at 128^2 with a flexible beam:
the mask and its velocity field after the start-up, then 40 steps of the coupled run.  The FP64
form must match the oracle within 1e-10 (relative L2) in the mask, the vorticity, the beam's
deflection and the drag/lift series; the FP32-compensated form within 1e-5."""
import numpy as np
import pytest

from conftest import rel, seeded_vorticity
from fsibe_2d_gb300 import make_params, FSIBE_FP32C

pytestmark = pytest.mark.gpu

N, NS, STEPS = 128, 32, 40

CASES = {
    "walls": dict(iWalls=1, h_channel=0.3),
    "cylinder": dict(iCylinder=1, R_cylinder=0.1),
    "walls+cylinder": dict(iWalls=1, h_channel=0.3, iCylinder=1, R_cylinder=0.1),
    "sponge1": dict(iSponge=1, SpongeSize=0.5, eps_sponge=1e-2),
    "sponge2": dict(iSponge=2, SpongeSize=0.5, eps_sponge=1e-2),
    "sponge3": dict(iSponge=3, SpongeSize=0.3, eps_sponge=1e-2),
    "sponge22": dict(iSponge=22, SpongeSize=0.3, eps_sponge=1e-2),
    "walls+sponge4": dict(iWalls=1, h_channel=0.3, iSponge=4, SpongeSize=0.5),
    "sponge10": dict(iSponge=10, SpongeSize=1.0, eps_sponge=0.1),   # columns 96..112 of 128
    # a fixed beam in an accelerating flow: the mask is redrawn until T_fullspeed, then kept
    "sponge4-accelerating": dict(iWalls=1, h_channel=0.3, iSponge=4, SpongeSize=0.5, iFLUSI=0,
                                 iMeanVelocity=1, T_fullspeed=0.02),
    "sponge22-accelerating": dict(iSponge=22, SpongeSize=0.3, eps_sponge=1e-2, iFLUSI=0,
                                  iMeanVelocity=2, T_fullspeed=0.02),
}


def _run_pair(oracle, precision, kw):
    import fsibe_2d_gb300 as F
    p = make_params(nx=N, ny=N, ns=NS, dt=1e-3, precision=precision, **kw)
    g, o = F.Run(p), oracle.OracleRun(make_params(nx=N, ny=N, ns=NS, dt=1e-3, **kw))
    w = seeded_vorticity(N, seed=7)
    g.init_fields(w); o.init_fields(w)
    return g, o


@pytest.mark.parametrize("name", list(CASES))
def test_features_fp64_match_the_oracle(oracle, name):
    g, o = _run_pair(oracle, 0, CASES[name])
    mg, mo = g.mask(), o.mask()
    for a, b in zip(mg, mo):                              # mask, us(:,:,1), us(:,:,2)
        assert np.abs(a - b).max() <= 1e-10 * max(1.0, np.abs(b).max()), name
    rg, ro = g.time_step(STEPS), o.time_step(STEPS)
    assert g.scalars().status == 0 and o.scalars().status == 0
    err = {"vorticity": rel(g.vort(), o.vort()), "deflection": rel(g.beam()[0][1], o.beam()[0][1]),
           "drag": rel(rg[:, 10], ro[:, 10]), "lift": rel(rg[:, 11], ro[:, 11])}
    print(name, "FP64 against the oracle after", STEPS, "steps:", err)
    assert max(err.values()) < 1e-10, (name, err)
    g.close(); o.close()


@pytest.mark.parametrize("name", ["walls+cylinder", "sponge22", "walls+sponge4", "sponge1", "sponge10"])
def test_features_fp32c_match_the_oracle(oracle, name):
    g, o = _run_pair(oracle, FSIBE_FP32C, CASES[name])
    rg, ro = g.time_step(STEPS), o.time_step(STEPS)
    assert g.scalars().status == 0
    err = {"vorticity": rel(g.vort(), o.vort()), "deflection": rel(g.beam()[0][1], o.beam()[0][1]),
           "drag": rel(rg[:, 10], ro[:, 10])}
    print(name, "FP32C against the oracle after", STEPS, "steps:", err)
    assert max(err.values()) < 1e-5, (name, err)
    g.close(); o.close()


def test_feature_parameters_are_checked():
    import fsibe_2d_gb300 as F
    from fsibe_2d_gb300._binding import FsibeError
    from fsibe_2d_gb300._abi import FSIBE_ERR_PARAM, FSIBE_ERR_UNSUPPORTED
    for kw, code in ((dict(iSponge=5, SpongeSize=0.5), FSIBE_ERR_PARAM),
                     (dict(iSponge=1, SpongeSize=0.0), FSIBE_ERR_PARAM),
                     (dict(iSponge=10, SpongeSize=4.0), FSIBE_ERR_PARAM),           # not inside the box
                     (dict(iSponge=1, iBeam=0, SpongeSize=0.5), FSIBE_ERR_UNSUPPORTED),
                     (dict(iWalls=2), FSIBE_ERR_PARAM)):
        with pytest.raises(FsibeError) as ex:
            F.Run(make_params(nx=64, ny=64, ns=16, **kw))
        assert ex.value.status == code, (kw, ex.value.status)


def test_surface_integral_with_walls_and_cylinder(oracle):
    """BeamForces.f90:331-336, 494-502: no surface integral with the leading-edge cylinder; with
    walls the file's penalization drag and lift columns are zero, the contour columns remain."""
    import ctypes as C
    from fsibe_2d_gb300._abi import FSIBE_ERR_UNSUPPORTED
    from fsibe_2d_gb300._binding import _ptr
    g, o = _run_pair(oracle, 0, CASES["walls"])
    g.time_step(5); o.time_step(5)
    t = g.scalars().time
    sg, so = g.BeamSurfaceIntegral(t), o.BeamSurfaceIntegral(t)
    assert sg[1] == 0.0 and sg[2] == 0.0 and so[1] == 0.0 and so[2] == 0.0
    scale = np.abs(so[3:]).max()
    assert np.abs(np.asarray(sg[3:]) - np.asarray(so[3:])).max() <= 1e-10 * scale
    g.close(); o.close()
    g, o = _run_pair(oracle, 0, CASES["cylinder"])
    out = np.zeros(11)
    for r in (g, o):
        assert getattr(r._lib, r._prefix + "surface_integral")(r._ctx, C.c_double(0.0), _ptr(out)) == FSIBE_ERR_UNSUPPORTED
    g.close(); o.close()
