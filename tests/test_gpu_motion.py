"""Prescribed leading-edge motions on the GPU against the oracle.

mouvement.f90:5-200 moves the leading edge (heaving 2, 201-213, 300-350, 401-413; impulsive
translation 4) or turns it (flapping 3).  The motion enters the mask, the drag window, the
forces, the beam solver's boundary terms and inertial terms, and integrate_position
(SolidSolver.f90:151-191, 565-660, 943-1045; integrate_position.f90; NavierStokes.f90:532-542).
With iFLUSI = 0 the beam only follows its leading edge (time_step.f90:211-216).  128^2, 40
steps: FP64 within 1e-10 of the oracle (relative L2) in vorticity, beam positions, drag, lift
and the records' mouvement rows; FP32-compensated within 1e-5."""
import numpy as np
import pytest

from conftest import rel, seeded_vorticity
from fsibe_2d_gb300 import make_params, FSIBE_FP32C

pytestmark = pytest.mark.gpu

N, NS, STEPS = 128, 32, 40


def _pair(oracle, precision, **kw):
    import fsibe_2d_gb300 as F
    base = dict(nx=N, ny=N, ns=NS, dt=2e-3, eps=1e-2, angle_beam=5.0)
    base.update(kw)
    g, o = F.Run(make_params(precision=precision, **base)), oracle.OracleRun(make_params(**base))
    w = seeded_vorticity(N, seed=5)
    g.init_fields(w); o.init_fields(w)
    return g, o


@pytest.mark.parametrize("flusi", [1, 0])
@pytest.mark.parametrize("m", [2, 3, 4, 201, 305, 401])
def test_motion_fp64_matches_the_oracle(oracle, m, flusi):
    g, o = _pair(oracle, 0, iMotion=m, iFLUSI=flusi)
    rg, ro = g.run_records(STEPS), o.run_records(STEPS)
    assert g.scalars().status == 0 and o.scalars().status == 0
    bg, bo = g.beam()[0], o.beam()[0]
    err = {"vorticity": rel(g.vort(), o.vort()), "x": rel(bg[0], bo[0]), "y": rel(bg[1], bo[1]),
           "vy": rel(bg[3], bo[3]) if np.abs(bo[3]).max() > 0 else np.abs(bg[3]).max(),
           "drag": rel(rg[:, 10], ro[:, 10]), "lift": rel(rg[:, 11], ro[:, 11]),
           "mouvement": float(np.abs(rg[:, 36:46] - ro[:, 36:46]).max() / max(1.0, np.abs(ro[:, 36:46]).max()))}
    print(f"iMotion={m} iFLUSI={flusi} FP64 against the oracle after {STEPS} steps:", err)
    assert max(err.values()) < 1e-10, (m, flusi, err)
    g.close(); o.close()


@pytest.mark.parametrize("m", [3, 201])
def test_motion_fp32c_matches_the_oracle(oracle, m):
    g, o = _pair(oracle, FSIBE_FP32C, iMotion=m, iFLUSI=1)
    rg, ro = g.time_step(STEPS), o.time_step(STEPS)
    assert g.scalars().status == 0
    err = {"vorticity": rel(g.vort(), o.vort()), "y": rel(g.beam()[0][1], o.beam()[0][1]),
           "drag": rel(rg[:, 10], ro[:, 10])}
    print(f"iMotion={m} FP32C against the oracle after {STEPS} steps:", err)
    assert max(err.values()) < 1e-5, (m, err)
    g.close(); o.close()


def test_motion_cases_are_checked():
    import fsibe_2d_gb300 as F
    from fsibe_2d_gb300._binding import FsibeError
    from fsibe_2d_gb300._abi import FSIBE_ERR_PARAM
    for m in (1, 5, 200, 214, 400, 414, 451):
        with pytest.raises(FsibeError) as ex:
            F.Run(make_params(nx=64, ny=64, ns=16, iMotion=m))
        assert ex.value.status == FSIBE_ERR_PARAM, (m, ex.value.status)
