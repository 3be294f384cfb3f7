"""The oracle's prescribed leading-edge motions (mouvement.f90:5-200) through the per-step
records' mouvement row (BeamIO.f90:229-238): the closed forms of each case at the times of
a run, and a fixed beam (iFLUSI = 0) that follows its leading edge (time_step.f90:211-216)."""
import math

import numpy as np
import pytest

from conftest import seeded_vorticity
from fsibe_2d_gb300 import make_params

PI = 4.0 * math.atan(1.0)


def _expected(m, t, x0, y0, angle):
    a0 = angle * PI / 180.0
    if m == 3:
        w = 2.0 * PI * 0.5
        am = 80.0 * PI / 180.0
        return [am * math.sin(w * t), am * math.cos(w * t) * w, -am * math.sin(w * t) * w * w, x0, y0, 0, 0, 0, 0]
    if m == 4:
        return [a0, 0, 0, x0 - t, y0, -1.0, 0, 0, 0]
    if m == 2 or 401 <= m <= 413:
        ym, tm = (0.5, 2.5) if m == 2 else (0.0333, [0.51, 0.34, 0.25, 0.20, 0.17, 0.14, 0.13, 0.11, 0.10, 0.09,
                                                      0.08, 0.08, 0.07][m - 401])
        w, arg = 2 * PI / tm, 2 * PI * t / tm + PI / 2
        return [a0, 0, 0, x0, y0 + ym * math.sin(arg), 0, ym * w * math.cos(arg), 0, -ym * w * w * math.sin(arg)]
    tm = [1.0, 1.09, 1.20, 1.29, 1.33, 1.4, 1.5, 1.71, 2.0, 2.4, 3.0, 4.0, 1.62][m - 201] if m < 300 else 1.62
    k = -20 * t**7 + 70 * t**6 - 84 * t**5 + 35 * t**4 if t <= 1 else 1.0
    kt = -140 * t**6 + 420 * t**5 - 420 * t**4 + 140 * t**3 if t <= 1 else 0.0
    ktt = -840 * t**5 + 2100 * t**4 - 1680 * t**3 + 420 * t**2 if t <= 1 else 0.0
    w, arg = 2 * PI / tm, 2 * PI * t / tm + PI / 2
    y, yt, ytt = 0.5 * math.sin(arg), 0.5 * w * math.cos(arg), -0.5 * w * w * math.sin(arg)
    return [a0, 0, 0, x0, y0 + k * y, 0, kt * y + yt * k, 0, ktt * y + ytt * k + 2 * kt * yt]


@pytest.mark.parametrize("m", [2, 3, 4, 201, 213, 305, 401, 413])
def test_mouvement_rows_follow_the_closed_forms(oracle, m):
    p = make_params(nx=64, ny=64, ns=16, iMotion=m, iFLUSI=0, dt=2e-3, eps=1e-2, angle_beam=5.0)
    o = oracle.OracleRun(p)
    o.init_fields(seeded_vorticity(64))
    rec = o.run_records(30)
    for r in rec:
        t = r[36]
        exp = _expected(m, t, p.x0, p.y0, p.angle_beam)
        got = [r[37], r[38], r[39], r[40], r[41], r[42], r[43], r[44], r[45]]
        assert np.allclose(got, exp, rtol=1e-12, atol=1e-12), (m, t, got, exp)
    assert np.isfinite(rec).all() and o.scalars().status == 0
    o.close()


def test_fixed_beam_follows_its_leading_edge(oracle):
    """iFLUSI = 0: integrate_position(time) after each step's forces: the beam is straight at
    the angle alpha(t) from the leading edge of the time before the step."""
    p = make_params(nx=64, ny=64, ns=16, iMotion=3, iFLUSI=0, dt=2e-3, eps=1e-2)
    o = oracle.OracleRun(p)
    o.init_fields(seeded_vorticity(64))
    rec = o.run_records(10)
    t_before = rec[-1, 21]
    alpha = 80.0 * PI / 180.0 * math.sin(PI * t_before)
    b = o.beam()[0]
    s = np.arange(p.ns) * (p.length / (p.ns - 1))
    assert np.allclose(b[0], p.x0 + s * math.cos(alpha), atol=1e-13)
    assert np.allclose(b[1], p.y0 + s * math.sin(alpha), atol=1e-13)
    o.close()


def test_paraz_cases_set_the_soft_startup(oracle):
    """mouvement.f90:102-104: tau = one period for the cases 401-413."""
    p = make_params(nx=64, ny=64, ns=16, iMotion=402, iFLUSI=1)
    o = oracle.OracleRun(p)
    o.init_fields(seeded_vorticity(64))
    o.time_step(3)
    assert o.scalars().status == 0
    o.close()
