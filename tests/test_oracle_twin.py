"""The C++ oracle's fluid step against an independent numpy restatement (oracle/py_twin.py,
numpy.fft instead of the oracle's FFT) on a fixed beam mask: vorticity, velocity, pressure
and drag/lift after a start-up and two AB2 steps agree to 1e-12."""
import numpy as np

from conftest import rel, seeded_vorticity
from fsibe_2d_gb300 import make_params


def test_fluid_step_matches_numpy_twin(oracle):
    from py_twin import FluidTwin
    n = 64
    p = make_params(nx=n, ny=n, ns=16, iFLUSI=0, iSaveBeam=3)
    r = oracle.OracleRun(p)
    w = seeded_vorticity(n, sigma=1e-2)
    r.init_fields(w)
    m, vx, vy = r.mask()
    b = r.beam()[0]
    tw = FluidTwin(p, m, vx, vy, b[0], b[1])
    vk = tw.coftxy(w)
    assert rel(vk, r.vortk()) < 1e-14
    u = tw.cal_velocity(0.0, vk)
    assert rel(u, r.u()) < 1e-13
    time = 0.0
    vk, nv, u, press, drag, dt1 = tw.explicit_step(time, vk, u)
    r.step()
    s = r.scalars()
    assert rel(vk, r.vortk()) < 1e-12 and rel(u, r.u()) < 1e-12 and rel(press, r.press()) < 1e-11
    assert abs(drag[0] - s.force[0]) < 1e-11 * abs(drag[0]) and abs(drag[1] - s.force[1]) < 1e-9 * abs(drag[0])
    time += dt1
    dt0 = dt1
    for _ in range(2):
        vk, nv, u, press, drag, dt1 = tw.ab2_step(time, dt0, vk, nv, u)
        r.step()
        time += dt1
        dt0 = dt1
    s = r.scalars()
    assert rel(vk, r.vortk()) < 1e-12 and rel(u, r.u()) < 1e-12 and rel(press, r.press()) < 1e-11
    assert rel(tw.vor_mean, r.vor_mean()) < 1e-12
    assert abs(drag[0] - s.force[0]) < 1e-11 * abs(drag[0])
    r.close()
