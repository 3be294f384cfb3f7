"""The oracle's channel walls, leading-edge cylinder and sponges (create_mask.f90:21-210,
223-470; NavierStokes.f90:142-164): known profiles and the behaviour of the sponge term."""
import math

import numpy as np

from conftest import seeded_vorticity
from fsibe_2d_gb300 import make_params


def _smooth_step(x, t, h):
    d = h * abs((math.exp(-4.0) - 1.0) / math.sqrt(math.pi))
    return 0.5 * (math.erf((t - x) / d) + math.erf((x + t) / d))


def test_wall_rows_follow_the_smooth_step(oracle):
    n, h = 64, 0.3
    p = make_params(nx=n, ny=n, ns=16, iWalls=1, h_channel=h)
    o = oracle.OracleRun(p)
    o.init_fields(seeded_vorticity(n))
    m = o.mask()[0] * p.eps
    dy = p.yl / n
    hs = h + p.N_smooth * dy
    for j in range(int(round(hs / dy)) + 1):           # bottom wall: every column alike
        assert np.allclose(m[j, :40], _smooth_step(j * dy, h, p.N_smooth * dy), rtol=0, atol=1e-15)
    for j in range(n - 1, int(round((p.yl - hs) / dy)) - 1, -1):
        assert np.allclose(m[j, :40], _smooth_step(abs(j * dy - p.yl), h, p.N_smooth * dy), rtol=0, atol=1e-15)
    o.close()


def test_cylinder_and_sponges_change_the_flow(oracle):
    n = 64
    w = seeded_vorticity(n, seed=4)
    base = oracle.OracleRun(make_params(nx=n, ny=n, ns=16))
    base.init_fields(w)
    ref = base.time_step(5)
    for kw in (dict(iCylinder=1, R_cylinder=0.1), dict(iSponge=1, SpongeSize=0.5, eps_sponge=1e-2),
               dict(iSponge=3, SpongeSize=0.3, eps_sponge=1e-2), dict(iSponge=22, SpongeSize=0.3, eps_sponge=1e-2),
               dict(iWalls=1, h_channel=0.3, iSponge=4, SpongeSize=0.5),
               dict(iSponge=10, SpongeSize=1.5, eps_sponge=0.1)):
        o = oracle.OracleRun(make_params(nx=n, ny=n, ns=16, **kw))
        o.init_fields(w)
        rows = o.time_step(5)
        assert np.isfinite(rows).all() and o.scalars().status == 0, kw
        assert np.abs(rows[:, 10] - ref[:, 10]).max() > 1e-8, kw        # the drag moved
        o.close()
    base.close()


def test_fixed_beam_mask_is_redrawn_only_while_the_flow_accelerates(oracle):
    """time_step.f90:124,187: with the velocity sponge and a beam that does not move, the mask
    follows the mean flow until T_fullspeed and is kept from then on."""
    n = 64
    p = make_params(nx=n, ny=n, ns=16, dt=1e-3, iWalls=1, h_channel=0.3, iSponge=4, SpongeSize=0.5,
                    iFLUSI=0, iMeanVelocity=1, T_fullspeed=0.01)
    o = oracle.OracleRun(p)
    o.init_fields(seeded_vorticity(n, seed=2))
    o.time_step(3)
    early = o.mask()[1].copy()
    o.time_step(12)
    t_late = o.scalars().time
    late = o.mask()[1].copy()
    o.time_step(10)
    assert t_late > p.T_fullspeed
    assert np.abs(late - early).max() > 1e-3          # the sponge's inflow profile grew
    assert np.array_equal(o.mask()[1], late)            # and is frozen after T_fullspeed
    o.close()


def test_pressure_snapshot_is_the_steps_pressure(oracle):
    """NavierStokes.f90:598-665 at the time after a step gives that step's pressure."""
    n = 64
    o = oracle.OracleRun(make_params(nx=n, ny=n, ns=16))
    o.init_fields(seeded_vorticity(n, seed=9))
    o.time_step(4)
    snap = o.ComputePressureSnapshot(o.scalars().time)
    p = o.press()
    assert np.abs(snap - p).max() <= 1e-12 * np.abs(p).max()
    o.close()
