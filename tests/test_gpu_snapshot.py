"""ComputePressureSnapshot (NavierStokes.f90:598-665) on the GPU against the oracle: the static
pressure of the current vorticity with the velocity at a given time (its mean flow) and the
current mask.  After a step, at the context's time, it is the step's own pressure."""
import numpy as np
import pytest

from conftest import rel, seeded_vorticity
from fsibe_2d_gb300 import make_params, FSIBE_FP32C

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,bound", [(0, 1e-10), (FSIBE_FP32C, 1e-5)])
def test_snapshot_matches_the_oracle(oracle, precision, bound):
    import fsibe_2d_gb300 as F
    kw = dict(nx=128, ny=128, ns=32, dt=1e-3, iMeanVelocity=1, T_fullspeed=0.5)   # an accelerating mean flow
    g, o = F.Run(make_params(precision=precision, **kw)), oracle.OracleRun(make_params(**kw))
    w = seeded_vorticity(128, seed=3)
    g.init_fields(w); o.init_fields(w)
    g.time_step(10); o.time_step(10)
    t = o.scalars().time
    for when in (t, t + 0.05):         # now, and with the mean flow of a later time
        sg, so = g.ComputePressureSnapshot(when), o.ComputePressureSnapshot(when)
        err = rel(sg, so)
        print(f"snapshot at {when:.4f}, precision {precision}: {err:.3e}")
        assert err < bound, (when, err)
    # the step's pressure, at the context's time
    if precision == 0:
        assert rel(g.ComputePressureSnapshot(t), g.press()) < 1e-12
    assert g.scalars().time == t        # the state is not changed
    g.close(); o.close()
