"""The benchmark configurations at their stated sizes and step counts.

C1 plain FP64 (256^2, ns=64, Re=100, dt=2e-4, 1000 steps): GPU against the oracle, relative L2
   <= 1e-10 in vorticity, beam deflection (y of every node) and the lift/drag time series.
C2 precision form (1024^2, ns=256, Re=500, dt=5e-5, 2000 steps): both forms against the
   oracle over all 2000 steps from the same seed -- FP64 within 1e-10, FP32-compensated within
   the stated 1e-5 -- in vorticity, deflection and the drag/lift time series; the FP64 form
   also against the oracle over the first 10 steps (1e-11).
C5 large run (4096^2, Lx=Ly=8, ns=1024, Re=2000, EI=0.05, mu=2, eta=1e-4, dt=1e-5): FP32 form
   against FP64 form over the first 100 steps (the bounded stand-in for 1000 steps)."""
import numpy as np
import pytest

from conftest import rel, seeded_vorticity
from fsibe_2d_gb300 import make_params, FSIBE_FP32C

pytestmark = pytest.mark.gpu


def test_c1_plain_fp64_1000_steps_match_oracle(oracle):
    import fsibe_2d_gb300 as F
    n, steps = 256, 1000
    p = make_params(nx=n, ny=n, ns=64, Re=100.0, dt=2e-4)
    g, o = F.Run(p), oracle.OracleRun(p)
    w = seeded_vorticity(n, K=8, sigma=1e-3, seed=0)
    g.init_fields(w); o.init_fields(w)
    rg, ro = g.time_step(steps), o.time_step(steps)
    assert g.scalars().status == 0
    assert rel(g.vort(), o.vort()) < 1e-10
    assert rel(g.beam()[0][1], o.beam()[0][1]) < 1e-10          # deflection line y(s)
    assert rel(rg[:, 10], ro[:, 10]) < 1e-10 and rel(rg[:, 11], ro[:, 11]) < 1e-10   # drag, lift
    assert rel(rg[:, 5], ro[:, 5]) < 1e-10                        # trailing-edge y
    g.close(); o.close()


def test_c2_both_forms_against_the_oracle_over_2000_steps(oracle):
    """C2 at its stated size and length: the FP64 form against the oracle within 1e-10, the
    FP32-compensated form against the oracle and against the FP64 form within 1e-5, in
    vorticity, deflection and the drag/lift time series (about 90 s of oracle time on 16
    host cores)."""
    import fsibe_2d_gb300 as F
    n, steps = 1024, 2000
    kw = dict(nx=n, ny=n, ns=256, Re=500.0, dt=5e-5)
    g64, g32 = F.Run(make_params(**kw)), F.Run(make_params(precision=FSIBE_FP32C, **kw))
    o = oracle.OracleRun(make_params(**kw))
    w = seeded_vorticity(n, K=8, sigma=1e-3, seed=0)
    g64.init_fields(w); g32.init_fields(w); o.init_fields(w)
    g64.use_graph(True); g32.use_graph(True)
    r64, r32, ro = g64.time_step(steps), g32.time_step(steps), o.time_step(steps)
    assert g64.scalars().status == 0 and g32.scalars().status == 0 and o.scalars().status == 0
    wo, yo = o.vort(), o.beam()[0][1]
    force = np.linalg.norm(ro[:, 10:12])
    err = {}
    for name, g, r in (("fp64", g64, r64), ("fp32c", g32, r32)):
        err[name] = {"vorticity": rel(g.vort(), wo), "deflection": rel(g.beam()[0][1], yo),
                     "drag": rel(r[:, 10], ro[:, 10]),
                     "lift_at_force_scale": float(np.linalg.norm(r[:, 11] - ro[:, 11]) / force)}
    print("C2, 2000 steps, relative L2 against the oracle:", err)
    assert max(err["fp64"].values()) < 1e-10, err
    assert max(err["fp32c"].values()) < 1e-5, err
    assert rel(g32.vort(), g64.vort()) < 1e-5
    g64.close(); g32.close(); o.close()


def test_c2_fp64_form_matches_oracle_first_steps(oracle):
    import fsibe_2d_gb300 as F
    n = 1024
    p = make_params(nx=n, ny=n, ns=256, Re=500.0, dt=5e-5)
    g, o = F.Run(p), oracle.OracleRun(p)
    w = seeded_vorticity(n)
    g.init_fields(w); o.init_fields(w)
    rg, ro = g.time_step(10), o.time_step(10)
    assert rel(g.vortk(), o.vortk()) < 1e-11
    assert rel(rg[:, 10:12], ro[:, 10:12]) < 1e-10
    g.close(); o.close()


def test_c5_large_run_fp32_vs_fp64_first_100_steps():
    import fsibe_2d_gb300 as F
    n, steps = 4096, 100
    kw = dict(nx=n, ny=n, ns=1024, xl=8.0, yl=8.0, Re=2000.0, dt=1e-5, EI=0.05, mu=2.0, eps=1e-4, x0=2.0, y0=4.0)
    g64, g32 = F.Run(make_params(**kw)), F.Run(make_params(precision=FSIBE_FP32C, **kw))
    w = seeded_vorticity(n, K=32, sigma=1e-3, seed=2)
    g64.init_fields(w); g32.init_fields(w)
    r64, r32 = g64.time_step(steps), g32.time_step(steps)
    assert g64.scalars().status == 0 and g32.scalars().status == 0
    assert rel(g32.vort(), g64.vort()) < 1e-5
    assert rel(r32[:, 10], r64[:, 10]) < 1e-5
    # the lift is small against the drag here: its error is measured at the force scale
    force = np.linalg.norm(r64[:, 10:12])
    assert np.linalg.norm(r32[:, 11] - r64[:, 11]) / force < 1e-5
    g64.close(); g32.close()
