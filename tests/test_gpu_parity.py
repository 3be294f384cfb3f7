"""GPU parity: the CUDA path through the C ABI against the CPU oracle on the same seeded inputs.

Tolerances: FP64 plain form -- relative L2 1e-13 for single transforms and operators, 1e-10 for
vorticity, deflection and lift/drag after the step counts below (the bar set for the plain
form); FP32-compensated form -- relative L2 5e-6 for transforms, 1e-5 for vorticity after
the stated steps."""
import numpy as np
import pytest

from conftest import rel, seeded_vorticity
from fsibe_2d_gb300 import make_params, FSIBE_FP32C

pytestmark = pytest.mark.gpu


def _runs(p, oracle):
    import fsibe_2d_gb300 as F
    return F.Run(p), oracle.OracleRun(p)


@pytest.mark.parametrize("nx,ny", [(64, 32), (128, 128), (256, 256), (1024, 1024)])
@pytest.mark.parametrize("prec,tol", [(0, 1e-13), (1, 5e-6)])
def test_transforms_and_packed_operators(oracle, nx, ny, prec, tol):
    g, o = _runs(make_params(nx=nx, ny=ny, ns=16, precision=prec), oracle)
    f = np.random.default_rng(nx * 7 + ny).standard_normal((ny, nx))
    fk_o = o.coftxy(f)
    assert rel(g.coftxy(f), fk_o) < tol
    assert rel(g.cofitxy(fk_o), o.cofitxy(fk_o)) < tol
    for name in ("cofdx", "cofdy", "cofdxdx", "cofdydy", "cofdxdy", "poisson"):
        assert rel(getattr(g, name)(fk_o), getattr(o, name)(fk_o)) < 1e-14, name
    assert rel(g.vis(2e-4), o.vis(2e-4)) < 1e-15
    assert np.array_equal(g.dealiase_mask(), o.dealiase_mask())
    g.close(); o.close()


def _state_errors(g, o):
    e = {}
    e["vortk"] = rel(g.vortk(), o.vortk())
    e["u"] = rel(g.u(), o.u())
    e["press"] = rel(g.press(), o.press())
    e["vor_mean"] = rel(g.vor_mean(), o.vor_mean())
    bg, bo = g.beam(), o.beam()
    e["beam"] = rel(bg[0], bo[0])
    e["theta"] = rel(bg[0][4], bo[0][4]) if np.any(bo[0][4]) else float(np.abs(bg[0][4]).max())
    e["p_new"] = rel(bg[2], bo[2])
    return e


def test_initial_state_and_mask(oracle):
    n = 256
    p = make_params(nx=n, ny=n, ns=64)
    g, o = _runs(p, oracle)
    w = seeded_vorticity(n)
    g.init_fields(w); o.init_fields(w)
    assert rel(g.vortk(), o.vortk()) < 1e-13
    assert rel(g.u(), o.u()) < 1e-13
    mg, mo = g.mask(), o.mask()
    assert rel(mg[0], mo[0]) < 1e-13
    assert np.abs(mg[1] - mo[1]).max() < 1e-12 and np.abs(mg[2] - mo[2]).max() < 1e-12
    g.close(); o.close()


@pytest.mark.parametrize("n,ns,steps", [(64, 16, 30), (256, 64, 60)])
def test_fsi_steps_fp64(oracle, n, ns, steps):
    p = make_params(nx=n, ny=n, ns=ns)
    g, o = _runs(p, oracle)
    w = seeded_vorticity(n)
    g.init_fields(w); o.init_fields(w)
    rg, ro = g.time_step(steps), o.time_step(steps)
    e = _state_errors(g, o)
    for k in ("vortk", "u", "press", "vor_mean", "beam", "p_new"):
        assert e[k] < 1e-10, (k, e)
    # beam_data rows: time, pressure samples, tip state, drag/lift, forces, energies
    scale = np.abs(ro).max(axis=0) + 1e-30
    colerr = (np.abs(rg - ro) / scale).max(axis=0)
    assert colerr.max() < 1e-9, colerr
    sg, so = g.scalars(), o.scalars()
    assert sg.status == 0 and sg.newton_iters == so.newton_iters
    for k in ("vor_rms", "kinetic", "dissipation", "porous_diss", "inflow_solid", "inflow_mean", "u_max"):
        assert abs(getattr(sg, k) - getattr(so, k)) <= 1e-10 * abs(getattr(so, k)) + 1e-300, k
    g.close(); o.close()


def test_routines_one_by_one_from_identical_states(oracle):
    """create_mask, the fluid step, GetForces and the solid step each match the oracle when
    both start from the same uploaded state (the state after 8 oracle steps)."""
    n, ns = 128, 32
    p = make_params(nx=n, ny=n, ns=ns)
    g, o = _runs(p, oracle)
    w = seeded_vorticity(n, seed=3)
    g.init_fields(w); o.init_fields(w)
    o.time_step(8); g.time_step(8)
    b, po, pn, to, tn = o.beam()
    b = b.copy(); b[4] += 1e-3 * np.sin(np.linspace(0, 3, ns)); b[4][0] = 0.0
    o.set_beam(b, po, pn, to, tn); g.set_beam(b, po, pn, to, tn)
    o.create_mask(0.0); g.create_mask(0.0)
    mg, mo = g.mask(), o.mask()
    assert rel(mg[0], mo[0]) < 1e-13
    o.set_u(o.u()); g.set_u(o.u())
    o.set_press(o.press()); g.set_press(o.press())
    o.GetForces(0.5); g.GetForces(0.5)
    assert rel(g.beam()[2], o.beam()[2]) < 1e-12
    assert rel(g.beam()[4], o.beam()[4]) < 1e-12
    g.close(); o.close()


def test_fp32_compensated_form_tracks_fp64(oracle):
    n, steps = 256, 60
    p64 = make_params(nx=n, ny=n, ns=64)
    p32 = make_params(nx=n, ny=n, ns=64, precision=FSIBE_FP32C)
    import fsibe_2d_gb300 as F
    g = F.Run(p32)
    o = oracle.OracleRun(p64)
    w = seeded_vorticity(n)
    g.init_fields(w); o.init_fields(w)
    rg, ro = g.time_step(steps), o.time_step(steps)
    assert rel(g.vort(), o.vort()) < 1e-5
    assert rel(rg[:, 10:12], ro[:, 10:12]) < 1e-5     # drag, lift
    g.close(); o.close()
