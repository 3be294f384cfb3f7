"""GPU parity at the sizes, grid shapes and options that the other GPU tests leave out.

* Transforms and packed operators at 2048^2, 4096^2 and the non-square 4096 x 1024 and
  1024 x 4096 (cof_fftw33.f90:142-243): each length has its own translation unit and launch
  bounds.  FP64 within 1e-13, FP32-compensated within 5e-6 (relative L2).
* Three FP64 steps of the large configuration (4096^2, ns = 1024) against the oracle: the
  vorticity spectrum, pressure and beam within 1e-11.
* Whole time steps (time_step.f90:178-228) on non-square grids, 256 x 128 and 128 x 256.
* Options of the reference that the benchmark configurations leave at their defaults:
  the sharp trailing edge (iSharpTrailing = 1, create_mask.f90:784-852), constant gravity and
  the gravity impulses (iImpulse 1 and 3, SolidSolver.f90:874-911), and the mean-flow modes
  1, 2, 4, 6 and 22 (mean_velocity.f90:4-84).
FP64 results within 1e-10 of the oracle after the stated steps; FP32-compensated within 1e-5."""
import numpy as np
import pytest

from conftest import rel, seeded_vorticity
from fsibe_2d_gb300 import make_params, FSIBE_FP32C

pytestmark = pytest.mark.gpu


def _runs(p, oracle):
    import fsibe_2d_gb300 as F
    return F.Run(p), oracle.OracleRun(p)


@pytest.mark.parametrize("nx,ny", [(2048, 2048), (4096, 4096), (4096, 1024), (1024, 4096)])
@pytest.mark.parametrize("prec,tol", [(0, 1e-13), (1, 5e-6)])
def test_transforms_large_and_non_square(oracle, nx, ny, prec, tol):
    g, o = _runs(make_params(nx=nx, ny=ny, ns=16, precision=prec), oracle)
    f = np.random.default_rng(nx * 3 + ny).standard_normal((ny, nx))
    fk_o = o.coftxy(f)
    assert rel(g.coftxy(f), fk_o) < tol
    assert rel(g.cofitxy(fk_o), o.cofitxy(fk_o)) < tol
    for name in ("cofdx", "cofdy", "cofdxdy", "poisson"):
        assert rel(getattr(g, name)(fk_o), getattr(o, name)(fk_o)) < 1e-14, name
    g.close(); o.close()


def _compare(g, o, rg, ro, tol, cols=(1, 5, 10, 11)):
    e = {"vortk": rel(g.vortk(), o.vortk()), "u": rel(g.u(), o.u()), "press": rel(g.press(), o.press())}
    bg, bo = g.beam()[0], o.beam()[0]
    e["beam_y"] = rel(bg[1], bo[1])
    e["beam_x"] = rel(bg[0], bo[0])
    for c in cols:
        e[f"row{c}"] = rel(rg[:, c], ro[:, c])
    assert max(e.values()) < tol, e
    return e


def test_large_configuration_three_fp64_steps_match_oracle(oracle):
    n = 4096
    p = make_params(nx=n, ny=n, ns=1024, xl=8.0, yl=8.0, Re=2000.0, dt=1e-5, EI=0.05, mu=2.0, eps=1e-4,
                    x0=2.0, y0=4.0)
    g, o = _runs(p, oracle)
    w = seeded_vorticity(n, K=32, sigma=1e-3, seed=2)
    g.init_fields(w); o.init_fields(w)
    rg, ro = g.time_step(3), o.time_step(3)
    assert g.scalars().status == 0 and o.scalars().status == 0
    e = _compare(g, o, rg, ro, 1e-11, cols=(1, 10))
    print("4096^2 FP64, 3 steps:", e)
    g.close(); o.close()


@pytest.mark.parametrize("nx,ny", [(256, 128), (128, 256)])
@pytest.mark.parametrize("prec", [0, 1])
def test_full_steps_on_non_square_grids(oracle, nx, ny, prec):
    import fsibe_2d_gb300 as F
    kw = dict(nx=nx, ny=ny, ns=32)
    g, o = F.Run(make_params(precision=prec, **kw)), oracle.OracleRun(make_params(**kw))
    w = seeded_vorticity(nx, ny=ny, seed=5)
    g.init_fields(w); o.init_fields(w)
    rg, ro = g.time_step(40), o.time_step(40)
    assert g.scalars().status == 0
    if prec == 0:
        _compare(g, o, rg, ro, 1e-10)
    else:
        assert rel(g.vort(), o.vort()) < 1e-5
        assert rel(rg[:, 10], ro[:, 10]) < 1e-5
    g.close(); o.close()


@pytest.mark.parametrize("prec", [0, 1])
def test_sharp_trailing_edge(oracle, prec):
    import fsibe_2d_gb300 as F
    kw = dict(nx=128, ny=128, ns=32, iSharpTrailing=1, angle_beam=5.0)
    g, o = F.Run(make_params(precision=prec, **kw)), oracle.OracleRun(make_params(**kw))
    w = seeded_vorticity(128, seed=6)
    g.init_fields(w); o.init_fields(w)
    mg, mo = g.mask()[0], o.mask()[0]
    assert rel(mg, mo) < (1e-13 if prec == 0 else 1e-6)
    rg, ro = g.time_step(40), o.time_step(40)
    assert g.scalars().status == 0
    if prec == 0:
        _compare(g, o, rg, ro, 1e-10)
    else:
        assert rel(g.vort(), o.vort()) < 1e-5
    g.close(); o.close()


def test_constant_gravity(oracle):
    p = make_params(nx=128, ny=128, ns=32, grav=0.5)
    g, o = _runs(p, oracle)
    w = seeded_vorticity(128, seed=7)
    g.init_fields(w); o.init_fields(w)
    rg, ro = g.time_step(40), o.time_step(40)
    _compare(g, o, rg, ro, 1e-10, cols=(1, 5, 10, 11, 19, 20))   # incl. the energies
    g.close(); o.close()


@pytest.mark.parametrize("mode,time", [(1, 0.8), (3, 2.5)])
def test_gravity_impulse_in_the_solid_step(oracle, mode, time):
    """GravityImpulse at a time inside the impulse's window: the solid step from identical
    states (after 6 steps of the oracle) must agree."""
    n, ns = 128, 32
    p = make_params(nx=n, ny=n, ns=ns, iImpulse=mode)
    g, o = _runs(p, oracle)
    w = seeded_vorticity(n, seed=8)
    g.init_fields(w); o.init_fields(w)
    o.time_step(6); g.time_step(6)
    b, po, pn, to, tn = o.beam()
    g.set_beam(b, po, pn, to, tn); o.set_beam(b, po, pn, to, tn)
    o.SolidSolverWrapper(time); g.SolidSolverWrapper(time)
    bg, bo = g.beam()[0], o.beam()[0]
    assert g.scalars().status == 0
    assert rel(bg[1], bo[1]) < 1e-10 and rel(bg[4], bo[4]) < 1e-10
    # the impulse moved the beam: the same call without it gives another state
    q = make_params(nx=n, ny=n, ns=ns)
    o2 = oracle.OracleRun(q)
    o2.init_fields(w); o2.time_step(6); o2.set_beam(b, po, pn, to, tn); o2.SolidSolverWrapper(time)
    assert rel(o2.beam()[0][4], bo[4]) > 1e-6
    g.close(); o.close(); o2.close()


@pytest.mark.parametrize("mode", [1, 2, 4, 6, 22])
@pytest.mark.parametrize("prec", [0, 1])
def test_mean_flow_modes(oracle, mode, prec):
    import fsibe_2d_gb300 as F
    kw = dict(nx=128, ny=128, ns=32, iMeanVelocity=mode, theta_inf=0.3)
    pg, po_ = make_params(precision=prec, **kw), make_params(**kw)
    for p in (pg, po_):
        p.T_fullspeed = 0.004   # the ramps of modes 1 and 2 span the first 20 steps
    g, o = F.Run(pg), oracle.OracleRun(po_)
    w = seeded_vorticity(128, seed=9)
    g.init_fields(w); o.init_fields(w)
    rg, ro = g.time_step(40), o.time_step(40)
    sg, so = g.scalars(), o.scalars()
    assert sg.status == 0
    if prec == 0:
        _compare(g, o, rg, ro, 1e-10)
        assert abs(sg.mean_ux - so.mean_ux) <= 1e-12 * max(1.0, abs(so.mean_ux))
    else:
        assert rel(g.vort(), o.vort()) < 1e-5
        assert rel(g.u(), o.u()) < 1e-5
    g.close(); o.close()
