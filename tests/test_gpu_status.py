"""Failure statuses through the C ABI, injected from the host.

Each case puts a state into a context that makes one of the reference's own checks fire,
and expects the same status from the GPU library as from the oracle:

| injection                                   | status            | reference check                  |
|---------------------------------------------|-------------------|----------------------------------|
| NaN pressure loads on the beam              | FSIBE_ERR_NAN     | SolidSolver.f90:539-546          |
| Newton limited to one iteration             | NEWTON_MAXIT      | SolidSolver.f90:291-301          |
| a beam whose rate of turn jumps by > 100     | BRAKE (soft)      | SolidSolver.f90:370-380          |
| a beam below the domain                     | MASK_OOB          | create_mask.f90:685-688          |
| a beam whose surface stencils leave the grid | INTERP_OOB        | Interpolation.f90:19-24          |
| bad parameters                              | PARAM/UNSUPPORTED | params.f90 checks                |
| a step before init_fields                   | STATE             | (call order)                     |

No case can fault the GPU: the kernels raise these flags on in-bounds data (the mask's
boxes are clipped to the grid, the interpolation skips stencils off the grid, the beam
kernels stop at their NaN tests).  After each failure the same context is initialised again
and must step cleanly, so a failure leaves the context usable."""
import numpy as np
import pytest

from conftest import seeded_vorticity
from fsibe_2d_gb300 import make_params, FSIBE_FP32C
from fsibe_2d_gb300._abi import (FSIBE_ERR_NAN, FSIBE_ERR_NEWTON_MAXIT, FSIBE_ERR_BRAKE, FSIBE_ERR_MASK_OOB,
                                 FSIBE_ERR_INTERP_OOB, FSIBE_ERR_PARAM, FSIBE_ERR_UNSUPPORTED, FSIBE_ERR_STATE)

pytestmark = pytest.mark.gpu

N, NS = 128, 32


def _pair(oracle, **kw):
    import fsibe_2d_gb300 as F
    p = make_params(nx=N, ny=N, ns=NS, **kw)
    g, o = F.Run(p), oracle.OracleRun(p)
    w = seeded_vorticity(N, seed=11)
    g.init_fields(w); o.init_fields(w)
    return g, o, w


def _status(run, name, *args):
    """The status of one routine call, without raising."""
    import ctypes as C
    fn = getattr(run._lib, run._prefix + name)
    return fn(run._ctx, *[C.c_double(a) if isinstance(a, float) else a for a in args])


def _usable_again(g, w, steps=3):
    g.init_fields(w)
    g.time_step(steps)
    assert g.scalars().status == 0


@pytest.mark.parametrize("cluster", ["16", "0"])
def test_nan_loads_raise_nan(oracle, monkeypatch, cluster):
    monkeypatch.setenv("FSIBE_BEAM_CLUSTER", cluster)   # the cluster and the single-CTA kernel
    g, o, w = _pair(oracle)
    g.time_step(2); o.time_step(2)
    b, po, pn, to, tn = o.beam()
    pn = pn.copy(); pn[NS // 2] = np.nan
    g.set_beam(b, po, pn, to, tn); o.set_beam(b, po, pn, to, tn)
    so, sg = _status(o, "solid_step", 0.001), _status(g, "solid_step", 0.001)
    assert so == FSIBE_ERR_NAN and sg == FSIBE_ERR_NAN, (so, sg)
    _usable_again(g, w)
    g.close(); o.close()


@pytest.mark.parametrize("cluster", ["16", "0"])
def test_newton_iteration_limit(oracle, monkeypatch, cluster):
    monkeypatch.setenv("FSIBE_BEAM_CLUSTER", cluster)
    g, o, w = _pair(oracle, newton_maxit=1, newton_tol=1e-14)
    so, sg = _status(o, "run", 2, None), _status(g, "run", 2, None)
    assert so == FSIBE_ERR_NEWTON_MAXIT and sg == FSIBE_ERR_NEWTON_MAXIT, (so, sg)
    g.close(); o.close()
    # the same parameters with the reference's limit step cleanly
    g2, o2, w = _pair(oracle, newton_tol=1e-14)
    assert _status(g2, "run", 2, None) == 0
    g2.close(); o2.close()


def test_emergency_brake_is_soft(oracle):
    g, o, w = _pair(oracle)
    g.time_step(2); o.time_step(2)
    b, po, pn, to, tn = o.beam()
    b = b.copy(); b[5][:] = 150.0     # theta_dot: the clamped node's rate of turn drops by 150
    g.set_beam(b, po, pn, to, tn); o.set_beam(b, po, pn, to, tn)
    so, sg = _status(o, "solid_step", 0.001), _status(g, "solid_step", 0.001)
    assert so == FSIBE_ERR_BRAKE and sg == FSIBE_ERR_BRAKE, (so, sg)
    # soft: the binding returns the status instead of raising (continue_timestep = .false.)
    assert g.SolidSolverWrapper(0.001) == FSIBE_ERR_BRAKE
    _usable_again(g, w)
    g.close(); o.close()


def test_beam_below_the_domain(oracle):
    g, o, w = _pair(oracle)
    b, po, pn, to, tn = o.beam()
    b = b.copy(); b[1] -= 2.5          # y from 2 to -0.5: the leading edge is below y = 0
    g.set_beam(b, po, pn, to, tn); o.set_beam(b, po, pn, to, tn)
    so, sg = _status(o, "create_mask", 0.0), _status(g, "create_mask", 0.0)
    assert so == FSIBE_ERR_MASK_OOB and sg == FSIBE_ERR_MASK_OOB, (so, sg)
    _usable_again(g, w)
    g.close(); o.close()


def test_interpolation_stencil_off_the_grid(oracle):
    g, o, w = _pair(oracle)
    g.time_step(1); o.time_step(1)
    b, po, pn, to, tn = o.beam()
    b = b.copy(); b[0] -= 0.98         # leading edge at x = 0.02: the 9-point stencils leave the grid
    g.set_beam(b, po, pn, to, tn); o.set_beam(b, po, pn, to, tn)
    so, sg = _status(o, "get_forces", 0.0), _status(g, "get_forces", 0.0)
    assert so == FSIBE_ERR_INTERP_OOB and sg == FSIBE_ERR_INTERP_OOB, (so, sg)
    _usable_again(g, w)
    g.close(); o.close()


def test_bad_parameters_are_rejected():
    import fsibe_2d_gb300 as F
    from fsibe_2d_gb300._binding import FsibeError
    cases = [(dict(ns=4), FSIBE_ERR_PARAM),                 # fewer than 8 beam nodes
             (dict(precision=7), FSIBE_ERR_PARAM),
             (dict(time_method_solid=3), FSIBE_ERR_PARAM),
             (dict(nx=100), FSIBE_ERR_UNSUPPORTED),          # not a power of two
             (dict(nx=8192), FSIBE_ERR_UNSUPPORTED)]
    for kw, code in cases:
        base = dict(nx=64, ny=64, ns=16)
        base.update(kw)
        with pytest.raises(FsibeError) as ex:
            F.Run(make_params(**base))
        assert ex.value.status == code, (kw, ex.value.status)
    # a valid context is still created afterwards
    r = F.Run(make_params(nx=64, ny=64, ns=16, precision=FSIBE_FP32C))
    r.close()


def test_step_before_init_fields(oracle):
    import fsibe_2d_gb300 as F
    g = F.Run(make_params(nx=64, ny=64, ns=16))
    assert _status(g, "step") == FSIBE_ERR_STATE
    assert _status(g, "fluid_step", 0) == FSIBE_ERR_STATE
    _usable_again(g, seeded_vorticity(64))
    g.close()
