"""Known-answer tests of the oracle derived from the mathematics the reference implements:
Taylor-Green decay under the integrating factor (NavierStokes.f90:422-508 with no mask),
the smoothed mask profile (create_mask.f90:475-520, 708-780), the phi4* kernel moments
(Interpolation.f90:82-91), exact interpolation of a linear pressure (BeamForces.f90:152-217)
and the analytic Newton Jacobian against central differences (the reference's own
Jacobi_num self-test, SolidSolver.f90:244-274)."""
import ctypes as C
import math

import numpy as np
import pytest

from conftest import rel, seeded_vorticity
from fsibe_2d_gb300 import make_params

dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731


def test_taylor_green_decays_exactly_under_the_integrating_factor(oracle):
    n, L, Re, dt = 64, 4.0, 50.0, 1e-3
    p = make_params(nx=n, ny=n, ns=16, xl=L, yl=L, Re=Re, dt=dt, iBeam=0, iFLUSI=0, iSaveBeam=0, iMeanVelocity=4)
    r = oracle.OracleRun(p)
    k0 = 2 * np.pi / L
    X, Y = np.meshgrid(np.arange(n) * L / n, np.arange(n) * L / n)
    w0 = np.sin(2 * k0 * X) * np.sin(2 * k0 * Y)
    r.init_fields(w0)
    vk0 = r.vortk()
    steps = 25
    r.time_step(steps)
    decay = math.exp(-p.nu * (8 * k0 ** 2) * dt * steps)  # start-up step included
    assert rel(r.vortk(), vk0 * decay) < 1e-12
    r.close()


def test_mask_profile_of_a_straight_beam(oracle):
    n = 64
    p = make_params(nx=n, ny=n, ns=16)
    r = oracle.OracleRun(p)
    r.init_fields(np.zeros((n, n)))
    m, vx, vy = r.mask()
    chi = m * p.eps
    dx = p.xl / n
    delta = p.N_smooth * dx * abs((math.exp(-4.0) - 1.0) / math.sqrt(math.pi))
    iy0 = int(round(p.y0 / dx))
    ix = int(round((p.x0 + 0.5 * p.length) / dx))
    # on the axis: SmoothStep(0) = erf(t/delta)
    assert abs(chi[iy0, ix] - math.erf(p.t_beam / delta)) < 1e-15
    # symmetric about the axis, zero far away, no velocity for a beam at rest
    for j in range(1, 8):
        assert chi[iy0 + j, ix] == chi[iy0 - j, ix]
    assert chi[iy0 + 20, ix] == 0.0 and np.all(vx == 0) and np.all(vy == 0)
    assert 0.0 <= chi.min() and chi.max() < 1.0
    r.close()


def test_phi4star_partition_of_unity_and_first_moment(oracle):
    L = oracle.lib()
    for x in np.random.default_rng(5).uniform(0, 1, 25):
        ks = np.arange(-4, 5)
        w = np.array([L.orc_delta_phi4star(abs(x - k)) for k in ks])
        assert abs(w.sum() - 1.0) < 1e-14
        assert abs(((x - ks) * w).sum()) < 1e-14


def test_linear_pressure_gives_exact_pressure_jump(oracle):
    n, ns = 64, 16
    p = make_params(nx=n, ny=n, ns=ns, iViscous=0)
    r = oracle.OracleRun(p)
    r.init_fields(np.zeros((n, n)))
    y = np.arange(n) * p.yl / n
    a = 0.7
    r.set_press(np.repeat((a * (y - p.y0))[:, None], n, axis=1))
    r.GetForces(1.0)  # time > T_release: full coupling
    b, po, pn, to, tn = r.beam()
    assert np.abs(pn - a * 2.0 * p.t_beam).max() < 1e-13
    s = r.scalars()
    ds = p.length / (ns - 1)
    assert abs(s.force_press[1] - ns * ds * a * 2.0 * p.t_beam) < 1e-12
    r.close()


def test_analytic_jacobian_matches_central_differences(oracle):
    L = oracle.lib()
    ns = 16
    n = 2 * ns + 4
    p = make_params(nx=64, ny=64, ns=ns)
    r = oracle.OracleRun(p)
    rng = np.random.default_rng(11)
    x = 1e-2 * rng.standard_normal(n)
    vecs = [1e-2 * rng.standard_normal(ns) for _ in range(7)]
    F = np.zeros(n)
    J = np.zeros(n * n)
    dt, dt_old = 2e-4, 2e-4
    for method in (2, 5):
        assert L.orc_newton_system(r._ctx, 0.1, dt, dt_old, method, dp(x), *[dp(v) for v in vecs], dp(F), dp(J)) == 0
        Jm = J.reshape(n, n).copy()
        Jfd = np.zeros((n, n))
        for j in range(n):
            h = 1e-6 * max(1.0, abs(x[j]))
            xp, xm = x.copy(), x.copy()
            xp[j] += h
            xm[j] -= h
            Fp, Fm = np.zeros(n), np.zeros(n)
            L.orc_newton_system(r._ctx, 0.1, dt, dt_old, method, dp(xp), *[dp(v) for v in vecs], dp(Fp), None)
            L.orc_newton_system(r._ctx, 0.1, dt, dt_old, method, dp(xm), *[dp(v) for v in vecs], dp(Fm), None)
            Jfd[:, j] = (Fp - Fm) / (2 * h)
        scale = np.abs(Jm).max(axis=1, keepdims=True)
        assert (np.abs(Jm - Jfd) / scale).max() < 1e-5
    r.close()


def test_short_fsi_run_is_deterministic_and_sane(oracle):
    n = 64
    p = make_params(nx=n, ny=n, ns=16)
    w = seeded_vorticity(n)
    rows = []
    for _ in range(2):
        r = oracle.OracleRun(p)
        r.init_fields(w)
        rows.append(r.time_step(6))
        s = r.scalars()
        assert s.newton_iters >= 3
        r.close()
    assert np.array_equal(rows[0], rows[1])
    assert np.all(np.isfinite(rows[0]))
    assert rows[0][-1, 10] > 0.0  # drag of an impulsively started plate is positive


def test_surface_integral_oracle(oracle):
    """BeamSurfaceIntegral (BeamForces.f90:306-509) on the oracle: finite, its time column,
    and the penalization drag/lift over the grid equal to the sum of mask (u - us) dx dy."""
    import numpy as np
    from conftest import seeded_vorticity
    from fsibe_2d_gb300 import make_params
    n = 128
    p = make_params(nx=n, ny=n, ns=32)
    o = oracle.OracleRun(p)
    o.init_fields(seeded_vorticity(n, seed=4))
    o.time_step(3)
    t = o.scalars().time
    o.create_mask(t); o.EvolveFluidAB2(); o.GetForces(t)
    out = o.BeamSurfaceIntegral(t)
    assert out.shape == (11,) and np.all(np.isfinite(out)) and out[0] == t
    m, mvx, mvy = o.mask()
    u = o.u().reshape(2, n, n)
    dx = p.xl / n
    assert abs(out[1] - np.sum(m * (u[0] - mvx)) * dx * dx) <= 1e-12 * max(1.0, abs(out[1]))
    assert out[3] == out[5] + out[6] + out[7] and out[4] == out[8] + out[9] + out[10]
    o.close()
