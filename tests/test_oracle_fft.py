"""The oracle's transforms and packed-layout operators against numpy.fft (pocketfft) and
against closed-form coefficients (cof_fftw33.f90:142-243, cofdx.f90, cofdy.f90, poisson.f90,
cal_vis.f90, dealiase_mask.f90, cofdxdy.f90)."""
import numpy as np
import pytest

from conftest import rel
from fsibe_2d_gb300 import make_params


def np_coftxy(f):
    """coftxy restated with numpy.fft: FFTW's r2c_2d ft(kx,ky) repacked with 1/(nx ny)."""
    ny, nx = f.shape
    ft = np.fft.fft(np.fft.rfft(f, axis=1), axis=0)
    norm = 1.0 / (nx * ny)
    fk = np.zeros_like(f)
    hx = nx // 2
    fk[0, 0::2] = ft[0, :hx].real * norm
    fk[0, 1::2] = ft[0, :hx].imag * norm
    for iy in range(1, ny // 2):
        p, m = ft[iy, :hx], ft[ny - iy, :hx]
        fk[2 * iy, 0::2] = 0.5 * (p.real + m.real) * norm
        fk[2 * iy + 1, 0::2] = 0.5 * (p.imag - m.imag) * norm
        fk[2 * iy, 1::2] = 0.5 * (p.imag + m.imag) * norm
        fk[2 * iy + 1, 1::2] = 0.5 * (-p.real + m.real) * norm
    return fk


def np_filtered(f):
    ny, nx = f.shape
    ft = np.fft.rfft2(f)
    ft[:, nx // 2] = 0.0
    ft[ny // 2, :] = 0.0
    return np.fft.irfft2(ft, s=f.shape)


@pytest.mark.parametrize("nx,ny", [(32, 32), (64, 32), (32, 128), (256, 256)])
def test_forward_and_inverse_match_numpy(oracle, nx, ny):
    r = oracle.OracleRun(make_params(nx=nx, ny=ny, ns=16))
    f = np.random.default_rng(nx + ny).standard_normal((ny, nx))
    fk = r.coftxy(f)
    assert rel(fk, np_coftxy(f)) < 1e-14
    # inverse of the packed coefficients is the Nyquist-filtered field (unnormalised c2r)
    assert rel(r.cofitxy(fk), np_filtered(f)) < 1e-14
    r.close()


def test_trig_monomials_have_exact_packed_coefficients(oracle):
    nx = ny = 64
    L = 4.0
    r = oracle.OracleRun(make_params(nx=nx, ny=ny, ns=16, xl=L, yl=L))
    x = np.arange(nx) * L / nx
    y = np.arange(ny) * L / ny
    X, Y = np.meshgrid(x, y)
    k0 = 2 * np.pi / L
    kx, ky = 3, 5
    # cos(kx x) cos(ky y): ft(kx, +-ky) = N/4 each -> a = fk(2kx,2ky) = 1/4
    fk = r.coftxy(np.cos(kx * k0 * X) * np.cos(ky * k0 * Y))
    assert abs(fk[2 * ky, 2 * kx] - 0.25) < 1e-15
    fk[2 * ky, 2 * kx] = 0.0
    assert np.abs(fk).max() < 1e-15
    # sin(kx x) sin(ky y) -> d = fk(2kx+1, 2ky+1) = 1/4  (ft(kx,+ky) = -N/4, ft(kx,-ky) = +N/4)
    fk = r.coftxy(np.sin(kx * k0 * X) * np.sin(ky * k0 * Y))
    assert abs(fk[2 * ky + 1, 2 * kx + 1] - 0.25) < 1e-15
    # ky = 0 row stores Re/Im directly: cos(kx x) -> fk(2kx, 0) = 1/2
    fk = r.coftxy(np.cos(kx * k0 * X))
    assert abs(fk[0, 2 * kx] - 0.5) < 1e-15
    r.close()


def test_spectral_derivatives_poisson_and_vis_on_trig_fields(oracle):
    nx, ny, L = 64, 32, 4.0
    p = make_params(nx=nx, ny=ny, ns=16, xl=L, yl=L, Re=50.0)
    r = oracle.OracleRun(p)
    X, Y = np.meshgrid(np.arange(nx) * L / nx, np.arange(ny) * L / ny)
    k0 = 2 * np.pi / L
    f = np.sin(3 * k0 * X) * np.cos(2 * k0 * Y) + 0.3 * np.cos(5 * k0 * X + 1 * k0 * Y)
    fk = r.coftxy(f)
    dfx = 3 * k0 * np.cos(3 * k0 * X) * np.cos(2 * k0 * Y) - 0.3 * 5 * k0 * np.sin(5 * k0 * X + k0 * Y)
    dfy = -2 * k0 * np.sin(3 * k0 * X) * np.sin(2 * k0 * Y) - 0.3 * k0 * np.sin(5 * k0 * X + k0 * Y)
    assert np.abs(r.cofitxy(r.cofdx(fk)) - dfx).max() < 1e-12
    assert np.abs(r.cofitxy(r.cofdy(fk)) - dfy).max() < 1e-12
    lap = -(9 + 4) * k0 ** 2 * np.sin(3 * k0 * X) * np.cos(2 * k0 * Y) - 0.3 * (25 + 1) * k0 ** 2 * np.cos(5 * k0 * X + k0 * Y)
    # poisson: f = -lap(ans)  <=>  ans_hat = f_hat/|k|^2
    assert np.abs(r.cofitxy(r.poisson(r.coftxy(-lap))) - f).max() < 1e-12
    assert np.abs(r.cofitxy(r.cofdxdx(fk)) + r.cofitxy(r.cofdydy(fk)) - lap).max() < 1e-10
    # cofdxdy returns MINUS the mixed derivative (reference quirk kept)
    assert np.abs(r.cofdxdy(fk) + r.cofdx(r.cofdy(fk))).max() < 1e-12
    dt = 1e-2
    w = r.vis(dt)
    nu = p.nu
    assert abs(w[2 * 2, 2 * 3] - np.exp(-nu * dt * (9 + 4) * k0 ** 2)) < 1e-15
    assert np.all(w[0:2, 0:2] == 1.0)
    r.close()


def test_dealiasing_mask_is_the_two_thirds_ellipse(oracle):
    nx, ny = 64, 32
    r = oracle.OracleRun(make_params(nx=nx, ny=ny, ns=16))
    d = r.dealiase_mask()
    kxt, kyt = 2.0 / 3.0 * (nx // 2 - 1), 2.0 / 3.0 * (ny // 2 - 1)
    for ky in range(ny // 2):
        for kx in range(nx // 2):
            keep = 0.0 if (kx ** 2 / kxt ** 2 + ky ** 2 / kyt ** 2) >= 1.0 else 1.0
            assert np.all(d[2 * ky:2 * ky + 2, 2 * kx:2 * kx + 2] == keep)
    r.close()
