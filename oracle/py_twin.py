"""numpy restatement of the reference's fluid step, used only to cross-check the C++ oracle.

TEST INFRASTRUCTURE ONLY.  Independent of oracle/fsibe_oracle.cpp: transforms go through
numpy.fft (pocketfft) instead of the oracle's own radix-2 FFT, operators are vectorised.
Covers coftxy/cofitxy (cof_fftw33.f90:142-243), cofdx/cofdy (cofdx.f90, cofdy.f90), poisson
(poisson.f90), vis (cal_vis.f90), dealiase_mask (dealiase_mask.f90), cal_nlk, cal_velocity,
pressure with cal_drag/cal_energy/time_avg_vort, EvolveFluidExplicit and EvolveFluidAB2
(NavierStokes.f90) for a fixed mask (no beam motion).
"""
import math

import numpy as np


class FluidTwin:
    def __init__(self, p, mask, maskvx, maskvy, x_beam, y_beam):
        self.p = p
        self.nx, self.ny = p.nx, p.ny
        self.dx, self.dy = p.xl / p.nx, p.yl / p.ny
        self.pi = 4.0 * math.atan(1.0)
        self.scalex = (2 * self.pi / p.xl) ** 2
        self.scaley = (2 * self.pi / p.yl) ** 2
        self.mask, self.mvx, self.mvy = mask, maskvx, maskvy
        self.xb, self.yb = x_beam, y_beam
        kx = np.arange(self.nx) // 2
        ky = np.arange(self.ny) // 2
        self.KX, self.KY = np.meshgrid(kx, ky)           # packed wavenumber of each slot
        self.XODD = (np.arange(self.nx) % 2)[None, :]
        self.YODD = (np.arange(self.ny) % 2)[:, None]
        kxt, kyt = 2.0 / 3.0 * (self.nx // 2 - 1), 2.0 / 3.0 * (self.ny // 2 - 1)
        self.dealiase = np.where(self.KX ** 2 / kxt ** 2 + self.KY ** 2 / kyt ** 2 >= 1.0, 0.0, 1.0)
        if p.idealis != 1:
            self.dealiase[:] = 1.0
        self.vor_mean = np.zeros((self.ny, self.nx))
        self.unst_old = None

    # -- transforms ------------------------------------------------------------------
    def coftxy(self, f):
        ny, nx = f.shape
        ft = np.fft.fft(np.fft.rfft(f, axis=1), axis=0)
        norm = 1.0 / (nx * ny)
        fk = np.zeros_like(f)
        hx = nx // 2
        fk[0, 0::2] = ft[0, :hx].real * norm
        fk[0, 1::2] = ft[0, :hx].imag * norm
        iy = np.arange(1, ny // 2)
        p, m = ft[iy, :hx], ft[ny - iy, :hx]
        fk[2 * iy, 0::2] = 0.5 * (p.real + m.real) * norm
        fk[2 * iy + 1, 0::2] = 0.5 * (p.imag - m.imag) * norm
        fk[2 * iy, 1::2] = 0.5 * (p.imag + m.imag) * norm
        fk[2 * iy + 1, 1::2] = 0.5 * (-p.real + m.real) * norm
        return fk

    def cofitxy(self, fk):
        ny, nx = fk.shape
        hx = nx // 2
        ft = np.zeros((ny, hx + 1), dtype=complex)
        ft[0, :hx] = fk[0, 0::2] + 1j * fk[0, 1::2]
        iy = np.arange(1, ny // 2)
        a, b = fk[2 * iy, 0::2], fk[2 * iy + 1, 0::2]
        c, d = fk[2 * iy, 1::2], fk[2 * iy + 1, 1::2]
        ft[iy, :hx] = (a - d) + 1j * (b + c)
        ft[ny - iy, :hx] = (a + d) + 1j * (-b + c)
        ft[:, 0] = ft[:, 0]
        g = np.fft.ifft(ft, axis=0) * ny
        g[:, 0] = g[:, 0].real
        return np.fft.irfft(g, n=nx, axis=1) * nx

    # -- packed operators ----------------------------------------------------------------
    def cofdx(self, fk):
        s1 = 2.0 * self.pi / self.p.xl
        out = np.empty_like(fk)
        out[:, 0::2] = -fk[:, 1::2] * self.KX[:, 0::2] * s1
        out[:, 1::2] = fk[:, 0::2] * self.KX[:, 1::2] * s1
        return out

    def cofdy(self, fk):
        s1 = 2.0 * self.pi / self.p.yl
        out = np.empty_like(fk)
        out[0::2, :] = -fk[1::2, :] * self.KY[0::2, :] * s1
        out[1::2, :] = fk[0::2, :] * self.KY[1::2, :] * s1
        return out

    def poisson(self, f):
        quot = self.KX ** 2 * self.scalex + self.KY ** 2 * self.scaley
        quot[0:2, 0:2] = 1.0
        ans = f / quot
        ans[0:2, 0:2] = 0.0
        return ans

    def vis(self, dt):
        coefx = -dt * self.p.nu * self.scalex
        coefy = -dt * self.p.nu * self.scaley
        return np.exp(coefx * self.KX ** 2 + coefy * self.KY ** 2)

    # -- NavierStokes.f90 ------------------------------------------------------------------
    def cal_velocity(self, time, vortk):
        stream = self.poisson(vortk)
        uy = self.cofitxy(self.cofdx(stream))
        ux = self.cofitxy(self.cofdy(stream))
        mux = math.cos(self.p.theta_inf) if self.p.iMeanVelocity == 3 else 0.0
        muy = math.sin(self.p.theta_inf) if self.p.iMeanVelocity == 3 else 0.0
        return np.stack([ux + mux, -uy + muy])

    def cal_nlk(self, time, vortk, u):
        vdx = self.cofitxy(self.cofdx(vortk))
        vdy = self.cofitxy(self.cofdy(vortk))
        nlk = self.coftxy(-u[0] * vdx - u[1] * vdy)
        umax = math.sqrt((u[0] ** 2 + u[1] ** 2).max())
        p = self.p
        dt1 = p.cfl * min(self.dx, self.dy) / umax
        if umax < 1e-10:
            dt1 = 1e-2
        if p.iBeam > 0:
            dt1 = min(0.9 * p.eps, dt1)
        if p.dt_fixed > 0:
            dt1 = min(p.dt_fixed, dt1)
        if p.time_end - time < dt1:
            dt1 = p.time_end - time
        pen1 = -self.mask * (u[0] - self.mvx)
        pen2 = -self.mask * (u[1] - self.mvy)
        pen2 = self.cofdx(self.coftxy(pen2))
        pen1 = self.cofdy(self.coftxy(pen1))
        return nlk + (pen2 - pen1), dt1

    def pressure(self, time, dt1, vortk):
        u = self.cal_velocity(time + dt1, vortk)
        pen = np.stack([self.mask * (u[0] - self.mvx), self.mask * (u[1] - self.mvy)])
        drag = self.cal_drag(time, dt1, pen)
        vor = self.cofitxy(vortk)
        self.vor_mean = (self.vor_mean * time + dt1 * vor) / (time + dt1)
        pen[0] = pen[0] - vor * u[1]
        pen[1] = pen[1] + vor * u[0]
        work = self.cofdx(self.coftxy(pen[0])) + self.cofdy(self.coftxy(pen[1]))
        q = self.cofitxy(self.poisson(work))
        press = q - 0.5 * (u[0] ** 2 + u[1] ** 2)
        return u, press, drag, vor

    def cal_drag(self, time, dt1, pen):
        p = self.p
        tb = p.t_beam
        iymax = int(max(self.yb.max() + 1.5 * tb, p.y0) / self.dy)
        iymin = int(min(self.yb.min() - 1.5 * tb, p.y0) / self.dy)
        ixmin = int(min(p.x0 - max(0.0, 1.5 * tb), self.xb.min() - 1.5 * tb) / self.dx)
        ixmax = int((self.xb.max() + 1.5 * tb) / self.dx)
        ixmin, ixmax = max(ixmin, 0), min(ixmax, self.nx - 1)
        iymin, iymax = max(iymin, 0), min(iymax, self.ny - 1)
        norm = self.dx * self.dy
        sl = (slice(iymin, iymax + 1), slice(ixmin, ixmax + 1))
        return pen[0][sl].sum() * norm, pen[1][sl].sum() * norm

    def explicit_step(self, time, vortk, u):
        nlk, dt1 = self.cal_nlk(time, vortk, u)
        work = self.vis(dt1)
        vk1 = (vortk + dt1 * nlk) * work * self.dealiase
        u1, press, drag, vor = self.pressure(time, dt1, vk1)
        return vk1, nlk * work, u1, press, drag, dt1

    def ab2_step(self, time, dt0, vortk, nlk_old_vis, u):
        nlk, dt1 = self.cal_nlk(time, vortk, u)
        b10 = dt1 / dt0 * (0.5 * dt1 + dt0)
        b11 = -0.5 * dt1 ** 2 / dt0
        work = self.vis(dt1)
        vk1 = (vortk + b10 * nlk + b11 * nlk_old_vis) * work * self.dealiase
        u1, press, drag, vor = self.pressure(time, dt1, vk1)
        return vk1, nlk * work, u1, press, drag, dt1
