/*
 * fsibe_oracle.cpp -- CPU restatement (FP64, C++17, OpenMP) of the FSIBE_2D hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: the GPU library is
 * checked against it, and bench.py times it as the CPU baseline.  No product code
 * path may link, load or call it.
 *
 * It restates, routine by routine, the reference's Fortran (tommy-engels/FSIBE_2D;
 * citations are file:line into that project) in the reference's own data layout:
 * physical fields (0:nx-1,0:ny-1) column-major, spectral fields in the packed
 * "Temperton" bicomplex layout written by coftxy.  The reference links FFTW/MKL for
 * its transforms and MKL LAPACK (dgetrf/dgetrs, dgttrf/dgttrs) for its beam
 * solves; none of that is vendored, so this file carries its own radix-2 FFT and
 * restates the published LAPACK algorithms (unblocked partial-pivot LU, dgetf2
 * order; tridiagonal LU with row interchanges, dgttrf/dgtts2 order).
 *
 * Parity pin: the reference ships no tests, fixtures or stored outputs.  This file
 * is pinned by the CPU tests against numpy.fft (pocketfft) and
 * scipy.linalg.lapack.{dgetrf,dgetrs,dgttrf,dgttrs}, and by known-answer tests
 * derived from the mathematics (trig monomials, Taylor-Green decay, the phi4*
 * partition of unity, analytic-vs-finite-difference Jacobian).
 */
#include "../include/fsibe.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct cplx { double re, im; };
static inline cplx cmul(cplx a, cplx b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
static inline cplx cadd(cplx a, cplx b) { return {a.re + b.re, a.im + b.im}; }
static inline cplx csub(cplx a, cplx b) { return {a.re - b.re, a.im - b.im}; }
static inline cplx cconj(cplx a) { return {a.re, -a.im}; }

/* exp(-2 pi i k / n), evaluated in long double and rounded once to double. */
static cplx twiddle(long k, long n) {
    const long double pi_l = 3.141592653589793238462643383279502884L;
    long double a = 2.0L * pi_l * (long double)k / (long double)n;
    return {(double)cosl(a), (double)(-sinl(a))};
}

/* Iterative radix-2 complex FFT of a power-of-two length (bit-reversal + DIT stages). */
struct CFFT {
    int n = 0;
    std::vector<cplx> tw;   /* tw[k] = exp(-2 pi i k/n), k < n/2 */
    std::vector<int> rev;
    void init(int n_) {
        n = n_;
        tw.resize(std::max(1, n / 2));
        for (int k = 0; k < n / 2; ++k) tw[k] = twiddle(k, n);
        rev.assign(n, 0);
        int lg = 0;
        while ((1 << lg) < n) ++lg;
        for (int i = 0; i < n; ++i) {
            int r = 0;
            for (int b = 0; b < lg; ++b) if (i & (1 << b)) r |= 1 << (lg - 1 - b);
            rev[i] = r;
        }
    }
    /* sign = -1 forward (exp(-i..)), +1 backward; unnormalized. */
    void run(cplx* a, int sign) const {
        for (int i = 0; i < n; ++i) if (i < rev[i]) std::swap(a[i], a[rev[i]]);
        for (int len = 2; len <= n; len <<= 1) {
            int half = len >> 1, step = n / len;
            for (int i = 0; i < n; i += len) {
                for (int j = 0; j < half; ++j) {
                    cplx w = tw[j * step];
                    if (sign > 0) w = cconj(w);
                    cplx u = a[i + j], v = cmul(a[i + j + half], w);
                    a[i + j] = cadd(u, v);
                    a[i + j + half] = csub(u, v);
                }
            }
        }
    }
};

/* Real FFT of length n through a complex FFT of length n/2 plus the split step. */
struct RFFT {
    int n = 0;
    CFFT half;
    std::vector<cplx> w;  /* exp(-2 pi i k/n), k <= n/2 */
    void init(int n_) {
        n = n_;
        half.init(n / 2);
        w.resize(n / 2 + 1);
        for (int k = 0; k <= n / 2; ++k) w[k] = twiddle(k, n);
    }
    /* X[k] = sum_j x[j] exp(-2 pi i jk/n), k = 0..n/2 */
    void forward(const double* x, cplx* X, cplx* z) const {
        const int m = n / 2;
        for (int j = 0; j < m; ++j) z[j] = {x[2 * j], x[2 * j + 1]};
        half.run(z, -1);
        for (int k = 0; k <= m; ++k) {
            cplx zk = z[k % m], zc = cconj(z[(m - k) % m]);
            cplx e = {0.5 * (zk.re + zc.re), 0.5 * (zk.im + zc.im)};
            cplx d = csub(zk, zc);                    /* 2i * O */
            cplx o = {0.5 * d.im, -0.5 * d.re};        /* d / (2i) */
            X[k] = cadd(e, cmul(w[k], o));
        }
    }
    /* x[j] = Re X[0] + 2 sum_{0<k<n/2} Re(X[k] e^{2 pi i jk/n}) + Re X[n/2] (-1)^j (unnormalized c2r;
     * the imaginary parts of the DC and Nyquist bins are ignored). */
    void inverse(const cplx* Xin, double* x, cplx* z) const {
        const int m = n / 2;
        for (int k = 0; k < m; ++k) {
            cplx a = Xin[k], b = Xin[m - k];
            if (k == 0) { a.im = 0.0; b.im = 0.0; }
            cplx bc = cconj(b);
            cplx e = cadd(a, bc);                      /* 2E */
            cplx o = cmul(csub(a, bc), cconj(w[k]));   /* 2 O */
            z[k] = {e.re - o.im, e.im + o.re};         /* 2E + i 2O */
        }
        half.run(z, +1);
        for (int j = 0; j < m; ++j) { x[2 * j] = z[j].re; x[2 * j + 1] = z[j].im; }
    }
};

struct Beam {
    std::vector<double> x, y, vx, vy, theta, theta_dot, ax, ay, p_old, p_new, tau_old, tau_new;
    std::vector<double> oldold;  /* (0:ns-1, 1:6) column-major */
    double Force[2] = {0, 0}, Force_unst[2] = {0, 0}, Force_press[2] = {0, 0}, Inertial[2] = {0, 0};
    double E_kin = 0, E_pot = 0, E_el = 0;
    double x0 = 0, y0 = 0, AngleBeam = 0, phase = 0, dt_old = 0;
    double drag_unst_new = 0, drag_unst_old = 0, lift_unst_new = 0, lift_unst_old = 0;
    bool StartupStep = true, UnstReady = false;
    int iMouvement = 0;
    void alloc(int ns) {
        for (auto* v : {&x, &y, &vx, &vy, &theta, &theta_dot, &ax, &ay, &p_old, &p_new, &tau_old, &tau_new})
            v->assign(ns, 0.0);
        oldold.assign((size_t)ns * 6, 0.0);
    }
};

}  // namespace

struct orc_ctx {
    fsibe_params P;
    int nx, ny, ns;
    double pi, scalex, scaley, ds, dx, dy;
    int TimeMethodSolid;
    bool ActuallyBDF2 = false;
    double grav;
    bool sharp;
    double U_mean_true = 1.0;
    std::vector<double> dealiase, mask, maskvx, maskvy, vor_mean;
    std::vector<double> mask_sponge, mask_frame;  /* vorticity sponge / eps_sponge; the frame of iSponge 22 */
    int n0 = 0, n1 = 1;
    double time = 0, dt0 = 0, dt1 = 0;
    std::vector<double> vortk[2], nlk[2], workvis[2], u, press;
    Beam beam;
    bool initialized = false, startup_done = false;
    fsibe_scalars sc;
    std::string err;
    RFFT rx;
    CFFT cy;
    std::vector<cplx> ft;  /* (0:nx/2-1, 0:ny-1), kx fastest */
};

namespace {

#define F2(a, ix, iy) (a)[(size_t)(iy) * c->nx + (ix)]

static int fail(orc_ctx* c, int code, const char* msg) {
    if (c) c->err = msg;
    return code;
}

/* ------------------------------------------------------------------------------
 * FFT backend: coftxy / cofitxy (cof_fftw33.f90:142-243)
 * ------------------------------------------------------------------------------ */

/* ft(kx,ky) = sum f(ix,iy) exp(-2 pi i (kx ix/nx + ky iy/ny)), kx < nx/2 (FFTW r2c_2d). */
static void r2c_2d(orc_ctx* c, const double* f) {
    const int nx = c->nx, ny = c->ny, hx = nx / 2;
    std::vector<cplx>& ft = c->ft;
#pragma omp parallel
    {
        std::vector<cplx> X(hx + 1), z(hx), col(ny);
#pragma omp for schedule(static)
        for (int iy = 0; iy < ny; ++iy) {
            c->rx.forward(f + (size_t)iy * nx, X.data(), z.data());
            for (int kx = 0; kx < hx; ++kx) ft[(size_t)iy * hx + kx] = X[kx];
        }
#pragma omp for schedule(static)
        for (int kx = 0; kx < hx; ++kx) {
            for (int iy = 0; iy < ny; ++iy) col[iy] = ft[(size_t)iy * hx + kx];
            c->cy.run(col.data(), -1);
            for (int ky = 0; ky < ny; ++ky) ft[(size_t)ky * hx + kx] = col[ky];
        }
    }
}

/* FFTW c2r_2d on ft with the kx = nx/2 column set to zero (unnormalized). */
static void c2r_2d(orc_ctx* c, double* f) {
    const int nx = c->nx, ny = c->ny, hx = nx / 2;
    std::vector<cplx>& ft = c->ft;
#pragma omp parallel
    {
        std::vector<cplx> X(hx + 1), z(hx), col(ny);
#pragma omp for schedule(static)
        for (int kx = 0; kx < hx; ++kx) {
            for (int ky = 0; ky < ny; ++ky) col[ky] = ft[(size_t)ky * hx + kx];
            c->cy.run(col.data(), +1);
            for (int iy = 0; iy < ny; ++iy) ft[(size_t)iy * hx + kx] = col[iy];
        }
#pragma omp for schedule(static)
        for (int iy = 0; iy < ny; ++iy) {
            for (int kx = 0; kx < hx; ++kx) X[kx] = ft[(size_t)iy * hx + kx];
            X[hx] = {0.0, 0.0};
            c->rx.inverse(X.data(), f + (size_t)iy * nx, z.data());
        }
    }
}

static void coftxy(orc_ctx* c, const double* f, double* fk) {
    const int nx = c->nx, ny = c->ny, hx = nx / 2;
    r2c_2d(c, f);
    const std::vector<cplx>& ft = c->ft;
    const double norm = 1.0 / ((double)nx * (double)ny);
#define FT(kx, ky) ft[(size_t)(ky) * hx + (kx)]
    for (int ix = 0; ix < hx; ++ix) {
        F2(fk, 2 * ix, 0) = FT(ix, 0).re * norm;
        F2(fk, 2 * ix + 1, 0) = FT(ix, 0).im * norm;
        F2(fk, 2 * ix, 1) = 0.0;
        F2(fk, 2 * ix + 1, 1) = 0.0;
    }
#pragma omp parallel for schedule(static)
    for (int iy = 1; iy < ny / 2; ++iy) {
        for (int kx = 0; kx < hx; ++kx) {
            cplx p = FT(kx, iy), m = FT(kx, ny - iy);
            F2(fk, 2 * kx, 2 * iy) = 0.5 * (p.re + m.re) * norm;
            F2(fk, 2 * kx, 2 * iy + 1) = 0.5 * (p.im - m.im) * norm;
            F2(fk, 2 * kx + 1, 2 * iy) = 0.5 * (p.im + m.im) * norm;
            F2(fk, 2 * kx + 1, 2 * iy + 1) = 0.5 * (-p.re + m.re) * norm;
        }
    }
#undef FT
}

static void cofitxy(orc_ctx* c, const double* fk, double* f) {
    const int nx = c->nx, ny = c->ny, hx = nx / 2;
    std::vector<cplx>& ft = c->ft;
#define FT(kx, ky) ft[(size_t)(ky) * hx + (kx)]
    for (int ix = 0; ix < hx; ++ix) {
        FT(ix, 0) = {F2(fk, 2 * ix, 0), F2(fk, 2 * ix + 1, 0)};
        FT(ix, ny / 2) = {0.0, 0.0};
    }
#pragma omp parallel for schedule(static)
    for (int iy = 1; iy < ny / 2; ++iy) {
        for (int kx = 0; kx < hx; ++kx) {
            double a = F2(fk, 2 * kx, 2 * iy), b = F2(fk, 2 * kx, 2 * iy + 1);
            double cc = F2(fk, 2 * kx + 1, 2 * iy), d = F2(fk, 2 * kx + 1, 2 * iy + 1);
            FT(kx, iy) = {a - d, b + cc};
            FT(kx, ny - iy) = {a + d, -b + cc};
        }
    }
#undef FT
    c2r_2d(c, f);
}

/* ------------------------------------------------------------------------------
 * Spectral operators in the packed layout
 * ------------------------------------------------------------------------------ */

static void cofdx(orc_ctx* c, const double* fk, double* out) {  /* cofdx.f90:16-27 */
    const double scale1 = 2.0 * c->pi / c->P.xl;
#pragma omp parallel for schedule(static)
    for (int ky = 0; ky < c->ny; ++ky) {
        for (int kx = 0; kx <= c->nx - 2; kx += 2) F2(out, kx, ky) = -F2(fk, kx + 1, ky) * (double)(kx / 2) * scale1;
        for (int kx = 1; kx <= c->nx - 1; kx += 2) F2(out, kx, ky) = F2(fk, kx - 1, ky) * (double)((kx - 1) / 2) * scale1;
    }
}

static void cofdy(orc_ctx* c, const double* fk, double* out) {  /* cofdy.f90:16-28 */
    const double scale1 = 2.0 * c->pi / c->P.yl;
#pragma omp parallel for schedule(static)
    for (int ky = 0; ky < c->ny; ++ky) {
        for (int kx = 0; kx < c->nx; ++kx) {
            if ((ky & 1) == 0) F2(out, kx, ky) = -F2(fk, kx, ky + 1) * (double)(ky / 2) * scale1;
            else F2(out, kx, ky) = F2(fk, kx, ky - 1) * (double)((ky - 1) / 2) * scale1;
        }
    }
}

static void cofdxdx(orc_ctx* c, const double* fk, double* out) {  /* cofdxdx.f90:16-25 */
    const double t = 2.0 * c->pi / c->P.xl, scale = t * t;
    for (int ky = 0; ky < c->ny; ++ky)
        for (int kx = 0; kx <= c->nx - 2; kx += 2) {
            double k = (double)(kx / 2);
            F2(out, kx, ky) = -F2(fk, kx, ky) * (k * k) * scale;
            F2(out, kx + 1, ky) = -F2(fk, kx + 1, ky) * (k * k) * scale;
        }
}

static void cofdydy(orc_ctx* c, const double* fk, double* out) {  /* cofdydy.f90:16-25 */
    const double t = 2.0 * c->pi / c->P.yl, scale = t * t;
    for (int kx = 0; kx < c->nx; ++kx)
        for (int ky = 0; ky <= c->ny - 2; ky += 2) {
            double k = (double)(ky / 2);
            F2(out, kx, ky) = -F2(fk, kx, ky) * (k * k) * scale;
            F2(out, kx, ky + 1) = -F2(fk, kx, ky + 1) * (k * k) * scale;
        }
}

/* cofdxdy.f90:16-30.  NB: this returns MINUS d2/dxdy in the packed layout (it equals
 * -cofdx(cofdy(.))); the reference's sign is kept. */
static void cofdxdy(orc_ctx* c, const double* fk, double* out) {
    const double scale = (2.0 * c->pi / c->P.xl) * (2.0 * c->pi / c->P.yl);
    for (int ky = 0; ky <= c->ny / 2 - 1; ++ky)
        for (int kx = 0; kx <= c->nx / 2 - 1; ++kx) {
            double fac = -(double)kx * (double)ky * scale;
            F2(out, 2 * kx, 2 * ky) = fac * F2(fk, 2 * kx + 1, 2 * ky + 1);
            F2(out, 2 * kx + 1, 2 * ky) = -fac * F2(fk, 2 * kx, 2 * ky + 1);
            F2(out, 2 * kx, 2 * ky + 1) = -fac * F2(fk, 2 * kx + 1, 2 * ky);
            F2(out, 2 * kx + 1, 2 * ky + 1) = fac * F2(fk, 2 * kx, 2 * ky);
        }
}

static void poisson(orc_ctx* c, const double* f, double* ans) {  /* poisson.f90:10-29 */
#pragma omp parallel for schedule(static)
    for (int ky = 0; ky <= c->ny / 2 - 1; ++ky)
        for (int kx = 0; kx <= c->nx / 2 - 1; ++kx) {
            if (kx == 0 && ky == 0) {
                F2(ans, 0, 0) = 0.0; F2(ans, 1, 0) = 0.0; F2(ans, 0, 1) = 0.0; F2(ans, 1, 1) = 0.0;
            } else {
                double quot = ((double)(kx * kx) * c->scalex + (double)(ky * ky) * c->scaley);
                F2(ans, 2 * kx, 2 * ky) = F2(f, 2 * kx, 2 * ky) / quot;
                F2(ans, 2 * kx + 1, 2 * ky) = F2(f, 2 * kx + 1, 2 * ky) / quot;
                F2(ans, 2 * kx, 2 * ky + 1) = F2(f, 2 * kx, 2 * ky + 1) / quot;
                F2(ans, 2 * kx + 1, 2 * ky + 1) = F2(f, 2 * kx + 1, 2 * ky + 1) / quot;
            }
        }
}

static void vis(orc_ctx* c, double dt, double* work) {  /* cal_vis.f90:14-34 */
    const double coefx = -dt * c->P.nu * c->scalex, coefy = -dt * c->P.nu * c->scaley;
#pragma omp parallel for schedule(static)
    for (int ky = 0; ky <= c->ny / 2 - 1; ++ky)
        for (int kx = 0; kx <= c->nx / 2 - 1; ++kx) {
            double e = std::exp(coefx * (double)(kx * kx) + coefy * (double)(ky * ky));
            F2(work, 2 * kx, 2 * ky) = e;
            F2(work, 2 * kx + 1, 2 * ky) = e;
            F2(work, 2 * kx, 2 * ky + 1) = e;
            F2(work, 2 * kx + 1, 2 * ky + 1) = e;
        }
}

static void dealiase_mask(orc_ctx* c) {  /* dealiase_mask.f90:9-26 */
    const int kx_max = c->nx / 2 - 1, ky_max = c->ny / 2 - 1;
    const double kx_trunc = 2.0 / 3.0 * (double)kx_max, ky_trunc = 2.0 / 3.0 * (double)ky_max;
    std::fill(c->dealiase.begin(), c->dealiase.end(), 1.0);
    if (c->P.idealis != 1) return;
    for (int ky = 0; ky <= ky_max; ++ky)
        for (int kx = 0; kx <= kx_max; ++kx)
            if ((double)kx * (double)kx / (kx_trunc * kx_trunc) + (double)ky * (double)ky / (ky_trunc * ky_trunc) >= 1.0) {
                F2(c->dealiase, 2 * kx, 2 * ky) = 0.0; F2(c->dealiase, 2 * kx + 1, 2 * ky) = 0.0;
                F2(c->dealiase, 2 * kx, 2 * ky + 1) = 0.0; F2(c->dealiase, 2 * kx + 1, 2 * ky + 1) = 0.0;
            }
}

/* mean_velocity.f90:4-84 (iMeanVelocity 1,2,3,4,6,22; 11 needs u_mean, not on this path) */
static double Mean_Ux(const orc_ctx* c, double time) {
    const fsibe_params& P = c->P;
    double tf;
    switch (P.iMeanVelocity) {
    case 1:
        tf = (time < P.T_fullspeed) ? (time * time * time) / (-0.5 * P.T_fullspeed * P.T_fullspeed * P.T_fullspeed) + 3.0 * (time * time) / (P.T_fullspeed * P.T_fullspeed) : 1.0;
        return std::cos(P.theta_inf) * tf;
    case 2:
        tf = (time < P.T_fullspeed) ? 0.5 * (1.0 - std::cos(0.5 * c->pi * time / P.T_fullspeed)) : 1.0;
        return std::cos(P.theta_inf) * tf;
    case 3: return std::cos(P.theta_inf);
    case 4: return 0.0;
    case 6: return time;
    case 22: return 0.1;
    default: return 0.0;
    }
}
static double Mean_Uy(const orc_ctx* c, double time) {
    const fsibe_params& P = c->P;
    double tf;
    switch (P.iMeanVelocity) {
    case 1:
        tf = (time < P.T_fullspeed) ? (time * time * time) / (-0.5 * P.T_fullspeed * P.T_fullspeed * P.T_fullspeed) + 3.0 * (time * time) / (P.T_fullspeed * P.T_fullspeed) : 1.0;
        return std::sin(P.theta_inf) * tf;
    case 2:
        tf = (time < P.T_fullspeed) ? 0.5 * (1.0 - std::cos(0.5 * c->pi * time / P.T_fullspeed)) : 1.0;
        return std::sin(P.theta_inf) * tf;
    case 3: return std::sin(P.theta_inf);
    default: return 0.0;
    }
}

/* ------------------------------------------------------------------------------
 * Motion and beam kinematics
 * ------------------------------------------------------------------------------ */

/* mouvement case 0, clamped leading edge (mouvement.f90:19-28). */
/* The heaving periods of mouvement cases 201-213 (and 300-350: 1.62) and 401-413. */
static const double kHeaveT[13] = {1.0, 1.09, 1.20, 1.29, 1.33, 1.4, 1.5, 1.71, 2.0, 2.4, 3.0, 4.0, 1.62};
static const double kParazT[13] = {0.51, 0.34, 0.25, 0.20, 0.17, 0.14, 0.13, 0.11, 0.10, 0.09, 0.08, 0.08, 0.07};

/* mouvement.f90:5-200: the leading edge's prescribed motion.  LE = x, y, vx, vy, ax, ay. */
static void mouvement(const orc_ctx* c, double time, double& alpha, double& alpha_t, double& alpha_tt, double LE[6],
                      const Beam& b) {
    const double pi = c->pi;
    const int m = c->P.iMotion;
    for (int i = 0; i < 6; ++i) LE[i] = 0.0;
    LE[0] = b.x0;
    LE[1] = b.y0;
    alpha = b.AngleBeam * pi / 180.0;
    alpha_t = 0.0;
    alpha_tt = 0.0;
    if ((m >= 201 && m <= 213) || (m >= 300 && m <= 350)) {  /* :29-76, heaving with a soft start */
        const double y_max = 0.5, t_max = (m < 300) ? kHeaveT[m - 201] : 1.62;
        double k = 1.0, kt = 0.0, ktt = 0.0;
        if (time <= 1.0) {
            const double a = -20.0, bb = 70.0, cc = -84.0, d = 35.0, t = time;
            const double t2 = t * t, t3 = t2 * t, t4 = t3 * t, t5 = t4 * t, t6 = t5 * t, t7 = t6 * t;
            k = a * t7 + bb * t6 + cc * t5 + d * t4;
            kt = 7.0 * a * t6 + 6.0 * bb * t5 + 5.0 * cc * t4 + 4.0 * d * t3;
            ktt = 42. * a * t5 + 30. * bb * t4 + 20. * cc * t3 + 12. * d * t2;
        }
        const double w = 2.0 * pi / t_max, arg = 2.0 * pi * time / t_max + pi / 2. + b.phase;
        const double y = y_max * std::sin(arg), yt = y_max * w * std::cos(arg), ytt = -y_max * (w * w) * std::sin(arg);
        LE[1] = b.y0 + k * y;
        LE[3] = kt * y + yt * k;
        LE[5] = ktt * y + ytt * k + 2. * kt * yt;
    } else if ((m >= 401 && m <= 413) || m == 2) {  /* :77-114 (Paraz), :116-130 (hard start) */
        const double y_max = (m == 2) ? 0.5 : 0.0333, t_max = (m == 2) ? 2.5 : kParazT[m - 401];
        const double w = 2.0 * pi / t_max, arg = 2.0 * pi * time / t_max + pi / 2;
        LE[1] = b.y0 + y_max * std::sin(arg);
        LE[3] = y_max * w * std::cos(arg);
        LE[5] = -y_max * (w * w) * std::sin(arg);
    } else if (m == 3) {  /* :131-143, flapping */
        const double angle_max = 80.0 * pi / 180.0, f = 0.5, w = 2.0 * pi * f;
        alpha = angle_max * std::sin(w * time);
        alpha_t = angle_max * std::cos(w * time) * w;
        alpha_tt = -1.0 * angle_max * std::sin(w * time) * (w * w);
    } else if (m == 4) {  /* :144-155, impulsive translation */
        const double u0 = -1.0;
        LE[0] = b.x0 + u0 * time;
        LE[2] = u0;
    }
}

/* integrate_position.f90:14-44: running sums of cos/sin(theta)*ds, rotated by alpha. */
static void integrate_position(const orc_ctx* c, double time, Beam& b) {
    double alpha, alpha_t, alpha_tt, LE[6];
    mouvement(c, time, alpha, alpha_t, alpha_tt, LE, b);
    const int ns = c->ns;
    const double ds = c->ds;
    double xrel = 0, yrel = 0, vxrel = 0, vyrel = 0;
    for (int s = 0; s < ns; ++s) {
        if (s > 0) {
            int i = s - 1;
            xrel = xrel + std::cos(b.theta[i]) * ds;
            yrel = yrel + std::sin(b.theta[i]) * ds;
            vxrel = vxrel - b.theta_dot[i] * std::sin(b.theta[i]) * ds;
            vyrel = vyrel + b.theta_dot[i] * std::cos(b.theta[i]) * ds;
        }
        const double ca = std::cos(alpha), sa = std::sin(alpha);
        b.x[s] = LE[0] + xrel * ca - yrel * sa;
        b.y[s] = LE[1] + yrel * ca + xrel * sa;
        b.vx[s] = LE[2] + ca * (vxrel - alpha_t * yrel) - sa * (vyrel + alpha_t * xrel);
        b.vy[s] = LE[3] + ca * (vyrel + alpha_t * xrel) + sa * (vxrel - alpha_t * yrel);
    }
}

/* init_beam.f90:24-120 (one beam) */
static void init_beams(orc_ctx* c) {
    Beam& b = c->beam;
    b = Beam();
    b.alloc(c->ns);
    b.x0 = c->P.x0;
    b.y0 = c->P.y0;
    b.iMouvement = c->P.iMotion;
    b.AngleBeam = c->P.angle_beam;
    b.phase = 0.0;
    double alpha, alpha_t, alpha_tt, LE[6];
    mouvement(c, 0.0, alpha, alpha_t, alpha_tt, LE, b);
    b.StartupStep = true;
    b.UnstReady = false;
    for (int n = 0; n < c->ns; ++n) {
        b.x[n] = LE[0] + (double)n * c->ds;
        b.y[n] = LE[1];
    }
    integrate_position(c, 0.0, b);
}

/* ------------------------------------------------------------------------------
 * Mask rasterisation (create_mask.f90)
 * ------------------------------------------------------------------------------ */

static inline double SmoothStep(const orc_ctx* c, double x, double t, double h) {  /* create_mask.f90:475-520 */
    if (!c->sharp) {
        const double GradientERF = std::fabs((std::exp(-(2.0 * 1.0) * (2.0 * 1.0)) - 1.0) / std::sqrt(c->pi));
        const double delta = h * GradientERF;
        return 0.5 * (std::erf((t - x) / delta) + std::erf((x + t) / delta));
    }
    return (x <= t) ? 1.0 : 0.0;
}

static inline double SmoothStep2(const orc_ctx* c, double x, double t, double h) {  /* create_mask.f90:523-545 */
    if (x <= t - h) return 1.0;
    if ((t - h) < x && x < (t + h)) return 0.5 * (1. + std::cos((x - t + h) * c->pi / (2.0 * h)));
    return 0.0;
}

static inline double ConvertAngle(const orc_ctx* c, double a) { return (a < 0.0) ? 2.0 * c->pi + a : a; }

static inline long nint(double v) { return std::lround(v); }

static void DrawBeamSegment(orc_ctx* c, double p1x, double p1y, double p2x, double p2y, double v1x, double v1y,
                            double v2x, double v2y, double t, double N) {  /* create_mask.f90:708-780 */
    const double dx = c->dx, dy = c->dy;
    const double t_star = t + 2.0 * N * std::max(dx, dy);
    const double alpha = -std::atan2((p2y - p1y), (p2x - p1x));
    long ixmin = nint((std::min(p1x, p2x) - t_star) / dx), ixmax = nint((std::max(p1x, p2x) + t_star) / dx);
    long iymin = nint((std::min(p1y, p2y) - t_star) / dy), iymax = nint((std::max(p1y, p2y) + t_star) / dy);
    ixmin = std::max(ixmin, 0L); ixmax = std::min(ixmax, (long)c->nx - 1);
    iymin = std::max(iymin, 0L); iymax = std::min(iymax, (long)c->ny - 1);
    const double ca = std::cos(alpha), sa = std::sin(alpha);
    const double p1s0 = ca * p1x - sa * p1y, p1s1 = sa * p1x + ca * p1y;
    const double p2s0 = ca * p2x - sa * p2y, p2s1 = sa * p2x + ca * p2y;
    const double h = N * std::max(dx, dy);
#pragma omp parallel for schedule(static)
    for (long i = ixmin; i <= ixmax; ++i)
        for (long j = iymin; j <= iymax; ++j) {
            double x_star = (double)i * dx * ca - (double)j * dy * sa;
            double y_star = (double)i * dx * sa + (double)j * dy * ca;
            if (x_star >= p1s0 && x_star <= p2s0 && y_star <= p1s1 + t_star && y_star >= p2s1 - t_star) {
                double temp = SmoothStep(c, std::fabs(y_star - p1s1), t, h);
                if (temp > F2(c->mask, i, j)) {
                    F2(c->mask, i, j) = temp;
                    F2(c->maskvx, i, j) = (v1x + (x_star - p1s0) * (v2x - v1x) / c->ds);
                    F2(c->maskvy, i, j) = (v1y + (x_star - p1s0) * (v2y - v1y) / c->ds);
                }
            }
        }
}

static void DrawSharpEnd(orc_ctx* c, double pex, double pey, double alpha, double vx, double vy, double t,
                         double N) {  /* create_mask.f90:784-852 */
    const double dx = c->dx, dy = c->dy, mx = std::max(dx, dy);
    const double t_star = t + 2.0 * N * mx;
    const double ca = std::cos(alpha), sa = std::sin(alpha);
    const double p1x = pex - 2.0 * mx * ca, p1y = pey - 2.0 * mx * sa;
    const double p2x = pex + 4.0 * mx * ca, p2y = pey + 4.0 * mx * sa;
    long ixmin = nint((std::min(p1x, p2x) - t_star) / dx), ixmax = nint((std::max(p1x, p2x) + t_star) / dx);
    long iymin = nint((std::min(p1y, p2y) - t_star) / dy), iymax = nint((std::max(p1y, p2y) + t_star) / dy);
    ixmin = std::max(ixmin, 0L); ixmax = std::min(ixmax, (long)c->nx - 1);
    iymin = std::max(iymin, 0L); iymax = std::min(iymax, (long)c->ny - 1);
    const double p1s0 = ca * p1x + sa * p1y, p1s1 = -sa * p1x + ca * p1y;
    const double p2s0 = ca * p2x + sa * p2y, p2s1 = -sa * p2x + ca * p2y;
    for (long i = ixmin; i <= ixmax; ++i)
        for (long j = iymin; j <= iymax; ++j) {
            double x_star = (double)i * dx * ca + (double)j * dy * sa;
            double y_star = -(double)i * dx * sa + (double)j * dy * ca;
            if (x_star >= p1s0 && x_star <= p2s0 && y_star <= p1s1 + t_star && y_star >= p2s1 - t_star) {
                double tmp2 = SmoothStep(c, x_star - p1s0, 2.0 * mx, N * mx);
                double temp = SmoothStep(c, std::fabs(y_star - p1s1), t, N * mx);
                F2(c->mask, i, j) = temp * tmp2;
                if (x_star - p1s0 >= 2.0 * mx) {
                    F2(c->maskvx, i, j) = vx;
                    F2(c->maskvy, i, j) = vy;
                }
            }
        }
}

static void DrawHinge(orc_ctx* c, double px, double py, double alpha1, double alpha2, double vx, double vy, double t,
                      double N) {  /* create_mask.f90:563-656 */
    const double dx = c->dx, dy = c->dy, mx = std::max(dx, dy);
    const double t_star = t + 2. * N * mx;
    long ixmin = nint((px - t_star) / dx), ixmax = nint((px + t_star) / dx);
    long iymin = nint((py - t_star) / dy), iymax = nint((py + t_star) / dy);
    ixmin = std::max(ixmin, 0L); ixmax = std::min(ixmax, (long)c->nx - 1);
    iymin = std::max(iymin, 0L); iymax = std::min(iymax, (long)c->ny - 1);
    const double beta1 = ConvertAngle(c, alpha1) * 180.0 / c->pi;
    const double beta2 = ConvertAngle(c, alpha2) * 180.0 / c->pi;
    for (long i = ixmin; i <= ixmax; ++i)
        for (long j = iymin; j <= iymax; ++j) {
            double R = std::sqrt(((double)i * dx - px) * ((double)i * dx - px) + ((double)j * dy - py) * ((double)j * dy - py));
            if (R <= t_star) {
                double gamma = std::atan2(((double)j * dy - py), ((double)i * dx - px));
                gamma = ConvertAngle(c, gamma) * 180.0 / c->pi;
                bool inside1 = false, inside2 = false;
                if (beta1 < 90.0) {
                    if ((gamma >= 0.0 && gamma <= 90.0 + beta1) || (gamma >= 270.0 + beta1 && gamma <= 360.0)) inside1 = true;
                } else if (beta1 >= 90.0 && beta1 < 270.0) {
                    if (gamma >= 270.0 + beta1 - 360.0 && gamma <= 90.0 + beta1) inside1 = true;
                } else if (beta1 >= 270.0) {
                    if ((gamma >= 0.0 && gamma <= 90.0 + beta1 - 360.0) || (gamma >= 270.0 + beta1 - 360.0 && gamma <= 360.0)) inside1 = true;
                }
                if (beta2 <= 90.0) {
                    if (gamma >= 90.0 + beta2 && gamma < 270.0 + beta2) inside2 = true;
                } else if (beta2 >= 90.0 && beta2 < 270.0) {
                    if ((gamma >= 0.0 && gamma <= 270.0 + beta2 - 360.0) || (gamma >= 90.0 + beta2 && gamma <= 360.0)) inside2 = true;
                } else if (beta2 >= 270.0) {
                    if (gamma >= 90.0 + beta2 - 360.0 && gamma < 270.0 + beta2 - 360.0) inside2 = true;
                }
                if (inside2 && inside1) {
                    double temp = SmoothStep(c, R, t, N * mx);
                    if (temp > F2(c->mask, i, j)) {
                        F2(c->mask, i, j) = temp;
                        F2(c->maskvx, i, j) = vx;
                        F2(c->maskvy, i, j) = vy;
                    }
                }
            }
        }
}

static int DrawADot(orc_ctx* c, double px, double py, double vx, double vy, double t, double N) {  /* create_mask.f90:663-704 */
    const double dx = c->dx, dy = c->dy, mx = std::max(dx, dy);
    if (py < 0.0) return fail(c, FSIBE_ERR_MASK_OOB, "Mask:: Beam Hinge. Index out of region");
#pragma omp parallel for schedule(static)
    for (int i = 0; i < c->nx; ++i)
        for (int j = 0; j < c->ny; ++j) {
            double R = std::sqrt(((double)i * dx - px) * ((double)i * dx - px) + ((double)j * dy - py) * ((double)j * dy - py));
            double temp = SmoothStep(c, R, t, N * mx);
            if (temp > F2(c->mask, i, j)) {
                F2(c->mask, i, j) = temp;
                F2(c->maskvx, i, j) = vx;
                F2(c->maskvy, i, j) = vy;
            }
        }
    return FSIBE_OK;
}

/* SmoothFrameAroundDomain (create_mask.f90:370-470): a level set phi of the distance to the
 * domain's edges with rounded corners, smoothed into a frame mask of the thickness 4 t_beam. */
static void SmoothFrameAroundDomain(orc_ctx* c, std::vector<double>& mask1) {
    const int nx = c->nx, ny = c->ny;
    const double dx = c->dx, dy = c->dy, xl = c->P.xl, yl = c->P.yl;
    std::vector<double> phi((size_t)nx * ny, 1000.0);
    const double thickness = 4.0 * c->P.t_beam, R1 = 0.0, R2 = 2.0 * thickness, RR = R1 + R2;
    const long ixmin = nint(RR / dx), ixmax = nx - nint(RR / dx), iymin = nint(RR / dy), iymax = ny - nint(RR / dy);
#define PHI(ix, iy) phi[(size_t)(iy) * nx + (ix)]
    for (long ix = ixmin; ix <= ixmax; ++ix)
        for (long iy = 0; iy <= ny - 1; ++iy) {
            const double y = (double)iy * dy;
            const double m = std::min(PHI(ix, iy), std::min(std::fabs(y - R1), std::fabs(y - (yl - R1))));
            PHI(ix, iy) = ((iy <= nint(R1 / dy)) || (iy >= ny - 1 - nint(R1 / dy))) ? -m : +m;
        }
    for (long ix = 0; ix <= nx - 1; ++ix)
        for (long iy = iymin; iy <= iymax; ++iy) {
            const double x = (double)ix * dx;
            const double m = std::min(PHI(ix, iy), std::min(std::fabs(x - R1), std::fabs(x - (xl - R1))));
            PHI(ix, iy) = ((ix <= nint(R1 / dx)) || (ix >= nx - 1 - nint(R1 / dx))) ? -m : +m;
        }
    auto corner = [&](long x0_, long x1_, long y0_, long y1_, double cx, double cy) {
        for (long ix = x0_; ix <= x1_; ++ix)
            for (long iy = y0_; iy <= y1_; ++iy) {
                const double x = (double)ix * dx, y = (double)iy * dy;
                PHI(ix, iy) = std::min(PHI(ix, iy), -(std::sqrt((x - cx) * (x - cx) + (y - cy) * (y - cy)) - R2));
            }
    };
    corner(0, ixmin, 0, iymin, RR, RR);
    corner(0, ixmin, iymax, ny - 1, RR, yl - RR);
    corner(ixmax, nx - 1, iymax, ny - 1, xl - RR, yl - RR);
    corner(ixmax, nx - 1, 0, iymin, xl - RR, RR);
    for (size_t k = 0; k < phi.size(); ++k) mask1[k] = SmoothStep2(c, phi[k], thickness / 2., thickness / 2.);
#undef PHI
}

static int create_mask(orc_ctx* c, double time) {  /* create_mask.f90:2-218 */
    const double N = c->P.N_smooth, dx = c->dx, dy = c->dy, yl = c->P.yl;
    std::fill(c->mask.begin(), c->mask.end(), 0.0);
    std::fill(c->maskvx.begin(), c->maskvx.end(), 0.0);
    std::fill(c->maskvy.begin(), c->maskvy.end(), 0.0);
    if (c->P.iWalls > 0) {  /* :30-54, walls in the y direction */
        const double h = c->P.h_channel, h_star = h + N * dy;
        for (long j = 0; j <= nint(h_star / dy); ++j) {
            const double temp = SmoothStep(c, (double)j * dy, h, N * dy);
            for (int i = 0; i < c->nx; ++i) F2(c->mask, i, j) = temp;
        }
        for (long j = c->ny - 1; j >= nint((yl - h_star) / dy); --j) {
            const double temp = SmoothStep(c, std::fabs((double)j * dy - yl), h, N * dy);
            for (int i = 0; i < c->nx; ++i) F2(c->mask, i, j) = temp;
        }
    }
    if (c->P.iCylinder == 1) {  /* :66-68 */
        const int st = DrawADot(c, c->P.x0 - c->P.R_cylinder, c->P.y0, 0.0, 0.0, c->P.R_cylinder, N);
        if (st) return st;
    }
    if (c->P.iBeam > 0) {
        Beam& b = c->beam;
        double alpha, alpha_t, alpha_tt, LE[6];
        mouvement(c, time, alpha, alpha_t, alpha_tt, LE, b);
        const int ns = c->ns;
        for (int i = 0; i <= ns - 2; ++i)
            DrawBeamSegment(c, b.x[i], b.y[i], b.x[i + 1], b.y[i + 1], b.vx[i], b.vy[i], b.vx[i + 1], b.vy[i + 1], c->P.t_beam, N);
        if (c->P.iSharpTrailing == 1)
            DrawSharpEnd(c, b.x[ns - 1], b.y[ns - 1], b.theta[ns - 1] + alpha, b.vx[ns - 1], b.vy[ns - 1], c->P.t_beam, N);
        for (int i = 1; i <= ns - 2; ++i) {
            double a1 = std::atan2((b.y[i] - b.y[i - 1]), (b.x[i] - b.x[i - 1]));
            double a2 = std::atan2((b.y[i + 1] - b.y[i]), (b.x[i + 1] - b.x[i]));
            DrawHinge(c, b.x[i], b.y[i], a1, a2, b.vx[i], b.vy[i], c->P.t_beam, N);
        }
        int st = DrawADot(c, b.x[0], b.y[0], b.vx[0], b.vy[0], c->P.t_beam, N);
        if (st) return st;
        if (c->P.iSharpTrailing == 0) {
            st = DrawADot(c, b.x[ns - 1], b.y[ns - 1], b.vx[ns - 1], b.vy[ns - 1], c->P.t_beam, N);
            if (st) return st;
        }
    }
    if (c->P.iSponge == 4) {  /* :131-181, velocity sponge at the inflow with a channel profile */
        const double sss = c->P.SpongeSize, ss = sss - 2.0 * N * dx, H_eff = yl - 2.0 * c->P.h_channel;
        const double U = Mean_Ux(c, time);
        auto column = [&](long ix, double x, double t, double h) {
            const double tmp = SmoothStep(c, x, t, h);
            for (int iy = 0; iy < c->ny; ++iy) {
                const double y_chan = (double)iy * dy - c->P.h_channel;
                if (F2(c->mask, ix, iy) < tmp) F2(c->mask, ix, iy) = tmp;
                F2(c->maskvx, ix, iy) = (y_chan > 0.0 && y_chan < H_eff)
                    ? 1.5 * U * y_chan * (H_eff - y_chan) / ((0.5 * H_eff) * (0.5 * H_eff)) : 0.0;
            }
        };
        for (long ix = 0; ix <= nint((0.5 * sss) / dx); ++ix) column(ix, 0.75 * sss - (double)ix * dx, ss * 0.5, 0.25 * ss);
        for (long ix = nint((0.5 * sss) / dx); ix <= nint((1.0 * sss) / dx); ++ix)
            column(ix, (double)ix * dx - 0.5 * sss, ss * 0.5, N * dx);
    }
    if (c->P.iSponge == 22) {  /* :188-204, the frame around the domain */
        if (*std::max_element(c->mask_frame.begin(), c->mask_frame.end()) < 1.0) SmoothFrameAroundDomain(c, c->mask_frame);
        const double f = c->P.eps / std::max(1.0e-3, c->P.eps);
        const double U = Mean_Ux(c, time), V = Mean_Uy(c, time);
        for (size_t k = 0; k < c->mask.size(); ++k) {
            c->mask[k] = c->mask[k] + c->mask_frame[k] * f;
            if (c->mask_frame[k] > 0.0) { c->maskvx[k] = U; c->maskvy[k] = V; }
        }
    }
    for (size_t k = 0; k < c->mask.size(); ++k) c->mask[k] = c->mask[k] / c->P.eps;
    return FSIBE_OK;
}

/* create_sponge_mask (create_mask.f90:223-364), once after the start-up mask: the vorticity
 * sponge of iSponge 1 (outflow), 2 (inflow, outside the obstacle), 3 (around the domain) and
 * 22 (a frame with a hole, outside the obstacle), divided by eps_sponge. */
static void create_sponge_mask(orc_ctx* c) {
    const double N = c->P.N_smooth, dx = c->dx, dy = c->dy, xl = c->P.xl, yl = c->P.yl, sss = c->P.SpongeSize;
    std::vector<double>& ms = c->mask_sponge;
    std::fill(ms.begin(), ms.end(), 0.0);
    const int isp = c->P.iSponge;
    if (isp == 1) {
        const double ss = sss - 2.0 * N * dx, begin = xl - sss;
        for (long ix = nint(begin / dx); ix <= nint((xl - 0.5 * sss) / dx); ++ix) {
            const double tmp = SmoothStep(c, xl - 0.5 * sss - (double)ix * dx, ss * 0.5, N * dx);
            for (int iy = 0; iy < c->ny; ++iy) F2(ms, ix, iy) = tmp;
        }
        for (long ix = nint((xl - 0.5 * sss) / dx); ix <= c->nx - 1; ++ix) {
            const double tmp = SmoothStep(c, (double)ix * dx - xl + 0.5 * sss - 1.0 * dx, ss * 0.4, N * dx);
            for (int iy = 0; iy < c->ny; ++iy) F2(ms, ix, iy) = tmp;
        }
    } else if (isp == 2) {
        const double ss = sss - 2.0 * N * dx;
        const long ixmax = nint((1.0 * sss) / dx);
        for (long ix = 0; ix <= nint((0.5 * sss) / dx); ++ix) {
            const double tmp = SmoothStep(c, 0.5 * sss - (double)ix * dx, ss * 0.5, N * dx);
            for (int iy = 0; iy < c->ny; ++iy) F2(ms, ix, iy) = tmp;
        }
        for (long ix = nint((0.5 * sss) / dx); ix <= ixmax; ++ix) {
            const double tmp = SmoothStep(c, (double)ix * dx - 0.5 * sss, ss * 0.5, N * dx);
            for (int iy = 0; iy < c->ny; ++iy) F2(ms, ix, iy) = tmp;
        }
        for (long ix = 0; ix <= ixmax; ++ix)
            for (int iy = 0; iy < c->ny; ++iy)
                if (F2(c->mask, ix, iy) * c->P.eps > 0.0) F2(ms, ix, iy) = F2(ms, ix, iy) * (1.0 - F2(c->mask, ix, iy) * c->P.eps);
    } else if (isp == 3) {
        const double ss = sss - N * dx;
        for (int ix = 0; ix < c->nx; ++ix)
            for (int iy = 0; iy < c->ny; ++iy) {
                const double t1 = SmoothStep(c, (double)ix * dx, ss, N * dx), t2 = SmoothStep(c, xl - (double)ix * dx, ss, N * dx);
                const double t3 = SmoothStep(c, (double)iy * dy, ss, N * dy), t4 = SmoothStep(c, yl - (double)iy * dy, ss, N * dy);
                F2(ms, ix, iy) = std::min(t1 + t2 + t3 + t4, 1.0);
            }
    } else if (isp == 22) {
        const long ixmin = nint(sss / dx), iymin = nint(sss / dy), ixmax = nint((xl - sss) / dx), iymax = nint((yl - sss) / dy);
        for (int ix = 0; ix < c->nx; ++ix)
            for (int iy = 0; iy < c->ny; ++iy) {
                const bool hole = ix >= ixmin && ix <= ixmax && iy >= iymin && iy <= iymax;
                F2(ms, ix, iy) = (hole || F2(c->mask, ix, iy) > 0.0) ? 0.0 : 1.0;
            }
    } else if (isp == 10) {  /* :276-281, the sharp outflow sponge */
        for (long ix = nint((xl - sss) / dx); ix <= c->nx - 1; ++ix)
            for (int iy = 0; iy < c->ny; ++iy) F2(ms, ix, iy) = 1.0;
    }
    for (double& v : ms) v = v / c->P.eps_sponge;
}

/* ------------------------------------------------------------------------------
 * Spectral fluid solver (NavierStokes.f90)
 * ------------------------------------------------------------------------------ */

static void cal_velocity(orc_ctx* c, double time, const double* vortk, double* u, double* stream) {  /* :181-212 */
    const size_t NN = (size_t)c->nx * c->ny;
    std::vector<double> work2(NN);
    poisson(c, vortk, stream);
    cofdx(c, stream, work2.data());
    cofitxy(c, work2.data(), u + NN);
    cofdy(c, stream, work2.data());
    cofitxy(c, work2.data(), u);
    const double mux = c->U_mean_true * Mean_Ux(c, time), muy = c->U_mean_true * Mean_Uy(c, time);
#pragma omp parallel for schedule(static)
    for (size_t k = 0; k < NN; ++k) {
        u[k] = u[k] + mux;
        u[NN + k] = -u[NN + k] + muy;
    }
}

static void cal_nlk(orc_ctx* c, double time, double& dt1, double* nlk, const double* vortk, const double* u) {  /* :9-177 */
    const size_t NN = (size_t)c->nx * c->ny;
    const double dx = c->dx, dy = c->dy;
    std::vector<double> vort_dx(NN), vort_dy(NN), work2(NN), pen1(NN), pen2(NN);
    cofdx(c, vortk, work2.data());
    cofitxy(c, work2.data(), vort_dx.data());
    cofdy(c, vortk, work2.data());
    cofitxy(c, work2.data(), vort_dy.data());
#pragma omp parallel for schedule(static)
    for (size_t k = 0; k < NN; ++k) work2[k] = -u[k] * vort_dx[k] - u[NN + k] * vort_dy[k];
    coftxy(c, work2.data(), nlk);
    double m = 0.0, su = 0.0, sv = 0.0;
    for (size_t k = 0; k < NN; ++k) {
        double w = u[k] * u[k] + u[NN + k] * u[NN + k];
        if (k == 0 || w > m) m = w;
    }
    for (size_t k = 0; k < NN; ++k) { su += u[k]; sv += u[NN + k]; }
    const double u_max = std::sqrt(m);
    dt1 = c->P.cfl * std::min(dx, dy) / u_max;
    if (u_max < 1.e-10) dt1 = 1.e-2;
    if (c->P.iBeam > 0 || c->P.iWalls > 0 || c->P.iCylinder > 0) dt1 = std::min(0.9 * c->P.eps, dt1);
    if (c->P.dt_fixed > 0.0) dt1 = std::min(c->P.dt_fixed, dt1);
    if ((c->P.time_end - time) < dt1) dt1 = c->P.time_end - time;
    c->sc.u_max = u_max;
    c->sc.mean_ux = su / (double)NN;
    c->sc.mean_uy = sv / (double)NN;
    if (c->P.iBeam > 0 || c->P.iWalls > 0 || c->P.iCylinder > 0 || c->P.iSponge == 22) {
#pragma omp parallel for schedule(static)
        for (size_t k = 0; k < NN; ++k) {
            pen1[k] = -c->mask[k] * (u[k] - c->maskvx[k]);
            pen2[k] = -c->mask[k] * (u[NN + k] - c->maskvy[k]);
        }
        if (c->P.iSponge == 10) {  /* :103-122: the integral along x of -mask_sponge du/dx */
            std::vector<double> wk(NN), dk(NN);
            coftxy(c, u, wk.data());
            cofdx(c, wk.data(), dk.data());
            cofitxy(c, dk.data(), work2.data());
            for (size_t k = 0; k < NN; ++k) work2[k] = -c->mask_sponge[k] * work2[k];
            const long ixmin = nint((c->P.xl - c->P.SpongeSize) / dx), ixmax = c->nx - 1 - 15;
#pragma omp parallel for schedule(static)
            for (int iy = 0; iy < c->ny; ++iy) {
                // the reference sums from ixmin for every ix; the running sum adds the same
                // terms in the same order
                double summe = 0.0;
                for (long ix = ixmin; ix <= ixmax; ++ix) {
                    if (ix > ixmin) summe = summe + 0.5 * (F2(work2, ix - 1, iy) + F2(work2, ix, iy)) * dx;
                    F2(pen1, ix, iy) = F2(pen1, ix, iy) + summe;
                }
            }
        }
        coftxy(c, pen2.data(), work2.data());
        cofdx(c, work2.data(), pen2.data());
        coftxy(c, pen1.data(), work2.data());
        cofdy(c, work2.data(), pen1.data());
    } else {
        std::fill(pen1.begin(), pen1.end(), 0.0);
        std::fill(pen2.begin(), pen2.end(), 0.0);
    }
#pragma omp parallel for schedule(static)
    for (size_t k = 0; k < NN; ++k) nlk[k] = nlk[k] + (pen2[k] - pen1[k]);
    const int isp = c->P.iSponge;
    if ((isp > 0 && isp < 4) || isp == 22) {  /* :142-160, the vorticity sponge */
        std::vector<double> penvortk(NN);
        cofitxy(c, vortk, work2.data());
#pragma omp parallel for schedule(static)
        for (size_t k = 0; k < NN; ++k) work2[k] = c->mask_sponge[k] * work2[k];
        coftxy(c, work2.data(), penvortk.data());
#pragma omp parallel for schedule(static)
        for (size_t k = 0; k < NN; ++k) nlk[k] = nlk[k] - penvortk[k];
    }
}

static void cal_energy(orc_ctx* c, double time, double dt1, const double* vor, const double* u, const double* pen) {  /* :222-263 */
    const size_t NN = (size_t)c->nx * c->ny;
    const double dx = c->dx, dy = c->dy;
    const double mux = Mean_Ux(c, time + dt1), muy = Mean_Uy(c, time + dt1);
    double s1 = 0, s2 = 0, s4 = 0, s5 = 0, s6 = 0;
    for (size_t k = 0; k < NN; ++k) {
        s1 += vor[k] * vor[k];
        s2 += ((u[k] - mux) * (u[k] - mux) + (u[NN + k] - muy) * (u[NN + k] - muy));
        double rx = u[k] - c->maskvx[k], ry = u[NN + k] - c->maskvy[k];
        s4 += c->mask[k] * (rx * rx + ry * ry);
        s5 += c->mask[k] * (c->maskvx[k] * rx + c->maskvy[k] * ry);
        s6 += mux * pen[k] + muy * pen[NN + k];
    }
    c->sc.vor_rms = dx * dy * std::sqrt(s1);
    c->sc.kinetic = 0.5 * dx * dy * s2;
    c->sc.dissipation = c->P.nu * dx * dy * s1;
    c->sc.porous_diss = dx * dy * s4;
    c->sc.inflow_solid = dx * dy * s5;
    c->sc.inflow_mean = dx * dy * c->U_mean_true * s6;
}

static void cal_drag(orc_ctx* c, double time, double dt1, const double* pen) {  /* :512-593 */
    const size_t NN = (size_t)c->nx * c->ny;
    const double dx = c->dx, dy = c->dy, norm = dx * dy;
    Beam& b = c->beam;
    double alpha, alpha_t, alpha_tt, LE[6];
    mouvement(c, time, alpha, alpha_t, alpha_tt, LE, b);
    const double r_cylinder = c->P.R_cylinder, tb = c->P.t_beam;
    double ymax = *std::max_element(b.y.begin(), b.y.end()), ymin = *std::min_element(b.y.begin(), b.y.end());
    double xmax = *std::max_element(b.x.begin(), b.x.end()), xmin = *std::min_element(b.x.begin(), b.x.end());
    long iymax = (long)((std::max(ymax + 1.5 * tb, LE[1] + 2.0 * r_cylinder)) / dy);
    long iymin = (long)((std::min(ymin - 1.5 * tb, LE[1] - 2.0 * r_cylinder)) / dy);
    long ixmin = (long)(std::min((LE[0] - std::max(2.5 * r_cylinder, 1.5 * tb)), (xmin - 1.5 * tb)) / dx);
    long ixmax = (long)((xmax + 1.5 * tb) / dx);
    if (c->P.iWalls > 0) {  /* :546-552, the window stays off the walls */
        const double h_star = c->P.h_channel + c->P.N_smooth * dy;
        if (ixmin < 0) ixmin = 0;
        if (ixmax > c->nx - 1) ixmax = c->nx - 1;
        if (iymin < nint(h_star / dy) + 2) iymin = nint(h_star / dy) + 2;
        if (iymax > nint((c->P.yl - h_star) / dy) - 2) iymax = nint((c->P.yl - h_star) / dy) - 2;
    }
    if (ixmin < 0) ixmin = 0;
    if (ixmax > c->nx - 1) ixmax = c->nx - 1;
    if (iymin < 0) iymin = 0;
    if (iymax > c->ny - 1) iymax = c->ny - 1;
    double f1 = 0, f2 = 0, d1 = 0, d2 = 0;
    for (long iy = iymin; iy <= iymax; ++iy)
        for (long ix = ixmin; ix <= ixmax; ++ix) {
            size_t k = (size_t)iy * c->nx + ix;
            f1 += pen[k];
            f2 += pen[NN + k];
            d1 += c->maskvx[k] * c->mask[k];
            d2 += c->maskvy[k] * c->mask[k];
        }
    b.Force[0] = f1 * norm;
    b.Force[1] = f2 * norm;
    b.drag_unst_new = d1 * norm * c->P.eps;
    b.lift_unst_new = d2 * norm * c->P.eps;
    if (b.UnstReady) {
        b.Force_unst[0] = (b.drag_unst_new - b.drag_unst_old) / dt1;
        b.Force_unst[1] = (b.lift_unst_new - b.lift_unst_old) / dt1;
    } else {
        b.Force_unst[0] = b.Force_unst[1] = 0.0;
    }
    b.drag_unst_old = b.drag_unst_new;
    b.lift_unst_old = b.lift_unst_new;
    b.UnstReady = true;
}

static void time_avg_vort(orc_ctx* c, double time, double dt, const double* vor) {  /* :670-683 */
#pragma omp parallel for schedule(static)
    for (size_t k = 0; k < c->vor_mean.size(); ++k) c->vor_mean[k] = (c->vor_mean[k] * time + dt * vor[k]) / (time + dt);
}

static void pressure(orc_ctx* c, double time, double dt1, const double* vortk, double* press, double* u) {  /* :273-403 */
    const size_t NN = (size_t)c->nx * c->ny;
    std::vector<double> work1(NN), work2(NN), pen(2 * NN);
    cal_velocity(c, time + dt1, vortk, u, work1.data());
#pragma omp parallel for schedule(static)
    for (size_t k = 0; k < NN; ++k) {
        pen[k] = c->mask[k] * (u[k] - c->maskvx[k]);
        pen[NN + k] = c->mask[k] * (u[NN + k] - c->maskvy[k]);
    }
    if (c->P.iBeam > 0) cal_drag(c, time, dt1, pen.data());
    cofitxy(c, vortk, work1.data());
    time_avg_vort(c, time, dt1, work1.data());
    cal_energy(c, time, dt1, work1.data(), u, pen.data());
    if (c->P.iFLUSI == 1 || c->P.iSaveBeam > 0) {
#pragma omp parallel for schedule(static)
        for (size_t k = 0; k < NN; ++k) {
            pen[k] = pen[k] - work1[k] * u[NN + k];
            pen[NN + k] = pen[NN + k] + work1[k] * u[k];
        }
        coftxy(c, pen.data(), work2.data());
        cofdx(c, work2.data(), pen.data());
        coftxy(c, pen.data() + NN, work2.data());
        cofdy(c, work2.data(), pen.data() + NN);
        for (size_t k = 0; k < NN; ++k) work1[k] = pen[k] + pen[NN + k];
        poisson(c, work1.data(), press);
        cofitxy(c, press, work1.data());
#pragma omp parallel for schedule(static)
        for (size_t k = 0; k < NN; ++k) press[k] = work1[k] - 0.5 * (u[k] * u[k] + u[NN + k] * u[NN + k]);
    } else {
        std::fill(press, press + NN, 0.0);
    }
}

static void EvolveFluidExplicit(orc_ctx* c) {  /* :422-459 */
    const size_t NN = (size_t)c->nx * c->ny;
    std::vector<double> stream(NN);
    const int n0 = c->n0, n1 = c->n1;
    cal_velocity(c, c->time, c->vortk[n0].data(), c->u.data(), stream.data());
    cal_nlk(c, c->time, c->dt1, c->nlk[n0].data(), c->vortk[n0].data(), c->u.data());
    vis(c, c->dt1, c->workvis[n1].data());
    const double dt1 = c->dt1;
#pragma omp parallel for schedule(static)
    for (size_t k = 0; k < NN; ++k)
        c->vortk[n1][k] = (c->vortk[n0][k] + dt1 * c->nlk[n0][k]) * c->workvis[n1][k] * c->dealiase[k];
    pressure(c, c->time, c->dt1, c->vortk[n1].data(), c->press.data(), c->u.data());
}

static void EvolveFluidAB2(orc_ctx* c) {  /* :463-508 */
    const size_t NN = (size_t)c->nx * c->ny;
    const int n0 = c->n0, n1 = c->n1;
#pragma omp parallel for schedule(static)
    for (size_t k = 0; k < NN; ++k) c->nlk[n1][k] = c->nlk[n1][k] * c->workvis[n0][k];
    cal_nlk(c, c->time, c->dt1, c->nlk[n0].data(), c->vortk[n0].data(), c->u.data());
    const double dt0 = c->dt0, dt1 = c->dt1;
    const double b10 = dt1 / dt0 * (0.5 * dt1 + dt0);
    const double b11 = -0.5 * dt1 * dt1 / dt0;
    vis(c, dt1, c->workvis[n1].data());
#pragma omp parallel for schedule(static)
    for (size_t k = 0; k < NN; ++k)
        c->vortk[n1][k] = (c->vortk[n0][k] + b10 * c->nlk[n0][k] + b11 * c->nlk[n1][k]) * c->workvis[n1][k] * c->dealiase[k];
    pressure(c, c->time, c->dt1, c->vortk[n1].data(), c->press.data(), c->u.data());
}

/* ------------------------------------------------------------------------------
 * Beam forces (BeamForces.f90, Interpolation.f90)
 * ------------------------------------------------------------------------------ */

static double delta_phi4star(double x, double dx, double pi) {  /* Interpolation.f90:51-101, "phi_4star" */
    double r = std::fabs(x / dx);
    if (r < 0.5) return (3. / 8.) + (pi / 32.) - 0.25 * (r * r);
    if (r >= 0.5 && r <= 1.5)
        return 0.25 + (1.0 - r) / 8. * std::sqrt(-2. + 8. * r - 4. * (r * r)) - std::asin(std::sqrt(2.) * (r - 1.)) / 8.;
    if (r >= 1.5 && r <= 2.5)
        return (17. / 16.) - (pi / 64.) - (3. * r / 4.) + ((r * r) / 8.) + (r - 2.) * std::sqrt(-14. + 16. * r - 4. * (r * r)) / 16. +
               std::asin(std::sqrt(2.) * (r - 2.)) / 16.;
    return 0.0;
}

/* Interpolation.f90:6-48 with typ="phi_4star" on the box (0,0)-(xl-dx,yl-dy). */
static int DeltaInterpolation(const orc_ctx* c, double xt, double yt, const double* field, double& out) {
    const double x1 = 0.0, y1 = 0.0, x2 = c->P.xl - c->dx, y2 = c->P.yl - c->dy;
    const double dx = (x2 - x1) / (double)(c->nx - 1), dy = (y2 - y1) / (double)(c->ny - 1);
    if (xt > x2 || xt < x1 || yt > y2 || yt < y1) return FSIBE_ERR_INTERP_OOB;
    const int i = (int)((xt - x1) / dx), j = (int)((yt - y1) / dy);
    const int NS = 4;
    if (i - NS < 0 || j - NS < 0 || i + NS > c->nx - 1 || j + NS > c->ny - 1) return FSIBE_ERR_INTERP_OOB;
    double R1 = 0.0;
    for (int ix = i - NS; ix <= i + NS; ++ix)
        for (int iy = j - NS; iy <= j + NS; ++iy) {
            double xl_ = (double)ix * dx + x1, yl_ = (double)iy * dy + y1;
            R1 = R1 + delta_phi4star(std::fabs(xl_ - xt), dx, c->pi) * delta_phi4star(std::fabs(yl_ - yt), dy, c->pi) *
                          field[(size_t)iy * c->nx + ix];
        }
    out = R1;
    return FSIBE_OK;
}

/* GetForces + GetForcesInterp with SPL=3 (BeamForces.f90:6-288); BeamSurfaceIntegral
 * (:306-509) is orc_surface_integral. */
static int GetForces(orc_ctx* c, double time) {
    const size_t NN = (size_t)c->nx * c->ny;
    const int ns = c->ns;
    Beam& b = c->beam;
    const bool viscous = (c->P.iViscous == 1);
    double alpha, alpha_t, alpha_tt, LE[6];
    mouvement(c, time, alpha, alpha_t, alpha_tt, LE, b);
    std::vector<double> pb(ns, 0.0), tb(ns, 0.0), sg(ns, 0.0), th(ns);
    std::vector<double> sa, sb;
    if (viscous) {
        std::vector<double> w1(NN), w2(NN), w3(NN);
        sa.resize(NN); sb.resize(NN);
        const double* u1 = c->u.data();
        const double* u2 = c->u.data() + NN;
        coftxy(c, u1, w1.data()); cofdx(c, w1.data(), w2.data()); cofitxy(c, w2.data(), sa.data());
        for (size_t k = 0; k < NN; ++k) sa[k] = 2.0 * c->P.nu * sa[k];
        coftxy(c, u1, w1.data()); cofdy(c, w1.data(), w2.data()); cofitxy(c, w2.data(), w3.data());
        coftxy(c, u2, w1.data()); cofdx(c, w1.data(), w2.data()); cofitxy(c, w2.data(), sb.data());
        for (size_t k = 0; k < NN; ++k) sb[k] = c->P.nu * (w3[k] + sb[k]);
    }
    for (int n = 0; n < ns; ++n) th[n] = b.theta[n] + alpha;
    const double off = c->P.t_beam + c->P.N_smooth * std::max(c->dy, c->dx);
    const double off1 = c->P.t_beam - 0.0 * c->P.N_smooth * std::max(c->dy, c->dx);
    int st = FSIBE_OK;
    for (int n = 0; n < ns; ++n) {
        const double s = std::sin(th[n]), co = std::cos(th[n]);
        double xu = b.x[n] - off * s, yu = b.y[n] + off * co, xb = b.x[n] + off * s, yb = b.y[n] - off * co;
        double xu1 = b.x[n] - off1 * s, yu1 = b.y[n] + off1 * co, xb1 = b.x[n] + off1 * s, yb1 = b.y[n] - off1 * co;
        double pu, pd;
        st |= DeltaInterpolation(c, xu1, yu1, c->press.data(), pu);
        st |= DeltaInterpolation(c, xb1, yb1, c->press.data(), pd);
        pb[n] = pu - pd;
        if (viscous) {
            double A1, B1, A2, B2;
            st |= DeltaInterpolation(c, xu, yu, sa.data(), A1);
            st |= DeltaInterpolation(c, xu, yu, sb.data(), B1);
            st |= DeltaInterpolation(c, xb, yb, sa.data(), A2);
            st |= DeltaInterpolation(c, xb, yb, sb.data(), B2);
            const double c2 = std::cos(2.0 * th[n]), s2 = std::sin(2.0 * th[n]);
            double sn1 = -A1 * c2 - B1 * s2, st1 = -A1 * s2 + B1 * c2;
            double sn2 = -A2 * c2 - B2 * s2, st2 = -A2 * s2 + B2 * c2;
            tb[n] = st1 - st2;
            sg[n] = -sn1 + sn2;
        }
    }
    if (st) return fail(c, FSIBE_ERR_INTERP_OOB, "DeltaInterpolation: target coordinates not in the field");
    if (viscous) for (int n = 0; n < ns; ++n) pb[n] = pb[n] + sg[n];
    else std::fill(tb.begin(), tb.end(), 0.0);
    double soft;
    if (time <= c->P.t_release) soft = 0.0;
    else if (time > c->P.t_release && time < c->P.t_release + c->P.tau) {
        double tr = time - c->P.t_release;
        soft = (tr * tr * tr) / (-0.5 * c->P.tau * c->P.tau * c->P.tau) + 3. * (tr * tr) / (c->P.tau * c->P.tau);
    } else soft = 1.0;
    for (int n = 0; n < ns; ++n) { pb[n] = pb[n] * soft; tb[n] = tb[n] * soft; }
    double fx = 0.0, fy = 0.0;
    for (int i = 0; i < ns; ++i) {
        fx = fx - (std::sin(th[i]) * pb[i] + std::cos(th[i]) * tb[i]) * c->ds;
        fy = fy + (std::cos(th[i]) * pb[i] + std::sin(th[i]) * tb[i]) * c->ds;
    }
    b.p_new = pb;
    b.tau_new = tb;
    b.Force_press[0] = fx;
    b.Force_press[1] = fy;
    return FSIBE_OK;
}

/* ------------------------------------------------------------------------------
 * Beam (IBES) solver (SolidSolver.f90)
 * ------------------------------------------------------------------------------ */

/* Differentiate1D + create_diff_matrices (SolidSolver.f90:1085-1233): the dense D matrices
 * restated row by row as stencils, coefficients divided by 2dx / dx^2 / 2dx^3 / dx^4 first,
 * then summed over increasing column index like matmul. */
static void Differentiate1D(const double* f, double* fd, int NN, double dx, int order) {
    const int N = NN - 1;
    auto apply = [&](int i, const int j0, const double* cf, int len, double den) {
        double s = 0.0;
        for (int q = 0; q < len; ++q) s += (cf[q] / den) * f[j0 + q];
        fd[i] = s;
    };
    if (order == 1) {
        const double den = 2.0 * dx;
        const double r0[3] = {-3., 4., -1.}, rN[3] = {1., -4., 3.}, in[3] = {-1., 0., 1.};
        apply(0, 0, r0, 3, den);
        for (int i = 1; i <= N - 1; ++i) apply(i, i - 1, in, 3, den);
        apply(N, N - 2, rN, 3, den);
    } else if (order == 2) {
        const double den = dx * dx;
        const double r0[4] = {2., -5., 4., -1.}, rN[4] = {-1., 4., -5., 2.}, in[3] = {1., -2., 1.};
        apply(0, 0, r0, 4, den);
        for (int i = 1; i <= N - 1; ++i) apply(i, i - 1, in, 3, den);
        apply(N, N - 3, rN, 4, den);
    } else if (order == 3) {
        const double den = 2.0 * (dx * dx * dx);
        const double r0[6] = {-17.0 / 2., 71.0 / 2., -59., 49., -41.0 / 2., 7.0 / 2.};
        const double rN[6] = {-7.0 / 2., 41.0 / 2., -49., 59., -71.0 / 2., 17.0 / 2.};
        const double in[5] = {-1., 2., 0., -2., 1.};
        apply(0, 0, r0, 6, den);
        apply(1, 1, r0, 6, den);
        for (int i = 2; i <= N - 2; ++i) apply(i, i - 2, in, 5, den);
        apply(N - 1, N - 6, rN, 6, den);
        apply(N, N - 5, rN, 6, den);
    } else {
        const double den = (dx * dx) * (dx * dx);
        const double r0[7] = {35.0 / 6., -31., 137.0 / 2., -242.0 / 3., 107.0 / 2., -19.0, 17.0 / 6.};
        const double rN[7] = {17.0 / 6.0, -19.0, 107.0 / 2.0, -242.0 / 3.0, 137.0 / 2.0, -31.0, 35.0 / 6.0};
        const double in[5] = {1., -4., 6., -4., 1.};
        apply(0, 0, r0, 7, den);
        apply(1, 1, r0, 7, den);
        for (int i = 2; i <= N - 2; ++i) apply(i, i - 2, in, 5, den);
        apply(N - 1, N - 7, rN, 7, den);
        apply(N, N - 6, rN, 7, den);
    }
}

/* LAPACK dgttrf + dgttrs (via dgtts2, NOTRANS, one right-hand side). */
static int gttrf_solve(int n, std::vector<double>& dl, std::vector<double>& d, std::vector<double>& du, double* b) {
    std::vector<double> du2(std::max(n - 2, 1), 0.0);
    std::vector<int> ipiv(n);
    for (int i = 0; i < n; ++i) ipiv[i] = i;
    for (int i = 0; i < n - 2; ++i) {
        if (std::fabs(d[i]) >= std::fabs(dl[i])) {
            if (d[i] != 0.0) {
                double fact = dl[i] / d[i];
                dl[i] = fact;
                d[i + 1] = d[i + 1] - fact * du[i];
            }
        } else {
            double fact = d[i] / dl[i];
            d[i] = dl[i];
            dl[i] = fact;
            double temp = du[i];
            du[i] = d[i + 1];
            d[i + 1] = temp - fact * d[i + 1];
            du2[i] = du[i + 1];
            du[i + 1] = -fact * du[i + 1];
            ipiv[i] = i + 1;
        }
    }
    if (n > 1) {
        int i = n - 2;
        if (std::fabs(d[i]) >= std::fabs(dl[i])) {
            if (d[i] != 0.0) {
                double fact = dl[i] / d[i];
                dl[i] = fact;
                d[i + 1] = d[i + 1] - fact * du[i];
            }
        } else {
            double fact = d[i] / dl[i];
            d[i] = dl[i];
            dl[i] = fact;
            double temp = du[i];
            du[i] = d[i + 1];
            d[i + 1] = temp - fact * d[i + 1];
            ipiv[i] = i + 1;
        }
    }
    for (int i = 0; i < n; ++i) if (d[i] == 0.0) return i + 1;
    for (int i = 0; i < n - 1; ++i) {
        if (ipiv[i] == i) b[i + 1] = b[i + 1] - dl[i] * b[i];
        else { double temp = b[i]; b[i] = b[i + 1]; b[i + 1] = temp - dl[i] * b[i]; }
    }
    b[n - 1] = b[n - 1] / d[n - 1];
    if (n > 1) b[n - 2] = (b[n - 2] - du[n - 2] * b[n - 1]) / d[n - 2];
    for (int i = n - 3; i >= 0; --i) b[i] = (b[i] - du[i] * b[i + 1] - du2[i] * b[i + 2]) / d[i];
    return 0;
}

/* LAPACK dgetrf (unblocked dgetf2 order) + dgetrs on a dense row-major n x n matrix. */
static int getrf_solve(int n, std::vector<double>& A, double* b) {
    std::vector<int> ipiv(n);
    for (int j = 0; j < n; ++j) {
        int p = j;
        double mx = std::fabs(A[(size_t)j * n + j]);
        for (int i = j + 1; i < n; ++i) {
            double v = std::fabs(A[(size_t)i * n + j]);
            if (v > mx) { mx = v; p = i; }
        }
        ipiv[j] = p;
        if (A[(size_t)p * n + j] == 0.0) return j + 1;
        if (p != j) for (int k = 0; k < n; ++k) std::swap(A[(size_t)j * n + k], A[(size_t)p * n + k]);
        const double r = 1.0 / A[(size_t)j * n + j];
        for (int i = j + 1; i < n; ++i) A[(size_t)i * n + j] *= r;
        for (int i = j + 1; i < n; ++i) {
            const double l = A[(size_t)i * n + j];
            if (l == 0.0) continue;
            double* Ai = &A[(size_t)i * n];
            const double* Aj = &A[(size_t)j * n];
            for (int k = j + 1; k < n; ++k) Ai[k] -= l * Aj[k];
        }
    }
    for (int j = 0; j < n; ++j) if (ipiv[j] != j) std::swap(b[j], b[ipiv[j]]);
    for (int j = 0; j < n; ++j) {
        if (b[j] != 0.0) for (int i = j + 1; i < n; ++i) b[i] -= b[j] * A[(size_t)i * n + j];
    }
    for (int j = n - 1; j >= 0; --j) {
        if (b[j] != 0.0) {
            b[j] = b[j] / A[(size_t)j * n + j];
            for (int i = 0; i < j; ++i) b[i] -= b[j] * A[(size_t)i * n + j];
        }
    }
    return 0;
}

static void solid_coeffs(int method, double dt, double dt_old, double& C1, double& C2, double& C3, double& C4) {
    if (method == FSIBE_EULER_IMPLICIT) { C1 = 1.0; C2 = 0.0; C3 = 1.0; C4 = 0.0; }
    else if (method == FSIBE_CRANK_NICHOLSON) { C1 = 2.0; C2 = 1.0; C3 = 1.0; C4 = 0.0; }
    else {
        double R = dt / dt_old;
        C1 = (1. + 2. * R) / (1. + R);
        C2 = 0.0;
        C3 = ((1. + R) * (1. + R)) / (1. + 2. * R);
        C4 = (-(R * R)) / (1. + 2. * R);
    }
}

/* Tension (SolidSolver.f90:1000-1081) */
static int Tension(orc_ctx* c, double time, double* T, double* T_s, const double* theta, const double* theta_dot,
                   const double* pressure, const double* tau) {
    const int ns = c->ns;
    const double ds = c->ds, eta = c->P.eta, mue = c->P.mue;
    double alpha, alpha_t, alpha_tt, LE[6];
    mouvement(c, time, alpha, alpha_t, alpha_tt, LE, c->beam);
    std::vector<double> th_s(ns), th_ss(ns), th_sss(ns), tau_s(ns), dmain(ns), dup(ns - 1), ddown(ns - 1), rhs(ns);
    Differentiate1D(theta, th_s.data(), ns, ds, 1);
    Differentiate1D(theta, th_ss.data(), ns, ds, 2);
    Differentiate1D(theta, th_sss.data(), ns, ds, 3);
    Differentiate1D(tau, tau_s.data(), ns, ds, 1);
    const double K1 = mue * (LE[4] * std::cos(alpha) + LE[5] * std::sin(alpha) + c->grav * std::sin(alpha)) - tau[0];
    const double T_s0 = -eta * th_ss[0] * th_s[0] + K1;
    const double ds2 = ds * ds;
    for (int i = 0; i < ns; ++i) dmain[i] = -2.0 / ds2 - th_s[i] * th_s[i];
    for (int i = 0; i < ns - 1; ++i) { dup[i] = 1.0 / ds2; ddown[i] = 1.0 / ds2; }
    dmain[ns - 1] = 1.0;
    ddown[ns - 2] = 0.0;
    dup[0] = 2.0 / ds2;
    for (int i = 0; i < ns; ++i) {
        double w = theta_dot[i] + alpha_t;
        rhs[i] = -(pressure[i] * th_s[i]) - (2. * eta * th_s[i] * th_sss[i]) - (eta * (th_ss[i] * th_ss[i])) - mue * (w * w) - tau_s[i];
    }
    rhs[ns - 1] = 0.0;
    rhs[0] = rhs[0] + T_s0 * 2.0 / ds;
    for (int i = 0; i < ns; ++i) rhs[i] = rhs[i] / dmain[i];
    for (int i = 0; i < ns - 1; ++i) {
        dup[i] = dup[i] / dmain[i];
        ddown[i] = ddown[i] / dmain[i + 1];
    }
    for (int i = 0; i < ns; ++i) dmain[i] = 1.0;
    int info = gttrf_solve(ns, ddown, dmain, dup, rhs.data());
    for (int i = 0; i < ns; ++i) T[i] = rhs[i];
    Differentiate1D(T, T_s, ns, ds, 1);
    T_s[0] = T_s0;
    if (info != 0) return fail(c, FSIBE_ERR_SINGULAR, "dgttrf: singular tension system");
    return FSIBE_OK;
}

/* RHS_beameqn (SolidSolver.f90:918-994): on return theta := theta_dot, theta_dot := theta_ddot. */
static int RHS_beameqn(orc_ctx* c, double time, double* theta, double* theta_dot, const double* pb, double* T,
                       const double* tau) {
    const int ns = c->ns;
    const double ds = c->ds, eta = c->P.eta, mue = c->P.mue, sigma = c->P.sigma;
    double alpha, alpha_t, alpha_tt, LE[6];
    mouvement(c, time, alpha, alpha_t, alpha_tt, LE, c->beam);
    theta[0] = 0.0;
    theta_dot[0] = 0.0;
    std::vector<double> T_s(ns);
    int st = Tension(c, time, T, T_s.data(), theta, theta_dot, pb, tau);
    if (st) return st;
    const double K2 = pb[0] + mue * (LE[5] * std::cos(alpha) - LE[4] * std::sin(alpha) + c->grav * std::cos(alpha));
    const double ds2 = ds * ds;
    const double C2 = 2.0 * ds * K2 - T[0] * theta[1] + (eta / ds2) * (10.0 * theta[0] - 12.0 * theta[1] + 6.0 * theta[2] - theta[3]);
    std::vector<double> te(ns + 3), te_s(ns + 3), te_ss(ns + 3), te_sss(ns + 3), te_ssss(ns + 3), p_s(ns);
    te[0] = C2 / ((3.0 * eta / ds2) - T[0]);
    for (int i = 0; i < ns; ++i) te[i + 1] = theta[i];
    const double A1 = theta[ns - 3] / 12. - 2. * theta[ns - 2] / 3.;
    const double A2 = -theta[ns - 3] / 12. + 4. * theta[ns - 2] / 3. - 5. * theta[ns - 1] / 2.;
    te[ns + 1] = 3. * (A1 - A2) / 2.;
    te[ns + 2] = 12. * (2. * A1 - A2);
    Differentiate1D(te.data(), te_s.data(), ns + 3, ds, 1);
    Differentiate1D(te.data(), te_ss.data(), ns + 3, ds, 2);
    Differentiate1D(te.data(), te_sss.data(), ns + 3, ds, 3);
    Differentiate1D(te.data(), te_ssss.data(), ns + 3, ds, 4);
    Differentiate1D(pb, p_s.data(), ns, ds, 1);
    std::vector<double> td_in(theta_dot, theta_dot + ns);
    for (int i = 0; i < ns; ++i) theta[i] = td_in[i];
    for (int i = 0; i < ns; ++i) {
        const double ts = te_s[i + 1], tss = te_ss[i + 1], tssss = te_ssss[i + 1];
        theta_dot[i] = (-p_s[i] - eta * tssss + tss * (T[i] + eta * (ts * ts)) + 2. * T_s[i] * ts - mue * alpha_tt -
                        sigma * td_in[i] + tau[i] * ts) / mue;
    }
    theta_dot[0] = 0.0;
    return FSIBE_OK;
}

/* x layout (Fortran 1-based): x(1:ns+3) = theta(-1:ns+1), x(ns+4:2ns+4) = T(-1:ns-1).
 * TH(i) / TT(i) address theta(i) / T(i) in a 0-based vector. */
#define TH(v, i) (v)[(i) + 1]
#define TT(v, i) (v)[ns + 3 + (i) + 1]

/* F_nonlinear (SolidSolver.f90:552-667); F is 0-based: F[k-1] = F(k). */
static int F_nonlinear(orc_ctx* c, double time, double dt, double dt_old, double* F, const double* theta_old,
                       const double* theta_dot_old, const double* x, const double* p, const double* old_rhs,
                       const double* theta_oldold, const double* theta_dot_oldold, const double* tau) {
    const int ns = c->ns;
    const double ds = c->ds, eta = c->P.eta, mue = c->P.mue, sigma = c->P.sigma;
    double alpha, alpha_t, alpha_tt, LE[6];
    std::vector<double> tau_s(ns), tdn(ns);
    Differentiate1D(tau, tau_s.data(), ns, ds, 1);
    mouvement(c, time + dt, alpha, alpha_t, alpha_tt, LE, c->beam);
    const double K1 = mue * (LE[4] * std::cos(alpha) + LE[5] * std::sin(alpha) + c->grav * std::sin(alpha)) - tau[0];
    const double K2 = p[0] + mue * (LE[5] * std::cos(alpha) - LE[4] * std::sin(alpha) + c->grav * std::cos(alpha));
    double C1, C2, C3, C4;
    solid_coeffs(c->TimeMethodSolid, dt, dt_old, C1, C2, C3, C4);
    for (int i = 0; i < ns; ++i) tdn[i] = (C1 / dt) * (TH(x, i) - C3 * theta_old[i] - C4 * theta_oldold[i]) - C2 * theta_dot_old[i];
    const double ds2 = ds * ds, ds3 = ds * ds * ds, ds4 = (ds * ds) * (ds * ds);
    F[0] = TH(x, 0);
    F[1] = (TT(x, 1) - TT(x, -1)) / (2.0 * ds) + (eta / (2.0 * ds3)) * (TH(x, -1) - 2.0 * TH(x, 0) + TH(x, 1)) * (TH(x, 1) - TH(x, -1)) - K1;
    F[2] = TT(x, 0) * (TH(x, 1) - TH(x, -1)) / (2.0 * ds) -
           (eta / (2.0 * ds3)) * (-3.0 * TH(x, -1) + 10.0 * TH(x, 0) - 12.0 * TH(x, 1) + 6.0 * TH(x, 2) - TH(x, 3)) - K2;
    F[3] = ((1.0 / 12.0) * TH(x, ns - 3) - (2.0 / 3.0) * TH(x, ns - 2) + (2.0 / 3.0) * TH(x, ns) - (1.0 / 12.0) * TH(x, ns + 1)) / ds;
    F[4] = ((-1.0 / 12.0) * TH(x, ns - 3) + (4.0 / 3.0) * TH(x, ns - 2) - 2.5 * TH(x, ns - 1) + (4.0 / 3.0) * TH(x, ns) +
            (-1.0 / 12.0) * TH(x, ns + 1)) / ds2;
    F[5] = TT(x, ns - 1);
    {
        const double d1 = (TH(x, 1) - TH(x, -1)) / (2.0 * ds);
        const double lap = (TH(x, 1) - 2.0 * TH(x, 0) + TH(x, -1)) / ds2;
        const double w = tdn[0] + alpha_t;
        F[6] = (TT(x, -1) - 2.0 * TT(x, 0) + TT(x, 1)) / ds2 - TT(x, 0) * (d1 * d1) + p[0] * d1 +
               (eta / ds4) * (TH(x, 1) - TH(x, -1)) * (-2.5 * TH(x, 0) + 9.0 * TH(x, 1) - 12.0 * TH(x, 2) + 7.0 * TH(x, 3) - 1.5 * TH(x, 4)) +
               eta * (lap * lap) + mue * (w * w) - tau_s[0];
    }
    {
        const int m = ns - 1;
        const double d1 = (TH(x, ns) - TH(x, ns - 2)) / (2. * ds);
        F[7] = C3 * theta_dot_old[m] + C4 * theta_dot_oldold[m] - tdn[m] +
               (dt / (C1 * mue)) *
                   (-(3. * p[m] - 4. * p[m - 1] + p[m - 2]) / (2. * ds) -
                    eta * (TH(x, ns + 1) - 4. * TH(x, ns) + 6. * TH(x, ns - 1) - 4. * TH(x, ns - 2) + TH(x, ns - 3)) / ds4 +
                    (TT(x, m) + eta * (d1 * d1)) * (TH(x, ns) - 2. * TH(x, ns - 1) + TH(x, ns - 2)) / ds2 +
                    (3. * TT(x, m) - 4. * TT(x, m - 1) + TT(x, m - 2)) * (TH(x, ns) - TH(x, ns - 2)) / (2. * ds2) -
                    alpha_tt * (mue * mue) - sigma * tdn[m] + tau[m] * (TH(x, ns) - TH(x, ns - 2)) / (2.0 * ds) +
                    C2 * mue * old_rhs[m]);
    }
    for (int i = 1; i <= ns - 2; ++i) {
        const double d1 = (TH(x, i + 1) - TH(x, i - 1)) / (2. * ds);
        F[8 + i - 1] = C3 * theta_dot_old[i] + C4 * theta_dot_oldold[i] - tdn[i] +
                       (dt / (C1 * mue)) *
                           (-1.0 * (p[i + 1] - p[i - 1]) / (2. * ds) -
                            eta * (TH(x, i + 2) - 4. * TH(x, i + 1) + 6. * TH(x, i) - 4. * TH(x, i - 1) + TH(x, i - 2)) / ds4 +
                            (TT(x, i) + eta * (d1 * d1)) * (TH(x, i + 1) - 2. * TH(x, i) + TH(x, i - 1)) / ds2 +
                            (TT(x, i + 1) - TT(x, i - 1)) * (TH(x, i + 1) - TH(x, i - 1)) / (2.0 * ds2) - alpha_tt * (mue * mue) -
                            sigma * tdn[i] + tau[i] * (TH(x, i + 1) - TH(x, i - 1)) / (2.0 * ds) + C2 * mue * old_rhs[i]);
        const double d1b = (TH(x, i + 1) - TH(x, i - 1)) / (2.0 * ds);
        const double lap = (TH(x, i + 1) - 2.0 * TH(x, i) + TH(x, i - 1)) / ds2;
        const double w = tdn[i] + alpha_t;
        F[8 + (ns - 2) + i - 1] = (TT(x, i - 1) - 2.0 * TT(x, i) + TT(x, i + 1)) / ds2 - TT(x, i) * (d1b * d1b) + p[i] * d1b +
                                  eta * (TH(x, i + 1) - TH(x, i - 1)) * (TH(x, i + 2) - 2.0 * TH(x, i + 1) + 2.0 * TH(x, i - 1) - TH(x, i - 2)) /
                                      (2.0 * ds4) +
                                  eta * (lap * lap) + mue * (w * w) - tau_s[i];
    }
    for (int k = 0; k < 2 * ns + 4; ++k)
        if (std::isnan(F[k])) return fail(c, FSIBE_ERR_NAN, "NaN in F_nonlinear");
    return FSIBE_OK;
}

/* Jacobi (SolidSolver.f90:671-863).  The reference fills J(var, eqn) and transposes before
 * dgetrf; here Jr[eqn][var] (row-major, 0-based) is filled directly. */
static int Jacobi(orc_ctx* c, double time, double dt, double dt_old, std::vector<double>& Jr, const double* x,
                  const double* theta_old, const double* theta_dot_old, const double* p, const double* theta_oldold,
                  const double* theta_dot_oldold, const double* tau) {
    const int ns = c->ns, n = 2 * ns + 4;
    const double ds = c->ds, eta = c->P.eta, mue = c->P.mue, sigma = c->P.sigma;
    double alpha, alpha_t, alpha_tt, LE[6];
    mouvement(c, time + dt, alpha, alpha_t, alpha_tt, LE, c->beam);
    double C1, C2, C3, C4;
    solid_coeffs(c->TimeMethodSolid, dt, dt_old, C1, C2, C3, C4);
    const double D = C1 / dt;
    std::vector<double> tdn(ns);
    for (int i = 0; i < ns; ++i) tdn[i] = (C1 / dt) * (TH(x, i) - C3 * theta_old[i] - C4 * theta_oldold[i]) - C2 * theta_dot_old[i];
    std::fill(Jr.begin(), Jr.end(), 0.0);
    /* J(l,k) in Fortran (1-based var l, eqn k) -> Jr[(k-1)*n + (l-1)] */
#define JF(l, k) Jr[(size_t)((k)-1) * n + ((l)-1)]
    const double ds2 = ds * ds, ds3 = ds * ds * ds, ds4 = (ds * ds) * (ds * ds);
    const int T0_index = ns + 4;
    JF(2, 1) = 1.0;
    JF(1, 2) = (eta / (2.0 * ds3)) * (-2.0 * TH(x, -1) + 2.0 * TH(x, 0));
    JF(2, 2) = -(eta / (ds3)) * (TH(x, 1) - TH(x, -1));
    JF(3, 2) = (eta / (2.0 * ds3)) * (-2.0 * TH(x, 0) + 2.0 * TH(x, 1));
    JF(T0_index, 2) = -0.5 / ds;
    JF(T0_index + 2, 2) = 0.5 / ds;
    JF(1, 3) = (-0.5 * eta / (ds3)) * (-3.0) - TT(x, 0) / (2.0 * ds);
    JF(2, 3) = (-0.5 * eta / (ds3)) * (10.0);
    JF(3, 3) = (-0.5 * eta / (ds3)) * (-12.0) + TT(x, 0) / (2.0 * ds);
    JF(4, 3) = (-0.5 * eta / (ds3)) * (6.0);
    JF(5, 3) = (-0.5 * eta / (ds3)) * (-1.0);
    JF(T0_index + 1, 3) = (TH(x, 1) - TH(x, -1)) / (2.0 * ds);
    JF(ns + 3, 4) = (-1.0 / 12.0) / ds;
    JF(ns + 2, 4) = (2.0 / 3.0) / ds;
    JF(ns, 4) = (-2.0 / 3.0) / ds;
    JF(ns - 1, 4) = (1.0 / 12.0) / ds;
    JF(ns + 3, 5) = (-1.0 / 12.0) / ds2;
    JF(ns + 2, 5) = (4.0 / 3.0) / ds2;
    JF(ns + 1, 5) = (-5.0 / 2.0) / ds2;
    JF(ns, 5) = (4.0 / 3.0) / ds2;
    JF(ns - 1, 5) = (-1.0 / 12.0) / ds2;
    JF(2 * ns + 4, 6) = 1.0;
    {
        const double t1m = TH(x, 1) - TH(x, -1);
        const double lap = TH(x, 1) - 2.0 * TH(x, 0) + TH(x, -1);
        const double q = -2.5 * TH(x, 0) + 9.0 * TH(x, 1) - 12.0 * TH(x, 2) + 7.0 * TH(x, 3) - 1.5 * TH(x, 4);
        JF(1, 7) = TT(x, 0) * t1m / (2.0 * ds2) - p[0] / (2.0 * ds) - (eta / ds4) * q + 2.0 * eta * lap / ds4;
        JF(2, 7) = -2.5 * eta * t1m / ds4 - 4.0 * eta * lap / ds4 + 2.0 * mue * (tdn[0] + alpha_t) * D;
        JF(3, 7) = -TT(x, 0) * t1m / (2.0 * ds2) + p[0] / (2.0 * ds) + (eta / ds4) * q + 9.0 * eta * t1m / ds4 + 2.0 * eta * lap / ds4;
        JF(4, 7) = -12.0 * eta * t1m / ds4;
        JF(5, 7) = 7.0 * eta * t1m / ds4;
        JF(6, 7) = -1.5 * eta * t1m / ds4;
        JF(ns + 4, 7) = 1.0 / ds2;
        JF(ns + 5, 7) = (-2.0 - (t1m * t1m) / 4.0) / ds2;
        JF(ns + 6, 7) = 1.0 / ds2;
    }
    {
        const double d0 = TH(x, ns) - TH(x, ns - 2);
        const double lap = TH(x, ns) - 2.0 * TH(x, ns - 1) + TH(x, ns - 2);
        const double Tp = TT(x, ns - 1) + eta * ((d0 / (2.0 * ds)) * (d0 / (2.0 * ds)));
        const double Tb = 3.0 * TT(x, ns - 1) - 4.0 * TT(x, ns - 2) + TT(x, ns - 3);
        const double g = dt / (C1 * mue);
        JF(2 * ns + 4, 8) = (dt / (C1 * mue * ds2)) * (lap + (3.0 / 2.0) * d0);
        JF(2 * ns + 3, 8) = -4.0 * g * d0 / (2.0 * ds2);
        JF(2 * ns + 2, 8) = 1.0 * g * d0 / (2.0 * ds2);
        JF(ns + 3, 8) = -dt * eta / ((C1 * mue) * ds4);
        JF(ns + 2, 8) = (dt / (C1 * mue * ds2)) * (4.0 * eta / ds2 + Tp + tau[ns - 1] * ds / (2.0) + eta * lap * d0 / (2.0 * ds2) + Tb / 2.0);
        JF(ns, 8) = (dt / (C1 * mue * ds2)) * (4.0 * eta / ds2 + Tp - tau[ns - 1] * ds / (2.0) - eta * lap * d0 / (2.0 * ds2) - Tb / 2.0);
        JF(ns + 1, 8) = -D + g * (-6.0 * eta / ds4 - 2.0 * Tp / ds2 - D * sigma);
        JF(ns - 1, 8) = -dt * eta / (C1 * mue * ds4);
    }
    for (int i = 1; i <= ns - 2; ++i) {
        const int k = 8 + i, l = i + 2, m = i + ns + 5;
        const double g = dt / (C1 * mue);
        const double d1 = TH(x, i + 1) - TH(x, i - 1);
        const double lap = TH(x, i + 1) - 2.0 * TH(x, i) + TH(x, i - 1);
        const double Tp = TT(x, i) + eta * ((d1 / (2.0 * ds)) * (d1 / (2.0 * ds)));
        const double dT = TT(x, i + 1) - TT(x, i - 1);
        JF(l, k) = -D + g * (-6.0 * eta / ds4 - (2.0 / ds2) * Tp - D * sigma);
        JF(l - 1, k) = g * (4.0 * eta / ds4 + Tp / ds2 - tau[i] / (2.0 * ds) - eta * lap * d1 / (2.0 * ds4) - dT / (2.0 * ds2));
        JF(l + 1, k) = g * (4.0 * eta / ds4 + Tp / ds2 + tau[i] / (2.0 * ds) + eta * lap * d1 / (2.0 * ds4) + dT / (2.0 * ds2));
        JF(l - 2, k) = -eta * dt / (C1 * mue * ds4);
        JF(l + 2, k) = -eta * dt / (C1 * mue * ds4);
        JF(m, k) = g * lap / ds2;
        JF(m - 1, k) = -g * d1 / (2.0 * ds2);
        JF(m + 1, k) = g * d1 / (2.0 * ds2);
    }
    for (int i = 1; i <= ns - 2; ++i) {
        const int k = 8 + ns - 2 + i, l = i + 2, m = i + ns + 5;
        const double d1 = TH(x, i + 1) - TH(x, i - 1);
        const double lap = TH(x, i + 1) - 2.0 * TH(x, i) + TH(x, i - 1);
        const double q = TH(x, i + 2) - 2.0 * TH(x, i + 1) + 2.0 * TH(x, i - 1) - TH(x, i - 2);
        JF(l, k) = -4.0 * eta * lap / ds4 + 2.0 * mue * (tdn[i] + alpha_t) * D;
        JF(l - 1, k) = TT(x, i) * d1 / (2.0 * ds2) - p[i] / (2.0 * ds) + eta * d1 / ds4 - eta * q / (2.0 * ds4) + 2.0 * eta * lap / ds4;
        JF(l + 1, k) = -TT(x, i) * d1 / (2.0 * ds2) + p[i] / (2.0 * ds) - eta * d1 / ds4 + eta * q / (2.0 * ds4) + 2.0 * eta * lap / ds4;
        JF(l - 2, k) = -eta * d1 / (2.0 * ds4);
        JF(l + 2, k) = eta * d1 / (2.0 * ds4);
        JF(m, k) = -2.0 / ds2 - ((d1 / (2.0 * ds)) * (d1 / (2.0 * ds)));
        JF(m - 1, k) = 1.0 / ds2;
        JF(m + 1, k) = 1.0 / ds2;
    }
#undef JF
    for (size_t q = 0; q < Jr.size(); ++q)
        if (std::isnan(Jr[q])) return fail(c, FSIBE_ERR_NAN, "NaN in Jacobian");
    return FSIBE_OK;
}

static void SolidEnergies(orc_ctx* c) {  /* SolidSolver.f90:76-92 */
    Beam& b = c->beam;
    const int ns = c->ns;
    std::vector<double> th_s(ns);
    Differentiate1D(b.theta.data(), th_s.data(), ns, c->ds, 1);
    double sk = 0, sp = 0, se = 0, sax = 0, say = 0;
    for (int i = 0; i < ns; ++i) {
        sk += b.vx[i] * b.vx[i] + b.vy[i] * b.vy[i];
        sp += b.y[i] - b.y0;
        se += th_s[i] * th_s[i];
        sax += b.ax[i];
        say += b.ay[i];
    }
    b.E_kin = c->P.mue * 0.5 * c->ds * sk;
    b.E_pot = c->P.mue * c->grav * c->ds * sp;
    b.E_el = c->P.eta * 0.5 * c->ds * se;
    b.Inertial[0] = c->P.mue * c->ds * sax;
    b.Inertial[1] = c->P.mue * c->ds * say;
}

static void GravityImpulse(orc_ctx* c, double time) {  /* SolidSolver.f90:874-911 */
    const int m = c->P.iImpulse;
    if (m == 1 || m == 2) {
        const double T0 = 0.75, T1 = 0.85, A = (m == 1) ? 1.00 : 4.00;
        c->grav = A * std::sin(c->pi * (time - T0) / (T1 - T0));
        if (time < T0) c->grav = 0.0;
        if (time > T1) c->grav = 0.0;
    } else if (m == 3) {
        const double T0 = 2.0, T1 = 3.0;
        double k = 0.0;
        if (time <= T0) k = 0.0;
        else if (time >= T0 && time <= T1) {
            const double a = -20.0, b = 70.0, cc = -84.0, d = 35.0, t = (time - T0) / (T1 - T0);
            const double t2 = t * t, t4 = t2 * t2;
            k = a * (t4 * t2 * t) + b * (t4 * t2) + cc * (t4 * t) + d * t4;
        } else if (time > T1) k = 1.0;
        c->grav = 0.7 * k;
    }
}

/* IBES_solver (SolidSolver.f90:99-414) for the single beam. */
static int IBES_solver(orc_ctx* c, double time, double dt) {
    Beam& b = c->beam;
    const int ns = c->ns, n = 2 * ns + 4;
    const double ds = c->ds, eta = c->P.eta, mue = c->P.mue;
    std::vector<double> bo5 = b.theta, bo6 = b.theta_dot, bo3 = b.vx, bo4 = b.vy;
    std::vector<double> oo5(b.oldold.begin() + 4 * ns, b.oldold.begin() + 5 * ns);
    std::vector<double> oo6(b.oldold.begin() + 5 * ns, b.oldold.begin() + 6 * ns);
    std::vector<double> beam_old_full(6 * (size_t)ns);
    for (int i = 0; i < ns; ++i) {
        beam_old_full[i] = b.x[i]; beam_old_full[ns + i] = b.y[i]; beam_old_full[2 * ns + i] = b.vx[i];
        beam_old_full[3 * ns + i] = b.vy[i]; beam_old_full[4 * ns + i] = b.theta[i]; beam_old_full[5 * ns + i] = b.theta_dot[i];
    }
    const double dt_old = b.dt_old;
    double alpha, alpha_t, alpha_tt, LE[6];
    mouvement(c, time + dt, alpha, alpha_t, alpha_tt, LE, b);
    if (b.StartupStep) {
        b.StartupStep = false;
        if (c->TimeMethodSolid == FSIBE_BDF2) { c->ActuallyBDF2 = true; c->TimeMethodSolid = FSIBE_CRANK_NICHOLSON; }
    }
    /* EE1 predictor (SolidSolver.f90:1309-1331) */
    std::vector<double> T(ns), th1 = b.theta, td1 = b.theta_dot;
    int st = RHS_beameqn(c, time, th1.data(), td1.data(), b.p_old.data(), T.data(), b.tau_old.data());
    if (st) return st;
    std::vector<double> g5(ns);
    for (int i = 0; i < ns; ++i) g5[i] = b.theta[i] + dt * th1[i];
    std::vector<double> thg(ns + 3), Tg(ns + 1);  /* thg[i+1] = theta(i), Tg[i+1] = T(i) */
    for (int i = 0; i < ns; ++i) thg[i + 1] = g5[i];
    const double ds2 = ds * ds;
    const double K2 = b.p_new[0] + mue * (LE[5] * std::cos(alpha) - LE[4] * std::sin(alpha) + c->grav * std::cos(alpha));
    const double C2v = 2.0 * ds * K2 - T[0] * thg[2] + (eta / ds2) * (10.0 * thg[1] - 12.0 * thg[2] + 6.0 * thg[3] - thg[4]);
    thg[0] = C2v / ((3.0 * eta / ds2) - T[0]);
    const double A1 = g5[ns - 3] / 12. - 2. * g5[ns - 2] / 3.;
    const double A2 = -g5[ns - 3] / 12. + 4. * g5[ns - 2] / 3. - 5. * g5[ns - 1] / 2.;
    thg[ns + 1] = 3. * (A1 - A2) / 2.;
    thg[ns + 2] = 12. * (2. * A1 - A2);
    const double K1 = mue * (LE[4] * std::cos(alpha) + LE[5] * std::sin(alpha) + c->grav * std::sin(alpha)) - b.tau_new[0];
    const double th_ss0 = (2.0 * thg[1] - 5.0 * thg[2] + 4.0 * thg[3] - 1.0 * thg[4]) / ds2;
    const double th_s0 = (-1.5 * thg[1] + 2.0 * thg[2] - 0.5 * thg[3]) / ds;
    const double T_s0 = -eta * th_ss0 * th_s0 + K1;
    Tg[0] = T[1] - 2.0 * ds * T_s0;
    for (int i = 0; i < ns; ++i) Tg[i + 1] = T[i];
    std::vector<double> x(n), xd(n), F(n), Jr((size_t)n * n), old_rhs(ns, 0.0);
    for (int i = 0; i < ns + 3; ++i) x[i] = thg[i];
    for (int i = 0; i < ns + 1; ++i) x[ns + 3 + i] = Tg[i];
    if (c->TimeMethodSolid == FSIBE_CRANK_NICHOLSON) {
        std::vector<double> th_o = bo5, Td(ns);
        old_rhs = bo6;
        st = RHS_beameqn(c, time, th_o.data(), old_rhs.data(), b.p_old.data(), Td.data(), b.tau_old.data());
        if (st) return st;
    }
    int iter = 0;
    bool iterate = true;
    const double tol = c->P.newton_tol;
    while (iterate) {
        st = F_nonlinear(c, time, dt, dt_old, F.data(), bo5.data(), bo6.data(), x.data(), b.p_new.data(), old_rhs.data(),
                         oo5.data(), oo6.data(), b.tau_new.data());
        if (st) return st;
        for (int k = 0; k < n; ++k) F[k] = -1.0 * F[k];
        st = Jacobi(c, time, dt, dt_old, Jr, x.data(), bo5.data(), bo6.data(), b.p_new.data(), oo5.data(), oo6.data(), b.tau_new.data());
        if (st) return st;
        xd = F;
        if (getrf_solve(n, Jr, xd.data()) != 0) return fail(c, FSIBE_ERR_SINGULAR, "dgetrf: singular Newton matrix");
        for (int k = 0; k < n; ++k) if (std::isnan(xd[k])) return fail(c, FSIBE_ERR_NAN, "NaN in the linear solve");
        iter = iter + 1;
        double sd = 0.0, sx = 0.0;
        for (int k = 0; k < n; ++k) x[k] = x[k] + xd[k];
        for (int k = 0; k < n; ++k) sd += xd[k] * xd[k];
        for (int k = 0; k < n; ++k) sx += x[k] * x[k];
        const double err = std::sqrt(sd);
        const double err_rel = std::fabs(std::sqrt(sd) / std::sqrt(sx));
        if ((err < tol || err_rel < tol) && iter > 2) iterate = false;
        if (iter > c->P.newton_maxit - 1) return fail(c, FSIBE_ERR_NEWTON_MAXIT, "IBES: Newton did not converge");
    }
    for (int i = 0; i < ns; ++i) b.theta[i] = x[1 + i];
    double C1, C2, C3, C4;
    solid_coeffs(c->TimeMethodSolid, dt, dt_old, C1, C2, C3, C4);
    for (int i = 0; i < ns; ++i) b.theta_dot[i] = (C1 / dt) * (b.theta[i] - C3 * bo5[i] - C4 * oo5[i]) - C2 * bo6[i];
    integrate_position(c, time + dt, b);
    for (int i = 0; i < ns; ++i) {
        b.ax[i] = (b.vx[i] - bo3[i]) / dt;
        b.ay[i] = (b.vy[i] - bo4[i]) / dt;
    }
    double mx = 0.0;
    for (int i = 0; i < ns; ++i) mx = std::max(mx, std::fabs(b.theta_dot[i] - bo6[i]));
    c->sc.newton_iters = iter;
    if (c->ActuallyBDF2) { c->TimeMethodSolid = FSIBE_BDF2; c->ActuallyBDF2 = false; }
    b.oldold = beam_old_full;
    b.dt_old = dt;
    if (mx > 100.0) return fail(c, FSIBE_ERR_BRAKE, "IBES: emergency brake, |d theta_dot| > 100");
    return FSIBE_OK;
}

static int SolidSolverWrapper(orc_ctx* c, double time, double dt) {  /* SolidSolver.f90:13-44 */
    int st = FSIBE_OK;
    if (time > c->P.t_release) st = IBES_solver(c, time, dt);
    else integrate_position(c, time + dt, c->beam);
    SolidEnergies(c);
    return st;
}

static void fill_scalars(orc_ctx* c) {
    Beam& b = c->beam;
    const int ns = c->ns;
    fsibe_scalars& s = c->sc;
    s.time = c->time; s.dt0 = c->dt0; s.dt1 = c->dt1;
    for (int q = 0; q < 2; ++q) {
        s.force[q] = b.Force[q]; s.force_unst[q] = b.Force_unst[q];
        s.force_press[q] = b.Force_press[q]; s.inertial_force[q] = b.Inertial[q];
    }
    s.e_kinetic = b.E_kin; s.e_elastic = b.E_el; s.e_pot = b.E_pot;
    const double row[21] = {c->time, b.p_new[ns - 1], b.p_new[3 * ns / 4], b.p_new[ns / 2], b.x[ns - 1], b.y[ns - 1],
                            b.vx[ns - 1], b.vy[ns - 1], b.theta[ns - 1], b.theta_dot[ns - 1], b.Force[0], b.Force[1],
                            b.Force_unst[0], b.Force_unst[1], b.Force_press[0], b.Force_press[1], b.Inertial[0],
                            b.Inertial[1], b.E_kin, b.E_el, b.E_pot};
    std::memcpy(s.beam_data, row, sizeof(row));
}

static bool is_pow2(int v) { return v >= 8 && (v & (v - 1)) == 0; }

/* Fortran sequential unformatted records (gfortran framing: a 4-byte length before and after
 * each record), as MakeRuntimeBackup writes them with -r8 (reals 8 bytes, integers and
 * logicals 4). */
struct RecWriter {
    std::vector<char> rec;
    FILE* f;
    void put(const void* p, size_t n) { const char* q = static_cast<const char*>(p); rec.insert(rec.end(), q, q + n); }
    void d(double v) { put(&v, 8); }
    void i(int32_t v) { put(&v, 4); }
    void dv(const double* p, size_t n) { put(p, 8 * n); }
    bool end() {
        const int32_t n = (int32_t)rec.size();
        const bool ok = fwrite(&n, 4, 1, f) == 1 && (rec.empty() || fwrite(rec.data(), 1, rec.size(), f) == rec.size()) &&
                        fwrite(&n, 4, 1, f) == 1;
        rec.clear();
        return ok;
    }
};
struct RecReader {
    std::vector<char> rec;
    size_t pos = 0;
    FILE* f;
    bool next() {
        int32_t n = 0, m = 0;
        if (fread(&n, 4, 1, f) != 1 || n < 0) return false;
        rec.resize((size_t)n);
        if (n > 0 && fread(rec.data(), 1, (size_t)n, f) != (size_t)n) return false;
        if (fread(&m, 4, 1, f) != 1 || m != n) return false;
        pos = 0;
        return true;
    }
    bool get(void* p, size_t n) {
        if (pos + n > rec.size()) return false;
        std::memcpy(p, rec.data() + pos, n);
        pos += n;
        return true;
    }
    bool d(double& v) { return get(&v, 8); }
    bool i(int32_t& v) { return get(&v, 4); }
    bool dv(double* p, size_t n) { return get(p, 8 * n); }
};

}  // namespace

/* ==================================================================================
 * C API of the oracle (same argument meaning as include/fsibe.h, prefix orc_)
 * ================================================================================== */
extern "C" {

int orc_create(const fsibe_params* p, orc_ctx** out) {
    if (!p || !out) return FSIBE_ERR_PARAM;
    if (!is_pow2(p->nx) || !is_pow2(p->ny) || p->ns < 8) return FSIBE_ERR_PARAM;
    orc_ctx* c = new orc_ctx();
    c->P = *p;
    c->nx = p->nx; c->ny = p->ny; c->ns = p->ns;
    c->pi = 4.0 * std::atan(1.0);
    c->scalex = (2.0 * c->pi / p->xl) * (2.0 * c->pi / p->xl);
    c->scaley = (2.0 * c->pi / p->yl) * (2.0 * c->pi / p->yl);
    c->ds = p->length / (double)(p->ns - 1);
    c->dx = p->xl / (double)p->nx;
    c->dy = p->yl / (double)p->ny;
    c->TimeMethodSolid = p->time_method_solid;
    c->grav = p->grav;
    c->sharp = std::fabs(p->N_smooth) < 1e-4;
    if (c->P.newton_tol <= 0.0) c->P.newton_tol = 1.0e-7;
    if (c->P.newton_maxit <= 0) c->P.newton_maxit = 50;
    /* mouvement.f90:102-104: the Paraz cases set the forces' soft start-up to one period */
    if (c->P.iMotion >= 401 && c->P.iMotion <= 413) c->P.tau = kParazT[c->P.iMotion - 401];
    const size_t NN = (size_t)c->nx * c->ny;
    for (auto* v : {&c->dealiase, &c->mask, &c->maskvx, &c->maskvy, &c->vor_mean, &c->press, &c->mask_sponge, &c->mask_frame})
        v->assign(NN, 0.0);
    for (int q = 0; q < 2; ++q) { c->vortk[q].assign(NN, 0.0); c->nlk[q].assign(NN, 0.0); c->workvis[q].assign(NN, 0.0); }
    c->u.assign(2 * NN, 0.0);
    c->ft.assign((size_t)(c->nx / 2) * c->ny, cplx{0, 0});
    c->rx.init(c->nx);
    c->cy.init(c->ny);
    dealiase_mask(c);
    std::memset(&c->sc, 0, sizeof(c->sc));
    *out = c;
    return FSIBE_OK;
}

int orc_destroy(orc_ctx* c) { delete c; return FSIBE_OK; }
const char* orc_last_error(const orc_ctx* c) { return c ? c->err.c_str() : ""; }
int orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n; return 1;
#endif
}

int orc_fft_forward(orc_ctx* c, const double* f, double* fk) { coftxy(c, f, fk); return FSIBE_OK; }
int orc_fft_inverse(orc_ctx* c, const double* fk, double* f) { cofitxy(c, fk, f); return FSIBE_OK; }
int orc_cofdx(orc_ctx* c, const double* a, double* b) { cofdx(c, a, b); return FSIBE_OK; }
int orc_cofdy(orc_ctx* c, const double* a, double* b) { cofdy(c, a, b); return FSIBE_OK; }
int orc_cofdxdx(orc_ctx* c, const double* a, double* b) { cofdxdx(c, a, b); return FSIBE_OK; }
int orc_cofdydy(orc_ctx* c, const double* a, double* b) { cofdydy(c, a, b); return FSIBE_OK; }
int orc_cofdxdy(orc_ctx* c, const double* a, double* b) { cofdxdy(c, a, b); return FSIBE_OK; }
int orc_poisson(orc_ctx* c, const double* a, double* b) { poisson(c, a, b); return FSIBE_OK; }
int orc_vis(orc_ctx* c, double dt, double* w) { vis(c, dt, w); return FSIBE_OK; }
int orc_dealiase_mask(orc_ctx* c, double* d) { std::memcpy(d, c->dealiase.data(), c->dealiase.size() * 8); return FSIBE_OK; }

int orc_init_fields(orc_ctx* c, const double* vort) {  /* time_step.f90:29-113 with inicond=111 */
    c->time = 0.0; c->dt1 = 0.0; c->dt0 = 0.0;
    c->TimeMethodSolid = c->P.time_method_solid;
    c->ActuallyBDF2 = false;
    c->grav = c->P.grav;
    init_beams(c);
    c->beam.StartupStep = true;
    const size_t NN = (size_t)c->nx * c->ny;
    for (int q = 0; q < 2; ++q) { std::fill(c->vortk[q].begin(), c->vortk[q].end(), 0.0); std::fill(c->nlk[q].begin(), c->nlk[q].end(), 0.0); }
    std::fill(c->vor_mean.begin(), c->vor_mean.end(), 0.0);
    std::fill(c->press.begin(), c->press.end(), 0.0);
    c->n1 = 1; c->n0 = 0;
    coftxy(c, vort, c->vortk[0].data());
    std::vector<double> stream(NN);
    c->U_mean_true = (c->P.iWalls == 1) ? 1.0 - 2.0 * c->P.h_channel / c->P.yl : 1.0;  /* time_step.f90:95-100 */
    cal_velocity(c, 0.0, c->vortk[0].data(), c->u.data(), stream.data());
    int st = create_mask(c, c->time);
    if (st) return st;
    create_sponge_mask(c);
    c->initialized = true;
    c->startup_done = false;
    std::memset(&c->sc, 0, sizeof(c->sc));
    fill_scalars(c);
    return FSIBE_OK;
}

int orc_create_mask(orc_ctx* c, double time) { return create_mask(c, time); }

int orc_fluid_step(orc_ctx* c, int explicit_step) {
    if (!c->initialized) return FSIBE_ERR_STATE;
    if (explicit_step) EvolveFluidExplicit(c);
    else EvolveFluidAB2(c);
    return FSIBE_OK;
}

int orc_get_forces(orc_ctx* c, double time) { return GetForces(c, time); }

int orc_solid_step(orc_ctx* c, double time) {
    GravityImpulse(c, time);
    return SolidSolverWrapper(c, time, c->dt1);
}

int orc_advance(orc_ctx* c) {
    std::swap(c->n0, c->n1);
    c->time = c->time + c->dt1;
    c->beam.p_old = c->beam.p_new;
    c->beam.tau_old = c->beam.tau_new;
    fill_scalars(c);
    c->sc.step += 1;
    return FSIBE_OK;
}

int orc_step(orc_ctx* c) {  /* time_step.f90:120-162 (startup) or :178-228 */
    if (!c->initialized) return FSIBE_ERR_STATE;
    const fsibe_params& P = c->P;
    int st = FSIBE_OK;
    if (!c->startup_done) {
        if (P.iFLUSI == 1 || P.iMotion > 0 || (P.iSponge >= 4 && c->time < P.T_fullspeed)) { st = create_mask(c, c->time); if (st) return st; }
        EvolveFluidExplicit(c);
        if (P.iFLUSI == 1 || P.iSaveBeam > 0) { st = GetForces(c, c->time); if (st) return st; }
        if (P.iFLUSI == 1) {
            GravityImpulse(c, c->time);
            st = SolidSolverWrapper(c, c->time, c->dt1);
        } else if (P.iMotion > 0) integrate_position(c, c->time, c->beam);
        orc_advance(c);
        c->startup_done = true;
        return st;
    }
    c->dt0 = c->dt1;
    if (P.iFLUSI == 1 || P.iMotion > 0 || (P.iSponge >= 4 && c->time < P.T_fullspeed)) { st = create_mask(c, c->time); if (st) return st; }
    EvolveFluidAB2(c);
    if (P.iFLUSI == 1 || P.iSaveBeam > 0) { st = GetForces(c, c->time); if (st) return st; }
    if (P.iFLUSI == 1) {
        GravityImpulse(c, c->time);
        st = SolidSolverWrapper(c, c->time, c->dt1);
    } else if (P.iMotion > 0) integrate_position(c, c->time, c->beam);
    orc_advance(c);
    return st;
}

int orc_run(orc_ctx* c, int nsteps, double* rows) {
    for (int s = 0; s < nsteps; ++s) {
        int st = orc_step(c);
        if (rows) std::memcpy(rows + (size_t)s * 21, c->sc.beam_data, 21 * sizeof(double));
        if (st) return st;
    }
    return FSIBE_OK;
}

/* The time loop with its per-step output (time_step.f90:178-236): per step the beam_data row
 * (BeamIO.f90:193-216), then the rows the step appends to u_max (NavierStokes.f90:80-82),
 * energies (:259-261) and IBES_iter (SolidSolver.f90:392-394), which carry the time before
 * the step. */
int orc_run_records(orc_ctx* c, int nsteps, double* rec) {
    for (int s = 0; s < nsteps; ++s) {
        const double t_before = c->time;
        int st = orc_step(c);
        if (rec) {
            double* r = rec + (size_t)s * FSIBE_RECORD_COLS;
            std::memcpy(r, c->sc.beam_data, 21 * sizeof(double));
            const fsibe_scalars& q = c->sc;
            double al, al_t, al_tt, LE[6];  /* BeamIO.f90:229-238: mouvement(time) after the step */
            mouvement(c, c->time, al, al_t, al_tt, LE, c->beam);
            const double tail[FSIBE_RECORD_COLS - 21] = {
                t_before, q.dt1, q.u_max, q.mean_ux, q.mean_uy,
                t_before, q.dt1, q.vor_rms, q.kinetic, q.dissipation, q.porous_diss, q.inflow_solid, q.inflow_mean,
                t_before, (double)q.newton_iters,
                c->time, al, al_t, al_tt, LE[0], LE[1], LE[2], LE[3], LE[4], LE[5]};
            std::memcpy(r + 21, tail, sizeof(tail));
        }
        if (st) return st;
    }
    return FSIBE_OK;
}

int orc_upload_vortk(orc_ctx* c, const double* v) { std::memcpy(c->vortk[c->n0].data(), v, c->vortk[0].size() * 8); return FSIBE_OK; }
int orc_download_vortk(orc_ctx* c, double* v) { std::memcpy(v, c->vortk[c->n0].data(), c->vortk[0].size() * 8); return FSIBE_OK; }
int orc_download_vort(orc_ctx* c, double* v) { cofitxy(c, c->vortk[c->n0].data(), v); return FSIBE_OK; }
int orc_upload_u(orc_ctx* c, const double* u) { std::memcpy(c->u.data(), u, c->u.size() * 8); return FSIBE_OK; }
int orc_download_u(orc_ctx* c, double* u) { std::memcpy(u, c->u.data(), c->u.size() * 8); return FSIBE_OK; }
int orc_download_press(orc_ctx* c, double* p) { std::memcpy(p, c->press.data(), c->press.size() * 8); return FSIBE_OK; }
int orc_upload_press(orc_ctx* c, const double* p) { std::memcpy(c->press.data(), p, c->press.size() * 8); return FSIBE_OK; }
int orc_download_vor_mean(orc_ctx* c, double* p) { std::memcpy(p, c->vor_mean.data(), c->vor_mean.size() * 8); return FSIBE_OK; }
int orc_upload_mask(orc_ctx* c, const double* m, const double* vx, const double* vy) {
    const size_t NN = c->mask.size() * 8;
    std::memcpy(c->mask.data(), m, NN); std::memcpy(c->maskvx.data(), vx, NN); std::memcpy(c->maskvy.data(), vy, NN);
    return FSIBE_OK;
}
int orc_download_mask(orc_ctx* c, double* m, double* vx, double* vy) {
    const size_t NN = c->mask.size() * 8;
    std::memcpy(m, c->mask.data(), NN); std::memcpy(vx, c->maskvx.data(), NN); std::memcpy(vy, c->maskvy.data(), NN);
    return FSIBE_OK;
}
int orc_upload_beam(orc_ctx* c, const double* beam, const double* po, const double* pn, const double* to, const double* tn) {
    Beam& b = c->beam;
    const int ns = c->ns;
    if (b.x.size() != (size_t)ns) b.alloc(ns);
    std::vector<double>* cols[6] = {&b.x, &b.y, &b.vx, &b.vy, &b.theta, &b.theta_dot};
    for (int q = 0; q < 6; ++q) std::memcpy(cols[q]->data(), beam + (size_t)q * ns, ns * 8);
    if (po) std::memcpy(b.p_old.data(), po, ns * 8);
    if (pn) std::memcpy(b.p_new.data(), pn, ns * 8);
    if (to) std::memcpy(b.tau_old.data(), to, ns * 8);
    if (tn) std::memcpy(b.tau_new.data(), tn, ns * 8);
    return FSIBE_OK;
}
int orc_download_beam(orc_ctx* c, double* beam, double* po, double* pn, double* to, double* tn) {
    Beam& b = c->beam;
    const int ns = c->ns;
    const std::vector<double>* cols[6] = {&b.x, &b.y, &b.vx, &b.vy, &b.theta, &b.theta_dot};
    if (beam) for (int q = 0; q < 6; ++q) std::memcpy(beam + (size_t)q * ns, cols[q]->data(), ns * 8);
    if (po) std::memcpy(po, b.p_old.data(), ns * 8);
    if (pn) std::memcpy(pn, b.p_new.data(), ns * 8);
    if (to) std::memcpy(to, b.tau_old.data(), ns * 8);
    if (tn) std::memcpy(tn, b.tau_new.data(), ns * 8);
    return FSIBE_OK;
}
int orc_get_scalars(orc_ctx* c, fsibe_scalars* s) {
    fill_scalars(c);
    *s = c->sc;
    s->time = c->time;
    return FSIBE_OK;
}

/* Building blocks exposed for the known-answer tests. */
double orc_delta_phi4star(double r) { return delta_phi4star(r, 1.0, 4.0 * std::atan(1.0)); }
int orc_differentiate1d(const double* f, double* fd, int n, double dx, int order) { Differentiate1D(f, fd, n, dx, order); return 0; }
int orc_gttrf_solve(int n, double* dl, double* d, double* du, double* b) {
    std::vector<double> vdl(dl, dl + n - 1), vd(d, d + n), vdu(du, du + n - 1);
    return gttrf_solve(n, vdl, vd, vdu, b);
}
int orc_getrf_solve(int n, double* A, double* b) {
    std::vector<double> vA(A, A + (size_t)n * n);
    return getrf_solve(n, vA, b);
}
/* F and the analytic Jacobian of the current Newton system at x, for the FD Jacobian test
 * (mirrors the self-test Jacobi_num, SolidSolver.f90:244-274). */
int orc_newton_system(orc_ctx* c, double time, double dt, double dt_old, int method, const double* x,
                      const double* theta_old, const double* theta_dot_old, const double* p, const double* old_rhs,
                      const double* theta_oldold, const double* theta_dot_oldold, const double* tau, double* F, double* J) {
    const int n = 2 * c->ns + 4;
    int save = c->TimeMethodSolid;
    c->TimeMethodSolid = method;
    int st = F_nonlinear(c, time, dt, dt_old, F, theta_old, theta_dot_old, x, p, old_rhs, theta_oldold, theta_dot_oldold, tau);
    std::vector<double> Jr((size_t)n * n);
    if (!st) st = Jacobi(c, time, dt, dt_old, Jr, x, theta_old, theta_dot_old, p, theta_oldold, theta_dot_oldold, tau);
    if (J) std::memcpy(J, Jr.data(), Jr.size() * 8);
    c->TimeMethodSolid = save;
    return st;
}
double orc_time(orc_ctx* c) { return c->time; }

/* BeamSurfaceIntegral (BeamForces.f90:306-509), the diagnostic GetForces runs when
 * viscous_tensions (:129): the stresses (as GetForces forms them from u, :105-118) and the
 * pressure interpolated with phi4* on the contour around the beam -- two half circles of
 * nc = 128 points at the ends, the top and bottom lines at t_beam + N_smooth max(dx,dy)
 * (pressure at t_beam) -- and the penalization drag/lift over the whole grid.
 * out[11]: time, drag, lift, drag_surf, lift_surf, Ft(1), Fn(1), Fp(1), Ft(2), Fn(2), Fp(2)
 * (the columns of the 'surface' file, :492-499). */
/* ComputePressureSnapshot (NavierStokes.f90:598-665): the static pressure of the state's
 * vorticity at `time` (its mean flow) and the current mask, outside the time step. */
int orc_pressure_snapshot(orc_ctx* c, double time, double* press) {
    if (!c || !press) return FSIBE_ERR_PARAM;
    if (!c->initialized) return fail(c, FSIBE_ERR_STATE, "pressure snapshot before init_fields");
    const size_t NN = (size_t)c->nx * c->ny;
    std::vector<double> u(2 * NN), work1(NN), work2(NN), work_dx(NN), work_dy(NN), pen1(NN), pen2(NN);
    const double* vortk = c->vortk[c->n0].data();
    cal_velocity(c, time, vortk, u.data(), work1.data());
    for (size_t k = 0; k < NN; ++k) {
        pen1[k] = c->mask[k] * (u[k] - c->maskvx[k]);
        pen2[k] = c->mask[k] * (u[NN + k] - c->maskvy[k]);
    }
    cofitxy(c, vortk, work1.data());
    coftxy(c, pen1.data(), work2.data());
    cofdx(c, work2.data(), pen1.data());
    coftxy(c, pen2.data(), work2.data());
    cofdy(c, work2.data(), pen2.data());
    for (size_t k = 0; k < NN; ++k) {
        work_dx[k] = -work1[k] * u[NN + k];
        work_dy[k] = +work1[k] * u[k];
    }
    coftxy(c, work_dx.data(), work1.data());
    cofdx(c, work1.data(), work_dx.data());
    coftxy(c, work_dy.data(), work1.data());
    cofdy(c, work1.data(), work_dy.data());
    for (size_t k = 0; k < NN; ++k) work1[k] = pen1[k] + pen2[k] + work_dy[k] + work_dx[k];
    std::vector<double> q(NN);
    poisson(c, work1.data(), q.data());
    cofitxy(c, q.data(), work1.data());
    for (size_t k = 0; k < NN; ++k) press[k] = work1[k] - 0.5 * (u[k] * u[k] + u[NN + k] * u[NN + k]);
    return FSIBE_OK;
}

int orc_surface_integral(orc_ctx* c, double time, double* out) {
    if (!c || !out) return FSIBE_ERR_PARAM;
    if (!c->initialized) return fail(c, FSIBE_ERR_STATE, "surface_integral before init_fields");
    if (c->P.iViscous != 1 || c->P.iBeam <= 0) return fail(c, FSIBE_ERR_PARAM, "BeamSurfaceIntegral needs iViscous = 1 and a beam");
    // BeamForces.f90:331-336: no surface integral with the leading-edge cylinder
    if (c->P.iCylinder == 1) return fail(c, FSIBE_ERR_UNSUPPORTED, "BeamSurfaceIntegral is not computed with a cylinder at the leading edge");
    const size_t NN = (size_t)c->nx * c->ny;
    const int ns = c->ns, nc = 128;
    const Beam& b = c->beam;
    const double pi = c->pi, dx = c->dx, dy = c->dy;
    std::vector<double> sa(NN), sb(NN), w1(NN), w2(NN), w3(NN);
    const double* u1 = c->u.data();
    const double* u2 = c->u.data() + NN;
    coftxy(c, u1, w1.data()); cofdx(c, w1.data(), w2.data()); cofitxy(c, w2.data(), sa.data());
    for (size_t k = 0; k < NN; ++k) sa[k] = 2.0 * c->P.nu * sa[k];
    coftxy(c, u1, w1.data()); cofdy(c, w1.data(), w2.data()); cofitxy(c, w2.data(), w3.data());
    coftxy(c, u2, w1.data()); cofdx(c, w1.data(), w2.data()); cofitxy(c, w2.data(), sb.data());
    for (size_t k = 0; k < NN; ++k) sb[k] = c->P.nu * (w3[k] + sb[k]);
    double alpha, alpha_t, alpha_tt, LE[6];
    mouvement(c, time, alpha, alpha_t, alpha_tt, LE, b);
    double Ft[2] = {0, 0}, Fn[2] = {0, 0}, Fp[2] = {0, 0};
    int st = FSIBE_OK;
    const double R = c->P.t_beam + c->P.N_smooth * std::max(dx, dy);
    const double dphi = pi / (double)(nc - 1), dL = dphi * R;
    for (int end = 0; end < 2; ++end) {  /* trailing edge (:341-377), leading edge (:379-420) */
        const int node = end == 0 ? ns - 1 : 0;
        const double beta = (end == 0 ? b.theta[ns - 1] : b.theta[1]) + alpha;
        for (int i = 0; i < nc; ++i) {
            const double phi = (end == 0 ? -(0.5 * pi - beta) : (0.5 * pi + beta)) + (double)i * dphi;
            const double xc = b.x[node] + R * std::cos(phi), yc = b.y[node] + R * std::sin(phi);
            double A, B, P;
            st |= DeltaInterpolation(c, xc, yc, sa.data(), A);
            st |= DeltaInterpolation(c, xc, yc, sb.data(), B);
            st |= DeltaInterpolation(c, xc, yc, c->press.data(), P);
            const double sn = +A * std::cos(2.0 * phi) + B * std::sin(2.0 * phi);
            const double stt = -A * std::sin(2.0 * phi) + B * std::cos(2.0 * phi);
            const double sp = -P;
            Ft[0] = Ft[0] + dL * stt * (-std::sin(phi));
            Ft[1] = Ft[1] + dL * stt * (+std::cos(phi));
            Fn[0] = Fn[0] + dL * sn * (+std::cos(phi));
            Fn[1] = Fn[1] + dL * sn * (+std::sin(phi));
            Fp[0] = Fp[0] + dL * sp * (+std::cos(phi));
            Fp[1] = Fp[1] + dL * sp * (+std::sin(phi));
        }
    }
    for (int side = 0; side < 2; ++side) {  /* top (:426-451), bottom (:456-480) */
        const double sg = side == 0 ? 1.0 : -1.0;
        for (int i = 0; i < ns; ++i) {
            const double th = b.theta[i] + alpha, s = std::sin(th), co = std::cos(th);
            const double x = b.x[i] - sg * R * s, y = b.y[i] + sg * R * co;
            const double x1 = b.x[i] - sg * c->P.t_beam * s, y1 = b.y[i] + sg * c->P.t_beam * co;
            double A, B, P;
            st |= DeltaInterpolation(c, x, y, sa.data(), A);
            st |= DeltaInterpolation(c, x, y, sb.data(), B);
            st |= DeltaInterpolation(c, x1, y1, c->press.data(), P);
            const double sn = -A * std::cos(2.0 * th) - B * std::sin(2.0 * th);
            const double stt = -A * std::sin(2.0 * th) + B * std::cos(2.0 * th);
            const double sp = -P;
            Ft[0] = Ft[0] + c->ds * stt * (sg * co);
            Ft[1] = Ft[1] + c->ds * stt * (sg * s);
            Fn[0] = Fn[0] + c->ds * sn * (-sg * s);
            Fn[1] = Fn[1] + c->ds * sn * (sg * co);
            Fp[0] = Fp[0] + c->ds * sp * (-sg * s);
            Fp[1] = Fp[1] + c->ds * sp * (sg * co);
        }
    }
    if (st) return fail(c, FSIBE_ERR_INTERP_OOB, "DeltaInterpolation: target coordinates not in the field");
    double drag = 0.0, lift = 0.0;
    for (size_t k = 0; k < NN; ++k) {
        drag += c->mask[k] * (u1[k] - c->maskvx[k]);
        lift += c->mask[k] * (u2[k] - c->maskvy[k]);
    }
    out[0] = time;
    out[1] = c->P.iWalls > 0 ? 0.0 : drag * dx * dy;  // with walls the file's drag and lift are 0 (:494-502)
    out[2] = c->P.iWalls > 0 ? 0.0 : lift * dx * dy;
    out[3] = Ft[0] + Fn[0] + Fp[0];
    out[4] = Ft[1] + Fn[1] + Fp[1];
    out[5] = Ft[0]; out[6] = Fn[0]; out[7] = Fp[0];
    out[8] = Ft[1]; out[9] = Fn[1]; out[10] = Fp[1];
    return FSIBE_OK;
}

/* MakeRuntimeBackup (save_fields.f90:109-152): the records of runtime_backup<n>.in for the
 * state between two steps (n0 the current level, n1 the previous one, after the level
 * switch of time_step.f90:152/222). */
int orc_write_backup(orc_ctx* c, const char* path) {
    if (!c || !path) return FSIBE_ERR_PARAM;
    if (!c->initialized) return fail(c, FSIBE_ERR_STATE, "write_backup before init_fields");
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(c, FSIBE_ERR_PARAM, "cannot open the backup file for writing");
    const size_t NN = (size_t)c->nx * c->ny;
    RecWriter w;
    w.f = f;
    bool ok = true;
    w.d(c->time); ok = ok && w.end();
    w.d(123.0); ok = ok && w.end();  /* checksum */
    w.i(c->n1); w.d(c->dt1);
    for (int q = 0; q < 2; ++q) w.dv(c->vortk[q].data(), NN);
    for (int q = 0; q < 2; ++q) w.dv(c->nlk[q].data(), NN);
    for (int q = 0; q < 2; ++q) w.dv(c->workvis[q].data(), NN);
    w.dv(c->mask.data(), NN); w.dv(c->maskvx.data(), NN); w.dv(c->maskvy.data(), NN);
    w.i(1);  /* ivideo */
    w.dv(c->u.data(), 2 * NN);
    ok = ok && w.end();
    w.i(c->ns); ok = ok && w.end();
    w.d(0.0); w.i(0); ok = ok && w.end();  /* colorscale, colorscale_done */
    if (c->P.iBeam > 0) {
        const Beam& b = c->beam;
        const size_t ns = (size_t)c->ns;
        for (const auto* v : {&b.x, &b.y, &b.vx, &b.vy, &b.theta, &b.theta_dot}) w.dv(v->data(), ns);
        ok = ok && w.end();
        for (const auto* v : {&b.p_new, &b.p_old, &b.tau_new, &b.tau_old}) w.dv(v->data(), ns);
        ok = ok && w.end();
        w.dv(b.Force, 2); w.dv(b.Force_unst, 2); w.dv(b.Force_press, 2);
        w.d(b.E_kin); w.d(b.E_pot); w.d(b.E_el); w.d(b.x0); w.d(b.y0);
        ok = ok && w.end();
        w.d(b.AngleBeam); w.i(b.iMouvement); w.d(b.drag_unst_new); w.d(b.drag_unst_old);
        w.d(b.lift_unst_new); w.d(b.lift_unst_old);
        ok = ok && w.end();
        w.i(b.UnstReady ? 1 : 0); w.d(b.dt_old); w.dv(b.oldold.data(), 6 * ns);
        ok = ok && w.end();
        w.dv(b.ax.data(), ns); w.dv(b.ay.data(), ns); w.dv(b.Inertial, 2);
        ok = ok && w.end();
    }
    w.dv(c->vor_mean.data(), NN); ok = ok && w.end();
    ok = (std::fclose(f) == 0) && ok;
    return ok ? FSIBE_OK : fail(c, FSIBE_ERR_PARAM, "writing the backup file failed");
}

/* Resume from a backup: init_fields with inicond = 2 (init_fields.f90:44-100) and what
 * time_step does around it (time_step.f90:60-84): init_beams, InitializeSolidSolver (the next
 * solid step is a start-up step), the records, n0 = 1 - n1, the start-up mask; no Euler
 * start-up step follows. */
int orc_read_backup(orc_ctx* c, const char* path) {
    if (!c || !path) return FSIBE_ERR_PARAM;
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(c, FSIBE_ERR_PARAM, "cannot open the backup file");
    const size_t NN = (size_t)c->nx * c->ny;
    c->TimeMethodSolid = c->P.time_method_solid;
    c->ActuallyBDF2 = false;
    c->grav = c->P.grav;
    init_beams(c);
    c->beam.StartupStep = true;
    RecReader r;
    r.f = f;
    bool ok = true;
    double time = 0.0, checksum = 0.0, dt1 = 0.0, colorscale = 0.0;
    int32_t n1 = 1, ivideo = 0, ns = 0, cdone = 0;
    ok = ok && r.next() && r.d(time);
    ok = ok && r.next() && r.d(checksum) && checksum == 123.0;
    ok = ok && r.next() && r.i(n1) && r.d(dt1) && (n1 == 0 || n1 == 1);
    for (int q = 0; q < 2 && ok; ++q) ok = r.dv(c->vortk[q].data(), NN);
    for (int q = 0; q < 2 && ok; ++q) ok = r.dv(c->nlk[q].data(), NN);
    for (int q = 0; q < 2 && ok; ++q) ok = r.dv(c->workvis[q].data(), NN);
    ok = ok && r.dv(c->mask.data(), NN) && r.dv(c->maskvx.data(), NN) && r.dv(c->maskvy.data(), NN);
    ok = ok && r.i(ivideo) && r.dv(c->u.data(), 2 * NN);
    ok = ok && r.next() && r.i(ns) && ns == c->ns;
    ok = ok && r.next() && r.d(colorscale) && r.i(cdone);
    if (ok && c->P.iBeam > 0) {
        Beam& b = c->beam;
        const size_t nsz = (size_t)c->ns;
        int32_t imv = 0, ready = 0;
        ok = r.next();
        for (auto* v : {&b.x, &b.y, &b.vx, &b.vy, &b.theta, &b.theta_dot}) ok = ok && r.dv(v->data(), nsz);
        ok = ok && r.next();
        for (auto* v : {&b.p_new, &b.p_old, &b.tau_new, &b.tau_old}) ok = ok && r.dv(v->data(), nsz);
        ok = ok && r.next() && r.dv(b.Force, 2) && r.dv(b.Force_unst, 2) && r.dv(b.Force_press, 2) && r.d(b.E_kin) &&
             r.d(b.E_pot) && r.d(b.E_el) && r.d(b.x0) && r.d(b.y0);
        ok = ok && r.next() && r.d(b.AngleBeam) && r.i(imv) && r.d(b.drag_unst_new) && r.d(b.drag_unst_old) &&
             r.d(b.lift_unst_new) && r.d(b.lift_unst_old);
        ok = ok && r.next() && r.i(ready) && r.d(b.dt_old) && r.dv(b.oldold.data(), 6 * nsz);
        ok = ok && r.next() && r.dv(b.ax.data(), nsz) && r.dv(b.ay.data(), nsz) && r.dv(b.Inertial, 2);
        b.iMouvement = imv;
        b.UnstReady = ready != 0;
    }
    ok = ok && r.next() && r.dv(c->vor_mean.data(), NN);
    std::fclose(f);
    if (!ok) return fail(c, FSIBE_ERR_PARAM, "not a runtime backup of this configuration (record, checksum or ns)");
    c->time = time;
    c->dt1 = dt1;
    c->dt0 = dt1;
    c->n1 = n1;
    c->n0 = 1 - n1;
    c->U_mean_true = (c->P.iWalls == 1) ? 1.0 - 2.0 * c->P.h_channel / c->P.yl : 1.0;
    const int st = create_mask(c, c->time);
    if (st) return st;
    create_sponge_mask(c);
    c->initialized = true;
    c->startup_done = true;
    std::memset(&c->sc, 0, sizeof(c->sc));
    fill_scalars(c);
    return FSIBE_OK;
}

}  // extern "C"
