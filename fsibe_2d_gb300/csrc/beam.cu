// beam.cu -- FP64 device code of the flexible beam (IBES_solver, SolidSolver.f90:13-414) on
// one CTA per kernel:
//   * k_beam_pre: gravity, the EE1 predictor with the tension solve (an FP32 tridiagonal
//     elimination preconditioning an FP64 iterative refinement), the initial guess and the
//     Crank-Nicolson right-hand side -- beside the fluid step, on a side stream,
//   * k_beam: Newton with the analytic Jacobian as a band (interleaved theta/T ordering,
//     kl = ku = 7); J dx = -F by FP64 iterative refinement preconditioned by an FP32 banded LU
//     with partial pivoting whose triangular solves run in chunks in parallel; positions and
//     energies,
//   * k_init_beam.
// FP64 issue is the bottleneck on this chip (one FP64 warp instruction per SMSP every ~64
// cycles, ~64-cycle latency, division ~660 cycles): FP64 work is spread over all warps, serial
// chains run in FP32, divisions are taken out of loops.
#include <math.h>

#include <mutex>

#include "solid.cuh"

namespace fsibe {

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

// ===================================================================================
// Beam solver
// ===================================================================================
// Differentiate1D (SolidSolver.f90:1085-1233): the rows of create_diff_matrices as stencils.
// Coefficients live in constant memory; each row is divided by 2dx / dx^2 / 2dx^3 / dx^4 first
// and summed over increasing column index, like the reference's matmul.
__constant__ double cD1[3][3] = {{-3., 4., -1.}, {1., -4., 3.}, {-1., 0., 1.}};
__constant__ double cD2[3][4] = {{2., -5., 4., -1.}, {-1., 4., -5., 2.}, {1., -2., 1., 0.}};
__constant__ double cD3[3][6] = {{-17.0 / 2., 71.0 / 2., -59., 49., -41.0 / 2., 7.0 / 2.},
                                 {-7.0 / 2., 41.0 / 2., -49., 59., -71.0 / 2., 17.0 / 2.},
                                 {-1., 2., 0., -2., 1., 0.}};
__constant__ double cD4[3][7] = {{35.0 / 6., -31., 137.0 / 2., -242.0 / 3., 107.0 / 2., -19.0, 17.0 / 6.},
                                 {17.0 / 6.0, -19.0, 107.0 / 2.0, -242.0 / 3.0, 137.0 / 2.0, -31.0, 35.0 / 6.0},
                                 {1., -4., 6., -4., 1., 0., 0.}};

namespace {
// The coefficient tables divided once by 2dx / dx^2 / 2dx^3 / dx^4: tab[order-1][row type][q]
struct D1DTab {
    double c[4][3][8];
};

__device__ void d1d_tables(D1DTab* t, double dx) {
    const double den[4] = {2.0 * dx, dx * dx, 2.0 * (dx * dx * dx), (dx * dx) * (dx * dx)};
    for (int e = threadIdx.x; e < 4 * 3 * 8; e += blockDim.x) {
        const int o = e / 24, r = (e / 8) % 3, q = e % 8;
        double v = 0.0;
        if (o == 0 && q < 3) v = cD1[r][q];
        else if (o == 1 && q < 4) v = cD2[r][q];
        else if (o == 2 && q < 6) v = cD3[r][q];
        else if (o == 3 && q < 7) v = cD4[r][q];
        t->c[o][r][q] = v / den[o];
    }
}

__device__ double d1d(const D1DTab* tab, const double* f, int N, int order, int i) {
    const int L = N - 1;
    int rt, j0, len;
    if (order == 1) {
        len = 3;
        if (i == 0) { rt = 0; j0 = 0; } else if (i == L) { rt = 1; j0 = L - 2; } else { rt = 2; j0 = i - 1; }
    } else if (order == 2) {
        if (i == 0) { rt = 0; j0 = 0; len = 4; } else if (i == L) { rt = 1; j0 = L - 3; len = 4; } else { rt = 2; j0 = i - 1; len = 3; }
    } else if (order == 3) {
        if (i == 0 || i == 1) { rt = 0; j0 = i; len = 6; }
        else if (i == L - 1) { rt = 1; j0 = L - 6; len = 6; }
        else if (i == L) { rt = 1; j0 = L - 5; len = 6; }
        else { rt = 2; j0 = i - 2; len = 5; }
    } else {
        if (i == 0 || i == 1) { rt = 0; j0 = i; len = 7; }
        else if (i == L - 1) { rt = 1; j0 = L - 7; len = 7; }
        else if (i == L) { rt = 1; j0 = L - 6; len = 7; }
        else { rt = 2; j0 = i - 2; len = 5; }
    }
    const double* cf = tab->c[order - 1][rt];
    double s = 0.0;
    for (int q = 0; q < len; ++q) s += cf[q] * f[j0 + q];
    return s;
}

struct BeamWS {
    // vectors of length ns (+3 where noted) carved from one workspace (shared memory when it fits)
    double *T, *T_s, *th_s, *th_ss, *th_sss, *tau_s, *dmain, *dup, *ddown, *rhs, *du2;
    double *te, *te_s, *te_ss, *te_ssss;  // ns+3
    double *p_s, *th1, *td1, *td_in, *old_rhs, *tdn, *taun_s, *bo3, *bo4, *bo5, *bo6, *oo5, *oo6;
    double *g5, *x, *F, *xd, *xdi, *bvec, *cs, *pre;  // x/F/xd/xdi/bvec length n; cs/pre length 4*(ns+8)
    float* tf;      // 6 (ns+8) floats: FP32 scratch of the tridiagonal solve
    double* band;   // n x 16: Jacobian band rows (15 used), FP64, kept for the residuals
    int* ipiv;
    // FP32 factor (shared memory when it fits): U rows [1/u_kk, u_k,k+1 .. u_k,k+14, -],
    // L rows [pivot offset (int bits), l_1 .. l_7], the biased exponents e of the row maxima
    // (row scale 2^(1023-e)), and the solve vector
    float *Uf, *Lf, *yf;
    int* rse;
    // chunked solves: chunk count, transfer matrices E (C x 8 x 8) and F (C x 14 x 16), response
    // columns G (n x 8) and H (n x 16), and scratch d, D (C x 8), head, S (C x 16), yl (n)
    int nch;
    float *Ec, *Fc, *Gc, *Hc, *cd, *cD, *chead, *cS, *yl;
    const D1DTab* dtab;
};

// The beam workspace has five parts, each placed in shared memory when it fits (in this
// order of priority) and otherwise in the global copy:
//   scr   FP32 scratch of the chunked solves (chunk states, solve vectors),
//   fact  the FP32 factor: U rows [1/u_kk, u_k,k+1 .. u_k,k+14, -], L rows [pivot offset,
//         l_1 .. l_7], row-scale exponents, and the chunk transfer matrices E (8x8) and
//         F (14x14, rows of 16),
//   vec   the FP64 vectors,
//   band  the FP64 Jacobian band (residuals only),
// and bulk (the chunk response columns G, n x 8, and H, n x 16), which stays in global
// memory: it is read only by the block-parallel corrections.  fact and bulk persist between
// steps in the global copy.
__host__ __device__ inline int beam_chunks(int n) {
    int c = 0;
    while (5 * (c + 1) * (c + 1) <= 3 * n) ++c;  // floor(sqrt(0.6 n))
    c = (c < n / 14) ? c : n / 14;
    c = (c < 64) ? c : 64;
    return (c > 1) ? c : 1;
}
__host__ __device__ inline int chunk_lo(int c, int n, int C) { return (int)(((long long)c * n) / C); }
__host__ __device__ inline size_t r4(size_t v) { return (v + 3) & ~(size_t)3; }
__host__ __device__ inline size_t beam_vec_doubles(int ns) {
    const int n = 2 * ns + 4, L = ns + 8;
    const size_t d = (size_t)29 * L + 5 * (size_t)(n + 8) + 11 * (size_t)L + (size_t)L + 64;
    return (d + 1) & ~(size_t)1;
}
__host__ __device__ inline size_t beam_band_doubles(int ns) { return (size_t)(2 * ns + 4 + 16) * 16; }
__host__ __device__ inline size_t beam_fact_floats(int ns) {
    const int n = 2 * ns + 4, C = beam_chunks(n);
    return r4((size_t)(n + 16) * 25 + (size_t)C * (64 + 224));
}
__host__ __device__ inline size_t beam_scr_floats(int ns) {
    const int n = 2 * ns + 4, C = beam_chunks(n);
    return r4((size_t)C * 48 + 2 * (size_t)(n + 16));
}
__host__ __device__ inline size_t beam_bulk_floats(int ns) { return (size_t)(2 * ns + 4 + 16) * 24; }
// bytes of each part, in the order scr, fact, vec, band
__host__ __device__ inline size_t beam_part_bytes(int ns, int part) {
    switch (part) {
        case 0: return 4 * beam_scr_floats(ns);
        case 1: return 4 * beam_fact_floats(ns);
        case 2: return 8 * beam_vec_doubles(ns);
        default: return 8 * beam_band_doubles(ns);
    }
}

struct BeamParts { double* vec; double* band; float* fact; float* scr; float* bulk; };

// Part addresses: those whose bit is set in mask (1 scr, 2 fact, 4 vec, 8 band) packed in
// shared memory in that order, the rest at their place in the global copy
// [vec | band | fact | scr | bulk].
__device__ BeamParts beam_parts(double* gws, double* smem, int mask, int ns) {
    BeamParts P;
    double* g = gws;
    P.vec = g; g += beam_vec_doubles(ns);
    P.band = g; g += beam_band_doubles(ns);
    float* gf = reinterpret_cast<float*>(g);
    P.fact = gf; gf += beam_fact_floats(ns);
    P.scr = gf; gf += beam_scr_floats(ns);
    P.bulk = gf;
    char* sp = reinterpret_cast<char*>(smem);
    if (mask & 1) { P.scr = reinterpret_cast<float*>(sp); sp += beam_part_bytes(ns, 0); }
    if (mask & 2) { P.fact = reinterpret_cast<float*>(sp); sp += beam_part_bytes(ns, 1); }
    if (mask & 4) { P.vec = reinterpret_cast<double*>(sp); sp += beam_part_bytes(ns, 2); }
    if (mask & 8) { P.band = reinterpret_cast<double*>(sp); }
    return P;
}

__device__ BeamWS carve(const BeamParts& P, int ns) {
    const int n = 2 * ns + 4, L = ns + 8, C = beam_chunks(n);
    BeamWS w;
    double* p = P.vec;
    double** one[] = {&w.T, &w.T_s, &w.th_s, &w.th_ss, &w.th_sss, &w.tau_s, &w.dmain, &w.dup, &w.ddown, &w.rhs, &w.du2,
                      &w.te, &w.te_s, &w.te_ss, &w.te_ssss, &w.p_s, &w.th1, &w.td1, &w.td_in, &w.old_rhs, &w.tdn,
                      &w.taun_s, &w.bo3, &w.bo4, &w.bo5, &w.bo6, &w.oo5, &w.oo6, &w.g5};
    for (unsigned k = 0; k < sizeof(one) / sizeof(one[0]); ++k) { *one[k] = p; p += L; }
    double** nn[] = {&w.x, &w.F, &w.xd, &w.xdi, &w.bvec};
    for (unsigned k = 0; k < sizeof(nn) / sizeof(nn[0]); ++k) { *nn[k] = p; p += n + 8; }
    w.cs = p; p += 4 * L;
    w.pre = p; p += 4 * L;
    w.tf = reinterpret_cast<float*>(p); p += 3 * L;
    w.ipiv = reinterpret_cast<int*>(p);
    w.band = P.band;
    float* f = P.fact;
    w.Uf = f; f += (size_t)(n + 16) * 16;
    w.Lf = f; f += (size_t)(n + 16) * 8;
    w.rse = reinterpret_cast<int*>(f); f += n + 16;
    w.Ec = f; f += (size_t)C * 64;
    w.Fc = f;
    f = P.scr;
    w.cd = f; f += (size_t)C * 8;
    w.cD = f; f += (size_t)C * 8;
    w.chead = f; f += (size_t)C * 16;
    w.cS = f; f += (size_t)C * 16;
    w.yf = f; f += n + 16;
    w.yl = f;
    w.Gc = P.bulk;
    w.Hc = P.bulk + (size_t)(n + 16) * 8;
    w.nch = C;
    return w;
}
}  // namespace

// Workspace length (doubles) of the global copy of the beam workspace for ns nodes.
__host__ size_t beam_ws_doubles(int ns) {
    return beam_vec_doubles(ns) + beam_band_doubles(ns) +
           (beam_fact_floats(ns) + beam_scr_floats(ns) + beam_bulk_floats(ns) + 1) / 2;
}

namespace {

__device__ void solid_coeffs(int method, double dt, double dt_old, double& C1, double& C2, double& C3, double& C4) {
    if (method == FSIBE_EULER_IMPLICIT) { C1 = 1.0; C2 = 0.0; C3 = 1.0; C4 = 0.0; }
    else if (method == FSIBE_CRANK_NICHOLSON) { C1 = 2.0; C2 = 1.0; C3 = 1.0; C4 = 0.0; }
    else {
        const double R = dt / dt_old;
        C1 = (1. + 2. * R) / (1. + R);
        C2 = 0.0;
        C3 = ((1. + R) * (1. + R)) / (1. + 2. * R);
        C4 = (-(R * R)) / (1. + 2. * R);
    }
}

// One pass of an FP64 iterative refinement driven by an FP32 solve (block-cooperative):
// x += c for the FP32 correction c in cf, then the block maxima of |c| and |x| decide.
// Returns 1 when converged (the correction, or the next one predicted from the contraction
// c_k / c_(k-1), is below 2^-44 of the solution, or the corrections stopped shrinking at the
// FP64 residual's rounding floor below 2^-30), -1 on a failure (10 passes, or a stall above
// that floor), 0 to go on.  rbuf: 16 doubles of shared memory.
__device__ int refine_step(double* x, const float* cf, int n, int pass, float& cprev, double* rbuf) {
    unsigned cm = 0;
    unsigned long long xm = 0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const float ck = cf[k];
        const double xn = (pass == 0) ? (double)ck : x[k] + (double)ck;
        x[k] = xn;
        const unsigned a = __float_as_uint(ck) & 0x7fffffffu;
        const unsigned long long ax = (unsigned long long)__double_as_longlong(xn) & 0x7fffffffffffffffull;
        cm = (a > cm) ? a : cm;
        xm = (ax > xm) ? ax : xm;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned c2 = __shfl_xor_sync(0xffffffffu, cm, o);
        const unsigned long long x2 = __shfl_xor_sync(0xffffffffu, xm, o);
        cm = (c2 > cm) ? c2 : cm;
        xm = (x2 > xm) ? x2 : xm;
    }
    if ((threadIdx.x & 31) == 0) {
        rbuf[threadIdx.x >> 5] = __longlong_as_double((long long)cm);
        rbuf[8 + (threadIdx.x >> 5)] = __longlong_as_double((long long)xm);
    }
    __syncthreads();
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) {
        const unsigned c2 = (unsigned)__double_as_longlong(rbuf[q]);
        const unsigned long long x2 = (unsigned long long)__double_as_longlong(rbuf[8 + q]);
        cm = (c2 > cm) ? c2 : cm;
        xm = (x2 > xm) ? x2 : xm;
    }
    const double cmd = (double)__uint_as_float(cm), cpd = (double)cprev;
    const double xmd = __longlong_as_double((long long)xm);
    const double tol = 0x1p-44 * xmd;
    const bool conv = !(cmd > tol) || (pass >= 1 && cmd * cmd <= tol * cpd);
    const bool stall = pass >= 2 && cmd > 0.5 * cpd;
    cprev = __uint_as_float(cm);
    __syncthreads();
    if (conv || (stall && cmd <= 0x1p-30 * xmd)) return 1;
    if (stall || pass >= 9) return -1;
    return 0;
}

// Tridiagonal system (dl, d, du) x = b (dl, du: n-1 entries) solved to the accuracy of
// LAPACK dgttrf + dgttrs: dgttrf's elimination with partial pivoting, in FP32 on one thread,
// preconditions an FP64 iterative refinement with block-cooperative residuals.  fs: 5n
// floats of scratch, ip: n ints.  Returns non-zero on an exactly zero pivot.
__device__ int tri_solve(int n, const double* dl, const double* d, const double* du, const double* b, double* x,
                         float* fs, int* ip) {
    float* __restrict__ fl = fs;
    float* __restrict__ fd = fs + n;
    float* __restrict__ fu = fs + 2 * n;
    float* __restrict__ fu2 = fs + 3 * n;
    float* __restrict__ fy = fs + 4 * n;
    __shared__ int info_s;
    __shared__ double rbuf[16];
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        fd[i] = __double2float_rn(d[i]);
        if (i < n - 1) { fl[i] = __double2float_rn(dl[i]); fu[i] = __double2float_rn(du[i]); }
        fu2[i] = 0.f;
        fy[i] = __double2float_rn(b[i]);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int info = 0;
        for (int i = 0; i < n - 1; ++i) {
            const float di = fd[i], li = fl[i];
            if (fabsf(di) >= fabsf(li)) {
                ip[i] = 0;
                if (di != 0.f) {
                    const float f = __fmul_rn(li, __frcp_rn(di));
                    fl[i] = f;
                    fd[i + 1] = __fmaf_rn(-f, fu[i], fd[i + 1]);
                }
            } else {
                const float f = __fmul_rn(di, __frcp_rn(li));
                fd[i] = li;
                fl[i] = f;
                const float t = fu[i];
                fu[i] = fd[i + 1];
                fd[i + 1] = __fmaf_rn(-f, fd[i + 1], t);
                if (i < n - 2) { fu2[i] = fu[i + 1]; fu[i + 1] = -f * fu[i + 1]; }
                ip[i] = 1;
            }
        }
        for (int i = 0; i < n; ++i) {
            if (fd[i] == 0.f) { info = i + 1; break; }
            fd[i] = __frcp_rn(fd[i]);
        }
        info_s = info;
    }
    __syncthreads();
    if (info_s) return info_s;
    float cprev = 0.f;
    for (int pass = 0;; ++pass) {
        if (pass > 0) {
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                double r = fma(-d[i], x[i], b[i]);
                if (i > 0) r = fma(-dl[i - 1], x[i - 1], r);
                if (i < n - 1) r = fma(-du[i], x[i + 1], r);
                fy[i] = __double2float_rn(r);
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            float bi = fy[0];
            for (int i = 0; i < n - 1; ++i) {
                const float bn = fy[i + 1];
                if (ip[i] == 0) { fy[i] = bi; bi = __fmaf_rn(-fl[i], bi, bn); }
                else { fy[i] = bn; bi = __fmaf_rn(-fl[i], bn, bi); }
            }
            float x1 = __fmul_rn(bi, fd[n - 1]);
            fy[n - 1] = x1;
            if (n > 1) {
                float x0 = __fmul_rn(__fmaf_rn(-fu[n - 2], x1, fy[n - 2]), fd[n - 2]);
                fy[n - 2] = x0;
                for (int i = n - 3; i >= 0; --i) {
                    const float xi = __fmul_rn(__fmaf_rn(-fu2[i], x1, __fmaf_rn(-fu[i], x0, fy[i])), fd[i]);
                    fy[i] = xi;
                    x1 = x0;
                    x0 = xi;
                }
            }
        }
        __syncthreads();
        if (refine_step(x, fy, n, pass, cprev, rbuf) != 0) break;
    }
    return 0;
}

// Tension (SolidSolver.f90:1000-1081), block-cooperative.
__device__ int tension(const BeamArgs& b, BeamWS& w, double* T, double* T_s, const double* th, const double* thd,
                       const double* p, const double* tau, double grav) {
    const int ns = b.ns;
    const double ds = b.ds, eta = b.eta, mue = b.mue;
    const double alpha_t = 0.0;
    const double LE4 = 0.0, LE5 = 0.0;  // leading-edge accelerations, mouvement case 0
    for (int i = threadIdx.x; i < ns; i += blockDim.x) {
        w.th_s[i] = d1d(w.dtab, th, ns, 1, i);
        w.th_ss[i] = d1d(w.dtab, th, ns, 2, i);
        w.th_sss[i] = d1d(w.dtab, th, ns, 3, i);
        w.tau_s[i] = d1d(w.dtab, tau, ns, 1, i);
    }
    __syncthreads();
    const double K1 = mue * (LE4 * b.cos_a + LE5 * b.sin_a + grav * b.sin_a) - tau[0];
    const double T_s0 = -eta * w.th_ss[0] * w.th_s[0] + K1;
    const double ds2 = ds * ds;
    for (int i = threadIdx.x; i < ns; i += blockDim.x) {
        auto dm = [&](int k) { return (k == ns - 1) ? 1.0 : (-2.0 / ds2 - w.th_s[k] * w.th_s[k]); };
        const double dmi = dm(i);
        const double wv = thd[i] + alpha_t;
        double r = -(p[i] * w.th_s[i]) - (2. * eta * w.th_s[i] * w.th_sss[i]) - (eta * (w.th_ss[i] * w.th_ss[i])) - mue * (wv * wv) - w.tau_s[i];
        if (i == ns - 1) r = 0.0;
        if (i == 0) r = r + T_s0 * 2.0 / ds;
        w.rhs[i] = r / dmi;
        if (i < ns - 1) {
            const double up = (i == 0) ? 2.0 / ds2 : 1.0 / ds2;
            const double dn = (i == ns - 2) ? 0.0 : 1.0 / ds2;
            w.dup[i] = up / dmi;
            w.ddown[i] = dn / dm(i + 1);
        }
        w.dmain[i] = 1.0;
    }
    __syncthreads();
    const int info = tri_solve(ns, w.ddown, w.dmain, w.dup, w.rhs, T, w.tf, w.ipiv);
    __syncthreads();
    for (int i = threadIdx.x; i < ns; i += blockDim.x) T_s[i] = (i == 0) ? T_s0 : d1d(w.dtab, T, ns, 1, i);
    __syncthreads();
    return info;
}

// RHS_beameqn (SolidSolver.f90:918-994): on return th := theta_dot, thd := theta_ddot.
__device__ int rhs_beameqn(const BeamArgs& b, BeamWS& w, double* th, double* thd, const double* p, double* T,
                           const double* tau, double grav) {
    const int ns = b.ns;
    const double ds = b.ds, eta = b.eta, mue = b.mue, sigma = b.sigma;
    const double alpha_tt = 0.0;
    const double LE4 = 0.0, LE5 = 0.0;
    if (threadIdx.x == 0) { th[0] = 0.0; thd[0] = 0.0; }
    __syncthreads();
    int st = tension(b, w, T, w.T_s, th, thd, p, tau, grav);
    if (st) return st;
    const double ds2 = ds * ds;
    if (threadIdx.x == 0) {
        const double K2 = p[0] + mue * (LE5 * b.cos_a - LE4 * b.sin_a + grav * b.cos_a);
        const double C2 = 2.0 * ds * K2 - T[0] * th[1] + (eta / ds2) * (10.0 * th[0] - 12.0 * th[1] + 6.0 * th[2] - th[3]);
        w.te[0] = C2 / ((3.0 * eta / ds2) - T[0]);
        const double A1 = th[ns - 3] / 12. - 2. * th[ns - 2] / 3.;
        const double A2 = -th[ns - 3] / 12. + 4. * th[ns - 2] / 3. - 5. * th[ns - 1] / 2.;
        w.te[ns + 1] = 3. * (A1 - A2) / 2.;
        w.te[ns + 2] = 12. * (2. * A1 - A2);
    }
    for (int i = threadIdx.x; i < ns; i += blockDim.x) w.te[i + 1] = th[i];
    __syncthreads();
    for (int i = threadIdx.x; i < ns; i += blockDim.x) {
        w.te_s[i + 1] = d1d(w.dtab, w.te, ns + 3, 1, i + 1);
        w.te_ss[i + 1] = d1d(w.dtab, w.te, ns + 3, 2, i + 1);
        w.te_ssss[i + 1] = d1d(w.dtab, w.te, ns + 3, 4, i + 1);
        w.p_s[i] = d1d(w.dtab, p, ns, 1, i);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < ns; i += blockDim.x) {
        const double tdi = thd[i];
        const double ts = w.te_s[i + 1], tss = w.te_ss[i + 1], tssss = w.te_ssss[i + 1];
        double acc = (-w.p_s[i] - eta * tssss + tss * (T[i] + eta * (ts * ts)) + 2. * w.T_s[i] * ts - mue * alpha_tt -
                      sigma * tdi + tau[i] * ts) / mue;
        if (i == 0) acc = 0.0;
        th[i] = tdi;
        thd[i] = acc;
    }
    __syncthreads();
    return 0;
}

// Fortran x index (0-based) of theta(j), T(j)
__device__ __forceinline__ int xi_th(int j) { return j + 1; }
__device__ __forceinline__ int xi_T(int ns, int j) { return ns + 4 + j; }
// interleaved column of a Fortran variable (1-based l)
__device__ __forceinline__ int col_of(int ns, int l) {
    if (l <= ns + 3) {
        const int j = l - 2;
        if (j <= ns - 1) return 2 * (j + 1);
        return (j == ns) ? 2 * ns + 2 : 2 * ns + 3;
    }
    const int j = l - ns - 5;
    return 2 * (j + 1) + 1;
}
// interleaved row of Fortran equation k (1-based)
__device__ __forceinline__ int row_of(int ns, int k) {
    switch (k) {
        case 1: return 0;
        case 2: return 1;
        case 3: return 2;
        case 7: return 3;
        case 8: return 2 * ns;
        case 6: return 2 * ns + 1;
        case 5: return 2 * ns + 2;
        case 4: return 2 * ns + 3;
        default: break;
    }
    if (k <= 8 + ns - 2) { const int i = k - 8; return 2 * (i + 1); }
    const int i = k - 8 - (ns - 2);
    return 2 * (i + 1) + 1;
}

#define KL 7
#define KU 7
#define BW 15  /* KL + KU + 1 */

struct NewtonCtx {
    double time, dt, dt_old, C1, C2, C3, C4, D, K1, K2, alpha_t, alpha_tt, grav;
    // reciprocal constants: the device evaluates F and J with multiplications only
    double i2ds, ids, ids2, i2ds2, ids4, e2ds3, eds4, e2ds4, g, gds2, gds4e, mue2;
};

// The reciprocal constants: those of ds alone come from the host (BeamArgs::k), those of the
// step's dt are formed here.
__device__ void newton_consts(NewtonCtx& c, const BeamArgs& b) {
    const double eta = b.eta, mue = b.mue, ds2 = b.ds * b.ds, ds4 = ds2 * ds2;
    c.ids = b.k.ids;
    c.i2ds = b.k.i2ds;
    c.ids2 = b.k.ids2;
    c.i2ds2 = b.k.i2ds2;
    c.ids4 = b.k.ids4;
    c.e2ds3 = b.k.e2ds3;
    c.eds4 = b.k.eds4;
    c.e2ds4 = b.k.e2ds4;
    c.g = c.dt / (c.C1 * mue);
    c.gds2 = c.dt / (c.C1 * mue * ds2);
    c.gds4e = c.dt * eta / (c.C1 * mue * ds4);
    c.mue2 = mue * mue;
}

// F_nonlinear (SolidSolver.f90:552-667) equation k (1-based) at x (Fortran order).
__device__ double f_eq(const BeamArgs& b, const BeamWS& w, const NewtonCtx& c, int k) {
    const int ns = b.ns;
    const double eta = b.eta, mue = b.mue, sigma = b.sigma;
    const double* x = w.x;
    const double* p = b.p_new;
    const double* tau = b.tau_new;
    auto TH = [&](int j) { return x[j + 1]; };
    auto TT = [&](int j) { return x[ns + 4 + j]; };
    switch (k) {
        case 1: return TH(0);
        case 2: return (TT(1) - TT(-1)) * c.i2ds + c.e2ds3 * (TH(-1) - 2.0 * TH(0) + TH(1)) * (TH(1) - TH(-1)) - c.K1;
        case 3: return TT(0) * (TH(1) - TH(-1)) * c.i2ds - c.e2ds3 * (-3.0 * TH(-1) + 10.0 * TH(0) - 12.0 * TH(1) + 6.0 * TH(2) - TH(3)) - c.K2;
        case 4: return ((1.0 / 12.0) * TH(ns - 3) - (2.0 / 3.0) * TH(ns - 2) + (2.0 / 3.0) * TH(ns) - (1.0 / 12.0) * TH(ns + 1)) * c.ids;
        case 5: return ((-1.0 / 12.0) * TH(ns - 3) + (4.0 / 3.0) * TH(ns - 2) - 2.5 * TH(ns - 1) + (4.0 / 3.0) * TH(ns) + (-1.0 / 12.0) * TH(ns + 1)) * c.ids2;
        case 6: return TT(ns - 1);
        case 7: {
            const double d1 = (TH(1) - TH(-1)) * c.i2ds;
            const double lap = (TH(1) - 2.0 * TH(0) + TH(-1)) * c.ids2;
            const double wv = w.tdn[0] + c.alpha_t;
            return (TT(-1) - 2.0 * TT(0) + TT(1)) * c.ids2 - TT(0) * (d1 * d1) + p[0] * d1 +
                   c.eds4 * (TH(1) - TH(-1)) * (-2.5 * TH(0) + 9.0 * TH(1) - 12.0 * TH(2) + 7.0 * TH(3) - 1.5 * TH(4)) +
                   eta * (lap * lap) + mue * (wv * wv) - w.taun_s[0];
        }
        case 8: {
            const int m = ns - 1;
            const double d1 = (TH(ns) - TH(ns - 2)) * c.i2ds;
            return c.C3 * w.bo6[m] + c.C4 * w.oo6[m] - w.tdn[m] +
                   c.g * (-(3. * p[m] - 4. * p[m - 1] + p[m - 2]) * c.i2ds -
                          c.eds4 * (TH(ns + 1) - 4. * TH(ns) + 6. * TH(ns - 1) - 4. * TH(ns - 2) + TH(ns - 3)) +
                          (TT(m) + eta * (d1 * d1)) * (TH(ns) - 2. * TH(ns - 1) + TH(ns - 2)) * c.ids2 +
                          (3. * TT(m) - 4. * TT(m - 1) + TT(m - 2)) * (TH(ns) - TH(ns - 2)) * c.i2ds2 - c.alpha_tt * c.mue2 -
                          sigma * w.tdn[m] + tau[m] * (TH(ns) - TH(ns - 2)) * c.i2ds + c.C2 * mue * w.old_rhs[m]);
        }
        default: break;
    }
    if (k <= 8 + ns - 2) {
        const int i = k - 8;
        const double d1 = (TH(i + 1) - TH(i - 1)) * c.i2ds;
        return c.C3 * w.bo6[i] + c.C4 * w.oo6[i] - w.tdn[i] +
               c.g * (-1.0 * (p[i + 1] - p[i - 1]) * c.i2ds -
                      c.eds4 * (TH(i + 2) - 4. * TH(i + 1) + 6. * TH(i) - 4. * TH(i - 1) + TH(i - 2)) +
                      (TT(i) + eta * (d1 * d1)) * (TH(i + 1) - 2. * TH(i) + TH(i - 1)) * c.ids2 +
                      (TT(i + 1) - TT(i - 1)) * (TH(i + 1) - TH(i - 1)) * c.i2ds2 - c.alpha_tt * c.mue2 - sigma * w.tdn[i] +
                      tau[i] * (TH(i + 1) - TH(i - 1)) * c.i2ds + c.C2 * mue * w.old_rhs[i]);
    }
    const int i = k - 8 - (ns - 2);
    const double d1b = (TH(i + 1) - TH(i - 1)) * c.i2ds;
    const double lap = (TH(i + 1) - 2.0 * TH(i) + TH(i - 1)) * c.ids2;
    const double wv = w.tdn[i] + c.alpha_t;
    return (TT(i - 1) - 2.0 * TT(i) + TT(i + 1)) * c.ids2 - TT(i) * (d1b * d1b) + p[i] * d1b +
           c.e2ds4 * (TH(i + 1) - TH(i - 1)) * (TH(i + 2) - 2.0 * TH(i + 1) + 2.0 * TH(i - 1) - TH(i - 2)) +
           eta * (lap * lap) + mue * (wv * wv) - w.taun_s[i];
}

// Jacobi (SolidSolver.f90:671-863): row k (1-based equation) of the Newton matrix, written into
// the band row of its interleaved position.  Returns non-zero for an entry outside the band.
__device__ int jac_row(const BeamArgs& b, const BeamWS& w, const NewtonCtx& c, int k) {
    const int ns = b.ns;
    const double eta = b.eta, mue = b.mue, sigma = b.sigma;
    const double* x = w.x;
    const double* p = b.p_new;
    const double* tau = b.tau_new;
    auto TH = [&](int j) { return x[j + 1]; };
    auto TT = [&](int j) { return x[ns + 4 + j]; };
    const int row = row_of(ns, k);
    double* Ab = w.band + (size_t)row * 16;
    for (int q = 0; q < 16; ++q) Ab[q] = 0.0;
    int bad = 0;
    // (a NaN entry needs a NaN in x, p or tau, which the residual F of the same row shows)
    auto put = [&](int l, double v) {
        const int cidx = col_of(ns, l) - row + KL;
        if (cidx < 0 || cidx >= BW) { bad = 1; return; }
        Ab[cidx] = v;
    };
    const int T0 = ns + 4;
    const double D = c.D;
    const double g = c.g;
    const double e2ds3 = c.e2ds3, eds4 = c.eds4;
    switch (k) {
        case 1: put(2, 1.0); return bad;
        case 2:
            put(1, e2ds3 * (-2.0 * TH(-1) + 2.0 * TH(0)));
            put(2, -(2.0 * e2ds3) * (TH(1) - TH(-1)));
            put(3, e2ds3 * (-2.0 * TH(0) + 2.0 * TH(1)));
            put(T0, -0.5 * c.ids);
            put(T0 + 2, 0.5 * c.ids);
            return bad;
        case 3:
            put(1, -e2ds3 * (-3.0) - TT(0) * c.i2ds);
            put(2, -e2ds3 * (10.0));
            put(3, -e2ds3 * (-12.0) + TT(0) * c.i2ds);
            put(4, -e2ds3 * (6.0));
            put(5, -e2ds3 * (-1.0));
            put(T0 + 1, (TH(1) - TH(-1)) * c.i2ds);
            return bad;
        case 4:
            put(ns + 3, (-1.0 / 12.0) * c.ids);
            put(ns + 2, (2.0 / 3.0) * c.ids);
            put(ns, (-2.0 / 3.0) * c.ids);
            put(ns - 1, (1.0 / 12.0) * c.ids);
            return bad;
        case 5:
            put(ns + 3, (-1.0 / 12.0) * c.ids2);
            put(ns + 2, (4.0 / 3.0) * c.ids2);
            put(ns + 1, (-5.0 / 2.0) * c.ids2);
            put(ns, (4.0 / 3.0) * c.ids2);
            put(ns - 1, (-1.0 / 12.0) * c.ids2);
            return bad;
        case 6: put(2 * ns + 4, 1.0); return bad;
        case 7: {
            const double t1m = TH(1) - TH(-1);
            const double lap = TH(1) - 2.0 * TH(0) + TH(-1);
            const double q = -2.5 * TH(0) + 9.0 * TH(1) - 12.0 * TH(2) + 7.0 * TH(3) - 1.5 * TH(4);
            put(1, TT(0) * t1m * c.i2ds2 - p[0] * c.i2ds - eds4 * q + 2.0 * eds4 * lap);
            put(2, -2.5 * eds4 * t1m - 4.0 * eds4 * lap + 2.0 * mue * (w.tdn[0] + c.alpha_t) * D);
            put(3, -TT(0) * t1m * c.i2ds2 + p[0] * c.i2ds + eds4 * q + 9.0 * eds4 * t1m + 2.0 * eds4 * lap);
            put(4, -12.0 * eds4 * t1m);
            put(5, 7.0 * eds4 * t1m);
            put(6, -1.5 * eds4 * t1m);
            put(ns + 4, c.ids2);
            put(ns + 5, (-2.0 - (t1m * t1m) * 0.25) * c.ids2);
            put(ns + 6, c.ids2);
            return bad;
        }
        case 8: {
            const double d0 = TH(ns) - TH(ns - 2);
            const double lap = TH(ns) - 2.0 * TH(ns - 1) + TH(ns - 2);
            const double h = d0 * c.i2ds;
            const double Tp = TT(ns - 1) + eta * (h * h);
            const double Tb = 3.0 * TT(ns - 1) - 4.0 * TT(ns - 2) + TT(ns - 3);
            const double ds = b.ds;
            put(2 * ns + 4, c.gds2 * (lap + 1.5 * d0));
            put(2 * ns + 3, -4.0 * g * d0 * c.i2ds2);
            put(2 * ns + 2, g * d0 * c.i2ds2);
            put(ns + 3, -c.gds4e);
            put(ns + 2, c.gds2 * (4.0 * eta * c.ids2 + Tp + tau[ns - 1] * ds * 0.5 + eta * lap * d0 * c.i2ds2 + Tb * 0.5));
            put(ns, c.gds2 * (4.0 * eta * c.ids2 + Tp - tau[ns - 1] * ds * 0.5 - eta * lap * d0 * c.i2ds2 - Tb * 0.5));
            put(ns + 1, -D + g * (-6.0 * eds4 - 2.0 * Tp * c.ids2 - D * sigma));
            put(ns - 1, -c.gds4e);
            return bad;
        }
        default: break;
    }
    if (k <= 8 + ns - 2) {
        const int i = k - 8, l = i + 2, m = i + ns + 5;
        const double d1 = TH(i + 1) - TH(i - 1);
        const double lap = TH(i + 1) - 2.0 * TH(i) + TH(i - 1);
        const double h = d1 * c.i2ds;
        const double Tp = TT(i) + eta * (h * h);
        const double dT = TT(i + 1) - TT(i - 1);
        put(l, -D + g * (-6.0 * eds4 - (2.0 * c.ids2) * Tp - D * sigma));
        put(l - 1, g * (4.0 * eds4 + Tp * c.ids2 - tau[i] * c.i2ds - c.e2ds4 * lap * d1 - dT * c.i2ds2));
        put(l + 1, g * (4.0 * eds4 + Tp * c.ids2 + tau[i] * c.i2ds + c.e2ds4 * lap * d1 + dT * c.i2ds2));
        put(l - 2, -c.gds4e);
        put(l + 2, -c.gds4e);
        put(m, g * lap * c.ids2);
        put(m - 1, -g * d1 * c.i2ds2);
        put(m + 1, g * d1 * c.i2ds2);
        return bad;
    }
    const int i = k - 8 - (ns - 2), l = i + 2, m = i + ns + 5;
    const double d1 = TH(i + 1) - TH(i - 1);
    const double lap = TH(i + 1) - 2.0 * TH(i) + TH(i - 1);
    const double q = TH(i + 2) - 2.0 * TH(i + 1) + 2.0 * TH(i - 1) - TH(i - 2);
    const double h = d1 * c.i2ds;
    put(l, -4.0 * eds4 * lap + 2.0 * mue * (w.tdn[i] + c.alpha_t) * D);
    put(l - 1, TT(i) * d1 * c.i2ds2 - p[i] * c.i2ds + eds4 * d1 - c.e2ds4 * q + 2.0 * eds4 * lap);
    put(l + 1, -TT(i) * d1 * c.i2ds2 + p[i] * c.i2ds - eds4 * d1 + c.e2ds4 * q + 2.0 * eds4 * lap);
    put(l - 2, -c.e2ds4 * d1);
    put(l + 2, c.e2ds4 * d1);
    put(m, -2.0 * c.ids2 - (h * h));
    put(m - 1, c.ids2);
    put(m + 1, c.ids2);
    return bad;
}

// Row scale 2^(1023-e) of a row whose largest entry has biased exponent e (1 for e = 0).
__device__ __forceinline__ double row_scale(int e) {
    return (e == 0) ? 1.0 : __longlong_as_double((long long)(2046 - e) << 52);
}

// Row scaling of band row `row` by the power of two that brings its largest entry into
// [1, 2) (exact in FP64), and its FP32 copy for the factorisation.  The maximum is taken on
// the IEEE bit patterns (integer compares only).
__device__ __forceinline__ void scale_row(const BeamWS& w, int row) {
    const double* Ab = w.band + (size_t)row * 16;
    unsigned long long m = 0;
#pragma unroll
    for (int q = 0; q < BW; ++q) {
        const unsigned long long a = (unsigned long long)__double_as_longlong(Ab[q]) & 0x7fffffffffffffffull;
        m = (a > m) ? a : m;
    }
    const int e = (int)(m >> 52);
    const double sc = row_scale(e);
    w.rse[row] = e;
    float4* U4 = reinterpret_cast<float4*>(w.Uf + (size_t)row * 16);
#pragma unroll
    for (int q = 0; q < 4; ++q)
        U4[q] = make_float4(__double2float_rn(Ab[4 * q] * sc), __double2float_rn(Ab[4 * q + 1] * sc),
                            __double2float_rn(Ab[4 * q + 2] * sc), __double2float_rn(Ab[4 * q + 3] * sc));
}

// FP32 banded LU with partial pivoting (dgbtrf semantics, kl = ku = 7) of the row-scaled
// Jacobian, in place in w.Uf; one warp.  Lane c < 16 owns the window column j with
// j = c (mod 16), so the window never shifts across lanes; registers v[r] hold window rows
// k..k+7.  U row k overwrites band row k (consumed 8 steps earlier): [1/u_kk, u_k,k+1 ..
// u_k,k+14]; L row k = [pivot offset, l_1 .. l_7] with the multipliers in window order after
// the interchange.  Returns non-zero on an exactly zero pivot (dgbtrf's INFO > 0).
__device__ int band_factor_f32(const BeamWS& w, int n) {
    const int lane = threadIdx.x & 31;
    const bool mat = lane < 16;
    float* U = w.Uf;
    float v[KL + 1];
#pragma unroll
    for (int r = 0; r <= KL; ++r) {
        const int ci = lane - r + KL;  // window [0, 15], column j = lane
        v[r] = (r < n && mat && ci >= 0 && ci < BW) ? U[r * 16 + ci] : 0.f;
    }
    int info = 0;
    for (int k = 0; k < n; ++k) {
        const int pl = k & 15;
        float col[KL + 1];
#pragma unroll
        for (int r = 0; r <= KL; ++r) col[r] = __shfl_sync(0xffffffffu, v[r], pl);
        int p = 0;
        unsigned best = __float_as_uint(col[0]) & 0x7fffffffu;
#pragma unroll
        for (int r = 1; r <= KL; ++r) {
            const unsigned a = __float_as_uint(col[r]) & 0x7fffffffu;
            if (k + r < n && a > best) { best = a; p = r; }
        }
        float t0 = v[0], c0 = col[0];
#pragma unroll
        for (int r = 1; r <= KL; ++r)
            if (r == p) {
                const float tmp = v[r]; v[r] = t0; t0 = tmp;
                const float cm = col[r]; col[r] = c0; c0 = cm;
            }
        v[0] = t0;
        if (c0 == 0.f) { info = k + 1; break; }  // c0 is the same in every lane
        const float rinv = __frcp_rn(c0);
        float l[KL + 1];
#pragma unroll
        for (int r = 1; r <= KL; ++r) l[r] = __fmul_rn(col[r], rinv);
        const int c = (lane - k) & 15;  // offset of this lane's column from k
        if (mat && c >= 1 && c <= 14) {
#pragma unroll
            for (int r = 1; r <= KL; ++r) v[r] = __fmaf_rn(-l[r], v[0], v[r]);
        }
        if (mat && c <= 14) U[(size_t)k * 16 + c] = (c == 0) ? rinv : v[0];
        if (lane == 16) {
            float4* L4 = reinterpret_cast<float4*>(w.Lf + (size_t)k * 8);
            L4[0] = make_float4(__int_as_float(p), l[1], l[2], l[3]);
            L4[1] = make_float4(l[4], l[5], l[6], l[7]);
        }
#pragma unroll
        for (int r = 0; r < KL; ++r) v[r] = v[r + 1];
        // next window [k+1, k+16]: the pivot lane now holds column k+16 (zero for every row),
        // the new row k+8 enters with its scaled band values
        const int r8 = k + 1 + KL;
        float nv = 0.f;
        if (r8 < n && mat) {
            const int cn = (lane - (k + 1)) & 15;
            if (cn < BW) nv = U[(size_t)r8 * 16 + cn];
        }
        if (lane == pl) {
#pragma unroll
            for (int r = 0; r < KL; ++r) v[r] = 0.f;
        }
        v[KL] = nv;
    }
    return __shfl_sync(0xffffffffu, info, 0);
}

// Forward elimination steps k0..k1-1 (dgbtrs order: the interchange, then the L update)
// from the window q = rows k..k+7, with b[k+8] entering at each step (b == nullptr: zero
// inputs).  Step k's output goes to out[(k - k0) * os]; q ends as the window at k1.
__device__ __forceinline__ void fwd_chunk(const float* __restrict__ L, int k0, int k1, int n, float* q,
                                          const float* __restrict__ b, float* __restrict__ out, int os) {
#pragma unroll 4
    for (int k = k0; k < k1; ++k) {
        const float4 la = *reinterpret_cast<const float4*>(L + (size_t)k * 8);
        const float4 lb = *reinterpret_cast<const float4*>(L + (size_t)k * 8 + 4);
        const int p = __float_as_int(la.x);
        float t = q[0];
        if (p != 0) {
            const float q0 = q[0];
#pragma unroll
            for (int r = 1; r <= KL; ++r)
                if (r == p) { t = q[r]; q[r] = q0; }
        }
        q[1] = __fmaf_rn(-la.y, t, q[1]);
        q[2] = __fmaf_rn(-la.z, t, q[2]);
        q[3] = __fmaf_rn(-la.w, t, q[3]);
        q[4] = __fmaf_rn(-lb.x, t, q[4]);
        q[5] = __fmaf_rn(-lb.y, t, q[5]);
        q[6] = __fmaf_rn(-lb.z, t, q[6]);
        q[7] = __fmaf_rn(-lb.w, t, q[7]);
        out[(size_t)(k - k0) * os] = t;
#pragma unroll
        for (int r = 0; r < KL; ++r) q[r] = q[r + 1];
        q[KL] = (b != nullptr && k + 1 + KL < n) ? b[k + 1 + KL] : 0.f;
    }
}

// Back substitution rows k1-1 .. k0 of U x = y with the incoming x_(k1) .. x_(k1+13) in
// xw[1..14] (y == nullptr: zero right-hand side); x_k goes to out[(k - k0) * os].  The row
// is a dot product with the far terms first, so only x_(k+1), x_(k+2) are on the recurrence.
__device__ __forceinline__ void bwd_chunk(const float* __restrict__ U, int k0, int k1, float* xw,
                                          const float* __restrict__ y, float* __restrict__ out, int os) {
#pragma unroll 4
    for (int k = k1 - 1; k >= k0; --k) {
        const float4* Uk = reinterpret_cast<const float4*>(U + (size_t)k * 16);
        const float4 u0 = Uk[0], u1 = Uk[1], u2 = Uk[2], u3 = Uk[3];
        float sa = __fmul_rn(u3.z, xw[14]);
        sa = __fmaf_rn(u3.y, xw[13], sa);
        sa = __fmaf_rn(u3.x, xw[12], sa);
        sa = __fmaf_rn(u2.w, xw[11], sa);
        sa = __fmaf_rn(u2.z, xw[10], sa);
        sa = __fmaf_rn(u2.y, xw[9], sa);
        sa = __fmaf_rn(u2.x, xw[8], sa);
        float sb = __fmul_rn(u1.w, xw[7]);
        sb = __fmaf_rn(u1.z, xw[6], sb);
        sb = __fmaf_rn(u1.y, xw[5], sb);
        sb = __fmaf_rn(u1.x, xw[4], sb);
        sb = __fmaf_rn(u0.w, xw[3], sb);
        float t = __fsub_rn((y != nullptr) ? y[k] : 0.f, __fadd_rn(sa, sb));
        t = __fmaf_rn(-u0.z, xw[2], t);
        t = __fmaf_rn(-u0.y, xw[1], t);
        const float xk = __fmul_rn(t, u0.x);
        out[(size_t)(k - k0) * os] = xk;
#pragma unroll
        for (int c = 14; c >= 2; --c) xw[c] = xw[c - 1];
        xw[1] = xk;
    }
}

__device__ __forceinline__ int chunk_of(int k, int n, int C) { return (int)((((long long)k + 1) * C - 1) / n); }

// Chunk responses of a new factor (block-cooperative): for chunk c and each unit initial
// window e_j of the forward elimination, the outputs (column j of G) and the final window
// (column j of E_c); for each unit incoming state e_j of the back substitution, the solution
// (column j of H) and its first 14 rows (column j of F_c).
__device__ void band_precompute(const BeamWS& w, int n) {
    const int C = w.nch;
    for (int job = threadIdx.x; job < C * 22; job += blockDim.x) {
        const int c = job / 22, j = job % 22;
        const int k0 = chunk_lo(c, n, C), k1 = chunk_lo(c + 1, n, C);
        if (j < 8) {
            float q[KL + 1];
#pragma unroll
            for (int r = 0; r <= KL; ++r) q[r] = (r == j) ? 1.f : 0.f;
            fwd_chunk(w.Lf, k0, k1, n, q, nullptr, w.Gc + (size_t)k0 * 8 + j, 8);
#pragma unroll
            for (int r = 0; r <= KL; ++r) w.Ec[c * 64 + r * 8 + j] = q[r];
        } else {
            const int jj = j - 8;
            float xw[15];
#pragma unroll
            for (int q = 0; q < 15; ++q) xw[q] = (q == jj + 1) ? 1.f : 0.f;
            bwd_chunk(w.Uf, k0, k1, xw, nullptr, w.Hc + (size_t)k0 * 16 + jj, 16);
            if (C > 1)
                for (int i = 0; i < 14; ++i) w.Fc[c * 224 + i * 16 + jj] = w.Hc[(size_t)(k0 + i) * 16 + jj];
        }
    }
    __syncthreads();
}

// Solve with the FP32 factor in place on w.yf, block-cooperative, in chunks: local forward
// eliminations with the chunk's own inputs, the sequential carry of the 8-value windows
// between chunks (D_(c+1) = d_c + E_c D_c), the correction y += G D; then local back
// substitutions with zero incoming state, the carry of the 14-value states from the last
// chunk down (S_(c-1) = head_c + F_c S_c), and the correction x += H S.
__device__ __forceinline__ void band_solve_chunked(const BeamWS& w, int n, long long* sub) {
    const int C = w.nch, lane = threadIdx.x & 31;
    long long t0 = clock64();
#define SUB(k) do { const long long t_ = clock64(); sub[k] += t_ - t0; t0 = t_; } while (0)
    if (threadIdx.x < C) {
        const int c = threadIdx.x, k0 = chunk_lo(c, n, C), k1 = chunk_lo(c + 1, n, C);
        float q[KL + 1];
#pragma unroll
        for (int r = 0; r <= KL; ++r) q[r] = (k0 + r < n) ? w.yf[k0 + r] : 0.f;
        fwd_chunk(w.Lf, k0, k1, n, q, w.yf, w.yl + k0, 1);
#pragma unroll
        for (int r = 0; r <= KL; ++r) w.cd[c * 8 + r] = q[r] - ((k1 + r < n) ? w.yf[k1 + r] : 0.f);
    }
    __syncthreads();
    SUB(0);
    if (threadIdx.x < 8) {
        float Di = 0.f;
        w.cD[lane] = 0.f;
        for (int c = 0; c + 1 < C; ++c) {
            const float4 e0 = *reinterpret_cast<const float4*>(w.Ec + c * 64 + lane * 8);
            const float4 e1 = *reinterpret_cast<const float4*>(w.Ec + c * 64 + lane * 8 + 4);
            const float d0 = __shfl_sync(0xffu, Di, 0), d1 = __shfl_sync(0xffu, Di, 1), d2 = __shfl_sync(0xffu, Di, 2),
                        d3 = __shfl_sync(0xffu, Di, 3), d4 = __shfl_sync(0xffu, Di, 4), d5 = __shfl_sync(0xffu, Di, 5),
                        d6 = __shfl_sync(0xffu, Di, 6), d7 = __shfl_sync(0xffu, Di, 7);
            float a0 = __fmaf_rn(e0.x, d0, w.cd[c * 8 + lane]);
            float a1 = __fmul_rn(e0.y, d1);
            a0 = __fmaf_rn(e0.z, d2, a0);
            a1 = __fmaf_rn(e0.w, d3, a1);
            a0 = __fmaf_rn(e1.x, d4, a0);
            a1 = __fmaf_rn(e1.y, d5, a1);
            a0 = __fmaf_rn(e1.z, d6, a0);
            a1 = __fmaf_rn(e1.w, d7, a1);
            Di = __fadd_rn(a0, a1);
            w.cD[(c + 1) * 8 + lane] = Di;
        }
    }
    __syncthreads();
    SUB(1);
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const int c = chunk_of(k, n, C);
        const float4 g0 = *reinterpret_cast<const float4*>(w.Gc + (size_t)k * 8);
        const float4 g1 = *reinterpret_cast<const float4*>(w.Gc + (size_t)k * 8 + 4);
        const float* D = w.cD + c * 8;
        float a = __fmaf_rn(g0.x, D[0], w.yl[k]);
        float e = __fmul_rn(g0.y, D[1]);
        a = __fmaf_rn(g0.z, D[2], a);
        e = __fmaf_rn(g0.w, D[3], e);
        a = __fmaf_rn(g1.x, D[4], a);
        e = __fmaf_rn(g1.y, D[5], e);
        a = __fmaf_rn(g1.z, D[6], a);
        e = __fmaf_rn(g1.w, D[7], e);
        w.yl[k] = __fadd_rn(a, e);
    }
    __syncthreads();
    SUB(2);
    if (threadIdx.x < C) {
        const int c = threadIdx.x, k0 = chunk_lo(c, n, C), k1 = chunk_lo(c + 1, n, C);
        float xw[15];
#pragma unroll
        for (int q = 0; q < 15; ++q) xw[q] = 0.f;
        bwd_chunk(w.Uf, k0, k1, xw, w.yl, w.yf + k0, 1);
        if (C > 1)
            for (int i = 0; i < 14; ++i) w.chead[c * 16 + i] = w.yf[k0 + i];
    }
    __syncthreads();
    SUB(3);
    if (threadIdx.x < 14) {
        float Si = 0.f;
        w.cS[(C - 1) * 16 + lane] = 0.f;
        for (int c = C - 1; c >= 1; --c) {
            const float* Fr = w.Fc + c * 224 + lane * 16;
            float sv[14];
#pragma unroll
            for (int j = 0; j < 14; ++j) sv[j] = __shfl_sync(0x3fffu, Si, j);
            float a0 = w.chead[c * 16 + lane], a1 = 0.f;
#pragma unroll
            for (int j = 0; j < 14; j += 2) {
                a0 = __fmaf_rn(Fr[j], sv[j], a0);
                a1 = __fmaf_rn(Fr[j + 1], sv[j + 1], a1);
            }
            Si = __fadd_rn(a0, a1);
            w.cS[(c - 1) * 16 + lane] = Si;
        }
    }
    __syncthreads();
    SUB(4);
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const int c = chunk_of(k, n, C);
        const float4* H4 = reinterpret_cast<const float4*>(w.Hc + (size_t)k * 16);
        const float4 h0 = H4[0], h1 = H4[1], h2 = H4[2], h3 = H4[3];
        const float* Sv = w.cS + c * 16;
        float a = __fmaf_rn(h0.x, Sv[0], w.yf[k]);
        float e = __fmul_rn(h0.y, Sv[1]);
        a = __fmaf_rn(h0.z, Sv[2], a);
        e = __fmaf_rn(h0.w, Sv[3], e);
        a = __fmaf_rn(h1.x, Sv[4], a);
        e = __fmaf_rn(h1.y, Sv[5], e);
        a = __fmaf_rn(h1.z, Sv[6], a);
        e = __fmaf_rn(h1.w, Sv[7], e);
        a = __fmaf_rn(h2.x, Sv[8], a);
        e = __fmaf_rn(h2.y, Sv[9], e);
        a = __fmaf_rn(h2.z, Sv[10], a);
        e = __fmaf_rn(h2.w, Sv[11], e);
        a = __fmaf_rn(h3.x, Sv[12], a);
        e = __fmaf_rn(h3.y, Sv[13], e);
        w.yf[k] = __fadd_rn(a, e);
    }
    __syncthreads();
    SUB(5);
#undef SUB
}

// FP64 residual of band row k at the current solution, row-scaled into the FP32 solve vector.
__device__ __forceinline__ void residual_row(const BeamWS& w, int n, int k) {
    const double* Bk = w.band + (size_t)k * 16;
    double acc = w.bvec[k];
#pragma unroll
    for (int ci = 0; ci < BW; ++ci) {
        const int j = k - KL + ci;
        if (j >= 0 && j < n) acc = fma(-Bk[ci], w.xdi[j], acc);
    }
    w.yf[k] = __double2float_rn(acc * row_scale(w.rse[k]));
}

}  // namespace

// Cycle counters of the beam kernel's phases (thread 0, registers; added to the scalars at the
// end of the kernel), read by fsibe_beam_phase_cycles.
#define PH(k) do { const long long t_ = clock64(); ph[k] += t_ - ph_t; ph_t = t_; } while (0)

// Block copy of m float4 with eight loads in flight per thread (the source may be in L2).
__device__ __forceinline__ void copy_f4(float4* __restrict__ d, const float4* __restrict__ g, size_t m) {
    size_t q = threadIdx.x;
    for (; q + 7 * blockDim.x < m; q += 8 * blockDim.x) {
        float4 v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = g[q + u * blockDim.x];
#pragma unroll
        for (int u = 0; u < 8; ++u) d[q + u * blockDim.x] = v[u];
    }
    for (; q < m; q += blockDim.x) d[q] = g[q];
}

// Doubles of the predictor's output: the initial guess x (n), the Crank-Nicolson right-hand
// side old_rhs, the EE1 angles g5 and the EE1 tension T (ns each).
__host__ size_t beam_pred_doubles(int ns) { return (size_t)(2 * ns + 4) + 3 * (size_t)ns + 8; }

// GravityImpulse (SolidSolver.f90:874-911)
__device__ double gravity_impulse(const BeamArgs& b, double time, double grav) {
    if (b.iImpulse == 1 || b.iImpulse == 2) {
        const double T0 = 0.75, T1 = 0.85, A = (b.iImpulse == 1) ? 1.00 : 4.00;
        grav = A * sin(b.pi * (time - T0) / (T1 - T0));
        if (time < T0) grav = 0.0;
        if (time > T1) grav = 0.0;
    } else if (b.iImpulse == 3) {
        const double T0 = 2.0, T1 = 3.0;
        double k = 0.0;
        if (time <= T0) k = 0.0;
        else if (time >= T0 && time <= T1) {
            const double t = (time - T0) / (T1 - T0), t2 = t * t, t4 = t2 * t2;
            k = -20.0 * (t4 * t2 * t) + 70.0 * (t4 * t2) - 84.0 * (t4 * t) + 35.0 * t4;
        } else k = 1.0;
        grav = 0.7 * k;
    }
    return grav;
}

// The part of IBES_solver that needs only the state at the start of the step and the
// previous step's loads (SolidSolver.f90:138-222): gravity, the start-up method switch, the
// EE1 predictor (RHS_beameqn with the tension solve), the initial guess except its two
// ghost values that use the new loads, and the Crank-Nicolson right-hand side.  It runs on a
// side stream while the fluid step of the same time step runs; its output goes to b.pred.
__global__ void __launch_bounds__(256) k_beam_pre(BeamArgs b) {
    extern __shared__ __align__(16) double smem_ws[];
    DevScalars* S = b.S;
    if (S->status != 0) return;
    const int ns = b.ns, n = 2 * ns + 4;
    const BeamParts parts = beam_parts(b.ws, smem_ws, b.use_smem, ns);
    BeamWS w = carve(parts, ns);
    const double time = S->time, dt = S->dt1;
    const double ds = b.ds;
    __shared__ D1DTab dtab;
    long long ph_t = clock64(), ph[4] = {0, 0, 0, 0};
    d1d_tables(&dtab, b.ds);
    w.dtab = &dtab;
    if (threadIdx.x == 0) S->grav = gravity_impulse(b, time, S->grav);
    __syncthreads();
    const double grav = S->grav;
    if (!(time > b.t_release)) return;
    if (threadIdx.x == 0 && S->startup_step) {
        S->startup_step = 0;
        if (S->method == FSIBE_BDF2) { S->actually_bdf2 = 1; S->method = FSIBE_CRANK_NICHOLSON; }
    }
    for (int i = threadIdx.x; i < ns; i += blockDim.x) { w.th1[i] = b.th[i]; w.td1[i] = b.thd[i]; }
    __syncthreads();
    const int method = S->method;
    PH(0);
    // EE1 predictor: th1 = theta, td1 = theta_dot -> RHS
    int st = rhs_beameqn(b, w, w.th1, w.td1, b.p_old, w.T, b.tau_old, grav);
    PH(1);
    if (st) { if (threadIdx.x == 0) set_status(S, FSIBE_ERR_SINGULAR); return; }
    double* px = b.pred;
    double* p_old_rhs = b.pred + n;
    double* pg5 = p_old_rhs + ns;
    double* pT = pg5 + ns;
    for (int i = threadIdx.x; i < ns; i += blockDim.x) {
        const double g5 = b.th[i] + dt * w.th1[i];
        w.g5[i] = g5;
        pg5[i] = g5;
        pT[i] = w.T[i];
        px[xi_th(i)] = g5;
        px[xi_T(ns, i)] = w.T[i];
        p_old_rhs[i] = 0.0;
    }
    __syncthreads();
    // initial guess, free-end ghost values (SolidSolver.f90:188-196)
    if (threadIdx.x == 0) {
        const double* g5 = w.g5;
        const double A1 = g5[ns - 3] / 12. - 2. * g5[ns - 2] / 3.;
        const double A2 = -g5[ns - 3] / 12. + 4. * g5[ns - 2] / 3. - 5. * g5[ns - 1] / 2.;
        px[xi_th(ns)] = 3. * (A1 - A2) / 2.;
        px[xi_th(ns + 1)] = 12. * (2. * A1 - A2);
    }
    PH(2);
    if (method == FSIBE_CRANK_NICHOLSON) {
        for (int i = threadIdx.x; i < ns; i += blockDim.x) { w.th1[i] = b.th[i]; w.old_rhs[i] = b.thd[i]; }
        __syncthreads();
        st = rhs_beameqn(b, w, w.th1, w.old_rhs, b.p_old, w.T, b.tau_old, grav);
        if (st) { if (threadIdx.x == 0) set_status(S, FSIBE_ERR_SINGULAR); return; }
        for (int i = threadIdx.x; i < ns; i += blockDim.x) p_old_rhs[i] = w.old_rhs[i];
    }
    PH(3);
    if (threadIdx.x == 0)
        for (int k = 0; k < 4; ++k) S->phase[k] += ph[k];
}

// IBES_solver / SolidSolverWrapper / SolidEnergies after the loads of the step are known:
// Newton with the banded Jacobian, positions, energies; one CTA.  k_beam_pre of the same
// step ran before it.
__global__ void __launch_bounds__(256) k_beam(BeamArgs b) {
    extern __shared__ __align__(16) double smem_ws[];
    DevScalars* S = b.S;
    if (S->status != 0) return;
    const int ns = b.ns, n = 2 * ns + 4;
    // use_smem: bit mask of the workspace parts in shared memory (1 scr, 2 fact, 4 vec, 8 band)
    const int mode = b.use_smem;
    const BeamParts parts = beam_parts(b.ws, smem_ws, mode, ns);
    BeamWS w = carve(parts, ns);
    const double time = S->time, dt = S->dt1;
    const double ds = b.ds, mue = b.mue, eta = b.eta;
    __shared__ double red[4][8];
    __shared__ int flag, stop_s;
    __shared__ D1DTab dtab;
    long long ph_t = clock64(), ph[24] = {};
    d1d_tables(&dtab, b.ds);
    w.dtab = &dtab;
    const double grav = S->grav;
    for (int i = threadIdx.x; i < ns; i += blockDim.x) {
        w.bo3[i] = b.vx[i]; w.bo4[i] = b.vy[i]; w.bo5[i] = b.th[i]; w.bo6[i] = b.thd[i];
        w.oo5[i] = b.oo[4 * ns + i]; w.oo6[i] = b.oo[5 * ns + i];
    }
    __syncthreads();

    bool released = time > b.t_release;
    if (released) {
        const double dt_old = S->dt_old;
        const int method = S->method;
        for (int i = threadIdx.x; i < n; i += blockDim.x) w.x[i] = b.pred[i];
        for (int i = threadIdx.x; i < ns; i += blockDim.x) {
            w.old_rhs[i] = b.pred[n + i];
            w.taun_s[i] = d1d(w.dtab, b.tau_new, ns, 1, i);
        }
        // initial guess, clamped-end ghost values from the new loads (SolidSolver.f90:175-187, 197-202)
        if (threadIdx.x == 0) {
            const double* g5 = b.pred + n + ns;
            const double* T = g5 + ns;
            const double ds2 = ds * ds;
            const double K2 = b.p_new[0] + mue * (0.0 * b.cos_a - 0.0 * b.sin_a + grav * b.cos_a);
            const double C2v = 2.0 * ds * K2 - T[0] * g5[1] + (eta / ds2) * (10.0 * g5[0] - 12.0 * g5[1] + 6.0 * g5[2] - g5[3]);
            w.x[xi_th(-1)] = C2v / ((3.0 * eta / ds2) - T[0]);
            const double K1 = mue * (0.0 * b.cos_a + 0.0 * b.sin_a + grav * b.sin_a) - b.tau_new[0];
            const double th_ss0 = (2.0 * g5[0] - 5.0 * g5[1] + 4.0 * g5[2] - 1.0 * g5[3]) * b.k.ids2;
            const double th_s0 = (-1.5 * g5[0] + 2.0 * g5[1] - 0.5 * g5[2]) * b.k.ids;
            const double T_s0 = -eta * th_ss0 * th_s0 + K1;
            w.x[xi_T(ns, -1)] = T[1] - 2.0 * ds * T_s0;
        }
        __syncthreads();
        // the step's Newton constants, evaluated once (divisions are long FP64 sequences here)
        __shared__ NewtonCtx cs;
        if (threadIdx.x == 0) {
            cs.time = time; cs.dt = dt; cs.dt_old = dt_old; cs.alpha_t = 0.0; cs.alpha_tt = 0.0; cs.grav = grav;
            solid_coeffs(method, dt, dt_old, cs.C1, cs.C2, cs.C3, cs.C4);
            cs.D = cs.C1 / dt;
            newton_consts(cs, b);
            cs.K1 = mue * (0.0 * b.cos_a + 0.0 * b.sin_a + grav * b.sin_a) - b.tau_new[0];
            cs.K2 = b.p_new[0] + mue * (0.0 * b.cos_a - 0.0 * b.sin_a + grav * b.cos_a);
        }
        __syncthreads();
        const NewtonCtx& c = cs;
        // the FP32 factor of an earlier step, when one is stored
        bool need_factor = (S->beam_fact == 0), factored = false;
        if (!need_factor && (mode & 2)) {
            const float4* g = reinterpret_cast<const float4*>(b.ws + beam_vec_doubles(ns) + beam_band_doubles(ns));
            float4* d = reinterpret_cast<float4*>(w.Uf);
            copy_f4(d, g, beam_fact_floats(ns) / 4);
            __syncthreads();
        }
        int iter = 0;
        bool iterate = true;
        PH(22);
        while (iterate) {
            if (threadIdx.x == 0) flag = 0;
            for (int i = threadIdx.x; i < ns; i += blockDim.x)
                w.tdn[i] = c.D * (w.x[xi_th(i)] - c.C3 * w.bo5[i] - c.C4 * w.oo5[i]) - c.C2 * w.bo6[i];
            __syncthreads();
            // F and the Jacobian row of each equation; the eight boundary equations (each its own
            // code path) go one per warp so that no warp serialises several of them
            auto assemble = [&](int k) {
                const double f = f_eq(b, w, c, k);
                if (isnan(f)) flag = FSIBE_ERR_NAN;
                w.bvec[row_of(ns, k)] = -1.0 * f;
                if (jac_row(b, w, c, k)) flag = FSIBE_ERR_NAN;
            };
            for (int r = threadIdx.x; r < n - 8; r += blockDim.x) assemble(9 + r);
            for (int q = threadIdx.x >> 5; q < 8; q += blockDim.x >> 5)
                if ((threadIdx.x & 31) == 0) assemble(1 + q);
            __syncthreads();
            if (flag) { if (threadIdx.x == 0) set_status(S, flag); return; }
            PH(4);
            // J dx = -F: FP32 LU of the row-scaled band as the preconditioner of an FP64
            // iterative refinement, run to the accuracy of an FP64 factorisation.  The factor is
            // kept across Newton iterations and steps while it still contracts fast (<= 5
            // solves); a stale factor that stops converging is replaced and the solve redone.
            int solves = 0;
            for (int attempt = 0; attempt < 2; ++attempt) {
                const bool fresh = need_factor;
                if (need_factor) {
                    for (int k = threadIdx.x; k < n; k += blockDim.x) scale_row(w, k);
                    __syncthreads();
                    if (threadIdx.x < 32) {
                        const int info = band_factor_f32(w, n);
                        if (threadIdx.x == 0 && info) flag = FSIBE_ERR_SINGULAR;
                    }
                    __syncthreads();
                    if (flag) { if (threadIdx.x == 0) set_status(S, flag); return; }
                    band_precompute(w, n);
                    need_factor = false;
                    factored = true;
                }
                PH(5);
                for (int k = threadIdx.x; k < n; k += blockDim.x)
                    w.yf[k] = __double2float_rn(w.bvec[k] * row_scale(w.rse[k]));
                __syncthreads();
                float cprev = 0.f;
                bool ok = false;
                for (int pass = 0;; ++pass) {
                    if (pass > 0) {
                        for (int k = threadIdx.x; k < n; k += blockDim.x) residual_row(w, n, k);
                        __syncthreads();
                    }
                    PH(11);
                    band_solve_chunked(w, n, ph + 16);
                    PH(12);
                    ++solves;
                    const int rs = refine_step(w.xdi, w.yf, n, pass, cprev, &red[2][0]);
                    PH(13);
                    if (rs != 0) { ok = rs > 0; break; }
                }
                if (ok || fresh) break;
                need_factor = true;
            }
            if (solves > 5) need_factor = true;
            if (threadIdx.x == 0) ph[10] += solves;
            PH(6);
            double sd = 0.0, sx = 0.0;
            for (int l = threadIdx.x; l < n; l += blockDim.x) {
                const double d = w.xdi[col_of(ns, l + 1)];
                if (isnan(d)) flag = FSIBE_ERR_NAN;
                const double xn = w.x[l] + d;
                w.x[l] = xn;
                sd += d * d;
                sx += xn * xn;
            }
            for (int o = 16; o > 0; o >>= 1) {
                sd += __shfl_xor_sync(0xffffffffu, sd, o);
                sx += __shfl_xor_sync(0xffffffffu, sx, o);
            }
            if ((threadIdx.x & 31) == 0) { red[0][threadIdx.x >> 5] = sd; red[1][threadIdx.x >> 5] = sx; }
            __syncthreads();
            if (flag) { if (threadIdx.x == 0) set_status(S, flag); return; }
            iter = iter + 1;
            // the norms and the convergence test on one warp (sqrt and division are long FP64
            // sequences here: one lane evaluates them once instead of every warp)
            if (threadIdx.x < 32) {
                const int nw = blockDim.x >> 5, ln = lane_id();
                double tsd = (ln < nw) ? red[0][ln] : 0.0, tsx = (ln < nw) ? red[1][ln] : 0.0;
                for (int o = 4; o > 0; o >>= 1) {
                    tsd += __shfl_xor_sync(0xffffffffu, tsd, o);
                    tsx += __shfl_xor_sync(0xffffffffu, tsx, o);
                }
                if (ln == 0) {
                    const double err = sqrt(tsd);
                    const double err_rel = fabs(sqrt(tsd) / sqrt(tsx));
                    stop_s = ((err < b.tol || err_rel < b.tol) && iter > 2) ? 1 : 0;
                }
            }
            __syncthreads();
            PH(23);
            if (stop_s) iterate = false;
            if (iter > b.maxit - 1) {
                if (threadIdx.x == 0) set_status(S, FSIBE_ERR_NEWTON_MAXIT);
                return;
            }
            __syncthreads();
        }
        for (int i = threadIdx.x; i < ns; i += blockDim.x) {
            const double th = w.x[xi_th(i)];
            b.th[i] = th;
            b.thd[i] = c.D * (th - c.C3 * w.bo5[i] - c.C4 * w.oo5[i]) - c.C2 * w.bo6[i];
        }
        if (factored) {
            if (mode & 2) {
                float4* g = reinterpret_cast<float4*>(b.ws + beam_vec_doubles(ns) + beam_band_doubles(ns));
                const float4* d = reinterpret_cast<const float4*>(w.Uf);
                copy_f4(g, d, beam_fact_floats(ns) / 4);
            }
            if (threadIdx.x == 0) S->beam_fact = 1;
        }
        if (threadIdx.x == 0) {
            S->newton_iters = iter;
            if (S->actually_bdf2) { S->method = FSIBE_BDF2; S->actually_bdf2 = 0; }
            S->dt_old = dt;
        }
        // beam_oldold = beam_old (the state at entry)
        for (int i = threadIdx.x; i < ns; i += blockDim.x) {
            b.oo[0 * ns + i] = b.x[i]; b.oo[1 * ns + i] = b.y[i]; b.oo[2 * ns + i] = w.bo3[i];
            b.oo[3 * ns + i] = w.bo4[i]; b.oo[4 * ns + i] = w.bo5[i]; b.oo[5 * ns + i] = w.bo6[i];
        }
        __syncthreads();
    }
    PH(7);
    // integrate_position(time + dt) (integrate_position.f90:14-44): running sums in order
    for (int i = threadIdx.x; i < ns; i += blockDim.x) {
        const double th = b.th[i], td = b.thd[i];
        double sn, cn;
        sincos(th, &sn, &cn);
        w.cs[i] = cn * ds;
        w.cs[ns + 8 + i] = sn * ds;
        w.cs[2 * (ns + 8) + i] = td * sn * ds;
        w.cs[3 * (ns + 8) + i] = td * cn * ds;
    }
    __syncthreads();
    // the four running sums in the reference's order: the positions decide grid-aligned
    // boxes (mask, drag window), so their roundings must be the reference's
    if (threadIdx.x < 4) {
        const int q = threadIdx.x;
        const double* src = w.cs + q * (ns + 8);
        double* dst = w.pre + q * (ns + 8);
        double s = 0.0;
        for (int i = 0; i < ns; ++i) {
            dst[i] = s;
            s = (q == 2) ? s - src[i] : s + src[i];
        }
    }
    __syncthreads();
    {
        const double ca = b.cos_a, sa = b.sin_a, alpha_t = 0.0, idt = 1.0 / dt;
        for (int i = threadIdx.x; i < ns; i += blockDim.x) {
            const double xrel = w.pre[i], yrel = w.pre[(ns + 8) + i];
            const double vxrel = w.pre[2 * (ns + 8) + i], vyrel = w.pre[3 * (ns + 8) + i];
            b.x[i] = b.x0 + xrel * ca - yrel * sa;
            b.y[i] = b.y0 + yrel * ca + xrel * sa;
            b.vx[i] = 0.0 + ca * (vxrel - alpha_t * yrel) - sa * (vyrel + alpha_t * xrel);
            b.vy[i] = 0.0 + ca * (vyrel + alpha_t * xrel) + sa * (vxrel - alpha_t * yrel);
            if (released) {
                b.ax[i] = (b.vx[i] - w.bo3[i]) * idt;
                b.ay[i] = (b.vy[i] - w.bo4[i]) * idt;
            }
        }
    }
    __syncthreads();
    // emergency brake (SolidSolver.f90:370-380)
    if (released) {
        double mx = 0.0;
        for (int i = threadIdx.x; i < ns; i += blockDim.x) mx = fmax(mx, fabs(b.thd[i] - w.bo6[i]));
        for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if ((threadIdx.x & 31) == 0) red[2][threadIdx.x >> 5] = mx;
        __syncthreads();
        if (threadIdx.x == 0) {
            double m = 0.0;
            for (int q = 0; q < (int)(blockDim.x >> 5); ++q) m = fmax(m, red[2][q]);
            if (m > 100.0) set_status(S, FSIBE_ERR_BRAKE);
        }
    }
    PH(8);
    // SolidEnergies (SolidSolver.f90:76-92): the five sums as block reductions (per-thread
    // partials, then a shuffle tree), since a serial FP64 loop costs a full warp issue slot
    // per addition on this chip
    {
        __shared__ double esum[5][8];
        double sk = 0, sp = 0, se = 0, sax = 0, say = 0;
        for (int i = threadIdx.x; i < ns; i += blockDim.x) {
            const double th_s = d1d(w.dtab, b.th, ns, 1, i);
            const double vx = b.vx[i], vy = b.vy[i];
            sk += vx * vx + vy * vy;
            sp += b.y[i] - b.y0;
            se += th_s * th_s;
            sax += b.ax[i];
            say += b.ay[i];
        }
        for (int o = 16; o > 0; o >>= 1) {
            sk += __shfl_xor_sync(0xffffffffu, sk, o);
            sp += __shfl_xor_sync(0xffffffffu, sp, o);
            se += __shfl_xor_sync(0xffffffffu, se, o);
            sax += __shfl_xor_sync(0xffffffffu, sax, o);
            say += __shfl_xor_sync(0xffffffffu, say, o);
        }
        if ((threadIdx.x & 31) == 0) {
            const int wv = threadIdx.x >> 5;
            esum[0][wv] = sk; esum[1][wv] = sp; esum[2][wv] = se; esum[3][wv] = sax; esum[4][wv] = say;
        }
        __syncthreads();
        if (threadIdx.x < 32) {
            const int nw = blockDim.x >> 5;
            double v[5];
#pragma unroll
            for (int q = 0; q < 5; ++q) v[q] = (lane_id() < nw) ? esum[q][lane_id()] : 0.0;
#pragma unroll
            for (int o = 4; o > 0; o >>= 1)
#pragma unroll
                for (int q = 0; q < 5; ++q) v[q] += __shfl_xor_sync(0xffffffffu, v[q], o);
            if (threadIdx.x == 0) {
                S->e_kinetic = mue * 0.5 * ds * v[0];
                S->e_pot = mue * grav * ds * v[1];
                S->e_elastic = eta * 0.5 * ds * v[2];
                S->inertial_force[0] = mue * ds * v[3];
                S->inertial_force[1] = mue * ds * v[4];
            }
        }
    }
    PH(9);
    if (threadIdx.x == 0)
        for (int k = 4; k < 24; ++k) S->phase[k] += ph[k];
}

// Beam start state (init_beam.f90:83-120): straight beam at the leading edge, at rest.
__global__ void k_init_beam(BeamArgs b) {
    const int ns = b.ns;
    if (threadIdx.x == 0) b.S->beam_fact = 0;
    const double ca = b.cos_a, sa = b.sin_a;
    for (int i = threadIdx.x; i < ns; i += blockDim.x) {
        b.th[i] = 0.0; b.thd[i] = 0.0; b.ax[i] = 0.0; b.ay[i] = 0.0;
        b.p_old[i] = 0.0; b.p_new[i] = 0.0; b.tau_old[i] = 0.0; b.tau_new[i] = 0.0;
        for (int q = 0; q < 6; ++q) b.oo[q * ns + i] = 0.0;
        b.vx[i] = 0.0; b.vy[i] = 0.0;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double xrel = 0.0, yrel = 0.0;
        for (int s = 0; s < ns; ++s) {
            if (s > 0) {
                xrel = xrel + cos(0.0) * b.ds;
                yrel = yrel + sin(0.0) * b.ds;
            }
            b.x[s] = b.x0 + xrel * ca - yrel * sa;
            b.y[s] = b.y0 + yrel * ca + xrel * sa;
            b.vx[s] = 0.0;
            b.vy[s] = 0.0;
        }
    }
}

// ===================================================================================
// Host launchers
// ===================================================================================
static size_t beam_smem_bytes(int ns, int mask) {
    size_t bytes = 0;
    for (int part = 0; part < 4; ++part)
        if (mask & (1 << part)) bytes += beam_part_bytes(ns, part);
    return bytes;
}
void launch_beam(const BeamArgs& b, cudaStream_t st) {
    k_beam<<<1, 256, beam_smem_bytes(b.ns, b.use_smem), st>>>(b);
}
void launch_beam_pre(const BeamArgs& b, cudaStream_t st) {
    k_beam_pre<<<1, 256, beam_smem_bytes(b.ns, b.use_smem), st>>>(b);
}
// The dynamic shared-memory limit of a kernel is one setting per function, shared by every
// context of the process: it is only ever raised, to the largest size any context needs.
static bool raise_smem_limit(const void* fn, size_t bytes, size_t* current) {
    static std::mutex mu;
    std::lock_guard<std::mutex> lock(mu);
    if (bytes <= *current) return true;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess) return false;
    *current = bytes;
    return true;
}
static size_t g_pre_smem = 0, g_beam_smem = 0;

// Shared-memory placement for the predictor kernel: the FP64 vectors when they fit.
int beam_pre_smem_setup(int ns) {
    const size_t bytes = beam_part_bytes(ns, 2);
    if (bytes > 216 * 1024) return 0;
    return raise_smem_limit((const void*)k_beam_pre, bytes, &g_pre_smem) ? 4 : 0;
}
// Shared-memory placement of the beam workspace: parts taken in the order scr, fact, vec,
// band, each one kept when it still fits in 216 KB.
int beam_smem_setup(int ns) {
    int mask = 0;
    size_t bytes = 0;
    for (int part = 0; part < 4; ++part) {
        const size_t pb = beam_part_bytes(ns, part);
        if (bytes + pb <= 216 * 1024) { mask |= 1 << part; bytes += pb; }
    }
    if (mask && !raise_smem_limit((const void*)k_beam, bytes, &g_beam_smem)) mask = 0;
    return mask;
}
void launch_init_beam(const BeamArgs& b, cudaStream_t st) { k_init_beam<<<1, 256, 0, st>>>(b); }

}  // namespace fsibe
