// beam_impl.cuh -- device routines of the beam solver (IBES_solver, SolidSolver.f90:13-414)
// shared by the single-CTA kernels (beam.cu) and the cluster kernel (beam_cluster.cu): the
// Differentiate1D stencils, the beam workspace, the tension solve, F_nonlinear and the Jacobian
// rows, the FP32 banded LU and its chunked triangular solves, and the FP64 residuals.
// Everything has internal linkage: each translation unit that includes it gets its own copy.
// FP64 issue is the bottleneck on this chip (one FP64 warp instruction per SMSP every ~64
// cycles, ~64-cycle latency, division ~660 cycles): FP64 work is spread over all warps, serial
// chains run in FP32, divisions are taken out of loops.
#pragma once
#include <math.h>

#include "solid.cuh"

namespace fsibe {
namespace {

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

// ===================================================================================
// Beam solver
// ===================================================================================
// Differentiate1D (SolidSolver.f90:1085-1233): the rows of create_diff_matrices as stencils,
// each divided by 2dx / dx^2 / 2dx^3 / dx^4 first and summed over increasing column index,
// like the reference's matmul.  The divided table tab[order-1][row type][q] is formed once on
// the host (beam_d1d_table) and copied into shared memory by each kernel.
struct D1DTab {
    double c[4][3][8];
};

__device__ __forceinline__ void d1d_load(D1DTab* t, const double* __restrict__ g) {
    double* d = &t->c[0][0][0];
    for (int e = threadIdx.x; e < 4 * 3 * 8; e += blockDim.x) d[e] = g[e];
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
// the FP32 LU factor (U rows of 16, L rows of 8), which the sequential chunk sweeps read
__host__ __device__ inline size_t beam_lu_floats(int ns) { return (size_t)(2 * ns + 4 + 16) * 24; }
// the rest of the factor: row exponents and the chunk-boundary responses E, F
__host__ __device__ inline size_t beam_fact_floats(int ns) {
    const int n = 2 * ns + 4, C = beam_chunks(n);
    return r4((size_t)(n + 16) + (size_t)C * (64 + 224));
}
__host__ __device__ inline size_t beam_scr_floats(int ns) {
    const int n = 2 * ns + 4, C = beam_chunks(n);
    return r4((size_t)C * 48 + 2 * (size_t)(n + 16));
}
__host__ __device__ inline size_t beam_bulk_floats(int ns) { return (size_t)(2 * ns + 4 + 16) * 24; }
// The workspace parts: 0 scr, 1 fact, 2 vec, 3 band, 4 lu (mask bit 1 << part)
constexpr int BEAM_PARTS = 5;
__host__ __device__ inline size_t beam_part_bytes(int ns, int part) {
    switch (part) {
        case 0: return 4 * beam_scr_floats(ns);
        case 1: return 4 * beam_fact_floats(ns);
        case 2: return 8 * beam_vec_doubles(ns);
        case 3: return 8 * beam_band_doubles(ns);
        default: return 4 * beam_lu_floats(ns);
    }
}
// The o-th part in the order in which parts are offered shared memory (and packed there): the
// small scratch vectors, the LU factor of the sequential sweeps, the rest of the factor, the
// FP64 vectors, the FP64 band
__host__ __device__ constexpr int beam_part_at(int o) { return o == 0 ? 0 : (o == 1 ? 4 : o - 1); }

struct BeamParts { double* vec; double* band; float* lu; float* fact; float* scr; float* bulk; };

// Part addresses: those whose bit is set in mask packed in shared memory in beam_part_at order,
// the rest at their place in the global copy [vec | band | lu | fact | scr | bulk].
__device__ BeamParts beam_parts(double* gws, double* smem, int mask, int ns) {
    BeamParts P;
    double* g = gws;
    P.vec = g; g += beam_vec_doubles(ns);
    P.band = g; g += beam_band_doubles(ns);
    float* gf = reinterpret_cast<float*>(g);
    P.lu = gf; gf += beam_lu_floats(ns);
    P.fact = gf; gf += beam_fact_floats(ns);
    P.scr = gf; gf += beam_scr_floats(ns);
    P.bulk = gf;
    char* sp = reinterpret_cast<char*>(smem);
    for (int o = 0; o < BEAM_PARTS; ++o) {
        const int part = beam_part_at(o);
        if (!(mask & (1 << part))) continue;
        switch (part) {
            case 0: P.scr = reinterpret_cast<float*>(sp); break;
            case 1: P.fact = reinterpret_cast<float*>(sp); break;
            case 2: P.vec = reinterpret_cast<double*>(sp); break;
            case 3: P.band = reinterpret_cast<double*>(sp); break;
            default: P.lu = reinterpret_cast<float*>(sp); break;
        }
        sp += beam_part_bytes(ns, part);
    }
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
    w.Uf = P.lu;
    w.Lf = P.lu + (size_t)(n + 16) * 16;
    float* f = P.fact;
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
// c_k / c_(k-1), is below tscale (2^-44) of the solution, or the corrections stopped shrinking
// at the FP64 residual's rounding floor below 2^-30), -1 on a failure (10 passes, or a stall
// above that floor), 0 to go on.  rbuf: 16 doubles of shared memory.
//
// The beam's Newton iteration passes tscale = 2^-30: a solve's error enters the iterate as
// 2^-30 |dx_k|.  Before convergence Newton's map is flat at the root, so that moves the next
// iterate by O(|x_k - x*| 2^-30 |dx_k|); in the last iteration |dx_k| is below the Newton
// tolerance, so the error is below FP64 rounding of the solution (the stopping test on |dx_k|
// moves by the same relative 2^-30).
__device__ int refine_step(double* x, const float* cf, int n, int pass, float& cprev, double* rbuf,
                           double tscale = 0x1p-44) {
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
    const double tol = tscale * xmd;
    const bool conv = !(cmd > tol) || (pass >= 1 && cmd * cmd <= tol * cpd);
    const bool stall = pass >= 2 && cmd > 0.5 * cpd;
    cprev = __uint_as_float(cm);
    __syncthreads();
    if (conv || (stall && cmd <= 0x1p-30 * xmd)) return 1;
    if (stall || pass >= 9) return -1;
    return 0;
}

// One warp solves the first-order recurrence v_i = a_i v_(i-1) + c_i, v_(-1) = 0, over
// i = 0..n-1 (rev: over i = n-1..0 with v_n = 0), and writes out_i = v_i (times scale_i when
// scale is given).  Lane L takes a chunk of consecutive terms: it composes the chunk's affine
// maps, a shuffle scan composes the chunks, and each lane replays its chunk from the value
// that enters it.  out may alias c (each lane reads and writes only its own chunk).
__device__ __forceinline__ void warp_affine_scan(const float* a, const float* c, float* out, const float* scale, int n,
                                                 bool rev) {
    const int lane = threadIdx.x & 31;
    const int k = (n + 31) / 32;
    const int s0 = lane * k < n ? lane * k : n, s1 = (s0 + k) < n ? s0 + k : n;
    float A = 1.f, C = 0.f;
    for (int s = s0; s < s1; ++s) {
        const int i = rev ? n - 1 - s : s;
        C = __fmaf_rn(a[i], C, c[i]);
        A = __fmul_rn(a[i], A);
    }
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const float Ap = __shfl_up_sync(0xffffffffu, A, o), Cp = __shfl_up_sync(0xffffffffu, C, o);
        if (lane >= o) {
            C = __fmaf_rn(A, Cp, C);
            A = __fmul_rn(A, Ap);
        }
    }
    float v = __shfl_up_sync(0xffffffffu, C, 1);
    if (lane == 0) v = 0.f;
    for (int s = s0; s < s1; ++s) {
        const int i = rev ? n - 1 - s : s;
        v = __fmaf_rn(a[i], v, c[i]);
        out[i] = scale ? __fmul_rn(v, scale[i]) : v;
    }
}

// Tridiagonal system (dl, d, du) x = b (dl, du: n-1 entries) solved to the accuracy of an FP64
// factorisation (LAPACK dgttrf + dgttrs): an FP32 LU without interchanges (the scaled tension
// system is diagonally dominant) preconditions an FP64 iterative refinement with
// block-cooperative residuals.  The LU is formed by one thread; every refinement pass applies
// it by two warp scans (forward y_i = b_i - l_i y_(i-1), backward x_i = y_i/u_i -
// (du_i/u_i) x_(i+1)).  fs: 5n floats of scratch.  Returns non-zero on a zero pivot.
__device__ int tri_solve(int n, const double* dl, const double* d, const double* du, const double* b, double* x,
                         float* fs, int*) {
    float* __restrict__ fa = fs;           // forward coefficients -l_i (fa_0 = 0); first the FP32 d
    float* __restrict__ fr = fs + n;       // 1/u_i
    float* __restrict__ fb = fs + 2 * n;   // backward coefficients -du_i/u_i (fb_(n-1) = 0); first dl
    float* __restrict__ fu = fs + 3 * n;   // du (FP32)
    float* __restrict__ fy = fs + 4 * n;   // right-hand side / correction
    __shared__ int info_s;
    __shared__ double rbuf[16];
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        fa[i] = __double2float_rn(d[i]);
        fb[i] = (i < n - 1) ? __double2float_rn(dl[i]) : 0.f;
        fu[i] = (i < n - 1) ? __double2float_rn(du[i]) : 0.f;
        fy[i] = __double2float_rn(b[i]);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int info = 0;
        float u = fa[0];
        if (u == 0.f) info = 1;
        float r = __frcp_rn(u);
        fr[0] = r;
        fa[0] = 0.f;
        for (int i = 1; i < n && !info; ++i) {
            const float l = __fmul_rn(fb[i - 1], r);
            const float di = fa[i];
            u = __fmaf_rn(-l, fu[i - 1], di);
            if (u == 0.f) { info = i + 1; break; }
            fb[i - 1] = -__fmul_rn(fu[i - 1], r);
            r = __frcp_rn(u);
            fr[i] = r;
            fa[i] = -l;
        }
        fb[n - 1] = 0.f;
        info_s = info;
    }
    __syncthreads();
    if (info_s) return info_s;
    float cprev = 0.f;
    for (int pass = 0;; ++pass) {
        if (pass > 0) {
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                double rr = fma(-d[i], x[i], b[i]);
                if (i > 0) rr = fma(-dl[i - 1], x[i - 1], rr);
                if (i < n - 1) rr = fma(-du[i], x[i + 1], rr);
                fy[i] = __double2float_rn(rr);
            }
            __syncthreads();
        }
        if (threadIdx.x < 32) {
            warp_affine_scan(fa, fy, fy, fr, n, false);  // y_i / u_i
            __syncwarp();
            warp_affine_scan(fb, fy, fy, nullptr, n, true);
        }
        __syncthreads();
        if (refine_step(x, fy, n, pass, cprev, rbuf) != 0) break;
    }
    return 0;
}

// Tension (SolidSolver.f90:1000-1081), block-cooperative.
// mo: the leading edge's motion at the time of the call (mouvement(time))
__device__ int tension(const BeamArgs& b, BeamWS& w, double* T, double* T_s, const double* th, const double* thd,
                       const double* p, const double* tau, double grav, const Motion& mo) {
    const int ns = b.ns;
    const double ds = b.ds, eta = b.eta, mue = b.mue;
    const double alpha_t = mo.alpha_t;
    const double LE4 = mo.le[4], LE5 = mo.le[5];  // leading-edge accelerations
    for (int i = threadIdx.x; i < ns; i += blockDim.x) {
        w.th_s[i] = d1d(w.dtab, th, ns, 1, i);
        w.th_ss[i] = d1d(w.dtab, th, ns, 2, i);
        w.th_sss[i] = d1d(w.dtab, th, ns, 3, i);
        w.tau_s[i] = d1d(w.dtab, tau, ns, 1, i);
    }
    __syncthreads();
    const double K1 = mue * (LE4 * mo.ca + LE5 * mo.sa + grav * mo.sa) - tau[0];
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
                           const double* tau, double grav, const Motion& mo) {
    const int ns = b.ns;
    const double ds = b.ds, eta = b.eta, mue = b.mue, sigma = b.sigma;
    const double alpha_tt = mo.alpha_tt;
    const double LE4 = mo.le[4], LE5 = mo.le[5];
    if (threadIdx.x == 0) { th[0] = 0.0; thd[0] = 0.0; }
    __syncthreads();
    int st = tension(b, w, T, w.T_s, th, thd, p, tau, grav, mo);
    if (st) return st;
    const double ds2 = ds * ds;
    if (threadIdx.x == 0) {
        const double K2 = p[0] + mue * (LE5 * mo.ca - LE4 * mo.sa + grav * mo.ca);
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

// Newton's stopping test with iter > 2 (SolidSolver.f90:285-291): sqrt(sd) < tol or
// sqrt(sd) / sqrt(sx) < tol, for the sums of squares sd of the update and sx of the iterate.
// The squared comparisons settle it unless a side lies within 2^-40 (relative) of its bound,
// where the square roots and the quotient are evaluated as the reference does.
__device__ int newton_stop(double sd, double sx, double tol) {
    const double t2 = tol * tol, lo = 1.0 - 0x1p-40, hi = 1.0 + 0x1p-40;
    int a;  // sqrt(sd) < tol
    if (sd < t2 * lo) a = 1;
    else if (sd > t2 * hi) a = 0;
    else a = sqrt(sd) < tol;
    if (a) return 1;
    const double b2 = t2 * sx;  // sqrt(sd) / sqrt(sx) < tol
    if (sd < b2 * lo) return 1;
    if (sd > b2 * hi) return 0;
    return fabs(sqrt(sd) / sqrt(sx)) < tol;
}

// Offset (doubles) in the predictor's output of the step constants it forms for the Newton
// kernel: C1..C4, D = C1/dt, g, gds2, gds4e, and den0 = 3 eta/ds^2 - T_0 with RN(1/den0)
// for the clamped-end ghost value.
__host__ __device__ inline size_t pred_consts(int ns) { return (size_t)(2 * ns + 4) + 3 * (size_t)ns; }

// The Newton constants from the predictor's step constants K (no divisions here).
__device__ void newton_consts_pre(NewtonCtx& c, const BeamArgs& b, const double* __restrict__ K) {
    c.C1 = K[0]; c.C2 = K[1]; c.C3 = K[2]; c.C4 = K[3]; c.D = K[4];
    c.ids = b.k.ids;
    c.i2ds = b.k.i2ds;
    c.ids2 = b.k.ids2;
    c.i2ds2 = b.k.i2ds2;
    c.ids4 = b.k.ids4;
    c.e2ds3 = b.k.e2ds3;
    c.eds4 = b.k.eds4;
    c.e2ds4 = b.k.e2ds4;
    c.g = K[5];
    c.gds2 = K[6];
    c.gds4e = K[7];
    c.mue2 = b.mue * b.mue;
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
// Ab, the 16-entry band row of its interleaved position.  Returns non-zero for an entry outside the band.
__device__ int jac_row(const BeamArgs& b, const BeamWS& w, const NewtonCtx& c, int k, double* Ab) {
    const int ns = b.ns;
    const double eta = b.eta, mue = b.mue, sigma = b.sigma;
    const double* x = w.x;
    const double* p = b.p_new;
    const double* tau = b.tau_new;
    auto TH = [&](int j) { return x[j + 1]; };
    auto TT = [&](int j) { return x[ns + 4 + j]; };
    const int row = row_of(ns, k);
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
__device__ __forceinline__ void scale_band_row(const double* __restrict__ Ab, float* __restrict__ Urow, int* e_out) {
    unsigned long long m = 0;
#pragma unroll
    for (int q = 0; q < BW; ++q) {
        const unsigned long long a = (unsigned long long)__double_as_longlong(Ab[q]) & 0x7fffffffffffffffull;
        m = (a > m) ? a : m;
    }
    const int e = (int)(m >> 52);
    const double sc = row_scale(e);
    *e_out = e;
    float4* U4 = reinterpret_cast<float4*>(Urow);
#pragma unroll
    for (int q = 0; q < 4; ++q)
        U4[q] = make_float4(__double2float_rn(Ab[4 * q] * sc), __double2float_rn(Ab[4 * q + 1] * sc),
                            __double2float_rn(Ab[4 * q + 2] * sc), __double2float_rn(Ab[4 * q + 3] * sc));
}
__device__ __forceinline__ void scale_row(const BeamWS& w, int row) {
    scale_band_row(w.band + (size_t)row * 16, w.Uf + (size_t)row * 16, w.rse + row);
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
// chunk rows of the boundary-carry sweeps in flight ahead of their use
constexpr int CARRY_PD = 4;

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
        // the E rows of the next CARRY_PD chunks are in flight in a register ring (they do not
        // depend on the carry; at large ns they live in global memory)
        float4 ea[CARRY_PD], eb[CARRY_PD];
#pragma unroll
        for (int d = 0; d < CARRY_PD; ++d) {
            ea[d] = eb[d] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (d < C - 1) {
                ea[d] = *reinterpret_cast<const float4*>(w.Ec + d * 64 + lane * 8);
                eb[d] = *reinterpret_cast<const float4*>(w.Ec + d * 64 + lane * 8 + 4);
            }
        }
        for (int c = 0; c + 1 < C; ++c) {
            const float4 e0 = ea[0], e1 = eb[0];
#pragma unroll
            for (int d = 0; d + 1 < CARRY_PD; ++d) { ea[d] = ea[d + 1]; eb[d] = eb[d + 1]; }
            if (c + CARRY_PD < C - 1) {
                ea[CARRY_PD - 1] = *reinterpret_cast<const float4*>(w.Ec + (c + CARRY_PD) * 64 + lane * 8);
                eb[CARRY_PD - 1] = *reinterpret_cast<const float4*>(w.Ec + (c + CARRY_PD) * 64 + lane * 8 + 4);
            }
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
        // the F rows of the next CARRY_PD chunks in a register ring, as the E rows above
        float Fq[CARRY_PD][14];
#pragma unroll
        for (int d = 0; d < CARRY_PD; ++d)
#pragma unroll
            for (int j = 0; j < 14; ++j) Fq[d][j] = (C - 1 - d >= 1) ? w.Fc[(C - 1 - d) * 224 + lane * 16 + j] : 0.f;
        for (int c = C - 1; c >= 1; --c) {
            float Fr[14];
#pragma unroll
            for (int j = 0; j < 14; ++j) Fr[j] = Fq[0][j];
#pragma unroll
            for (int d = 0; d + 1 < CARRY_PD; ++d)
#pragma unroll
                for (int j = 0; j < 14; ++j) Fq[d][j] = Fq[d + 1][j];
            if (c - CARRY_PD >= 1) {
#pragma unroll
                for (int j = 0; j < 14; ++j) Fq[CARRY_PD - 1][j] = w.Fc[(c - CARRY_PD) * 224 + lane * 16 + j];
            }
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

}  // namespace
}  // namespace fsibe
