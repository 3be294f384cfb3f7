// solid.cu -- FP64 device code of the solid side of the step:
//   * create_mask (create_mask.f90:2-218): primitive set-up + tile-culled rasteriser,
//   * GetForces / GetForcesInterp with SPL=3 (BeamForces.f90:6-288) and the phi4* delta
//     interpolation (Interpolation.f90:6-101),
//   * SolidSolverWrapper / IBES_solver (SolidSolver.f90:13-414) as one persistent CTA:
//     EE1 predictor with the tridiagonal tension solve, analytic Jacobian assembled as a band
//     (interleaved theta/T ordering, kl = ku = 7) and a warp-level banded LU with partial
//     pivoting in place of the reference's dense dgetrf/dgetrs.
// Built with -fmad=false so the geometric tests of the mask see the same roundings as the
// reference's separate multiply/add.
#include <math.h>

#include "solid.cuh"

namespace fsibe {

// ===================================================================================
// Mask
// ===================================================================================
__device__ __forceinline__ int dnint(double v) { return (int)llround(v); }  // Fortran NINT

__device__ __forceinline__ double smooth_step(double x, double t, double h, int sharp, double gerf) {
    if (!sharp) {
        const double delta = h * gerf;
        return 0.5 * (erf((t - x) / delta) + erf((x + t) / delta));
    }
    return (x <= t) ? 1.0 : 0.0;
}

__device__ __forceinline__ double convert_angle(double a, double pi) { return (a < 0.0) ? 2.0 * pi + a : a; }

__device__ __forceinline__ void clip_box(int* bx, int nx, int ny) {
    bx[0] = max(bx[0], 0);
    bx[1] = min(bx[1], nx - 1);
    bx[2] = max(bx[2], 0);
    bx[3] = min(bx[3], ny - 1);
}

// Per-primitive parameters in drawing order: segments, sharp end, hinges, dots.
__global__ void k_mask_prep(MaskArgs a, double gerf) {
    const int ns = a.ns;
    const double dx = a.dx, dy = a.dy, mx = fmax(dx, dy), t = a.t_beam, N = a.N_smooth;
    const double t_star = t + 2.0 * N * mx;
    const double alpha = a.angle_deg * a.pi / 180.0;  // mouvement case 0
    const int nseg = ns - 1, nsharp = (a.sharp_trailing == 1) ? 1 : 0, nh = ns - 2;
    const int ndot = (a.sharp_trailing == 0) ? 2 : 1;
    const int total = nseg + nsharp + nh + ndot;
    __shared__ int rect[4];
    if (threadIdx.x == 0) { rect[0] = a.nx; rect[1] = -1; rect[2] = a.ny; rect[3] = -1; }
    __syncthreads();
    for (int q = threadIdx.x; q < total; q += blockDim.x) {
        Prim P;
        for (int k = 0; k < 12; ++k) P.p[k] = 0.0;
        if (q < nseg) {
            const int i = q;
            const double p1x = a.x[i], p1y = a.y[i], p2x = a.x[i + 1], p2y = a.y[i + 1];
            const double al = -atan2((p2y - p1y), (p2x - p1x));
            P.type = PRIM_SEGMENT;
            P.box[0] = dnint((fmin(p1x, p2x) - t_star) / dx);
            P.box[1] = dnint((fmax(p1x, p2x) + t_star) / dx);
            P.box[2] = dnint((fmin(p1y, p2y) - t_star) / dy);
            P.box[3] = dnint((fmax(p1y, p2y) + t_star) / dy);
            const double ca = cos(al), sa = sin(al);
            P.p[0] = ca; P.p[1] = sa;
            P.p[2] = ca * p1x - sa * p1y; P.p[3] = sa * p1x + ca * p1y;
            P.p[4] = ca * p2x - sa * p2y; P.p[5] = sa * p2x + ca * p2y;
            P.p[6] = a.vx[i]; P.p[7] = a.vy[i]; P.p[8] = a.vx[i + 1]; P.p[9] = a.vy[i + 1];
        } else if (q < nseg + nsharp) {
            const int e = ns - 1;
            const double al = a.th[e] + alpha;
            const double ca = cos(al), sa = sin(al);
            const double p1x = a.x[e] - 2.0 * mx * ca, p1y = a.y[e] - 2.0 * mx * sa;
            const double p2x = a.x[e] + 4.0 * mx * ca, p2y = a.y[e] + 4.0 * mx * sa;
            P.type = PRIM_SHARP;
            P.box[0] = dnint((fmin(p1x, p2x) - t_star) / dx);
            P.box[1] = dnint((fmax(p1x, p2x) + t_star) / dx);
            P.box[2] = dnint((fmin(p1y, p2y) - t_star) / dy);
            P.box[3] = dnint((fmax(p1y, p2y) + t_star) / dy);
            P.p[0] = ca; P.p[1] = sa;
            P.p[2] = ca * p1x + sa * p1y; P.p[3] = -sa * p1x + ca * p1y;
            P.p[4] = ca * p2x + sa * p2y; P.p[5] = -sa * p2x + ca * p2y;
            P.p[6] = a.vx[e]; P.p[7] = a.vy[e];
        } else if (q < nseg + nsharp + nh) {
            const int i = q - nseg - nsharp + 1;
            const double px = a.x[i], py = a.y[i];
            const double a1 = atan2((a.y[i] - a.y[i - 1]), (a.x[i] - a.x[i - 1]));
            const double a2 = atan2((a.y[i + 1] - a.y[i]), (a.x[i + 1] - a.x[i]));
            P.type = PRIM_HINGE;
            P.box[0] = dnint((px - t_star) / dx);
            P.box[1] = dnint((px + t_star) / dx);
            P.box[2] = dnint((py - t_star) / dy);
            P.box[3] = dnint((py + t_star) / dy);
            P.p[0] = px; P.p[1] = py;
            P.p[2] = convert_angle(a1, a.pi) * 180.0 / a.pi;
            P.p[3] = convert_angle(a2, a.pi) * 180.0 / a.pi;
            P.p[4] = a.vx[i]; P.p[5] = a.vy[i];
        } else {
            // DrawADot runs over the whole grid in the reference; SmoothStep is exactly zero once
            // both erf arguments exceed ~6 (erf rounds to 1), so the box is cut at t + 10 delta.
            const int e = (q == total - ndot) ? 0 : ns - 1;
            const double px = a.x[e], py = a.y[e];
            if (py < 0.0) set_status(a.S, FSIBE_ERR_MASK_OOB);
            const double rcut = t + 10.0 * (N * mx) * gerf;
            P.type = PRIM_DOT;
            P.box[0] = (int)floor((px - rcut) / dx) - 1;
            P.box[1] = (int)ceil((px + rcut) / dx) + 1;
            P.box[2] = (int)floor((py - rcut) / dy) - 1;
            P.box[3] = (int)ceil((py + rcut) / dy) + 1;
            P.p[0] = px; P.p[1] = py; P.p[2] = a.vx[e]; P.p[3] = a.vy[e];
        }
        clip_box(P.box, a.nx, a.ny);
        a.prims[q] = P;
        if (P.box[0] <= P.box[1] && P.box[2] <= P.box[3]) {
            atomicMin(&rect[0], P.box[0]);
            atomicMax(&rect[1], P.box[1]);
            atomicMin(&rect[2], P.box[2]);
            atomicMax(&rect[3], P.box[3]);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 0; k < 4; ++k) a.rect[k] = rect[k];
        *a.nprims = total;
    }
}

#define MASK_TX 16
#define MASK_TY 8
#define MASK_NT (MASK_TX * MASK_TY)

// DrawHinge's angular test (create_mask.f90:623-641): both half-circle sectors contain gamma.
// near (optional) is set when gamma lies within `margin` degrees of an interval end.
template <typename T>
__device__ __forceinline__ bool hinge_inside(T gamma, T beta1, T beta2, T margin, bool* near) {
    bool in1 = false, in2 = false;
    auto ge = [&](T a, T b) { if (near && fabs(a - b) < margin) *near = true; return a >= b; };
    auto le = [&](T a, T b) { if (near && fabs(a - b) < margin) *near = true; return a <= b; };
    auto lt = [&](T a, T b) { if (near && fabs(a - b) < margin) *near = true; return a < b; };
    if (beta1 < (T)90) {
        if ((ge(gamma, (T)0) && le(gamma, (T)90 + beta1)) || (ge(gamma, (T)270 + beta1) && le(gamma, (T)360))) in1 = true;
    } else if (beta1 >= (T)90 && beta1 < (T)270) {
        if (ge(gamma, (T)270 + beta1 - (T)360) && le(gamma, (T)90 + beta1)) in1 = true;
    } else if (beta1 >= (T)270) {
        if ((ge(gamma, (T)0) && le(gamma, (T)90 + beta1 - (T)360)) || (ge(gamma, (T)270 + beta1 - (T)360) && le(gamma, (T)360))) in1 = true;
    }
    if (beta2 <= (T)90) {
        if (ge(gamma, (T)90 + beta2) && lt(gamma, (T)270 + beta2)) in2 = true;
    } else if (beta2 >= (T)90 && beta2 < (T)270) {
        if ((ge(gamma, (T)0) && le(gamma, (T)270 + beta2 - (T)360)) || (ge(gamma, (T)90 + beta2) && le(gamma, (T)360))) in2 = true;
    } else if (beta2 >= (T)270) {
        if (ge(gamma, (T)90 + beta2 - (T)360) && lt(gamma, (T)270 + beta2 - (T)360)) in2 = true;
    }
    return in1 && in2;
}

// FP32 pre-test data of one primitive: a cell that fails the pre-test is outside the primitive
// by more than the margin, so the exact FP64 test (the reference's arithmetic) is skipped.
struct PrimF {
    float4 a;  // segment/sharp: (cos, sin, x*_lo, x*_hi)   hinge/dot: (px, py, R^2 limit, 0)
    float2 b;  // segment/sharp: (y*_hi, y*_lo)
};

template <typename R>
__global__ void __launch_bounds__(MASK_NT) k_mask_raster(MaskArgs a, double gerf) {
    const int tx = threadIdx.x % MASK_TX, ty = threadIdx.x / MASK_TX;
    const int ix0 = blockIdx.x * MASK_TX, iy0 = blockIdx.y * MASK_TY;
    const int i = ix0 + tx, j = iy0 + ty;
    R* mk_ = reinterpret_cast<R*>(a.mask);
    R* vx_ = reinterpret_cast<R*>(a.mvx);
    R* vy_ = reinterpret_cast<R*>(a.mvy);
    const size_t cell = (size_t)j * a.nx + i;
    const int r0 = a.rect[0], r1 = a.rect[1], r2 = a.rect[2], r3 = a.rect[3];
    const int ix1 = ix0 + MASK_TX - 1, iy1 = iy0 + MASK_TY - 1;
    if (r1 < ix0 || r0 > ix1 || r3 < iy0 || r2 > iy1) {
        mk_[cell] = (R)0; vx_[cell] = (R)0; vy_[cell] = (R)0;
        return;
    }
    __shared__ Prim sp[MASK_NT];
    __shared__ PrimF sf[MASK_NT];
    __shared__ int wcount[MASK_NT / 32];
    __shared__ int nlist;
    const double dx = a.dx, dy = a.dy, mxd = fmax(dx, dy), t = a.t_beam, N = a.N_smooth;
    const double t_star = t + 2.0 * N * mxd, h = N * mxd;
    const double rcut = t + 10.0 * h * gerf;
    const float mg = 1.0e-5f * (float)fmax((double)a.nx * dx, (double)a.ny * dy);
    const double xi = (double)i * dx, yj = (double)j * dy;
    const float xf = (float)xi, yf = (float)yj;
    double m = 0.0, vx = 0.0, vy = 0.0;
    const int total = *a.nprims;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int base = 0; base < total; base += MASK_NT) {
        const int q = base + threadIdx.x;
        bool hit = false;
        Prim P;
        if (q < total) {
            P = a.prims[q];
            const int* bx = P.box;
            hit = !(bx[1] < ix0 || bx[0] > ix1 || bx[3] < iy0 || bx[2] > iy1) && bx[0] <= bx[1] && bx[2] <= bx[3];
        }
        const unsigned bal = __ballot_sync(0xffffffffu, hit);
        if (lane == 0) wcount[warp] = __popc(bal);
        __syncthreads();
        int off = 0;
        for (int w = 0; w < warp; ++w) off += wcount[w];
        if (hit) {
            const int e = off + __popc(bal & ((1u << lane) - 1u));
            sp[e] = P;
            PrimF F;
            if (P.type == PRIM_SEGMENT || P.type == PRIM_SHARP) {
                F.a = make_float4((float)P.p[0], (float)P.p[1], (float)P.p[2] - mg, (float)P.p[4] + mg);
                F.b = make_float2((float)(P.p[3] + t_star) + mg, (float)(P.p[5] - t_star) - mg);
            } else {
                const float lim = (float)((P.type == PRIM_HINGE) ? t_star : rcut) + mg;
                F.a = make_float4((float)P.p[0], (float)P.p[1], lim * lim, 0.f);
                F.b = make_float2(0.f, 0.f);
            }
            sf[e] = F;
        }
        if (threadIdx.x == 0) {
            int s = 0;
            for (int w = 0; w < MASK_NT / 32; ++w) s += wcount[w];
            nlist = s;
        }
        __syncthreads();
        const int nl = nlist;
        for (int e = 0; e < nl; ++e) {
            const Prim& Q = sp[e];
            if (i < Q.box[0] || i > Q.box[1] || j < Q.box[2] || j > Q.box[3]) continue;
            const PrimF F = sf[e];
            if (Q.type == PRIM_SEGMENT) {
                const float xs_f = xf * F.a.x - yf * F.a.y, ys_f = xf * F.a.y + yf * F.a.x;
                if (xs_f < F.a.z || xs_f > F.a.w || ys_f > F.b.x || ys_f < F.b.y) continue;
                const double ca = Q.p[0], sa = Q.p[1];
                const double xs = xi * ca - yj * sa, ys = xi * sa + yj * ca;
                if (xs >= Q.p[2] && xs <= Q.p[4] && ys <= (Q.p[3] + t_star) && ys >= (Q.p[5] - t_star)) {
                    const double temp = smooth_step(fabs(ys - Q.p[3]), t, h, a.sharp, gerf);
                    if (temp > m) {
                        m = temp;
                        vx = (Q.p[6] + (xs - Q.p[2]) * (Q.p[8] - Q.p[6]) / a.ds);
                        vy = (Q.p[7] + (xs - Q.p[2]) * (Q.p[9] - Q.p[7]) / a.ds);
                    }
                }
            } else if (Q.type == PRIM_SHARP) {
                const float xs_f = xf * F.a.x + yf * F.a.y, ys_f = -xf * F.a.y + yf * F.a.x;
                if (xs_f < F.a.z || xs_f > F.a.w || ys_f > F.b.x || ys_f < F.b.y) continue;
                const double ca = Q.p[0], sa = Q.p[1];
                const double xs = xi * ca + yj * sa, ys = -xi * sa + yj * ca;
                if (xs >= Q.p[2] && xs <= Q.p[4] && ys <= (Q.p[3] + t_star) && ys >= (Q.p[5] - t_star)) {
                    const double tmp2 = smooth_step(xs - Q.p[2], 2.0 * mxd, h, a.sharp, gerf);
                    const double temp = smooth_step(fabs(ys - Q.p[3]), t, h, a.sharp, gerf);
                    m = temp * tmp2;
                    if (xs - Q.p[2] >= 2.0 * mxd) { vx = Q.p[6]; vy = Q.p[7]; }
                }
            } else {
                const float ex = xf - F.a.x, ey = yf - F.a.y;
                if (ex * ex + ey * ey > F.a.z) continue;
                const double ddx = xi - Q.p[0], ddy = yj - Q.p[1];
                if (Q.type == PRIM_HINGE) {
                    // angular wedge first: FP32 atan2 of the FP64 offsets, exact FP64 only near an end
                    const float beta1f = (float)Q.p[2], beta2f = (float)Q.p[3];
                    float gf = atan2f((float)ddy, (float)ddx);
                    if (gf < 0.f) gf = 6.28318530717958647692f + gf;
                    gf = gf * 57.2957795130823208768f;
                    bool near = (fabsf(gf) < 1e-3f) || (fabsf(gf - 360.f) < 1e-3f) || (ddx == 0.0 && ddy == 0.0);
                    bool inw = hinge_inside<float>(gf, beta1f, beta2f, 1e-3f, &near);
                    if (near) {
                        const double gamma = convert_angle(atan2(ddy, ddx), a.pi) * 180.0 / a.pi;
                        inw = hinge_inside<double>(gamma, Q.p[2], Q.p[3], 0.0, nullptr);
                    }
                    if (!inw) continue;
                    const double Rr = sqrt(ddx * ddx + ddy * ddy);
                    if (Rr <= t_star) {
                        const double temp = smooth_step(Rr, t, h, a.sharp, gerf);
                        if (temp > m) { m = temp; vx = Q.p[4]; vy = Q.p[5]; }
                    }
                } else {
                    const double Rr = sqrt(ddx * ddx + ddy * ddy);
                    const double temp = smooth_step(Rr, t, h, a.sharp, gerf);
                    if (temp > m) { m = temp; vx = Q.p[2]; vy = Q.p[3]; }
                }
            }
        }
        __syncthreads();
    }
    mk_[cell] = (R)(m / a.eps);
    vx_[cell] = (R)vx;
    vy_[cell] = (R)vy;
}

// ===================================================================================
// Forces: phi4* delta interpolation of p and the viscous stresses at the beam surface
// ===================================================================================
__device__ __forceinline__ double delta_phi4star(double x, double dx, double pi) {
    const double r = fabs(x / dx);
    if (r < 0.5) return (3. / 8.) + (pi / 32.) - 0.25 * (r * r);
    if (r >= 0.5 && r <= 1.5)
        return 0.25 + (1.0 - r) / 8. * sqrt(-2. + 8. * r - 4. * (r * r)) - asin(sqrt(2.) * (r - 1.)) / 8.;
    if (r >= 1.5 && r <= 2.5)
        return (17. / 16.) - (pi / 64.) - (3. * r / 4.) + ((r * r) / 8.) + (r - 2.) * sqrt(-14. + 16. * r - 4. * (r * r)) / 16. +
               asin(sqrt(2.) * (r - 2.)) / 16.;
    return 0.0;
}

__device__ __forceinline__ double fld(const void* f, int fp32, size_t k) {
    return fp32 ? (double)reinterpret_cast<const float*>(f)[k] : reinterpret_cast<const double*>(f)[k];
}

__global__ void __launch_bounds__(128) k_forces(ForceArgs a, double dxi, double dyi) {
    const int n = blockIdx.x;
    __shared__ double dl[4][18];
    __shared__ int ij[4][2];
    __shared__ double res[6];
    const double alpha = a.angle_deg * a.pi / 180.0;
    const double thn = a.th[n] + alpha;
    const double s = sin(thn), c = cos(thn);
    const double mx = fmax(a.dy, a.dx);
    const double off = a.t_beam + a.N_smooth * mx;
    const double off1 = a.t_beam - 0.0 * a.N_smooth * mx;
    const double x = a.x[n], y = a.y[n];
    double px[4], py[4];
    px[0] = x - off1 * s; py[0] = y + off1 * c;
    px[1] = x + off1 * s; py[1] = y - off1 * c;
    px[2] = x - off * s; py[2] = y + off * c;
    px[3] = x + off * s; py[3] = y - off * c;
    const double x2 = a.xl - a.dx, y2 = a.yl - a.dy;
    if (threadIdx.x < 4) {
        const int p = threadIdx.x;
        const double xt = px[p], yt = py[p];
        const int i = (int)((xt - 0.0) / dxi), j = (int)((yt - 0.0) / dyi);
        ij[p][0] = i; ij[p][1] = j;
        if (xt > x2 || xt < 0.0 || yt > y2 || yt < 0.0 || i - 4 < 0 || j - 4 < 0 || i + 4 > a.nx - 1 || j + 4 > a.ny - 1)
            set_status(a.S, FSIBE_ERR_INTERP_OOB);
    }
    __syncthreads();
    if (threadIdx.x < 72) {
        const int p = threadIdx.x / 18, d = threadIdx.x % 18;
        if (d < 9) {
            const double xl_ = (double)(ij[p][0] - 4 + d) * dxi + 0.0;
            dl[p][d] = delta_phi4star(fabs(xl_ - px[p]), dxi, a.pi);
        } else {
            const double yl_ = (double)(ij[p][1] - 4 + d - 9) * dyi + 0.0;
            dl[p][d] = delta_phi4star(fabs(yl_ - py[p]), dyi, a.pi);
        }
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int k = threadIdx.x;
        const int p = (k < 2) ? k : (k < 4 ? 2 : 3);
        const void* f = (k < 2) ? a.press : ((k & 1) == 0 ? a.sa : a.sb);
        double R1 = 0.0;
        const int i = ij[p][0], j = ij[p][1];
        const bool ok = !(i - 4 < 0 || j - 4 < 0 || i + 4 > a.nx - 1 || j + 4 > a.ny - 1);
        if (ok && (k < 2 || a.viscous)) {
            for (int dxk = 0; dxk < 9; ++dxk)
                for (int dyk = 0; dyk < 9; ++dyk)
                    R1 = R1 + dl[p][dxk] * dl[p][9 + dyk] * fld(f, a.fp32, (size_t)(j - 4 + dyk) * a.nx + (i - 4 + dxk));
        }
        res[k] = R1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double pb = res[0] - res[1], tb = 0.0;
        if (a.viscous) {
            const double A1 = res[2], B1 = res[3], A2 = res[4], B2 = res[5];
            const double c2 = cos(2.0 * thn), s2 = sin(2.0 * thn);
            const double sn1 = -A1 * c2 - B1 * s2, st1 = -A1 * s2 + B1 * c2;
            const double sn2 = -A2 * c2 - B2 * s2, st2 = -A2 * s2 + B2 * c2;
            tb = st1 - st2;
            const double sg = -sn1 + sn2;
            pb = pb + sg;
        }
        const double time = a.S->time;
        double soft;
        if (time <= a.t_release) soft = 0.0;
        else if (time > a.t_release && time < a.t_release + a.tau) {
            const double tr = time - a.t_release;
            soft = (tr * tr * tr) / (-0.5 * a.tau * a.tau * a.tau) + 3. * (tr * tr) / (a.tau * a.tau);
        } else soft = 1.0;
        a.p_new[n] = pb * soft;
        a.tau_new[n] = tb * soft;
        // this node's term of the force integral (BeamForces.f90:264-267), summed below in order
        const double pn = pb * soft, tn = tb * soft;
        a.fterm[2 * n] = (sin(thn) * pn + cos(thn) * tn) * a.ds;
        a.fterm[2 * n + 1] = (cos(thn) * pn + sin(thn) * tn) * a.ds;
        __threadfence();
        const unsigned done = atomicAdd(a.counter, 1u);
        if (done == (unsigned)a.ns - 1) {
            // last block: Force_press = the sequential sum of the node terms, like the reference
            __threadfence();
            const volatile double* ft = a.fterm;
            double fx = 0.0, fy = 0.0;
            for (int i = 0; i < a.ns; ++i) {
                fx = fx - ft[2 * i];
                fy = fy + ft[2 * i + 1];
            }
            a.S->force_press[0] = fx;
            a.S->force_press[1] = fy;
            *a.counter = 0u;
        }
    }
}

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
    const D1DTab* dtab;
};

// The workspace has three parts: the FP64 vectors, the FP64 Jacobian band, the FP32 factor.
__host__ __device__ inline size_t beam_vec_doubles(int ns) {
    const int n = 2 * ns + 4, L = ns + 8;
    const size_t d = (size_t)29 * L + 5 * (size_t)(n + 8) + 11 * (size_t)L + (size_t)L + 64;
    return (d + 1) & ~(size_t)1;
}
__host__ __device__ inline size_t beam_band_doubles(int ns) { return (size_t)(2 * ns + 4 + 16) * 16; }
__host__ __device__ inline size_t beam_f32_floats_(int ns) {
    const int n = 2 * ns + 4;
    return ((size_t)(n + 16) * 16 + (size_t)(n + 16) * 8 + 2 * (size_t)(n + 16) + 3) & ~(size_t)3;
}
// Floats of the FP32 factor that persist between steps (U, L, row exponents).
__host__ __device__ inline size_t beam_fact_floats(int ns) { return ((size_t)(2 * ns + 4 + 16) * 25 + 3) & ~(size_t)3; }

__device__ BeamWS carve(double* p, double* band, float* f, int ns) {
    const int n = 2 * ns + 4, L = ns + 8;
    BeamWS w;
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
    w.band = band;
    w.Uf = f; f += (size_t)(n + 16) * 16;
    w.Lf = f; f += (size_t)(n + 16) * 8;
    w.rse = reinterpret_cast<int*>(f); f += n + 16;
    w.yf = f;
    return w;
}
}  // namespace

// Workspace length (doubles) of the global copy of the beam workspace for ns nodes.
__host__ size_t beam_ws_doubles(int ns) {
    return beam_vec_doubles(ns) + beam_band_doubles(ns) + (beam_f32_floats_(ns) + 1) / 2;
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
    const double alpha = b.angle_deg * b.pi / 180.0, alpha_t = 0.0;
    const double LE4 = 0.0, LE5 = 0.0;  // leading-edge accelerations, mouvement case 0
    for (int i = threadIdx.x; i < ns; i += blockDim.x) {
        w.th_s[i] = d1d(w.dtab, th, ns, 1, i);
        w.th_ss[i] = d1d(w.dtab, th, ns, 2, i);
        w.th_sss[i] = d1d(w.dtab, th, ns, 3, i);
        w.tau_s[i] = d1d(w.dtab, tau, ns, 1, i);
    }
    __syncthreads();
    const double K1 = mue * (LE4 * cos(alpha) + LE5 * sin(alpha) + grav * sin(alpha)) - tau[0];
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
    const double alpha = b.angle_deg * b.pi / 180.0, alpha_tt = 0.0;
    const double LE4 = 0.0, LE5 = 0.0;
    if (threadIdx.x == 0) { th[0] = 0.0; thd[0] = 0.0; }
    __syncthreads();
    int st = tension(b, w, T, w.T_s, th, thd, p, tau, grav);
    if (st) return st;
    const double ds2 = ds * ds;
    if (threadIdx.x == 0) {
        const double K2 = p[0] + mue * (LE5 * cos(alpha) - LE4 * sin(alpha) + grav * cos(alpha));
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

__device__ void newton_consts(NewtonCtx& c, double ds, double eta, double mue) {
    const double ds2 = ds * ds, ds3 = ds * ds * ds, ds4 = (ds * ds) * (ds * ds);
    c.ids = 1.0 / ds;
    c.i2ds = 1.0 / (2.0 * ds);
    c.ids2 = 1.0 / ds2;
    c.i2ds2 = 1.0 / (2.0 * ds2);
    c.ids4 = 1.0 / ds4;
    c.e2ds3 = eta / (2.0 * ds3);
    c.eds4 = eta / ds4;
    c.e2ds4 = eta / (2.0 * ds4);
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
// the band row of its interleaved position.  Returns non-zero when a NaN is produced.
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
    auto put = [&](int l, double v) {
        const int cidx = col_of(ns, l) - row + KL;
        if (isnan(v) || cidx < 0 || cidx >= BW) { bad = 1; return; }
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

// Solve with the FP32 factor in place on w.yf (one thread): the interchanges and L
// eliminations in the order dgbtrf made them (dgbtrs), then U x = y with the row written as
// a dot product, far terms first, so only x_{k+1} and x_{k+2} are on the recurrence.
__device__ void band_solve_f32(const BeamWS& w, int n) {
    float* __restrict__ y = w.yf;
    const float* __restrict__ L = w.Lf;
    const float* __restrict__ U = w.Uf;
    float q[KL + 1];
#pragma unroll
    for (int r = 0; r <= KL; ++r) q[r] = (r < n) ? y[r] : 0.f;
#pragma unroll 4
    for (int k = 0; k < n; ++k) {
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
        y[k] = t;
#pragma unroll
        for (int r = 0; r < KL; ++r) q[r] = q[r + 1];
        q[KL] = (k + 1 + KL < n) ? y[k + 1 + KL] : 0.f;
    }
    float xw[15];  // xw[c] = x_{k+c}
#pragma unroll
    for (int c = 0; c < 15; ++c) xw[c] = 0.f;
#pragma unroll 4
    for (int k = n - 1; k >= 0; --k) {
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
        float t = __fsub_rn(y[k], __fadd_rn(sa, sb));
        t = __fmaf_rn(-u0.z, xw[2], t);
        t = __fmaf_rn(-u0.y, xw[1], t);
        const float xk = __fmul_rn(t, u0.x);
        y[k] = xk;
#pragma unroll
        for (int c = 14; c >= 2; --c) xw[c] = xw[c - 1];
        xw[1] = xk;
    }
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

// IBES_solver / SolidSolverWrapper / SolidEnergies / the force integral, one CTA.
__global__ void __launch_bounds__(256) k_beam(BeamArgs b) {
    extern __shared__ __align__(16) double smem_ws[];
    DevScalars* S = b.S;
    if (S->status != 0) return;
    const int ns = b.ns, n = 2 * ns + 4;
    // use_smem: which workspace parts live in shared memory (0 none, 1 the FP32 factor,
    // 2 also the FP64 vectors, 3 also the FP64 band); the others in the global copy
    const int mode = b.use_smem;
    const size_t nv = beam_vec_doubles(ns), nb = beam_band_doubles(ns);
    double* vec = (mode >= 2) ? smem_ws : b.ws;
    double* band = (mode >= 3) ? smem_ws + nv : b.ws + nv;
    float* f32 = reinterpret_cast<float*>(mode == 3 ? smem_ws + nv + nb : (mode == 2 ? smem_ws + nv : (mode == 1 ? smem_ws : b.ws + nv + nb)));
    BeamWS w = carve(vec, band, f32, ns);
    const double time = S->time, dt = S->dt1;
    const double ds = b.ds, mue = b.mue, eta = b.eta;
    const double alpha = b.angle_deg * b.pi / 180.0;
    __shared__ double red[4][8];
    __shared__ int flag;
    __shared__ D1DTab dtab;
    long long ph_t = clock64(), ph[14] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    d1d_tables(&dtab, b.ds);
    w.dtab = &dtab;
    __syncthreads();

    if (threadIdx.x == 0) {
        // GravityImpulse (SolidSolver.f90:874-911)
        double grav = S->grav;
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
        S->grav = grav;
    }
    __syncthreads();
    const double grav = S->grav;

    for (int i = threadIdx.x; i < ns; i += blockDim.x) {
        w.bo3[i] = b.vx[i]; w.bo4[i] = b.vy[i]; w.bo5[i] = b.th[i]; w.bo6[i] = b.thd[i];
        w.oo5[i] = b.oo[4 * ns + i]; w.oo6[i] = b.oo[5 * ns + i];
    }
    __syncthreads();

    bool released = time > b.t_release;
    if (released) {
        const double dt_old = S->dt_old;
        if (threadIdx.x == 0) {
            if (S->startup_step) {
                S->startup_step = 0;
                if (S->method == FSIBE_BDF2) { S->actually_bdf2 = 1; S->method = FSIBE_CRANK_NICHOLSON; }
            }
        }
        __syncthreads();
        const int method = S->method;
        // EE1 predictor: th1 = theta, td1 = theta_dot -> RHS
        for (int i = threadIdx.x; i < ns; i += blockDim.x) { w.th1[i] = b.th[i]; w.td1[i] = b.thd[i]; }
        __syncthreads();
        PH(0);
        int st = rhs_beameqn(b, w, w.th1, w.td1, b.p_old, w.T, b.tau_old, grav);
        PH(1);
        if (st) { if (threadIdx.x == 0) set_status(S, FSIBE_ERR_SINGULAR); return; }
        for (int i = threadIdx.x; i < ns; i += blockDim.x) w.g5[i] = b.th[i] + dt * w.th1[i];
        __syncthreads();
        // initial guess with ghost points (SolidSolver.f90:175-202)
        if (threadIdx.x == 0) {
            const double* g5 = w.g5;
            const double* T = w.T;
            const double ds2 = ds * ds;
            const double K2 = b.p_new[0] + mue * (0.0 * cos(alpha) - 0.0 * sin(alpha) + grav * cos(alpha));
            const double C2v = 2.0 * ds * K2 - T[0] * g5[1] + (eta / ds2) * (10.0 * g5[0] - 12.0 * g5[1] + 6.0 * g5[2] - g5[3]);
            w.x[xi_th(-1)] = C2v / ((3.0 * eta / ds2) - T[0]);
            const double A1 = g5[ns - 3] / 12. - 2. * g5[ns - 2] / 3.;
            const double A2 = -g5[ns - 3] / 12. + 4. * g5[ns - 2] / 3. - 5. * g5[ns - 1] / 2.;
            w.x[xi_th(ns)] = 3. * (A1 - A2) / 2.;
            w.x[xi_th(ns + 1)] = 12. * (2. * A1 - A2);
            const double K1 = mue * (0.0 * cos(alpha) + 0.0 * sin(alpha) + grav * sin(alpha)) - b.tau_new[0];
            const double th_ss0 = (2.0 * g5[0] - 5.0 * g5[1] + 4.0 * g5[2] - 1.0 * g5[3]) / ds2;
            const double th_s0 = (-1.5 * g5[0] + 2.0 * g5[1] - 0.5 * g5[2]) / ds;
            const double T_s0 = -eta * th_ss0 * th_s0 + K1;
            w.x[xi_T(ns, -1)] = T[1] - 2.0 * ds * T_s0;
        }
        for (int i = threadIdx.x; i < ns; i += blockDim.x) {
            w.x[xi_th(i)] = w.g5[i];
            w.x[xi_T(ns, i)] = w.T[i];
            w.old_rhs[i] = 0.0;
            w.taun_s[i] = d1d(w.dtab, b.tau_new, ns, 1, i);
        }
        __syncthreads();
        PH(2);
        if (method == FSIBE_CRANK_NICHOLSON) {
            for (int i = threadIdx.x; i < ns; i += blockDim.x) { w.th1[i] = w.bo5[i]; w.old_rhs[i] = w.bo6[i]; }
            __syncthreads();
            st = rhs_beameqn(b, w, w.th1, w.old_rhs, b.p_old, w.T, b.tau_old, grav);
            if (st) { if (threadIdx.x == 0) set_status(S, FSIBE_ERR_SINGULAR); return; }
        }
        NewtonCtx c;
        c.time = time; c.dt = dt; c.dt_old = dt_old; c.alpha_t = 0.0; c.alpha_tt = 0.0; c.grav = grav;
        solid_coeffs(method, dt, dt_old, c.C1, c.C2, c.C3, c.C4);
        c.D = c.C1 / dt;
        newton_consts(c, ds, eta, mue);
        c.K1 = mue * (0.0 * cos(alpha) + 0.0 * sin(alpha) + grav * sin(alpha)) - b.tau_new[0];
        c.K2 = b.p_new[0] + mue * (0.0 * cos(alpha) - 0.0 * sin(alpha) + grav * cos(alpha));
        // the FP32 factor of an earlier step, when one is stored
        bool need_factor = (S->beam_fact == 0), factored = false;
        if (!need_factor && mode >= 1) {
            const float4* g = reinterpret_cast<const float4*>(b.ws + beam_vec_doubles(ns) + beam_band_doubles(ns));
            float4* d = reinterpret_cast<float4*>(w.Uf);
            for (size_t q = threadIdx.x; q < beam_fact_floats(ns) / 4; q += blockDim.x) d[q] = g[q];
            __syncthreads();
        }
        int iter = 0;
        bool iterate = true;
        PH(3);
        while (iterate) {
            if (threadIdx.x == 0) flag = 0;
            for (int i = threadIdx.x; i < ns; i += blockDim.x)
                w.tdn[i] = (c.C1 / dt) * (w.x[xi_th(i)] - c.C3 * w.bo5[i] - c.C4 * w.oo5[i]) - c.C2 * w.bo6[i];
            __syncthreads();
            for (int k = 1 + threadIdx.x; k <= n; k += blockDim.x) {
                const double f = f_eq(b, w, c, k);
                if (isnan(f)) flag = FSIBE_ERR_NAN;
                w.bvec[row_of(ns, k)] = -1.0 * f;
                if (jac_row(b, w, c, k)) flag = FSIBE_ERR_NAN;
            }
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
                    if (threadIdx.x == 0) band_solve_f32(w, n);
                    __syncthreads();
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
            double tsd = 0.0, tsx = 0.0;
            for (int q = 0; q < (int)(blockDim.x >> 5); ++q) { tsd += red[0][q]; tsx += red[1][q]; }
            iter = iter + 1;
            const double err = sqrt(tsd);
            const double err_rel = fabs(sqrt(tsd) / sqrt(tsx));
            if ((err < b.tol || err_rel < b.tol) && iter > 2) iterate = false;
            if (iter > b.maxit - 1) {
                if (threadIdx.x == 0) set_status(S, FSIBE_ERR_NEWTON_MAXIT);
                return;
            }
            __syncthreads();
        }
        double C1, C2, C3, C4;
        solid_coeffs(method, dt, dt_old, C1, C2, C3, C4);
        for (int i = threadIdx.x; i < ns; i += blockDim.x) {
            const double th = w.x[xi_th(i)];
            b.th[i] = th;
            b.thd[i] = (C1 / dt) * (th - C3 * w.bo5[i] - C4 * w.oo5[i]) - C2 * w.bo6[i];
        }
        if (factored) {
            if (mode >= 1) {
                float4* g = reinterpret_cast<float4*>(b.ws + beam_vec_doubles(ns) + beam_band_doubles(ns));
                const float4* d = reinterpret_cast<const float4*>(w.Uf);
                for (size_t q = threadIdx.x; q < beam_fact_floats(ns) / 4; q += blockDim.x) g[q] = d[q];
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
        w.cs[i] = cos(th) * ds;
        w.cs[ns + 8 + i] = sin(th) * ds;
        w.cs[2 * (ns + 8) + i] = td * sin(th) * ds;
        w.cs[3 * (ns + 8) + i] = td * cos(th) * ds;
    }
    __syncthreads();
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
        const double ca = cos(alpha), sa = sin(alpha), alpha_t = 0.0;
        for (int i = threadIdx.x; i < ns; i += blockDim.x) {
            const double xrel = w.pre[i], yrel = w.pre[(ns + 8) + i];
            const double vxrel = w.pre[2 * (ns + 8) + i], vyrel = w.pre[3 * (ns + 8) + i];
            b.x[i] = b.x0 + xrel * ca - yrel * sa;
            b.y[i] = b.y0 + yrel * ca + xrel * sa;
            b.vx[i] = 0.0 + ca * (vxrel - alpha_t * yrel) - sa * (vyrel + alpha_t * xrel);
            b.vy[i] = 0.0 + ca * (vyrel + alpha_t * xrel) + sa * (vxrel - alpha_t * yrel);
            if (released) {
                b.ax[i] = (b.vx[i] - w.bo3[i]) / dt;
                b.ay[i] = (b.vy[i] - w.bo4[i]) / dt;
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
    // SolidEnergies (SolidSolver.f90:76-92)
    for (int i = threadIdx.x; i < ns; i += blockDim.x) w.T_s[i] = d1d(w.dtab, b.th, ns, 1, i);
    __syncthreads();
    if (threadIdx.x == 0) {
        double sk = 0, sp = 0, se = 0, sax = 0, say = 0;
        for (int i = 0; i < ns; ++i) {
            sk += b.vx[i] * b.vx[i] + b.vy[i] * b.vy[i];
            sp += b.y[i] - b.y0;
            se += w.T_s[i] * w.T_s[i];
            sax += b.ax[i];
            say += b.ay[i];
        }
        S->e_kinetic = mue * 0.5 * ds * sk;
        S->e_pot = mue * grav * ds * sp;
        S->e_elastic = eta * 0.5 * ds * se;
        S->inertial_force[0] = mue * ds * sax;
        S->inertial_force[1] = mue * ds * say;
    }
    PH(9);
    if (threadIdx.x == 0)
        for (int k = 0; k < 14; ++k) S->phase[k] += ph[k];
}

// Beam start state (init_beam.f90:83-120): straight beam at the leading edge, at rest.
__global__ void k_init_beam(BeamArgs b) {
    const int ns = b.ns;
    if (threadIdx.x == 0) b.S->beam_fact = 0;
    const double alpha = b.angle_deg * b.pi / 180.0, ca = cos(alpha), sa = sin(alpha);
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
void launch_mask(const MaskArgs& a, double gerf, bool fp32, cudaStream_t st) {
    k_mask_prep<<<1, 256, 0, st>>>(a, gerf);
    dim3 grid(a.nx / MASK_TX, a.ny / MASK_TY);
    if (fp32) k_mask_raster<float><<<grid, MASK_NT, 0, st>>>(a, gerf);
    else k_mask_raster<double><<<grid, MASK_NT, 0, st>>>(a, gerf);
}

void launch_forces(const ForceArgs& a, double dxi, double dyi, cudaStream_t st) {
    k_forces<<<a.ns, 128, 0, st>>>(a, dxi, dyi);
}

static size_t beam_smem_bytes(int ns, int mode) {
    const size_t f = 4 * beam_f32_floats_(ns), v = 8 * beam_vec_doubles(ns), bd = 8 * beam_band_doubles(ns);
    if (mode == 3) return v + bd + f;
    if (mode == 2) return v + f;
    if (mode == 1) return f;
    return 0;
}
void launch_beam(const BeamArgs& b, cudaStream_t st) {
    k_beam<<<1, 256, beam_smem_bytes(b.ns, b.use_smem), st>>>(b);
}
// Shared-memory placement of the beam workspace: the largest set of parts that fits in
// 216 KB, in the order FP32 factor, FP64 vectors, FP64 band.
int beam_smem_setup(int ns) {
    for (int mode = 3; mode >= 1; --mode) {
        const size_t bytes = beam_smem_bytes(ns, mode);
        if (bytes > 216 * 1024) continue;
        if (cudaFuncSetAttribute(k_beam, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) == cudaSuccess) return mode;
    }
    return 0;
}
void launch_init_beam(const BeamArgs& b, cudaStream_t st) { k_init_beam<<<1, 256, 0, st>>>(b); }

}  // namespace fsibe
