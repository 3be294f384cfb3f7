// solid.cu -- FP64 device code of the fluid-solid interface (the beam solver is in beam.cu):
//   * create_mask (create_mask.f90:2-218): primitive set-up + tile-culled rasteriser,
//   * GetForces / GetForcesInterp with SPL=3 (BeamForces.f90:6-288) and the phi4* delta
//     interpolation (Interpolation.f90:6-101).
// Built with -fmad=false so the geometric tests of the mask see the same roundings as the
// reference's separate multiply/add.
#include <math.h>

#include "solid.cuh"

namespace fsibe {

// ===================================================================================
// Mask
// ===================================================================================
__device__ __forceinline__ int dnint(double v) { return (int)llround(v); }  // Fortran NINT


__device__ __forceinline__ double convert_angle(double a, double pi) { return (a < 0.0) ? 2.0 * pi + a : a; }
// the same in FP32, in degrees (the FP32 form's raster: the angle of a cell about a hinge)
__device__ __forceinline__ float deg_f(float a) {
    if (a < 0.f) a = 6.28318530717958647692f + a;
    return a * 57.2957795130823208768f;
}

__device__ __forceinline__ void clip_box(int* bx, int nx, int ny) {
    bx[0] = max(bx[0], 0);
    bx[1] = min(bx[1], nx - 1);
    bx[2] = max(bx[2], 0);
    bx[3] = min(bx[3], ny - 1);
}

// Per-primitive parameters in drawing order: segments, sharp end, hinges, dots (create_mask.f90:
// 2-218, DrawBeamSegment/DrawHinge/DrawADot).  A block of four warps handles 32 nodes i, the
// FP64 work of a node spread over the four SMSPs: warp 0 segment i; warp 1 the direction angle
// of segment i-1 (the hinge's first angle); warp 2 that of segment i (its second); warp 3 the
// hinge's box, then the sharp end and the dots.  After one barrier warp 1 finishes the hinge.
// The bounding box of all primitives is reduced with atomics; the last block publishes it with
// its union with the previous step's box and resets the accumulator.
__global__ void __launch_bounds__(128) k_mask_prep(MaskArgs a, double gerf) {
    pdl_wait();     // the previous kernel of the stream has completed
    if (a.until_full && a.S->time >= a.T_fullspeed) return;
    __shared__ double ang2[32];
    __shared__ int hbox[32][4];
    __shared__ int wbox[4][4];
    const int ns = a.ns, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const double dx = a.dx, dy = a.dy, mx = fmax(dx, dy), t = a.t_beam, N = a.N_smooth;
    const double t_star = t + 2.0 * N * mx;
    const double rdx = a.rdx, rdy = a.rdy;
    const int nseg = ns - 1, nsharp = (a.sharp_trailing == 1) ? 1 : 0, nh = ns - 2;
    const int ndot = (a.sharp_trailing == 0) ? 2 : 1;
    const int total = nseg + nsharp + nh + ndot;
    const int i = blockIdx.x * 32 + lane;
    int bx0 = a.nx, bx1 = -1, by0 = a.ny, by1 = -1;
    // the FP32 raster's per-primitive data (the raster's expressions for its constants)
    const double rcut_g = t + 10.0 * (N * mx) * gerf;
    const float mg = 1.0e-5f * (float)fmax((double)a.nx * dx, (double)a.ny * dy);
    auto emit = [&](int q, Prim& P) {
        clip_box(P.box, a.nx, a.ny);
        a.prims[q] = P;
        if (a.primg && P.type != PRIM_SHARP) {
            PrimG G;
            if (P.type == PRIM_SEGMENT) {
                G.a = make_float4((float)P.p[0], (float)P.p[1], 0.f, 0.f);
                G.b = make_float4((float)(P.p[4] - P.p[2]), (float)((P.p[5] - P.p[3]) - t_star), 0.f, 0.f);
                G.c = make_float4((float)P.p[6], (float)P.p[7], (float)((P.p[8] - P.p[6]) * a.inv_ds),
                                  (float)((P.p[9] - P.p[7]) * a.inv_ds));
            } else {
                const float lim = (float)((P.type == PRIM_HINGE) ? t_star : rcut_g) + mg;
                G.a = make_float4(0.f, 0.f, lim * lim, 0.f);
                G.b = make_float4((float)P.p[2], (float)P.p[3], 0.f, 0.f);
                G.c = (P.type == PRIM_HINGE) ? make_float4((float)P.p[4], (float)P.p[5], 0.f, 0.f)
                                             : make_float4((float)P.p[2], (float)P.p[3], 0.f, 0.f);
            }
            a.primg[q] = G;
        }
        if (P.box[0] <= P.box[1] && P.box[2] <= P.box[3]) {
            bx0 = min(bx0, P.box[0]); bx1 = max(bx1, P.box[1]);
            by0 = min(by0, P.box[2]); by1 = max(by1, P.box[3]);
        }
    };
    const bool hinge = (i >= 1 && i <= ns - 2);
    double a1 = 0.0;
    if (warp == 0) {
        if (i < nseg) {
            const double p1x = a.x[i], p1y = a.y[i], p2x = a.x[i + 1], p2y = a.y[i + 1];
            // al = -atan2(p2y - p1y, p2x - p1x): cos(al), sin(al) from the normalised direction
            const double ddx = p2x - p1x, ddy = p2y - p1y;
            const double rl = 1.0 / sqrt(ddx * ddx + ddy * ddy);
            Prim P;
            for (int k = 0; k < 12; ++k) P.p[k] = 0.0;
            P.type = PRIM_SEGMENT;
            P.box[0] = dnint(div_cr(fmin(p1x, p2x) - t_star, dx, rdx));
            P.box[1] = dnint(div_cr(fmax(p1x, p2x) + t_star, dx, rdx));
            P.box[2] = dnint(div_cr(fmin(p1y, p2y) - t_star, dy, rdy));
            P.box[3] = dnint(div_cr(fmax(p1y, p2y) + t_star, dy, rdy));
            const double ca = ddx * rl, sa = -ddy * rl;
            P.p[0] = ca; P.p[1] = sa;
            P.p[2] = ca * p1x - sa * p1y; P.p[3] = sa * p1x + ca * p1y;
            P.p[4] = ca * p2x - sa * p2y; P.p[5] = sa * p2x + ca * p2y;
            P.p[6] = a.vx[i]; P.p[7] = a.vy[i]; P.p[8] = a.vx[i + 1]; P.p[9] = a.vy[i + 1];
            P.p[10] = p1x; P.p[11] = p1y;  // the FP32 raster works relative to the start point
            emit(i, P);
        }
    } else if (warp == 1) {
        // the hinge's two angles: FP32 in the FP32 form, whose raster tests its wedges in FP32
        if (hinge) {
            const double ddy = a.y[i] - a.y[i - 1], ddx = a.x[i] - a.x[i - 1];
            a1 = a.primg ? (double)atan2f((float)ddy, (float)ddx) : atan2(ddy, ddx);
        }
    } else if (warp == 2) {
        if (hinge) {
            const double ddy = a.y[i + 1] - a.y[i], ddx = a.x[i + 1] - a.x[i];
            ang2[lane] = a.primg ? (double)atan2f((float)ddy, (float)ddx) : atan2(ddy, ddx);
        }
    } else {
        if (hinge) {
            const double px = a.x[i], py = a.y[i];
            hbox[lane][0] = dnint(div_cr(px - t_star, dx, rdx));
            hbox[lane][1] = dnint(div_cr(px + t_star, dx, rdx));
            hbox[lane][2] = dnint(div_cr(py - t_star, dy, rdy));
            hbox[lane][3] = dnint(div_cr(py + t_star, dy, rdy));
        }
        if (i == ns && nsharp) {
            const int e = ns - 1;
            const double al = a.th[e] + motion_at(a.mo, a.S->time).alpha;  // mouvement(time)
            double sa, ca;
            sincos(al, &sa, &ca);
            const double p1x = a.x[e] - 2.0 * mx * ca, p1y = a.y[e] - 2.0 * mx * sa;
            const double p2x = a.x[e] + 4.0 * mx * ca, p2y = a.y[e] + 4.0 * mx * sa;
            Prim P;
            for (int k = 0; k < 12; ++k) P.p[k] = 0.0;
            P.type = PRIM_SHARP;
            P.box[0] = dnint(div_cr(fmin(p1x, p2x) - t_star, dx, rdx));
            P.box[1] = dnint(div_cr(fmax(p1x, p2x) + t_star, dx, rdx));
            P.box[2] = dnint(div_cr(fmin(p1y, p2y) - t_star, dy, rdy));
            P.box[3] = dnint(div_cr(fmax(p1y, p2y) + t_star, dy, rdy));
            P.p[0] = ca; P.p[1] = sa;
            P.p[2] = ca * p1x + sa * p1y; P.p[3] = -sa * p1x + ca * p1y;
            P.p[4] = ca * p2x + sa * p2y; P.p[5] = -sa * p2x + ca * p2y;
            P.p[6] = a.vx[e]; P.p[7] = a.vy[e];
            emit(nseg, P);
        }
        if (i >= ns + 1 && i < ns + 1 + ndot) {
            // DrawADot runs over the whole grid in the reference; SmoothStep is exactly zero once
            // both erf arguments exceed ~6 (erf rounds to 1), so the box is cut at t + 10 delta.
            const int d = i - (ns + 1);
            const int e = (d == 0) ? 0 : ns - 1;
            const double px = a.x[e], py = a.y[e];
            if (py < 0.0) set_status(a.S, FSIBE_ERR_MASK_OOB);
            const double rcut = t + 10.0 * (N * mx) * gerf;
            Prim P;
            for (int k = 0; k < 12; ++k) P.p[k] = 0.0;
            P.type = PRIM_DOT;
            P.box[0] = (int)floor(div_cr(px - rcut, dx, rdx)) - 1;
            P.box[1] = (int)ceil(div_cr(px + rcut, dx, rdx)) + 1;
            P.box[2] = (int)floor(div_cr(py - rcut, dy, rdy)) - 1;
            P.box[3] = (int)ceil(div_cr(py + rcut, dy, rdy)) + 1;
            P.p[0] = px; P.p[1] = py; P.p[2] = a.vx[e]; P.p[3] = a.vy[e];
            emit(nseg + nsharp + nh + d, P);
        }
    }
    __syncthreads();
    if (warp == 1 && hinge) {
        const double px = a.x[i], py = a.y[i];
        const double a2 = ang2[lane];
        Prim P;
        for (int k = 0; k < 12; ++k) P.p[k] = 0.0;
        P.type = PRIM_HINGE;
        P.box[0] = hbox[lane][0]; P.box[1] = hbox[lane][1]; P.box[2] = hbox[lane][2]; P.box[3] = hbox[lane][3];
        P.p[0] = px; P.p[1] = py;
        if (a.primg) {  // degrees as the FP32 raster forms a cell's angle
            P.p[2] = (double)deg_f((float)a1);
            P.p[3] = (double)deg_f((float)a2);
        } else {
            P.p[2] = div_cr(convert_angle(a1, a.pi) * 180.0, a.pi, a.rpi);
            P.p[3] = div_cr(convert_angle(a2, a.pi) * 180.0, a.pi, a.rpi);
        }
        P.p[4] = a.vx[i]; P.p[5] = a.vy[i];
        emit(nseg + nsharp + (i - 1), P);
    }
    // the box of all primitives: warp reductions, the block's four warps, then atomics on the
    // accumulator rect[8..11]
    bx0 = __reduce_min_sync(0xffffffffu, bx0);
    bx1 = __reduce_max_sync(0xffffffffu, bx1);
    by0 = __reduce_min_sync(0xffffffffu, by0);
    by1 = __reduce_max_sync(0xffffffffu, by1);
    if (lane == 0) { wbox[warp][0] = bx0; wbox[warp][1] = bx1; wbox[warp][2] = by0; wbox[warp][3] = by1; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 1; q < 4; ++q) {
            bx0 = min(bx0, wbox[q][0]); bx1 = max(bx1, wbox[q][1]);
            by0 = min(by0, wbox[q][2]); by1 = max(by1, wbox[q][3]);
        }
        if (bx0 <= bx1) {
            atomicMin(&a.rect[8], bx0); atomicMax(&a.rect[9], bx1);
            atomicMin(&a.rect[10], by0); atomicMax(&a.rect[11], by1);
        }
        __threadfence();
        const unsigned done = atomicAdd(reinterpret_cast<unsigned*>(&a.rect[12]), 1u);
        if (done == gridDim.x - 1) {
            __threadfence();
            volatile int* R = a.rect;
            const int n0 = R[8], n1 = R[9], n2 = R[10], n3 = R[11];
            const int p0 = R[0], p1 = R[1], p2 = R[2], p3 = R[3];
            R[0] = n0; R[1] = n1; R[2] = n2; R[3] = n3;
            R[4] = min(n0, p0); R[5] = max(n1, p1); R[6] = min(n2, p2); R[7] = max(n3, p3);
            if (a.full) { R[4] = 0; R[5] = a.nx - 1; R[6] = 0; R[7] = a.ny - 1; }  // walls, sponges: every cell
            R[8] = a.nx; R[9] = -1; R[10] = a.ny; R[11] = -1;
            R[12] = 0;
            *a.nprims = total;
        }
    }
}

// Raster tiles: 8 x 4 cells, one block of MASK_WARPS warps each; blocks stride over the tiles
// of the union of this step's and the previous step's primitive box, so every other cell keeps
// its zero.  The few tiles along the beam carry all the FP64 work: the primitives of a tile are
// dealt to its warps round-robin by index (every warp holds all 32 cells), so a tile's work
// spreads over the four SMSPs of its SM, and the warps' partial results are combined with the
// draw-order rule.
#define MASK_TX 8
#define MASK_TY 4
#define MASK_WARPS 4

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

// SmoothStep in FP32 from the FP64 distance: the FP32 form's value, and for the FP64 form an
// estimate within 1e-6 of the FP64 value (the argument is rounded once, |erf'| <= 2/sqrt(pi),
// erff is within 2 ulp).
__device__ __forceinline__ float smooth_step_f(double x, double t, double inv_delta, int sharp) {
    if (sharp) return (x <= t) ? 1.f : 0.f;
    const float a1 = (float)((t - x) * inv_delta), a2 = (float)((x + t) * inv_delta);
    return 0.5f * (erff(a1) + erff(a2));
}
// The FP64 value as the reference evaluates it (SmoothStep, create_mask.f90:697-717).
__device__ __forceinline__ double smooth_step_d(double x, double t, double inv_delta, int sharp) {
    if (sharp) return (x <= t) ? 1.0 : 0.0;
    return 0.5 * (erf((t - x) * inv_delta) + erf((x + t) * inv_delta));
}

// Per-cell fold state of one warp over its share of the primitives: the largest SmoothStep so
// far, its velocity and primitive index (INT_MAX: none yet), and an FP32 lower bound of m.
// T: double in the FP64 form, float in the FP32 form.
template <typename T>
struct MaskFold {
    T m, vx, vy;
    int idx;
    float mlow;
};

// Draw order keeps the first of equal values (strict >); over a subset taken in any order the
// same winner is the largest value with the smallest index among its ties.
template <typename T>
__device__ __forceinline__ void fold_take(MaskFold<T>& f, T temp, T vx, T vy, int q) {
    if (temp > f.m || (temp == f.m && f.idx != 0x7fffffff && q < f.idx)) {
        f.m = temp; f.vx = vx; f.vy = vy; f.idx = q;
        if constexpr (sizeof(T) == 8) f.mlow = __double2float_rd(temp);
    }
}

// SmoothStep in FP32 from FP32 arguments (the FP32 form's raster).
__device__ __forceinline__ float smooth_step_ff(float x, float t, float inv_delta, int sharp) {
    if (sharp) return (x <= t) ? 1.f : 0.f;
    return 0.5f * (erff((t - x) * inv_delta) + erff((x + t) * inv_delta));
}

// Segment, hinge or dot q for the lane's cell at (cx, cy) from the tile origin, all in FP32:
// the FP32 form's mask is continuous across every primitive's edge (a segment's end meets its
// hinge's disc with the same value and velocity, the outer edges have SmoothStep ~ 0), so the
// exact FP64 edge tests of the FP64 form are not needed for its tolerance.
__device__ __forceinline__ void mask_prim_f(const MaskArgs& a, const Prim& Q, const PrimG& G, int q, int i, int j,
                                            float cx, float cy, float tf, float tsf, float idf, MaskFold<float>& f) {
    if (i < Q.box[0] || i > Q.box[1] || j < Q.box[2] || j > Q.box[3]) return;
    if (Q.type == PRIM_SEGMENT) {
        const float xr = cx - G.a.z, yr = cy - G.a.w;
        const float u = G.a.x * xr - G.a.y * yr, w = G.a.y * xr + G.a.x * yr;
        if (u < 0.f || u > G.b.x || w > tsf || w < G.b.y) return;
        const float temp = smooth_step_ff(fabsf(w), tf, idf, a.sharp);
        if (temp >= f.m) fold_take<float>(f, temp, G.c.x + u * G.c.z, G.c.y + u * G.c.w, q);
        return;
    }
    const float ddx = cx - G.a.x, ddy = cy - G.a.y, r2 = ddx * ddx + ddy * ddy;
    if (r2 > G.a.z) return;
    if (Q.type == PRIM_HINGE) {
        const float gf = deg_f(atan2f(ddy, ddx));
        if (!hinge_inside<float>(gf, G.b.x, G.b.y, 0.f, nullptr)) return;
        const float Rr = sqrtf(r2);
        if (Rr <= tsf) fold_take<float>(f, smooth_step_ff(Rr, tf, idf, a.sharp), G.c.x, G.c.y, q);
        return;
    }
    fold_take<float>(f, smooth_step_ff(sqrtf(r2), tf, idf, a.sharp), G.c.x, G.c.y, q);
}

// Segment, hinge or dot q for the lane's cell (i, j), FP32 pre-test first.  R = float: the FP32
// form, SmoothStep in FP32.  R = double: SmoothStep in FP64, evaluated only when its FP32
// estimate (within 1e-6) could exceed the cell's current value by the margin 1e-5 -- a
// candidate that cannot win changes nothing under the draw-order rule.
template <typename R>
__device__ __forceinline__ void mask_prim(const MaskArgs& a, const Prim& Q, const PrimF& F, int q, int i, int j,
                                          double xi, double yj, float xf, float yf, double t, double t_star,
                                          double inv_delta, double inv_ds, MaskFold<double>& f) {
    if (i < Q.box[0] || i > Q.box[1] || j < Q.box[2] || j > Q.box[3]) return;
    if (Q.type == PRIM_SEGMENT) {
        const float xs_f = xf * F.a.x - yf * F.a.y, ys_f = xf * F.a.y + yf * F.a.x;
        if (xs_f < F.a.z || xs_f > F.a.w || ys_f > F.b.x || ys_f < F.b.y) return;
        const double ca = Q.p[0], sa = Q.p[1];
        const double xs = xi * ca - yj * sa, ys = xi * sa + yj * ca;
        if (xs >= Q.p[2] && xs <= Q.p[4] && ys <= (Q.p[3] + t_star) && ys >= (Q.p[5] - t_star)) {
            const double dist = fabs(ys - Q.p[3]);
            const float tf = smooth_step_f(dist, t, inv_delta, a.sharp);
            double temp;
            if (sizeof(R) == 4) temp = tf;
            else {
                if (tf + 1e-5f <= f.mlow) return;
                temp = smooth_step_d(dist, t, inv_delta, a.sharp);
            }
            if (temp >= f.m)
                fold_take(f, temp, (Q.p[6] + (xs - Q.p[2]) * (Q.p[8] - Q.p[6]) * inv_ds),
                          (Q.p[7] + (xs - Q.p[2]) * (Q.p[9] - Q.p[7]) * inv_ds), q);
        }
        return;
    }
    const float ex = xf - F.a.x, ey = yf - F.a.y;
    if (ex * ex + ey * ey > F.a.z) return;
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
        if (!inw) return;
        const double Rr = sqrt(ddx * ddx + ddy * ddy);
        if (Rr <= t_star) {
            const float tf = smooth_step_f(Rr, t, inv_delta, a.sharp);
            double temp;
            if (sizeof(R) == 4) temp = tf;
            else {
                if (tf + 1e-5f <= f.mlow) return;
                temp = smooth_step_d(Rr, t, inv_delta, a.sharp);
            }
            fold_take(f, temp, Q.p[4], Q.p[5], q);
        }
        return;
    }
    const double Rr = sqrt(ddx * ddx + ddy * ddy);
    const float tf = smooth_step_f(Rr, t, inv_delta, a.sharp);
    double temp;
    if (sizeof(R) == 4) temp = tf;
    else {
        if (tf + 1e-5f <= f.mlow) return;
        temp = smooth_step_d(Rr, t, inv_delta, a.sharp);
    }
    fold_take(f, temp, Q.p[2], Q.p[3], q);
}

// SmoothStep (create_mask.f90:475-520) with the reference's divisions, for the static parts.
__device__ __forceinline__ double smooth_step_div(double x, double t, double h, int sharp, double gerf) {
    if (sharp) return (x <= t) ? 1.0 : 0.0;
    const double delta = h * gerf;
    return 0.5 * (erf((t - x) / delta) + erf((x + t) / delta));
}
// SmoothStep2 (create_mask.f90:523-545)
__device__ __forceinline__ double smooth_step2(double x, double t, double h, double pi) {
    if (x <= t - h) return 1.0;
    if ((t - h) < x && x < (t + h)) return 0.5 * (1. + cos((x - t + h) * pi / (2.0 * h)));
    return 0.0;
}

// The parts drawn after the beam (create_mask.f90:131-204) on the unscaled value m and the
// velocity of cell (i, j): the velocity sponge of iSponge = 4 (both halves, in the reference's
// order) and the frame of iSponge = 22.  U, V: Mean_ux, Mean_uy of the time.
__device__ __forceinline__ void mask_finish(const MaskArgs& a, double gerf, int i, int j, size_t cell, double U, double V,
                                            double& m, double& vx, double& vy) {
    if (a.sponge4) {
        auto column = [&](double x, double t, double h) {
            const double tmp = smooth_step_div(x, t, h, a.sharp, gerf);
            if (m < tmp) m = tmp;
            const double yc = (double)j * a.dy - a.h_channel;
            vx = (yc > 0.0 && yc < a.H_eff) ? 1.5 * U * yc * (a.H_eff - yc) / ((0.5 * a.H_eff) * (0.5 * a.H_eff)) : 0.0;
        };
        if (i <= a.s4_l1) column(0.75 * a.s4_star - (double)i * a.dx, a.s4_size * 0.5, 0.25 * a.s4_size);
        if (i >= a.s4_r0 && i <= a.s4_r1) column((double)i * a.dx - 0.5 * a.s4_star, a.s4_size * 0.5, a.N_smooth * a.dx);
    }
    if (a.frame) {
        const double fr = a.frame[cell];
        m = m + fr * a.frame_c;
        if (fr > 0.0) { vx = U; vy = V; }
    }
}

// The primitives in draw order, per cell (create_mask.f90:2-218): segments and then hinges and
// dots keep the largest SmoothStep (the first of equal values); the sharp end between them
// overwrites the value.  Each warp folds its share of a range of primitives; the block
// combines the partial folds after the segments (then applies the sharp end) and after the
// hinges and dots.
template <typename R>
__global__ void __launch_bounds__(32 * MASK_WARPS) k_mask_raster(MaskArgs a, double gerf) {
    pdl_wait();     // the previous kernel of the stream has completed
    if (a.until_full && a.S->time >= a.T_fullspeed) return;
    constexpr bool F32 = sizeof(R) == 4;
    using T = R;  // the fold's arithmetic: FP32 in the FP32 form, FP64 in the FP64 form
    __shared__ Prim sp[MASK_WARPS][32];
    __shared__ PrimF sf[MASK_WARPS][F32 ? 1 : 32];
    __shared__ PrimG sg[MASK_WARPS][F32 ? 32 : 1];
    __shared__ double cmv[MASK_WARPS][3][32];
    __shared__ int cidx[MASK_WARPS][32];
    R* mk_ = reinterpret_cast<R*>(a.mask);
    R* vx_ = reinterpret_cast<R*>(a.mvx);
    R* vy_ = reinterpret_cast<R*>(a.mvy);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int r0 = a.rect[0], r1 = a.rect[1], r2 = a.rect[2], r3 = a.rect[3];
    const int u0 = a.rect[4], u1 = a.rect[5], u2 = a.rect[6], u3 = a.rect[7];
    if (u1 < u0 || u3 < u2) return;
    const int tx0 = u0 / MASK_TX, ty0 = u2 / MASK_TY;
    const int ntx = u1 / MASK_TX - tx0 + 1, nty = u3 / MASK_TY - ty0 + 1;
    const double dx = a.dx, dy = a.dy, mxd = fmax(dx, dy), t = a.t_beam, N = a.N_smooth;
    const double t_star = t + 2.0 * N * mxd, h = N * mxd;
    const double rcut = t + 10.0 * h * gerf;
    const double inv_delta = a.inv_delta, inv_ds = a.inv_ds, inv_eps = a.inv_eps;  // FP64 quotients from the host
    const double two_mxd = 2.0 * mxd;
    const float mg = 1.0e-5f * (float)fmax((double)a.nx * dx, (double)a.ny * dy);
    const int total = *a.nprims;
    // Mean_ux, Mean_uy of the time, for the velocity sponge and the frame
    const double Um = a.full ? mean_flow_x(a.iMeanVelocity, a.S->time, a.cos_ti, a.T_fullspeed, a.pi) : 0.0;
    const double Vm = a.full ? mean_flow_y(a.iMeanVelocity, a.S->time, a.sin_ti, a.T_fullspeed, a.pi) : 0.0;
    const int nseg = a.ns - 1, nsharp = (a.sharp_trailing == 1) ? 1 : 0;
    // FP32 form: the cell's offset from its tile's origin and the SmoothStep constants
    const float cx = (float)((double)(lane % MASK_TX) * dx), cy = (float)((double)(lane / MASK_TX) * dy);
    const float tf = (float)t, tsf = (float)t_star, idf = (float)inv_delta;
    for (int tile = blockIdx.x; tile < ntx * nty; tile += gridDim.x) {
        const int ix0 = (tx0 + tile % ntx) * MASK_TX, iy0 = (ty0 + tile / ntx) * MASK_TY;
        const int ix1 = ix0 + MASK_TX - 1, iy1 = iy0 + MASK_TY - 1;
        const int i = ix0 + (lane % MASK_TX), j = iy0 + (lane / MASK_TX);
        const size_t cell = (size_t)j * a.nx + i;
        if (r1 < ix0 || r0 > ix1 || r3 < iy0 || r2 > iy1) {
            if (warp == 0) {
                if (a.full) {
                    double m = a.bg ? a.bg[cell] : 0.0, vx = 0.0, vy = 0.0;
                    mask_finish(a, gerf, i, j, cell, Um, Vm, m, vx, vy);
                    mk_[cell] = (R)(m * inv_eps); vx_[cell] = (R)vx; vy_[cell] = (R)vy;
                } else {
                    mk_[cell] = (R)0; vx_[cell] = (R)0; vy_[cell] = (R)0;
                }
            }
            continue;
        }
        const double xi = (double)i * dx, yj = (double)j * dy;
        const float xf = (float)xi, yf = (float)yj;
        const double x0 = (double)ix0 * dx, y0 = (double)iy0 * dy;
        MaskFold<T> f;
        f.m = (T)0; f.vx = (T)0; f.vy = (T)0; f.idx = 0x7fffffff; f.mlow = 0.f;
        if (a.bg) {  // walls and cylinder come first in the draw order (velocity 0)
            const double b0 = a.bg[cell];
            f.m = (T)b0;
            f.mlow = __double2float_rd(b0);
        }
        // this warp's primitives of [q0, q1): q = q0 + MASK_WARPS (32 c + lane) + warp, staged
        // per round of 32 with their FP32 pre-test data
        auto fold_range = [&](int q0, int q1) {
            for (int base = q0; base < q1; base += 32 * MASK_WARPS) {
                const int q = base + MASK_WARPS * lane + warp;
                bool hit = false;
                Prim P;
                if (q < q1) {
                    P = a.prims[q];
                    const int* bx = P.box;
                    hit = !(bx[1] < ix0 || bx[0] > ix1 || bx[3] < iy0 || bx[2] > iy1) && bx[0] <= bx[1] && bx[2] <= bx[3];
                }
                const unsigned bal = __ballot_sync(0xffffffffu, hit);
                if (hit) {
                    const int e = __popc(bal & ((1u << lane) - 1u));
                    sp[warp][e] = P;
                    if constexpr (F32) {
                        // k_mask_prep's data, with this tile's offsets (two FP64 subtractions)
                        PrimG G = a.primg[q];
                        const bool seg = P.type == PRIM_SEGMENT;
                        const float ox = (float)((seg ? P.p[10] : P.p[0]) - x0), oy = (float)((seg ? P.p[11] : P.p[1]) - y0);
                        if (seg) { G.a.z = ox; G.a.w = oy; }
                        else { G.a.x = ox; G.a.y = oy; }
                        sg[warp][e] = G;
                    } else {
                        PrimF F;
                        if (P.type == PRIM_SEGMENT || P.type == PRIM_SHARP) {
                            F.a = make_float4((float)P.p[0], (float)P.p[1], (float)P.p[2] - mg, (float)P.p[4] + mg);
                            F.b = make_float2((float)(P.p[3] + t_star) + mg, (float)(P.p[5] - t_star) - mg);
                        } else {
                            const float lim = (float)((P.type == PRIM_HINGE) ? t_star : rcut) + mg;
                            F.a = make_float4((float)P.p[0], (float)P.p[1], lim * lim, 0.f);
                            F.b = make_float2(0.f, 0.f);
                        }
                        sf[warp][e] = F;
                    }
                    cidx[warp][e] = q;
                }
                __syncwarp();
                const int nl = __popc(bal);
                for (int e = 0; e < nl; ++e) {
                    if constexpr (F32)
                        mask_prim_f(a, sp[warp][e], sg[warp][e], cidx[warp][e], i, j, cx, cy, tf, tsf, idf, f);
                    else
                        mask_prim<R>(a, sp[warp][e], sf[warp][e], cidx[warp][e], i, j, xi, yj, xf, yf, t, t_star,
                                     inv_delta, inv_ds, f);
                }
                __syncwarp();
            }
        };
        // the block's partial folds -> the combined state in every warp
        auto combine = [&]() {
            cmv[warp][0][lane] = f.m; cmv[warp][1][lane] = f.vx; cmv[warp][2][lane] = f.vy;
            const int my = f.idx;
            __syncthreads();
            cidx[warp][lane] = my;
            __syncthreads();
            for (int w = 0; w < MASK_WARPS; ++w) {
                const T mw = (T)cmv[w][0][lane];
                const int iw = cidx[w][lane];
                if (mw > f.m || (mw == f.m && iw < f.idx)) {
                    f.m = mw; f.vx = (T)cmv[w][1][lane]; f.vy = (T)cmv[w][2][lane]; f.idx = iw;
                }
            }
            if constexpr (!F32) f.mlow = __double2float_rd(f.m);
            __syncthreads();
        };
        fold_range(0, nseg);
        combine();
        if (nsharp) {
            const Prim& Q = a.prims[nseg];
            if (!(i < Q.box[0] || i > Q.box[1] || j < Q.box[2] || j > Q.box[3])) {
                const double ca = Q.p[0], sa = Q.p[1];
                const double xs = xi * ca + yj * sa, ys = -xi * sa + yj * ca;
                if (xs >= Q.p[2] && xs <= Q.p[4] && ys <= (Q.p[3] + t_star) && ys >= (Q.p[5] - t_star)) {
                    double tmp2, temp;
                    if (sizeof(R) == 4) {
                        tmp2 = smooth_step_f(xs - Q.p[2], two_mxd, inv_delta, a.sharp);
                        temp = smooth_step_f(fabs(ys - Q.p[3]), t, inv_delta, a.sharp);
                    } else {
                        tmp2 = smooth_step_d(xs - Q.p[2], two_mxd, inv_delta, a.sharp);
                        temp = smooth_step_d(fabs(ys - Q.p[3]), t, inv_delta, a.sharp);
                    }
                    f.m = (T)(temp * tmp2);
                    f.mlow = __double2float_rd(temp * tmp2);
                    if (xs - Q.p[2] >= two_mxd) { f.vx = (T)Q.p[6]; f.vy = (T)Q.p[7]; }
                }
            }
        }
        f.idx = 0x7fffffff;  // the state after the sharp end is no primitive of the next range
        fold_range(nseg + nsharp, total);
        combine();
        if (warp == 0) {
            double m = (double)f.m, vx = (double)f.vx, vy = (double)f.vy;
            if (a.full) mask_finish(a, gerf, i, j, cell, Um, Vm, m, vx, vy);
            mk_[cell] = (R)(m * inv_eps);
            vx_[cell] = (R)vx;
            vy_[cell] = (R)vy;
        }
    }
}

// ===================================================================================
// Forces: phi4* delta interpolation of p and the viscous stresses at the beam surface
// ===================================================================================
// phi4* (BeamForces.f90): the branch of r = |x/dx| chosen arithmetically, so a warp whose lanes
// fall in different branches runs one square root and one arcsine instead of one per branch;
// each branch keeps the reference's expression.  rdx = RN(1/dx).
__device__ __forceinline__ double delta_phi4star(double x, double dx, double rdx, double pi) {
    const double r = fabs(div_cr(x, dx, rdx));
    if (r < 0.5) return (3. / 8.) + (pi / 32.) - 0.25 * (r * r);
    if (!(r <= 2.5)) return 0.0;
    const bool b2 = r <= 1.5;
    const double sq = sqrt(b2 ? (-2. + 8. * r - 4. * (r * r)) : (-14. + 16. * r - 4. * (r * r)));
    const double as = asin(b2 ? sqrt(2.) * (r - 1.) : sqrt(2.) * (r - 2.));
    if (b2) return 0.25 + (1.0 - r) / 8. * sq - as / 8.;
    return (17. / 16.) - (pi / 64.) - (3. * r / 4.) + ((r * r) / 8.) + (r - 2.) * sq / 16. + as / 16.;
}

__device__ __forceinline__ double fld(const void* f, int fp32, size_t k) {
    return fp32 ? (double)reinterpret_cast<const float*>(f)[k] : reinterpret_cast<const double*>(f)[k];
}

// One block per beam node.  The trigonometric values are evaluated once per block; the six
// 9 x 9 interpolation sums run as 54 nine-term partial sums; the force integral of all nodes
// is a block reduction in the last block.  Summation orders differ from the reference's
// sequential loops (relative differences of a few ulps).
// The geometry of the interpolation at node n (BeamForces.f90:105-124): the trigonometric
// values, the four surface points' cells and their phi4* weights.  It depends only on the beam
// state, so the step computes it beside the fluid kernels; k_forces then reads it.
// Per node in a.geo: trig[4], dl[4][18]; in a.gij: ij[4][2].
__global__ void __launch_bounds__(128) k_forces_geo(ForceArgs a, double dxi, double dyi) {
    const int n = blockIdx.x;
    __shared__ double dl[4][18];
    __shared__ int ij[4][2];
    __shared__ double trig[4];  // sin, cos of theta + alpha and of twice it
    __shared__ double px[4], py[4];
    // the two sincos on two warps (SMSPs)
    if (threadIdx.x == 0 || threadIdx.x == 32) {
        const double thn = a.th[n] + motion_at(a.mo, a.S->time).alpha;  // mouvement(time)
        double sv, cv;
        if (threadIdx.x == 0) {
            sincos(thn, &sv, &cv);
            trig[0] = sv; trig[1] = cv;
            const double mx = fmax(a.dy, a.dx);
            const double off = a.t_beam + a.N_smooth * mx;
            const double off1 = a.t_beam - 0.0 * a.N_smooth * mx;
            const double x = a.x[n], y = a.y[n];
            px[0] = x - off1 * sv; py[0] = y + off1 * cv;
            px[1] = x + off1 * sv; py[1] = y - off1 * cv;
            px[2] = x - off * sv; py[2] = y + off * cv;
            px[3] = x + off * sv; py[3] = y - off * cv;
        } else {
            sincos(2.0 * thn, &sv, &cv);
            trig[2] = sv; trig[3] = cv;
        }
    }
    __syncthreads();
    const double x2 = a.xl - a.dx, y2 = a.yl - a.dy;
    if (threadIdx.x < 4) {
        const int p = threadIdx.x;
        const double xt = px[p], yt = py[p];
        const int i = (int)div_cr((xt - 0.0), dxi, a.rdxi), j = (int)div_cr((yt - 0.0), dyi, a.rdyi);
        ij[p][0] = i; ij[p][1] = j;
        if (xt > x2 || xt < 0.0 || yt > y2 || yt < 0.0 || i - 4 < 0 || j - 4 < 0 || i + 4 > a.nx - 1 || j + 4 > a.ny - 1)
            set_status(a.S, FSIBE_ERR_INTERP_OOB);
    }
    __syncthreads();
    if (threadIdx.x < 72) {
        const int p = threadIdx.x / 18, d = threadIdx.x % 18;
        if (d < 9) {
            const double xl_ = (double)(ij[p][0] - 4 + d) * dxi + 0.0;
            dl[p][d] = delta_phi4star(fabs(xl_ - px[p]), dxi, a.rdxi, a.pi);
        } else {
            const double yl_ = (double)(ij[p][1] - 4 + d - 9) * dyi + 0.0;
            dl[p][d] = delta_phi4star(fabs(yl_ - py[p]), dyi, a.rdyi, a.pi);
        }
    }
    __syncthreads();
    double* g = a.geo + (size_t)n * 76;
    if (threadIdx.x < 4) g[threadIdx.x] = trig[threadIdx.x];
    if (threadIdx.x < 72) g[4 + threadIdx.x] = dl[threadIdx.x / 18][threadIdx.x % 18];
    if (threadIdx.x < 8) a.gij[(size_t)n * 8 + threadIdx.x] = ij[threadIdx.x / 2][threadIdx.x % 2];
}

__global__ void __launch_bounds__(128) k_forces(ForceArgs a, double dxi, double dyi) {
    pdl_wait();     // the previous kernel of the stream has completed
    pdl_trigger();  // the beam kernel may start its set-up (it waits for this kernel's results)
    const int n = blockIdx.x;
    __shared__ double dl[4][18];
    __shared__ int ij[4][2];
    __shared__ double part[6][9];
    __shared__ double trig[4];  // sin, cos of theta + alpha and of twice it
    __shared__ int last;
    {
        const double* g = a.geo + (size_t)n * 76;
        if (threadIdx.x < 4) trig[threadIdx.x] = g[threadIdx.x];
        if (threadIdx.x < 72) dl[threadIdx.x / 18][threadIdx.x % 18] = g[4 + threadIdx.x];
        if (threadIdx.x < 8) ij[threadIdx.x / 2][threadIdx.x % 2] = a.gij[(size_t)n * 8 + threadIdx.x];
    }
    __syncthreads();
    if (threadIdx.x < 54) {
        // sum k (0, 1: pressure at the two surface points; 2..5: the stresses), column dxk
        const int k = threadIdx.x / 9, dxk = threadIdx.x % 9;
        const int p = (k < 2) ? k : (k < 4 ? 2 : 3);
        const void* f = (k < 2) ? a.press : ((k & 1) == 0 ? a.sa : a.sb);
        double R1 = 0.0;
        const int i = ij[p][0], j = ij[p][1];
        const bool ok = !(i - 4 < 0 || j - 4 < 0 || i + 4 > a.nx - 1 || j + 4 > a.ny - 1);
        if (ok && (k < 2 || a.viscous)) {
            // the column's nine field values loaded together, then the reference's sum in order
            const double dxv = dl[p][dxk];
            double fv[9];
#pragma unroll
            for (int dyk = 0; dyk < 9; ++dyk) fv[dyk] = fld(f, a.fp32, (size_t)(j - 4 + dyk) * a.nx + (i - 4 + dxk));
#pragma unroll
            for (int dyk = 0; dyk < 9; ++dyk) R1 = R1 + dxv * dl[p][9 + dyk] * fv[dyk];
        }
        part[k][dxk] = R1;
    }
    __syncthreads();
    __shared__ double res[6];
    if (threadIdx.x < 6) {
        double r = 0.0;
        for (int q = 0; q < 9; ++q) r += part[threadIdx.x][q];
        res[threadIdx.x] = r;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double pb = res[0] - res[1], tb = 0.0;
        if (a.viscous) {
            const double A1 = res[2], B1 = res[3], A2 = res[4], B2 = res[5];
            const double c2 = trig[3], s2 = trig[2];
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
        // this node's term of the force integral (BeamForces.f90:264-267)
        const double pn = pb * soft, tn = tb * soft, s = trig[0], c = trig[1];
        a.fterm[2 * n] = (s * pn + c * tn) * a.ds;
        a.fterm[2 * n + 1] = (c * pn + s * tn) * a.ds;
        __threadfence();
        const unsigned done = atomicAdd(a.counter, 1u);
        last = (done == (unsigned)a.ns - 1) ? 1 : 0;
    }
    __syncthreads();
    if (last) {
        // last block: Force_press = -sum of the x terms, sum of the y terms (block reduction)
        __threadfence();
        const volatile double* ft = a.fterm;
        double fx = 0.0, fy = 0.0;
        for (int i = threadIdx.x; i < a.ns; i += blockDim.x) {
            fx = fx - ft[2 * i];
            fy = fy + ft[2 * i + 1];
        }
        for (int o = 16; o > 0; o >>= 1) {
            fx += __shfl_xor_sync(0xffffffffu, fx, o);
            fy += __shfl_xor_sync(0xffffffffu, fy, o);
        }
        __shared__ double wsum[2][4];
        if ((threadIdx.x & 31) == 0) { wsum[0][threadIdx.x >> 5] = fx; wsum[1][threadIdx.x >> 5] = fy; }
        __syncthreads();
        if (threadIdx.x == 0) {
            double sx = 0.0, sy = 0.0;
            for (int q = 0; q < (int)(blockDim.x >> 5); ++q) { sx += wsum[0][q]; sy += wsum[1][q]; }
            a.S->force_press[0] = sx;
            a.S->force_press[1] = sy;
            *a.counter = 0u;
        }
    }
}

// ===================================================================================
// Host launchers
// ===================================================================================
void launch_mask_prep(const MaskArgs& a, double gerf, cudaStream_t st, bool pdl) {
    launch_k(k_mask_prep, dim3((a.ns + 3 + 31) / 32), dim3(128), 0, st, pdl, a, gerf);
}
// The walls (create_mask.f90:30-54: each wall row assigned its SmoothStep) and the leading-edge
// cylinder (:66-68, DrawADot with the strict > rule), and the frame of iSponge = 22
// (SmoothFrameAroundDomain, :370-470: the level set of the distance to the domain's edges with
// rounded corners, each pass of the reference applied to the cell in its order), per cell.
__global__ void k_static_masks(StaticMaskArgs a, double gerf) {
    const size_t n = (size_t)a.nx * a.ny;
    for (size_t cell = blockIdx.x * (size_t)blockDim.x + threadIdx.x; cell < n; cell += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(cell % a.nx), j = (int)(cell / a.nx);
        const double x = (double)i * a.dx, y = (double)j * a.dy, mx = fmax(a.dx, a.dy);
        if (a.bg) {
            double m = 0.0;
            if (a.iWalls > 0) {
                const double h = a.h_channel, hs = h + a.N * a.dy;
                if (j <= (int)llround(hs / a.dy)) m = smooth_step_div(y, h, a.N * a.dy, a.sharp, gerf);
                if (j >= (int)llround((a.yl - hs) / a.dy)) m = smooth_step_div(fabs(y - a.yl), h, a.N * a.dy, a.sharp, gerf);
            }
            if (a.iCylinder == 1) {
                const double px = a.x0 - a.R_cylinder, py = a.y0;
                const double Rr = sqrt((x - px) * (x - px) + (y - py) * (y - py));
                const double temp = smooth_step_div(Rr, a.R_cylinder, a.N * mx, a.sharp, gerf);
                if (temp > m) m = temp;
            }
            a.bg[cell] = m;
        }
        if (a.frame) {
            const double th = 4.0 * a.t_beam, R1 = 0.0, R2 = 2.0 * th, RR = R1 + R2;
            const int ixmin = (int)llround(RR / a.dx), ixmax = a.nx - (int)llround(RR / a.dx);
            const int iymin = (int)llround(RR / a.dy), iymax = a.ny - (int)llround(RR / a.dy);
            double phi = 1000.0;
            if (i >= ixmin && i <= ixmax) {
                const double m = fmin(phi, fmin(fabs(y - R1), fabs(y - (a.yl - R1))));
                phi = ((j <= (int)llround(R1 / a.dy)) || (j >= a.ny - 1 - (int)llround(R1 / a.dy))) ? -m : +m;
            }
            if (j >= iymin && j <= iymax) {
                const double m = fmin(phi, fmin(fabs(x - R1), fabs(x - (a.xl - R1))));
                phi = ((i <= (int)llround(R1 / a.dx)) || (i >= a.nx - 1 - (int)llround(R1 / a.dx))) ? -m : +m;
            }
            auto corner = [&](int x0_, int x1_, int y0_, int y1_, double cx, double cy) {
                if (i >= x0_ && i <= x1_ && j >= y0_ && j <= y1_)
                    phi = fmin(phi, -(sqrt((x - cx) * (x - cx) + (y - cy) * (y - cy)) - R2));
            };
            corner(0, ixmin, 0, iymin, RR, RR);
            corner(0, ixmin, iymax, a.ny - 1, RR, a.yl - RR);
            corner(ixmax, a.nx - 1, iymax, a.ny - 1, a.xl - RR, a.yl - RR);
            corner(ixmax, a.nx - 1, 0, iymin, a.xl - RR, RR);
            a.frame[cell] = smooth_step2(phi, th / 2., th / 2., a.pi);
        }
    }
}

// The vorticity sponge (create_sponge_mask, create_mask.f90:223-364) after the start-up mask:
// iSponge 1 (outflow), 2 (inflow, reduced inside the obstacle), 3 (around the domain), 22 (a
// frame with a hole, zero on the obstacle); divided by eps_sponge.
template <typename Rt>
__global__ void k_sponge_mask(StaticMaskArgs a, double gerf) {
    const size_t n = (size_t)a.nx * a.ny;
    Rt* out = reinterpret_cast<Rt*>(a.spg);
    const Rt* mk = reinterpret_cast<const Rt*>(a.mask);
    const double dx = a.dx, dy = a.dy, N = a.N, sss = a.SpongeSize, xl = a.xl, yl = a.yl;
    for (size_t cell = blockIdx.x * (size_t)blockDim.x + threadIdx.x; cell < n; cell += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(cell % a.nx), j = (int)(cell / a.nx);
        double v = 0.0;
        if (a.iSponge == 1) {
            const double ss = sss - 2.0 * N * dx;
            const int l0 = (int)llround((xl - sss) / dx), l1 = (int)llround((xl - 0.5 * sss) / dx);
            if (i >= l0 && i <= l1) v = smooth_step_div(xl - 0.5 * sss - (double)i * dx, ss * 0.5, N * dx, a.sharp, gerf);
            if (i >= l1) v = smooth_step_div((double)i * dx - xl + 0.5 * sss - 1.0 * dx, ss * 0.4, N * dx, a.sharp, gerf);
        } else if (a.iSponge == 2) {
            const double ss = sss - 2.0 * N * dx;
            const int l1 = (int)llround((0.5 * sss) / dx), r1 = (int)llround((1.0 * sss) / dx);
            if (i <= l1) v = smooth_step_div(0.5 * sss - (double)i * dx, ss * 0.5, N * dx, a.sharp, gerf);
            if (i >= l1 && i <= r1) v = smooth_step_div((double)i * dx - 0.5 * sss, ss * 0.5, N * dx, a.sharp, gerf);
            if (i <= r1) {
                const double me = (double)mk[cell] * a.eps;
                if (me > 0.0) v = v * (1.0 - me);
            }
        } else if (a.iSponge == 3) {
            const double ss = sss - N * dx;
            const double t1 = smooth_step_div((double)i * dx, ss, N * dx, a.sharp, gerf);
            const double t2 = smooth_step_div(xl - (double)i * dx, ss, N * dx, a.sharp, gerf);
            const double t3 = smooth_step_div((double)j * dy, ss, N * dy, a.sharp, gerf);
            const double t4 = smooth_step_div(yl - (double)j * dy, ss, N * dy, a.sharp, gerf);
            v = fmin(t1 + t2 + t3 + t4, 1.0);
        } else if (a.iSponge == 22) {
            const int x0 = (int)llround(sss / dx), y0 = (int)llround(sss / dy);
            const int x1 = (int)llround((xl - sss) / dx), y1 = (int)llround((yl - sss) / dy);
            const bool hole = i >= x0 && i <= x1 && j >= y0 && j <= y1;
            v = (hole || mk[cell] > (Rt)0) ? 0.0 : 1.0;
        }
        out[cell] = (Rt)(v / a.eps_sponge);
    }
}

void launch_static_masks(const StaticMaskArgs& a, double gerf, cudaStream_t st) {
    k_static_masks<<<1024, 256, 0, st>>>(a, gerf);
}
void launch_sponge_mask(const StaticMaskArgs& a, double gerf, cudaStream_t st) {
    if (a.fp32) k_sponge_mask<float><<<1024, 256, 0, st>>>(a, gerf);
    else k_sponge_mask<double><<<1024, 256, 0, st>>>(a, gerf);
}

void launch_mask(const MaskArgs& a, double gerf, bool fp32, cudaStream_t st, bool pdl) {
    // four-warp blocks, two per SM: a tile's primitives over the four SMSPs of an SM
    const int blocks = 2 * a.nsm;
    if (fp32) launch_k(k_mask_raster<float>, dim3(blocks), dim3(32 * MASK_WARPS), 0, st, pdl, a, gerf);
    else launch_k(k_mask_raster<double>, dim3(blocks), dim3(32 * MASK_WARPS), 0, st, pdl, a, gerf);
}

// BeamSurfaceIntegral (BeamForces.f90:306-509)
// ===================================================================================
// phi4* interpolation of one field at (xt, yt) on the box (0,0)-(xl-dx, yl-dy)
// (Interpolation.f90:6-48); false when the 9 x 9 stencil leaves the field.
__device__ bool surf_interp(const ForceArgs& a, const void* f, double xt, double yt, double dxi, double dyi,
                            double& out) {
    const double x2 = a.xl - a.dx, y2 = a.yl - a.dy;
    const int i = (int)div_cr(xt, dxi, a.rdxi), j = (int)div_cr(yt, dyi, a.rdyi);
    if (xt > x2 || xt < 0.0 || yt > y2 || yt < 0.0 || i - 4 < 0 || j - 4 < 0 || i + 4 > a.nx - 1 || j + 4 > a.ny - 1)
        return false;
    double dlx[9], r = 0.0;
    for (int d = 0; d < 9; ++d) dlx[d] = delta_phi4star(fabs((double)(i - 4 + d) * dxi - xt), dxi, a.rdxi, a.pi);
    for (int e = 0; e < 9; ++e) {
        const double dly = delta_phi4star(fabs((double)(j - 4 + e) * dyi - yt), dyi, a.rdyi, a.pi);
        const size_t row = (size_t)(j - 4 + e) * a.nx + (i - 4);
        for (int d = 0; d < 9; ++d) r += dlx[d] * dly * fld(f, a.fp32, row + d);
    }
    out = r;
    return true;
}

// The penalization drag / lift sums over the grid, one partial pair per block:
// sum mask (u - maskvx), sum mask (v - maskvy) (:483-486).  The FP32 form stores u - U.
__global__ void __launch_bounds__(256) k_surface_fields(SurfArgs s) {
    const size_t NN = (size_t)s.nx * s.ny;
    const double Uc = s.fp32 ? s.mean[0] : 0.0, Vc = s.fp32 ? s.mean[1] : 0.0;
    double d = 0.0, l = 0.0;
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < NN; k += (size_t)gridDim.x * blockDim.x) {
        const double m = fld(s.mask, s.fp32, k);
        d += m * ((fld(s.u, s.fp32, k) + Uc) - fld(s.mvx, s.fp32, k));
        l += m * ((fld(s.v, s.fp32, k) + Vc) - fld(s.mvy, s.fp32, k));
    }
    __shared__ double sm[2][8];
    for (int o = 16; o > 0; o >>= 1) { d += __shfl_xor_sync(0xffffffffu, d, o); l += __shfl_xor_sync(0xffffffffu, l, o); }
    if ((threadIdx.x & 31) == 0) { sm[0][threadIdx.x >> 5] = d; sm[1][threadIdx.x >> 5] = l; }
    __syncthreads();
    if (threadIdx.x < 2) {
        double t = 0.0;
        for (int w = 0; w < 8; ++w) t += sm[threadIdx.x][w];
        s.part[2 * blockIdx.x + threadIdx.x] = t;
    }
}

// The contour: two half circles of nc points at the ends (:341-420), the top and bottom lines
// (:426-480), a point a thread; six force sums reduced over the block; out[11] as the
// 'surface' file's columns.  One block of 256 threads.
__global__ void __launch_bounds__(256) k_surface_integral(ForceArgs a, SurfArgs s, double dxi, double dyi, double time) {
    const int nc = 128, ns = a.ns, npts = 2 * nc + 2 * ns;
    const double pi = a.pi;
    const double R = a.t_beam + a.N_smooth * fmax(a.dx, a.dy);
    const double dphi = pi / (double)(nc - 1), dL = dphi * R;
    const double alpha = motion_at(a.mo, time).alpha;  // mouvement(time) (BeamForces.f90:344)
    double F[6] = {0, 0, 0, 0, 0, 0};  // Ft(1), Fn(1), Fp(1), Ft(2), Fn(2), Fp(2)
    bool ok = true;
    for (int p = threadIdx.x; p < npts; p += blockDim.x) {
        double A = 0.0, B = 0.0, P = 0.0;
        if (p < 2 * nc) {
            const int end = p / nc, i = p % nc, node = end == 0 ? ns - 1 : 0;
            const double beta = a.th[end == 0 ? ns - 1 : 1] + alpha;
            const double phi = (end == 0 ? -(0.5 * pi - beta) : (0.5 * pi + beta)) + (double)i * dphi;
            double sp_, cp_, s2, c2;
            sincos(phi, &sp_, &cp_);
            sincos(2.0 * phi, &s2, &c2);
            const double xc = a.x[node] + R * cp_, yc = a.y[node] + R * sp_;
            ok &= surf_interp(a, a.sa, xc, yc, dxi, dyi, A);
            ok &= surf_interp(a, a.sb, xc, yc, dxi, dyi, B);
            ok &= surf_interp(a, a.press, xc, yc, dxi, dyi, P);
            const double sn = +A * c2 + B * s2, st = -A * s2 + B * c2, sp = -P;
            F[0] += dL * st * (-sp_); F[3] += dL * st * (+cp_);
            F[1] += dL * sn * (+cp_); F[4] += dL * sn * (+sp_);
            F[2] += dL * sp * (+cp_); F[5] += dL * sp * (+sp_);
        } else {
            const int q = p - 2 * nc, i = q % ns;
            const double sg = q < ns ? 1.0 : -1.0;
            const double th = a.th[i] + alpha;
            double sn_, cs_, s2, c2;
            sincos(th, &sn_, &cs_);
            sincos(2.0 * th, &s2, &c2);
            const double x = a.x[i] - sg * R * sn_, y = a.y[i] + sg * R * cs_;
            const double x1 = a.x[i] - sg * a.t_beam * sn_, y1 = a.y[i] + sg * a.t_beam * cs_;
            ok &= surf_interp(a, a.sa, x, y, dxi, dyi, A);
            ok &= surf_interp(a, a.sb, x, y, dxi, dyi, B);
            ok &= surf_interp(a, a.press, x1, y1, dxi, dyi, P);
            const double sn = -A * c2 - B * s2, st = -A * s2 + B * c2, sp = -P;
            F[0] += a.ds * st * (sg * cs_); F[3] += a.ds * st * (sg * sn_);
            F[1] += a.ds * sn * (-sg * sn_); F[4] += a.ds * sn * (sg * cs_);
            F[2] += a.ds * sp * (-sg * sn_); F[5] += a.ds * sp * (sg * cs_);
        }
    }
    if (!ok) set_status(a.S, FSIBE_ERR_INTERP_OOB);
    __shared__ double sm[8][8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int k = 0; k < 6; ++k) {
        double v = F[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) sm[k][warp] = v;
    }
    // the grid sums of k_surface_fields, one warp each
    if (warp < 2) {
        double v = 0.0;
        for (int b = lane; b < s.nblk; b += 32) v += s.part[2 * b + warp];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) sm[6 + warp][0] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t[6];
        for (int k = 0; k < 6; ++k) {
            t[k] = 0.0;
            for (int w = 0; w < 8; ++w) t[k] += sm[k][w];
        }
        double* o = s.out;
        o[0] = time;
        o[1] = sm[6][0] * a.dx * a.dy;
        o[2] = sm[7][0] * a.dx * a.dy;
        o[3] = t[0] + t[1] + t[2];
        o[4] = t[3] + t[4] + t[5];
        for (int k = 0; k < 6; ++k) o[5 + k] = t[k];
    }
}

void launch_surface_integral(const ForceArgs& a, const SurfArgs& s, double dxi, double dyi, double time, cudaStream_t st) {
    k_surface_fields<<<s.nblk, 256, 0, st>>>(s);
    k_surface_integral<<<1, 256, 0, st>>>(a, s, dxi, dyi, time);
}

void launch_forces_geo(const ForceArgs& a, double dxi, double dyi, cudaStream_t st) {
    k_forces_geo<<<a.ns, 128, 0, st>>>(a, dxi, dyi);
}
void launch_forces(const ForceArgs& a, double dxi, double dyi, cudaStream_t st, bool pdl) {
    launch_k(k_forces, dim3(a.ns), dim3(128), 0, st, pdl, a, dxi, dyi);
}

}  // namespace fsibe
