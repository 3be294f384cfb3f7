// api.cu -- the C ABI of include/fsibe.h: run context, step orchestration, state transfer.
//
// One fsibe_ctx holds every field of one run in HBM and a CUDA stream.  A step is a fixed
// sequence of kernel launches whose time-dependent inputs (time, dt, AB2 weights, drag
// window, status) live in a device struct, so a step needs no host round trip and can be
// captured once in a CUDA graph and replayed.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "adjoint.cuh"
#include "fluid.cuh"
#include "solid.cuh"

namespace fsibe {
void fill_sizes_32(SizeKernels<double>&, SizeKernels<float>&);
void fill_sizes_64(SizeKernels<double>&, SizeKernels<float>&);
void fill_sizes_128(SizeKernels<double>&, SizeKernels<float>&);
void fill_sizes_256(SizeKernels<double>&, SizeKernels<float>&);
void fill_sizes_512(SizeKernels<double>&, SizeKernels<float>&);
void fill_sizes_1024(SizeKernels<double>&, SizeKernels<float>&);
void fill_sizes_2048(SizeKernels<double>&, SizeKernels<float>&);
void fill_sizes_4096(SizeKernels<double>&, SizeKernels<float>&);
size_t beam_ws_doubles(int ns);
void launch_mask_prep(const MaskArgs& a, double gerf, cudaStream_t st, bool pdl);
void launch_mask(const MaskArgs& a, double gerf, bool fp32, cudaStream_t st, bool pdl);
void launch_forces(const ForceArgs& a, double dxi, double dyi, cudaStream_t st, bool pdl);
void launch_static_masks(const StaticMaskArgs& a, double gerf, cudaStream_t st);
void launch_sponge_mask(const StaticMaskArgs& a, double gerf, cudaStream_t st);
void launch_forces_geo(const ForceArgs& a, double dxi, double dyi, cudaStream_t st);
void launch_surface_integral(const ForceArgs& a, const SurfArgs& s, double dxi, double dyi, double time, cudaStream_t st);
void launch_beam(const BeamArgs& b, cudaStream_t st);
void launch_beam_pre(const BeamArgs& b, cudaStream_t st);
int beam_pre_smem_setup(int ns);
size_t beam_pred_doubles(int ns);
void beam_d1d_table(double ds, double* out);
void launch_init_beam(const BeamArgs& b, cudaStream_t st);
void launch_move_beam(const BeamArgs& b, cudaStream_t st);
int beam_smem_setup(int ns);
int beam_cluster_setup(int ns, int want, size_t* smem_out, int* big_out);
cudaError_t launch_running_sums(const double* src, double* dst, int n, int* nserial, cudaStream_t st);
size_t beam_cluster_fact_floats(int ns, int R);
void launch_beam_cluster(const BeamArgs& b, int R, size_t smem, cudaStream_t st, bool pdl);
size_t beam_cluster_minv_floats(int ns, int R);

static bool get_sizes(int N, SizeKernels<double>& d, SizeKernels<float>& f) {
    switch (N) {
        case 32: fill_sizes_32(d, f); return true;
        case 64: fill_sizes_64(d, f); return true;
        case 128: fill_sizes_128(d, f); return true;
        case 256: fill_sizes_256(d, f); return true;
        case 512: fill_sizes_512(d, f); return true;
        case 1024: fill_sizes_1024(d, f); return true;
        case 2048: fill_sizes_2048(d, f); return true;
        case 4096: fill_sizes_4096(d, f); return true;
        default: return false;
    }
}

// ---------------------------------------------------------------------------------
// Scalar kernels of the step
// ---------------------------------------------------------------------------------
struct StepArgs {
    DevScalars* S;
    const double* red;
    int nblk, explicit_step, iBeam, iMeanVelocity, ns, nx, ny;
    double cfl, dx, dy, eps, dt_fixed, time_end, theta_inf, T_fullspeed, U_mean_true, pi, nu;
    double x0, y0, t_beam, NN, scalex, scaley;
    double cos_ti, sin_ti;  // cos and sin of theta_inf, from the host
    MotionArgs mo;          // the leading edge's motion (the drag window follows it)
    double rdx, rdy, rNN;   // RN(1/dx), RN(1/dy), RN(1/NN)
    const double *bx, *by;
    double* etab;
    float2* etabf;
    int hx;
    double soff, rdyi;      // the stress points' offset from the beam; 1 / interpolation spacing
    int walls_or_cyl;       // walls or a cylinder clamp the step like a beam (NavierStokes.f90:71)
    double r_cyl;           // R_cylinder in the drag window (NavierStokes.f90:538-545)
    int wall_row0, wall_row1;  // iWalls: the window's rows stay within [row0, row1] (:546-552)
};

__device__ double mean_ux(int mode, double time, double cos_ti, double Tf, double pi) {  // mean_velocity.f90:4-42
    double tf;
    switch (mode) {
        case 1:
            tf = (time < Tf) ? (time * time * time) / (-0.5 * Tf * Tf * Tf) + 3.0 * (time * time) / (Tf * Tf) : 1.0;
            return cos_ti * tf;
        case 2:
            tf = (time < Tf) ? 0.5 * (1.0 - cos(0.5 * pi * time / Tf)) : 1.0;
            return cos_ti * tf;
        case 3: return cos_ti;
        case 6: return time;
        case 22: return 0.1;
        default: return 0.0;
    }
}
__device__ double mean_uy(int mode, double time, double sin_ti, double Tf, double pi) {  // mean_velocity.f90:46-84
    double tf;
    switch (mode) {
        case 1:
            tf = (time < Tf) ? (time * time * time) / (-0.5 * Tf * Tf * Tf) + 3.0 * (time * time) / (Tf * Tf) : 1.0;
            return sin_ti * tf;
        case 2:
            tf = (time < Tf) ? 0.5 * (1.0 - cos(0.5 * pi * time / Tf)) : 1.0;
            return sin_ti * tf;
        case 3: return sin_ti;
        default: return 0.0;
    }
}

// Start of a fluid step: the CFL/penalization/fixed dt of cal_nlk (NavierStokes.f90:59-78)
// from the velocity statistics of the previous step, the AB2 weights (:488-489), the mean
// flow at time+dt1 and the drag window of cal_drag (:539-564).
__global__ void __launch_bounds__(256) k_step_begin(StepArgs a) {
    // one warp per statistic (FP64 adds and compares are slow here: each warp reduces its own
    // quantity with shuffles): 0 max |u|^2, 1 sum u, 2 sum v, 3 min x, 4 max x, 5 min y, 6 max y
    __shared__ double q[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nblk = ((volatile DevScalars*)a.S)->nred;  // partials of the last x-pass kernel
    if (warp < 3) {
        const int slot = (warp == 0) ? RED_UMAX2 : (warp == 1 ? RED_SUM_U : RED_SUM_V);
        double v = 0.0;
        for (int b = lane; b < nblk; b += 32) {
            const double r = a.red[(size_t)b * RED_NSLOTS + slot];
            v = (warp == 0) ? fmax(v, r) : v + r;
        }
        for (int o = 16; o > 0; o >>= 1) {
            const double t = __shfl_xor_sync(0xffffffffu, v, o);
            v = (warp == 0) ? fmax(v, t) : v + t;
        }
        if (lane == 0) q[warp] = v;
    } else if (warp < 7) {
        const int w = warp - 3;
        const double* src = (w < 2) ? a.bx : a.by;
        const bool mx = (w & 1) != 0;
        double v = mx ? -1e300 : 1e300;
        for (int i = lane; i < a.ns; i += 32) v = mx ? fmax(v, src[i]) : fmin(v, src[i]);
        for (int o = 16; o > 0; o >>= 1) {
            const double t = __shfl_xor_sync(0xffffffffu, v, o);
            v = mx ? fmax(v, t) : fmin(v, t);
        }
        if (lane == 0) q[warp] = v;
    }
    __syncthreads();
    const double smax = q[0], su = q[1], sv = q[2];
    const double bminx = q[3], bmaxx = q[4], bminy = q[5], bmaxy = q[6];
    DevScalars* S = a.S;
    __shared__ double dts[2];
    // the scalars, each chain on its own warp (SMSP): dt1 (warp 0), the mean velocities
    // (warps 1, 2), the drag window (warps 3, 4); the quotients by constants use their host
    // reciprocals (div_cr: the correctly rounded quotient, like the division)
    if (threadIdx.x == 0) {
        const double time = S->time;
        const double dt0 = a.explicit_step ? S->dt0 : S->dt1;
        const double u_max = sqrt(smax);
        double dt1 = a.cfl * fmin(a.dx, a.dy) / u_max;
        if (u_max < 1.e-10) dt1 = 1.e-2;
        if (a.iBeam > 0 || a.walls_or_cyl) dt1 = fmin(0.9 * a.eps, dt1);
        if (a.dt_fixed > 0.0) dt1 = fmin(a.dt_fixed, dt1);
        if ((a.time_end - time) < dt1) dt1 = a.time_end - time;
        if (!a.explicit_step) S->dt0 = dt0;
        S->dt1 = dt1;
        S->u_max = u_max;
        S->umax2 = smax;
        S->explicit_step = a.explicit_step;
        dts[0] = dt1;
        dts[1] = dt0;
    } else if (threadIdx.x == 32) {
        S->mean_ux = div_cr(su, a.NN, a.rNN);
    } else if (threadIdx.x == 64) {
        S->mean_uy = div_cr(sv, a.NN, a.rNN);
    } else if (threadIdx.x == 96 || threadIdx.x == 128) {
        const double r_cyl = a.r_cyl, tb = a.t_beam;
        const Motion mo = motion_at(a.mo, S->time);  // LeadingEdge (NavierStokes.f90:532)
        if (threadIdx.x == 96) {
            int ixmin = 0, ixmax = a.nx - 1;
            if (a.iBeam > 0) {
                ixmin = (int)div_cr(fmin((mo.le[0] - fmax(2.5 * r_cyl, 1.5 * tb)), (bminx - 1.5 * tb)), a.dx, a.rdx);
                ixmax = (int)div_cr((bmaxx + 1.5 * tb), a.dx, a.rdx);
                if (ixmin < 0) ixmin = 0;
                if (ixmax > a.nx - 1) ixmax = a.nx - 1;
            }
            S->win[0] = ixmin; S->win[1] = ixmax;
        } else {
            int iymin = 0, iymax = a.ny - 1;
            if (a.iBeam > 0) {
                iymax = (int)div_cr((fmax(bmaxy + 1.5 * tb, mo.le[1] + 2.0 * r_cyl)), a.dy, a.rdy);
                iymin = (int)div_cr((fmin(bminy - 1.5 * tb, mo.le[1] - 2.0 * r_cyl)), a.dy, a.rdy);
                if (iymin < 0) iymin = 0;
                if (iymax > a.ny - 1) iymax = a.ny - 1;
                // the rows of the cells j of the forces' stress points (within soff of the
                // beam's y range, BeamForces.f90:105-124) and their 9 x 9 stencils, with two rows
                // of margin for the rounding of the cell index: k_stress_x leaves the others
                const double j0 = floor((bminy - a.soff) * a.rdyi) - 6.0, j1 = floor((bmaxy + a.soff) * a.rdyi) + 6.0;
                S->srow[0] = (int)fmax(j0, -1.0);
                S->srow[1] = (int)fmin(j1, (double)a.ny);
            } else {
                S->srow[0] = 0; S->srow[1] = a.ny - 1;
            }
            if (a.wall_row1 >= 0) {
                if (iymin < a.wall_row0) iymin = a.wall_row0;
                if (iymax > a.wall_row1) iymax = a.wall_row1;
            }
            S->win[2] = iymin; S->win[3] = iymax;
        }
    }
    __syncthreads();
    // after dt1: the AB2 weights (warps 0, 1) and the mean flow at time + dt1 (warps 2, 3)
    {
        const double dt1 = dts[0], dt0 = dts[1];
        if (threadIdx.x == 0) S->b10 = a.explicit_step ? dt1 : dt1 / dt0 * (0.5 * dt1 + dt0);
        else if (threadIdx.x == 32) S->b11 = a.explicit_step ? 0.0 : -0.5 * (dt1 * dt1) / dt0;
        else if (threadIdx.x == 64)
            S->mean_u_next = a.U_mean_true * mean_ux(a.iMeanVelocity, S->time + dt1, a.cos_ti, a.T_fullspeed, a.pi);
        else if (threadIdx.x == 96)
            S->mean_v_next = a.U_mean_true * mean_uy(a.iMeanVelocity, S->time + dt1, a.sin_ti, a.T_fullspeed, a.pi);
    }
    __syncthreads();
    // integrating factor exp(-nu dt |k|^2) = exp(coefx kx^2) exp(coefy ky^2) (cal_vis.f90:183-189),
    // one table per direction, FP64 and split FP32 hi + lo
    // (rebuilt only when dt changed: the tables of the same coefficients are already in place)
    const double dt1 = ((volatile DevScalars*)S)->dt1;
    const double coefx = -dt1 * a.nu * a.scalex, coefy = -dt1 * a.nu * a.scaley;
    const volatile DevScalars* VS = S;
    if (VS->etab_valid && VS->etab_cx == coefx && VS->etab_cy == coefy) return;
    const int ntab = a.hx + a.ny / 2 + 1;
    for (int i = threadIdx.x; i < ntab; i += blockDim.x) {
        const double e = (i < a.hx) ? exp(coefx * (double)(i * i)) : exp(coefy * (double)((i - a.hx) * (i - a.hx)));
        a.etab[i] = e;
        const float h = (float)e;
        a.etabf[i] = make_float2(h, (float)(e - (double)h));
    }
    __syncthreads();
    if (threadIdx.x == 0) { S->etab_cx = coefx; S->etab_cy = coefy; S->etab_valid = 1; }
}

// End of the fluid part: cal_energy (NavierStokes.f90:222-263) and cal_drag (:566-589)
// from the per-block partial sums, summed in a fixed order.
__global__ void __launch_bounds__(256) k_fluid_finish(StepArgs a) {
    // one warp per slot group: warp w reduces slots w and w + 8 with shuffles
    __shared__ double sm[RED_NSLOTS][1];
    const int lane = threadIdx.x & 31;
    const int nblk = ((volatile DevScalars*)a.S)->nred;  // partials of the last x-pass kernel
    for (int s = threadIdx.x >> 5; s < RED_NSLOTS; s += blockDim.x >> 5) {
        double v = 0.0;
        for (int b = lane; b < nblk; b += 32) {
            const double r = a.red[(size_t)b * RED_NSLOTS + s];
            v = (s == RED_UMAX2) ? fmax(v, r) : v + r;
        }
        for (int o = 16; o > 0; o >>= 1) {
            const double t = __shfl_xor_sync(0xffffffffu, v, o);
            v = (s == RED_UMAX2) ? fmax(v, t) : v + t;
        }
        if (lane == 0) sm[s][0] = v;
    }
    DevScalars* S = a.S;
    const int ready = ((volatile DevScalars*)S)->unst_ready;
    __syncthreads();
    // the scalars on three warps (SMSPs): energies (warp 0), drag (warp 1), lift (warp 2)
    const double dx = a.dx, dy = a.dy, norm = dx * dy;
    if (threadIdx.x == 0) {
        S->mean_u_cur = S->mean_u_next;
        S->mean_v_cur = S->mean_v_next;
        S->vor_rms = dx * dy * sqrt(sm[RED_OMEGA2][0]);
        S->kinetic = 0.5 * dx * dy * sm[RED_KIN][0];
        S->dissipation = a.nu * dx * dy * sm[RED_OMEGA2][0];
        S->porous_diss = dx * dy * sm[RED_POROUS][0];
        S->inflow_solid = dx * dy * sm[RED_INFLOW_SOLID][0];
        S->inflow_mean = dx * dy * a.U_mean_true * sm[RED_INFLOW_MEAN][0];
    } else if (a.iBeam > 0 && (threadIdx.x == 32 || threadIdx.x == 64)) {
        const int c = (threadIdx.x == 32) ? 0 : 1;
        S->force[c] = sm[c == 0 ? RED_DRAG_X : RED_DRAG_Y][0] * norm;
        const double dn = sm[c == 0 ? RED_UNST_X : RED_UNST_Y][0] * norm * a.eps;
        double* old = (c == 0) ? &S->drag_unst_old : &S->lift_unst_old;
        S->force_unst[c] = ready ? (dn - *old) / S->dt1 : 0.0;
        *old = dn;
    }
    __syncthreads();
    if (threadIdx.x == 0 && a.iBeam > 0) S->unst_ready = 1;
}

// time_step.f90:152-161 / :222-236 (advance_state in solid.cuh) as its own kernel.
__global__ void __launch_bounds__(256) k_advance(AdvArgs a) { advance_state(a); }

// ---- the packed Temperton layout (ABI boundary only) ---------------------------------
// unpack: fk (Fortran (0:nx-1,0:ny-1)) -> S[kx][ky]   (cof_fftw33.f90:214-233)
template <typename R>
__device__ __forceinline__ void put_split(C2<R>* hi, C2<R>* lo, size_t i, double re, double im) {
    const R h0 = (R)re, h1 = (R)im;
    hi[i] = mk<R>(h0, h1);
    if (lo) lo[i] = mk<R>((R)(re - (double)h0), (R)(im - (double)h1));
}
template <typename R>
__global__ void k_unpack(const double* fk, C2<R>* H, C2<R>* Hlo, int nx, int ny) {
    const int kx = blockIdx.x;
    const size_t r0 = (size_t)kx * ny;
    for (int l = threadIdx.x; l <= ny / 2; l += blockDim.x) {
        if (l == 0) {
            put_split<R>(H, Hlo, r0, fk[2 * kx], fk[2 * kx + 1]);
        } else if (l == ny / 2) {
            put_split<R>(H, Hlo, r0 + ny / 2, 0.0, 0.0);
        } else {
            const double a = fk[(size_t)(2 * l) * nx + 2 * kx], b = fk[(size_t)(2 * l + 1) * nx + 2 * kx];
            const double c = fk[(size_t)(2 * l) * nx + 2 * kx + 1], d = fk[(size_t)(2 * l + 1) * nx + 2 * kx + 1];
            put_split<R>(H, Hlo, r0 + l, a - d, b + c);
            put_split<R>(H, Hlo, r0 + ny - l, a + d, -b + c);
        }
    }
}
// pack: S[kx][ky] -> fk   (cof_fftw33.f90:168-190)
template <typename R>
__device__ __forceinline__ double2 get_sum(const C2<R>* hi, const C2<R>* lo, size_t i) {
    const C2<R> h = hi[i];
    double2 r = make_double2((double)h.x, (double)h.y);
    if (lo) { const C2<R> l = lo[i]; r.x += (double)l.x; r.y += (double)l.y; }
    return r;
}
template <typename R>
__global__ void k_pack(const C2<R>* H, const C2<R>* Hlo, double* fk, int nx, int ny) {
    const int kx = blockIdx.x;
    const size_t r0 = (size_t)kx * ny;
    for (int l = threadIdx.x; l < ny / 2; l += blockDim.x) {
        if (l == 0) {
            const double2 z = get_sum<R>(H, Hlo, r0);
            fk[2 * kx] = z.x;
            fk[2 * kx + 1] = z.y;
            fk[(size_t)nx + 2 * kx] = 0.0;
            fk[(size_t)nx + 2 * kx + 1] = 0.0;
        } else {
            const double2 p = get_sum<R>(H, Hlo, r0 + l), m = get_sum<R>(H, Hlo, r0 + ny - l);
            fk[(size_t)(2 * l) * nx + 2 * kx] = 0.5 * (p.x + m.x);
            fk[(size_t)(2 * l + 1) * nx + 2 * kx] = 0.5 * (p.y - m.y);
            fk[(size_t)(2 * l) * nx + 2 * kx + 1] = 0.5 * (p.y + m.y);
            fk[(size_t)(2 * l + 1) * nx + 2 * kx + 1] = 0.5 * (-p.x + m.x);
        }
    }
}

// Pointwise spectral operators directly on packed arrays (cofdx.f90, cofdy.f90, cofdxdx.f90,
// cofdydy.f90, cofdxdy.f90, poisson.f90, cal_vis.f90, dealiase_mask.f90).
enum PackedOp { PK_DX = 0, PK_DY, PK_DXDX, PK_DYDY, PK_DXDY, PK_POISSON, PK_VIS, PK_DEALIAS };
__global__ void k_packed_op(const double* in, double* out, int op, int nx, int ny, double xl, double yl, double pi,
                            double scalex, double scaley, double nu, double dt, int idealis) {
    const size_t N = (size_t)nx * ny;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N; e += (size_t)gridDim.x * blockDim.x) {
        const int kx = (int)(e % nx), ky = (int)(e / nx);
        auto IN = [&](int x, int y) { return in[(size_t)y * nx + x]; };
        double r = 0.0;
        switch (op) {
            case PK_DX: {
                const double s1 = 2.0 * pi / xl;
                r = ((kx & 1) == 0) ? -IN(kx + 1, ky) * (double)(kx / 2) * s1 : IN(kx - 1, ky) * (double)((kx - 1) / 2) * s1;
                break;
            }
            case PK_DY: {
                const double s1 = 2.0 * pi / yl;
                r = ((ky & 1) == 0) ? -IN(kx, ky + 1) * (double)(ky / 2) * s1 : IN(kx, ky - 1) * (double)((ky - 1) / 2) * s1;
                break;
            }
            case PK_DXDX: {
                const double t = 2.0 * pi / xl, k = (double)(kx / 2);
                r = -IN(kx, ky) * (k * k) * (t * t);
                break;
            }
            case PK_DYDY: {
                const double t = 2.0 * pi / yl, k = (double)(ky / 2);
                r = -IN(kx, ky) * (k * k) * (t * t);
                break;
            }
            case PK_DXDY: {
                const int a = kx / 2, b = ky / 2, ia = kx & 1, ib = ky & 1;
                const double fac = -(double)a * (double)b * ((2.0 * pi / xl) * (2.0 * pi / yl));
                if (!ia && !ib) r = fac * IN(2 * a + 1, 2 * b + 1);
                else if (ia && !ib) r = -fac * IN(2 * a, 2 * b + 1);
                else if (!ia && ib) r = -fac * IN(2 * a + 1, 2 * b);
                else r = fac * IN(2 * a, 2 * b);
                break;
            }
            case PK_POISSON: {
                const int a = kx / 2, b = ky / 2;
                if (a == 0 && b == 0) r = 0.0;
                else r = IN(kx, ky) / ((double)(a * a) * scalex + (double)(b * b) * scaley);
                break;
            }
            case PK_VIS: {
                const int a = kx / 2, b = ky / 2;
                const double coefx = -dt * nu * scalex, coefy = -dt * nu * scaley;
                r = exp(coefx * (double)(a * a) + coefy * (double)(b * b));
                break;
            }
            default: {
                const int a = kx / 2, b = ky / 2;
                const double kxt = 2.0 / 3.0 * (double)(nx / 2 - 1), kyt = 2.0 / 3.0 * (double)(ny / 2 - 1);
                r = 1.0;
                if (idealis == 1 && (double)a * (double)a / (kxt * kxt) + (double)b * (double)b / (kyt * kyt) >= 1.0) r = 0.0;
                break;
            }
        }
        out[e] = r;
    }
}

template <typename R>
__global__ void k_convert(const R* in, double* out, size_t n, const double* offset) {
    const double o = offset ? *offset : 0.0;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) out[e] = (double)in[e] + o;
}
template <typename R>
__global__ void k_convert_in(const double* in, R* out, size_t n, const double* offset) {
    const double o = offset ? *offset : 0.0;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) out[e] = (R)(in[e] - o);
}

}  // namespace fsibe

using namespace fsibe;

enum PhysIdx { PH_U = 0, PH_V, PH_MASK, PH_MVX, PH_MVY, PH_VORMEAN, PH_PRESS, PH_SA, PH_SB, PH_0, PH_N };
enum SpecIdx { SP_W = 0, SP_M, SP_WLO, SP_A, SP_B, SP_TU, SP_TV, SP_TW, SP_TSA, SP_TSB, SP_TDX, SP_TDY, SP_P1, SP_P2, SP_TQ, SP_0, SP_1, SP_N };
enum BeamIdx { B_X = 0, B_Y, B_VX, B_VY, B_TH, B_THD, B_AX, B_AY, B_PO, B_PN, B_TO, B_TN, B_N };

struct fsibe_ctx {
    fsibe_params P;
    Geometry g;
    bool fp32 = false;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    SizeKernels<double> kxd{}, kyd{};
    SizeKernels<float> kxf{}, kyf{};
    void* phys[PH_N] = {};
    void* spec[SP_N] = {};
    void *twX = nullptr, *twR = nullptr, *twY = nullptr;
    DevScalars* S = nullptr;
    double* red = nullptr;
    double* beam[B_N] = {};
    double* oo = nullptr;
    double* ws = nullptr;
    Prim* prims = nullptr;
    PrimG* primg = nullptr;       // the FP32 raster's per-primitive data (FP32 form)
    int *nprims = nullptr, *rect = nullptr;
    unsigned* counter = nullptr;
    double* fterm = nullptr;
    double* rows = nullptr;
    bool press_partial = false;  // the last fused step formed the pressure on the forces' rows only
    bool adv_ready = false;      // the next step's advection part ran (launched by the previous fused step)
    bool adv_pipe = false;       // fused steps launch the next step's advection part (from 2048^2)
    void* snap = nullptr;   // ComputePressureSnapshot's workspace (5 fields and 2 spectra of R), on first use
    int rows_cap = 0;
    double* etab = nullptr;       // integrating-factor tables (hx + ny/2 + 1)
    float2* etabf = nullptr;
    int* dcut = nullptr;          // dealiasing cut per kx
    float* kxw = nullptr;         // (float)(kx kxs), kx in [0, hx]: the FP32 kernels' wavenumbers
    int kcut = 0;                 // first kx whose row is entirely removed by the 2/3 rule
    double* dscratch = nullptr;   // 2*nx*ny doubles (ABI transfers, packed arrays)
    double* dscratch2 = nullptr;  // nx*ny doubles
    double gerf = 0.0;
    double U_mean_true = 1.0;
    // walls, cylinder and sponges: static fields, formed once (null when not used)
    bool full_mask = false;       // every cell of the mask is drawn each step
    double* bg = nullptr;         // walls + cylinder, unscaled
    double* frame = nullptr;      // iSponge = 22
    void* spg = nullptr;          // vorticity sponge / eps_sponge (R)
    void* s10 = nullptr;          // iSponge = 10: the integral term of the x penalization (R)
    void* s10_dudx = nullptr;     // and du/dx in physical space (R)
    int s10_ixmin = 0, s10_ixmax = -1;
    int* rect_full = nullptr;     // rows of the whole grid, for the penalization part of cal_nlk
    int beam_smem = 0;      // beam workspace parts in shared memory (bit mask, see k_beam)
    int beam_pre_smem = 0;  // the same for the predictor kernel
    int beam_cl = 0;        // CTAs of the cluster form of the beam kernel (0: the single-CTA form)
    int beam_cl_big = 0;    // its large-beam form (factor and M^-1 in global memory)
    float* clws = nullptr;  // the large-beam form's per-CTA factor copies
    size_t beam_cl_smem = 0;
    float* minv = nullptr;  // cluster form: rows of the preconditioner inverse, kept between steps
    int* minv_rse = nullptr;
    double* d1d = nullptr;  // Differentiate1D table of the beam (4 x 3 x 8)
    double* fgeo = nullptr;  // interpolation geometry of the forces, 76 doubles a node
    int* fgij = nullptr;     // its cells, 8 ints a node
    cudaEvent_t ev_geo = nullptr;
    cudaEvent_t ev_adv = nullptr;  // the advection part of k_nl_x, run beside the mask kernels
    bool nl_split = true;          // split k_nl_x in fsibe_step (FSIBE_NL_SPLIT=0: one launch)
    bool pdl = true;               // programmatic dependent launches on the main stream (FSIBE_PDL=0: off)
    bool stress_split = true;      // viscous stresses in k_stress_x beside k_press_x (FSIBE_STRESS_SPLIT=0: off)
    cudaEvent_t ev_ny = nullptr;   // k_nl_y done: k_stress_x may start
    double* pred = nullptr; // predictor output
    cudaStream_t side = nullptr;  // the beam predictor runs here beside the fluid step
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cudaStream_t side2 = nullptr;                     // the fluid step's scalar reductions run here
    cudaEvent_t ev_ff = nullptr, ev_ffj = nullptr, ev_sb0 = nullptr, ev_sb = nullptr;
    bool pre_launched = false;    // the predictor of the current step is in flight
    struct AdjWork* adj = nullptr;  // adjoint buffers and checkpoints (allocated on first use)
    bool initialized = false, startup_done = false;
    bool use_graph = false, graph_ready = false;
    cudaGraphExec_t gexec = nullptr;
    cudaGraph_t graph = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::string err;
    int launches = 0;
    int nsm = 152;                // SMs of the device
    int xv_nl = 1, xv_px = 1, xv_fin = 1;  // tile-height variants of the fused x kernels (1: default)
    int py_eng = 0;                        // k_press_y's transform engine (FP32: 0 paired, 1 one butterfly)
    // per-kernel event timing (fsibe_kernel_times)
    bool profiling = false;
    std::vector<cudaEvent_t> pool;
    size_t pool_used = 0;
    std::vector<std::pair<const char*, size_t>> prof;  // name, index of the start event
};

static void prof_begin(fsibe_ctx* c, const char* name, cudaStream_t st = nullptr) {
    if (!c->profiling) return;
    while (c->pool.size() < c->pool_used + 2) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        c->pool.push_back(e);
    }
    cudaEventRecord(c->pool[c->pool_used], st ? st : c->stream);
    c->prof.push_back({name, c->pool_used});
    c->pool_used += 2;
}
static void prof_end(fsibe_ctx* c, cudaStream_t st = nullptr) {
    if (!c->profiling) return;
    cudaEventRecord(c->pool[c->prof.back().second + 1], st ? st : c->stream);
}

static std::string g_err;

#define CK(ctx, call)                                                                   \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) {                                                        \
            (ctx)->err = std::string(#call) + ": " + cudaGetErrorString(e_);            \
            return FSIBE_ERR_CUDA;                                                      \
        }                                                                               \
    } while (0)

#define CKL(ctx)                                                                        \
    do {                                                                                \
        cudaError_t e_ = cudaGetLastError();                                            \
        if (e_ != cudaSuccess) {                                                        \
            (ctx)->err = std::string("kernel launch: ") + cudaGetErrorString(e_);       \
            return FSIBE_ERR_CUDA;                                                      \
        }                                                                               \
    } while (0)

static bool pow2_ok(int n) { return n >= 32 && n <= 4096 && (n & (n - 1)) == 0; }

template <typename T>
static void make_table(std::vector<T>& out, long n, long count) {
    const long double pi_l = 3.141592653589793238462643383279502884L;
    out.resize(count);
    for (long m = 0; m < count; ++m) {
        const long double a = 2.0L * pi_l * (long double)m / (long double)n;
        out[m].x = (decltype(out[m].x))cosl(a);
        out[m].y = (decltype(out[m].y))(-sinl(a));
    }
}

template <typename R>
static KArgs<R> kargs(fsibe_ctx* c) {
    KArgs<R> a;
    std::memset(&a, 0, sizeof(a));
    a.g = c->g;
    a.nu = c->P.nu;
    a.eps = c->P.eps;
    R** ph[] = {&a.u, &a.v, &a.mask, &a.mvx, &a.mvy, &a.vor_mean, &a.press, &a.sa, &a.sb, &a.phys0};
    for (int i = 0; i < PH_N; ++i) *ph[i] = reinterpret_cast<R*>(c->phys[i]);
    C2<R>** sp[] = {&a.W, &a.M, &a.Wlo, &a.A, &a.B, &a.Tu, &a.Tv, &a.Tw, &a.Tsa, &a.Tsb, &a.Tdx, &a.Tdy, &a.P1, &a.P2, &a.Tq, &a.spec0, &a.spec1};
    for (int i = 0; i < SP_N; ++i) *sp[i] = reinterpret_cast<C2<R>*>(c->spec[i]);
    a.twX = reinterpret_cast<const C2<R>*>(c->twX);
    a.twR = reinterpret_cast<const C2<R>*>(c->twR);
    a.twY = reinterpret_cast<const C2<R>*>(c->twY);
    a.S = c->S;
    a.red = c->red;
    a.etab = c->etab;
    a.etabf = c->etabf;
    a.dcut = c->dcut;
    a.kxw = c->kxw;
    a.kcut = c->kcut;
    a.spg = reinterpret_cast<const R*>(c->spg);
    a.s10 = reinterpret_cast<const R*>(c->s10);
    a.viscous = c->P.iViscous == 1;
    a.pressure_on = (c->P.iFLUSI == 1 || c->P.iSaveBeam > 0);
    a.penalize = c->P.iBeam > 0;
    a.op = OP_ID;
    return a;
}

template <typename R> static SizeKernels<R>& kx_of(fsibe_ctx* c);
template <> SizeKernels<double>& kx_of<double>(fsibe_ctx* c) { return c->kxd; }
template <> SizeKernels<float>& kx_of<float>(fsibe_ctx* c) { return c->kxf; }
template <typename R> static SizeKernels<R>& ky_of(fsibe_ctx* c);
template <> SizeKernels<double>& ky_of<double>(fsibe_ctx* c) { return c->kyd; }
template <> SizeKernels<float>& ky_of<float>(fsibe_ctx* c) { return c->kyf; }

// launch helpers (count launches for the bench's gpu_launches)
template <typename R>
static void launch_x(fsibe_ctx* c, void (*k)(KArgs<R>), int smem, const KArgs<R>& a, const char* name = "x_pass",
                     int nfields = 1) {
    const SizeKernels<R>& K = kx_of<R>(c);
    prof_begin(c, name);
    k<<<dim3(c->g.ny / K.x_rows, nfields), K.x_threads, smem, c->stream>>>(a);
    prof_end(c);
    c->launches++;
}
template <typename R>
// pdl: a programmatic dependent launch (only for kernels that begin with pdl_wait)
static void launch_y(fsibe_ctx* c, void (*k)(KArgs<R>), int smem, const KArgs<R>& a, const char* name = "y_pass",
                     int nfields = 1, bool pdl = false, int threads = 0) {
    const SizeKernels<R>& K = ky_of<R>(c);
    prof_begin(c, name);
    launch_k(k, dim3(c->g.hx, nfields), dim3(threads > 0 ? threads : K.y_threads), smem, c->stream, pdl && c->pdl, a);
    prof_end(c);
    c->launches++;
}

// a fused x kernel with one of its tile-height variants (nbuf row buffers of shared memory);
// on the main stream a programmatic dependent launch (the fused x kernels begin with pdl_wait)
template <typename R>
static void launch_xv(fsibe_ctx* c, void (*k)(KArgs<R>), const typename SizeKernels<R>::XVariant& v, int nbuf,
                      const KArgs<R>& a, const char* name, cudaStream_t st = nullptr, int grid = 0) {
    if (!st) st = c->stream;
    prof_begin(c, name, st);
    launch_k(k, dim3(grid > 0 ? grid : c->g.ny / v.rows), dim3(v.threads), nbuf == 3 ? v.smem3 : nbuf * v.smem1, st,
             c->pdl && st == c->stream, a);
    prof_end(c, st);
    c->launches++;
}

// The leading edge's motion (mouvement.f90:5-200): the case, its fixed position and angle (the
// angle's cosine and sine from the host), and the phase of the single beam (init_beam.f90:48).
static MotionArgs motion_args(const fsibe_ctx* c) {
    MotionArgs m;
    m.iMotion = c->P.iMotion;
    m.x0 = c->P.x0; m.y0 = c->P.y0;
    m.pi = c->g.pi;
    m.alpha0 = c->P.angle_beam * c->g.pi / 180.0;
    m.cos0 = std::cos(m.alpha0);
    m.sin0 = std::sin(m.alpha0);
    m.phase = 0.0;
    return m;
}

static StepArgs step_args(fsibe_ctx* c, int explicit_step, int nblk) {
    StepArgs a;
    std::memset(&a, 0, sizeof(a));
    a.S = c->S;
    a.red = c->red;
    a.nblk = nblk;
    a.explicit_step = explicit_step;
    a.iBeam = c->P.iBeam;
    a.iMeanVelocity = c->P.iMeanVelocity;
    a.ns = c->P.ns;
    a.nx = c->P.nx;
    a.ny = c->P.ny;
    a.cfl = c->P.cfl;
    a.dx = c->g.dx;
    a.dy = c->g.dy;
    a.eps = c->P.eps;
    a.dt_fixed = c->P.dt_fixed;
    a.time_end = c->P.time_end;
    a.theta_inf = c->P.theta_inf;
    a.T_fullspeed = c->P.T_fullspeed;
    a.U_mean_true = c->U_mean_true;
    a.pi = c->g.pi;
    a.nu = c->P.nu;
    a.x0 = c->P.x0;
    a.y0 = c->P.y0;
    a.mo = motion_args(c);
    a.t_beam = c->P.t_beam;
    a.NN = (double)c->P.nx * (double)c->P.ny;
    a.rdx = 1.0 / a.dx;
    a.rdy = 1.0 / a.dy;
    a.rNN = 1.0 / a.NN;
    a.bx = c->beam[B_X];
    a.by = c->beam[B_Y];
    a.scalex = c->g.scalex;
    a.scaley = c->g.scaley;
    a.cos_ti = std::cos(c->P.theta_inf);
    a.sin_ti = std::sin(c->P.theta_inf);
    a.etab = c->etab;
    a.etabf = c->etabf;
    a.hx = c->g.hx;
    a.soff = c->P.t_beam + c->P.N_smooth * std::fmax(c->g.dx, c->g.dy);
    a.rdyi = (double)(c->P.ny - 1) / (c->P.yl - c->g.dy);
    a.walls_or_cyl = (c->P.iWalls > 0 || c->P.iCylinder > 0) ? 1 : 0;
    a.r_cyl = c->P.R_cylinder;
    a.wall_row0 = 0; a.wall_row1 = -1;
    if (c->P.iWalls > 0) {
        const double h_star = c->P.h_channel + c->P.N_smooth * c->g.dy;
        a.wall_row0 = (int)std::lround(h_star / c->g.dy) + 2;
        a.wall_row1 = (int)std::lround((c->P.yl - h_star) / c->g.dy) - 2;
    }
    return a;
}

static BeamArgs beam_args(fsibe_ctx* c) {
    BeamArgs b;
    std::memset(&b, 0, sizeof(b));
    b.S = c->S;
    b.ns = c->P.ns; b.iImpulse = c->P.iImpulse; b.maxit = c->P.newton_maxit; b.iFLUSI = c->P.iFLUSI;
    b.ds = c->g.ds; b.eta = c->P.eta; b.mue = c->P.mue; b.sigma = c->P.sigma;
    b.t_release = c->P.t_release; b.tau = c->P.tau; b.tol = c->P.newton_tol; b.pi = c->g.pi;
    b.x0 = c->P.x0; b.y0 = c->P.y0; b.angle_deg = c->P.angle_beam;
    b.mo = motion_args(c);
    {
        const double ds = b.ds, eta = b.eta, ds2 = ds * ds, ds3 = ds * ds * ds, ds4 = (ds * ds) * (ds * ds);
        b.k.ids = 1.0 / ds;
        b.k.i2ds = 1.0 / (2.0 * ds);
        b.k.ids2 = 1.0 / ds2;
        b.k.i2ds2 = 1.0 / (2.0 * ds2);
        b.k.ids4 = 1.0 / ds4;
        b.k.e2ds3 = eta / (2.0 * ds3);
        b.k.eds4 = eta / ds4;
        b.k.e2ds4 = eta / (2.0 * ds4);
    }
    b.x = c->beam[B_X]; b.y = c->beam[B_Y]; b.vx = c->beam[B_VX]; b.vy = c->beam[B_VY];
    b.th = c->beam[B_TH]; b.thd = c->beam[B_THD]; b.ax = c->beam[B_AX]; b.ay = c->beam[B_AY];
    b.p_old = c->beam[B_PO]; b.p_new = c->beam[B_PN]; b.tau_old = c->beam[B_TO]; b.tau_new = c->beam[B_TN];
    b.oo = c->oo;
    b.ws = c->ws;
    b.use_smem = c->beam_smem;
    b.pred = c->pred;
    b.minv = c->minv;
    b.minv_rse = c->minv_rse;
    b.cl_big = c->beam_cl_big;
    b.clws = c->clws;
    b.d1d = c->d1d;
    return b;
}

// The beam predictor of the current step (k_beam_pre) on the side stream, forked from the
// main stream after the step's time step is known; solid_step joins it.
static int beam_predict(fsibe_ctx* c) {
    BeamArgs b = beam_args(c);
    b.use_smem = c->beam_pre_smem;
    CK(c, cudaEventRecord(c->ev_fork, c->stream));
    CK(c, cudaStreamWaitEvent(c->side, c->ev_fork, 0));
    prof_begin(c, "beam_pre", c->side);
    launch_beam_pre(b, c->side);
    prof_end(c, c->side);
    CKL(c);
    CK(c, cudaEventRecord(c->ev_join, c->side));
    c->launches++;
    c->pre_launched = true;
    return FSIBE_OK;
}



template <typename R>
static int x_blocks(fsibe_ctx* c) { return c->g.ny / kx_of<R>(c).x_rows; }

template <typename R>
static int sponge10_term(fsibe_ctx* c);  // the sharp outflow sponge's integral (below)

// The advection part of cal_nlk (NavierStokes.f90:88-132 without the penalization) on the
// second side stream, forked from the main stream at the start of the step: it reads the
// state the previous step left (u, v, the vorticity's derivatives) and no mask, so it runs
// beside the mask kernels.  fluid_step_t(adv_forked) joins it (ev_adv).
template <typename R>
static void nl_advect_t(fsibe_ctx* c, int explicit_step) {
    KArgs<R> a = kargs<R>(c);
    SizeKernels<R>& KX = kx_of<R>(c);
    a.explicit_step = explicit_step;
    // up to two tiles a SM: one block a SM, each taking tiles in turn (k_nl_x), so that the
    // mask raster launched after it finds room on every SM.  Beyond that the kernel is long
    // beside the raster, and a block a tile keeps more of it in flight (4096²: 281 µs against
    // 513 µs with one block a SM).
    // a run with the vorticity sponge takes the default tile, the one instantiated with it
    const auto& V = c->spg ? KX.xv[1] : KX.xv[c->xv_nl];
    const int tiles = c->g.ny / V.rows;
    launch_xv<R>(c, c->spg ? V.nl_adv_spg : V.nl_adv, V, 2, a, "nl_adv", c->side2,
                 tiles <= 2 * c->nsm ? (tiles < c->nsm ? tiles : c->nsm) : tiles);
}

// EvolveFluidExplicit / EvolveFluidAB2 + pressure (NavierStokes.f90:422-508, 273-403)
// stress_rows: the forces that follow use this beam state, so k_stress_x may leave the rows
// their stencils cannot reach
// adv_forked: the advection part of k_nl_x ran on the second side stream (ev_adv: this step's
// launch, joined here; or, with adv_prev, the previous step's launch, already ordered before
// this step).  adv_next: launch the next step's advection part on that stream after the
// fluid step's scalars, beside the pressure, the forces and the beam (the caller joins it).
template <typename R>
static int fluid_step_t(fsibe_ctx* c, int explicit_step, bool adv_forked = false, bool stress_rows = false,
                        bool adv_prev = false, bool adv_next = false) {
    KArgs<R> a = kargs<R>(c);
    SizeKernels<R>& KX = kx_of<R>(c);
    SizeKernels<R>& KY = ky_of<R>(c);
    const int nblk = x_blocks<R>(c);
    StepArgs sa = step_args(c, explicit_step, nblk);
    a.explicit_step = explicit_step;
    // the step's scalars (dt, AB2 weights, mean flow, drag window, integrating factor) on the
    // side stream beside nl_x, which reads none of them; the beam predictor follows them there
    CK(c, cudaEventRecord(c->ev_sb0, c->stream));
    CK(c, cudaStreamWaitEvent(c->side, c->ev_sb0, 0));
    prof_begin(c, "step_begin", c->side);
    k_step_begin<<<1, 256, 0, c->side>>>(sa);
    prof_end(c, c->side);
    CK(c, cudaEventRecord(c->ev_sb, c->side));
    c->launches++;
    if (c->P.iFLUSI == 1) { const int st = beam_predict(c); if (st) return st; }
    if (c->s10) { const int st = sponge10_term<R>(c); if (st) return st; }
    if (adv_forked) {
        // the advection part ran beside the mask kernels: add the penalization on the rows
        // of the mask's box
        if (!adv_prev) CK(c, cudaStreamWaitEvent(c->stream, c->ev_adv, 0));
        KArgs<R> p = a;
        // walls, sponges and the outflow sponge's integral: every row is penalized
        p.rect = (c->full_mask || c->s10) ? c->rect_full : c->rect;
        if (c->s10) launch_xv<R>(c, KX.xv[1].nl_pen_s10, KX.xv[1], 2, p, "nl_pen");
        else launch_xv<R>(c, KX.xv[c->xv_nl].nl_pen, KX.xv[c->xv_nl], 2, p, "nl_pen");
    } else if (c->spg) {
        launch_xv<R>(c, KX.xv[1].nl_x_spg, KX.xv[1], 3, a, "nl_x");  // the default tile carries the sponge
    } else if (c->s10) {
        launch_xv<R>(c, KX.xv[1].nl_x_s10, KX.xv[1], 3, a, "nl_x");
    } else {
        launch_xv<R>(c, KX.xv[c->xv_nl].nl_x, KX.xv[c->xv_nl], 3, a, "nl_x");
    }
    CK(c, cudaStreamWaitEvent(c->stream, c->ev_sb, 0));
    launch_y<R>(c, KY.nl_y, KY.y_smem_nl, a, "nl_y", 1, true);
    if (a.viscous && c->stress_split) {
        // the viscous stresses, read only by GetForces, on the second side stream beside the
        // pressure kernels (joined with ev_ffj below)
        CK(c, cudaEventRecord(c->ev_ny, c->stream));
        CK(c, cudaStreamWaitEvent(c->side2, c->ev_ny, 0));
        KArgs<R> s = a;
        s.srows = (stress_rows && c->P.iBeam > 0) ? 1 : 0;  // the row range k_step_begin formed
        const int vs = c->xv_px < 4 ? c->xv_px : 1;  // the paired press_x leaves the stresses to the default tile
        launch_xv<R>(c, KX.xv[vs].stress_x, KX.xv[vs], 2, s, "stress_x", c->side2);
        a.stress_split = 1;
    }
    if (c->xv_px == 4 && KX.xp.press_x && (a.stress_split || !a.viscous))
        launch_xv<R>(c, KX.xp.press_x, KX.xp, 3, a, "press_x");  // the paired FP32 kernel
    else {
        const int vp = c->xv_px < 4 ? c->xv_px : 1;
        launch_xv<R>(c, KX.xv[vp].press_x, KX.xv[vp], 3, a, "press_x");
    }
    // the energies, drag and unsteady forces from press_x's partial sums feed only scalars read
    // after the fluid step: a second side stream runs them beside the pressure transforms
    CK(c, cudaEventRecord(c->ev_ff, c->stream));
    CK(c, cudaStreamWaitEvent(c->side2, c->ev_ff, 0));
    prof_begin(c, "fluid_finish", c->side2);
    k_fluid_finish<<<1, 256, 0, c->side2>>>(sa);
    prof_end(c, c->side2);
    CK(c, cudaEventRecord(c->ev_ffj, c->side2));
    c->launches++;
    if (adv_next) {
        // the next step's advection part: it reads this step's new state (u, v from k_press_x,
        // the vorticity's derivatives from k_nl_y, the mean flow k_fluid_finish just stored) and
        // writes the spectra A, B, which k_nl_y has consumed
        nl_advect_t<R>(c, 0);
        CK(c, cudaEventRecord(c->ev_adv, c->side2));
    }
    if (a.pressure_on) {
        if (c->py_eng == 1 && KY.press_y1)  // the one-butterfly engine, where the autotuner found it faster
            launch_y<R>(c, KY.press_y1, KY.press_y1_smem, a, "press_y", 1, true, KY.y_threads);
        else
            launch_y<R>(c, KY.press_y, KY.y_smem2, a, "press_y", 1, true, KY.press_y_threads);
        KArgs<R> f = a;
        f.srows = (stress_rows && c->P.iBeam > 0) ? 1 : 0;  // the forces' rows only (k_press_fin)
        launch_xv<R>(c, KX.xv[c->xv_fin].press_fin, KX.xv[c->xv_fin], 1, f, "press_fin");
    } else {
        CK(c, cudaMemsetAsync(c->phys[PH_PRESS], 0, sizeof(R) * (size_t)c->g.nx * c->g.ny, c->stream));
    }
    CK(c, cudaStreamWaitEvent(c->stream, c->ev_ffj, 0));
    CKL(c);
    return FSIBE_OK;
}

static int fluid_step(fsibe_ctx* c, int explicit_step, bool adv_forked = false, bool stress_rows = false,
                      bool adv_prev = false, bool adv_next = false) {
    return c->fp32 ? fluid_step_t<float>(c, explicit_step, adv_forked, stress_rows, adv_prev, adv_next)
                   : fluid_step_t<double>(c, explicit_step, adv_forked, stress_rows, adv_prev, adv_next);
}

static MaskArgs mask_args(fsibe_ctx* c) {
    MaskArgs m;
    std::memset(&m, 0, sizeof(m));
    m.S = c->S;
    m.nx = c->P.nx; m.ny = c->P.ny; m.ns = c->P.ns;
    m.sharp_trailing = c->P.iSharpTrailing;
    m.sharp = std::fabs(c->P.N_smooth) < 1e-4;
    m.dx = c->g.dx; m.dy = c->g.dy; m.ds = c->g.ds;
    m.t_beam = c->P.t_beam; m.N_smooth = c->P.N_smooth; m.eps = c->P.eps; m.pi = c->g.pi;
    m.angle_deg = c->P.angle_beam;
    m.x = c->beam[B_X]; m.y = c->beam[B_Y]; m.vx = c->beam[B_VX]; m.vy = c->beam[B_VY]; m.th = c->beam[B_TH];
    m.prims = c->prims; m.primg = c->fp32 ? c->primg : nullptr; m.nprims = c->nprims; m.rect = c->rect; m.nsm = c->nsm;
    m.rdx = 1.0 / m.dx; m.rdy = 1.0 / m.dy; m.rpi = 1.0 / m.pi;
    m.inv_delta = 1.0 / ((m.N_smooth * std::fmax(m.dx, m.dy)) * c->gerf);
    m.inv_ds = 1.0 / m.ds;
    m.inv_eps = 1.0 / m.eps;
    m.mo = motion_args(c);
    m.mask = c->phys[PH_MASK]; m.mvx = c->phys[PH_MVX]; m.mvy = c->phys[PH_MVY];
    m.full = c->full_mask ? 1 : 0;
    m.bg = c->bg;
    m.frame = c->frame;
    m.frame_c = c->P.eps / std::max(1.0e-3, c->P.eps);
    m.sponge4 = c->P.iSponge == 4 ? 1 : 0;
    if (m.sponge4) {
        const double sss = c->P.SpongeSize;
        m.s4_star = sss;
        m.s4_size = sss - 2.0 * c->P.N_smooth * c->g.dx;
        m.s4_l1 = (int)std::lround((0.5 * sss) / c->g.dx);
        m.s4_r0 = m.s4_l1;
        m.s4_r1 = (int)std::lround((1.0 * sss) / c->g.dx);
        m.h_channel = c->P.h_channel;
        m.H_eff = c->P.yl - 2.0 * c->P.h_channel;
    }
    m.iMeanVelocity = c->P.iMeanVelocity;
    m.T_fullspeed = c->P.T_fullspeed;
    m.cos_ti = std::cos(c->P.theta_inf);
    m.sin_ti = std::sin(c->P.theta_inf);
    return m;
}

static StaticMaskArgs static_mask_args(fsibe_ctx* c) {
    StaticMaskArgs a;
    std::memset(&a, 0, sizeof(a));
    a.nx = c->P.nx; a.ny = c->P.ny;
    a.sharp = std::fabs(c->P.N_smooth) < 1e-4;
    a.iWalls = c->P.iWalls; a.iCylinder = c->P.iCylinder; a.iSponge = c->P.iSponge;
    a.dx = c->g.dx; a.dy = c->g.dy; a.xl = c->P.xl; a.yl = c->P.yl; a.N = c->P.N_smooth; a.pi = c->g.pi;
    a.h_channel = c->P.h_channel; a.R_cylinder = c->P.R_cylinder; a.x0 = c->P.x0; a.y0 = c->P.y0;
    a.t_beam = c->P.t_beam; a.SpongeSize = c->P.SpongeSize; a.eps = c->P.eps; a.eps_sponge = c->P.eps_sponge;
    a.bg = c->bg; a.frame = c->frame; a.spg = c->spg; a.mask = c->phys[PH_MASK];
    a.fp32 = c->fp32 ? 1 : 0;
    return a;
}

// create_sponge_mask (create_mask.f90:223-364) from the start-up mask, once per start
static int sponge_mask(fsibe_ctx* c) {
    if (!c->spg) return FSIBE_OK;
    StaticMaskArgs a = static_mask_args(c);
    a.bg = nullptr; a.frame = nullptr;
    launch_sponge_mask(a, c->gerf, c->stream);
    CKL(c);
    return FSIBE_OK;
}

// until_full: the step's redraw for the velocity sponge or the frame of a run whose beam does
// not move; the kernels keep the previous mask from T_fullspeed on (time_step.f90:187)
static int create_mask(fsibe_ctx* c, bool until_full = false) {
    if (c->P.iBeam <= 0) {
        const size_t bytes = (c->fp32 ? 4 : 8) * (size_t)c->g.nx * c->g.ny;
        for (int q : {PH_MASK, PH_MVX, PH_MVY}) CK(c, cudaMemsetAsync(c->phys[q], 0, bytes, c->stream));
        return FSIBE_OK;
    }
    MaskArgs m = mask_args(c);
    m.until_full = until_full ? 1 : 0;
    prof_begin(c, "mask_prep");
    launch_mask_prep(m, c->gerf, c->stream, c->pdl);
    prof_end(c);
    prof_begin(c, "mask");
    launch_mask(m, c->gerf, c->fp32, c->stream, c->pdl);
    prof_end(c);
    c->launches += 2;
    CKL(c);
    return FSIBE_OK;
}

static ForceArgs force_args(fsibe_ctx* c, double& dxi, double& dyi) {
    ForceArgs f;
    std::memset(&f, 0, sizeof(f));
    f.S = c->S;
    f.nx = c->P.nx; f.ny = c->P.ny; f.ns = c->P.ns; f.viscous = c->P.iViscous == 1;
    f.xl = c->P.xl; f.yl = c->P.yl; f.dx = c->g.dx; f.dy = c->g.dy; f.ds = c->g.ds;
    f.t_beam = c->P.t_beam; f.N_smooth = c->P.N_smooth; f.pi = c->g.pi; f.angle_deg = c->P.angle_beam;
    f.t_release = c->P.t_release; f.tau = c->P.tau;
    f.x = c->beam[B_X]; f.y = c->beam[B_Y]; f.th = c->beam[B_TH];
    f.press = c->phys[PH_PRESS]; f.sa = c->phys[PH_SA]; f.sb = c->phys[PH_SB];
    f.p_new = c->beam[B_PN]; f.tau_new = c->beam[B_TN];
    f.counter = c->counter;
    f.fterm = c->fterm;
    f.fp32 = c->fp32 ? 1 : 0;
    dxi = (c->P.xl - c->g.dx) / (double)(c->P.nx - 1);
    dyi = (c->P.yl - c->g.dy) / (double)(c->P.ny - 1);
    f.geo = c->fgeo;
    f.gij = c->fgij;
    f.mo = motion_args(c);
    f.rdxi = 1.0 / dxi;
    f.rdyi = 1.0 / dyi;
    return f;
}

// The interpolation geometry of the forces (k_forces_geo), from the beam state alone.
static void forces_geo(fsibe_ctx* c, cudaStream_t st) {
    double dxi, dyi;
    const ForceArgs f = force_args(c, dxi, dyi);
    prof_begin(c, "forces_geo", st);
    launch_forces_geo(f, dxi, dyi, st);
    prof_end(c, st);
    c->launches++;
}

// GetForces; geo_done: the step already formed the geometry beside the fluid kernels (ev_geo).
static int get_forces(fsibe_ctx* c, bool geo_done = false) {
    double dxi, dyi;
    const ForceArgs f = force_args(c, dxi, dyi);
    if (geo_done) CK(c, cudaStreamWaitEvent(c->stream, c->ev_geo, 0));
    else forces_geo(c, c->stream);
    prof_begin(c, "forces");
    launch_forces(f, dxi, dyi, c->stream, c->pdl);
    prof_end(c);
    c->launches++;
    CKL(c);
    return FSIBE_OK;
}

static AdvArgs adv_args(fsibe_ctx* c) {
    AdvArgs a;
    a.S = c->S;
    a.ns = c->P.ns;
    a.x = c->beam[B_X]; a.y = c->beam[B_Y]; a.vx = c->beam[B_VX]; a.vy = c->beam[B_VY];
    a.th = c->beam[B_TH]; a.thd = c->beam[B_THD];
    a.p_old = c->beam[B_PO]; a.p_new = c->beam[B_PN]; a.tau_old = c->beam[B_TO]; a.tau_new = c->beam[B_TN];
    a.rows = c->rows;
    a.mo = motion_args(c);
    return a;
}

// The solid step; with end_step and the cluster form, the cluster kernel also ends the time
// step (advance_state) and *advanced is set.
static int solid_step(fsibe_ctx* c, bool end_step = false, bool* advanced = nullptr) {
    if (!c->pre_launched) { const int st = beam_predict(c); if (st) return st; }
    CK(c, cudaStreamWaitEvent(c->stream, c->ev_join, 0));
    c->pre_launched = false;
    prof_begin(c, "beam");
    if (c->beam_cl) {
        BeamArgs b = beam_args(c);
        if (end_step) {
            b.fuse_adv = 1;
            b.adv = adv_args(c);
            if (advanced) *advanced = true;
        }
        launch_beam_cluster(b, c->beam_cl, c->beam_cl_smem, c->stream, c->pdl);
    } else {
        launch_beam(beam_args(c), c->stream);
    }
    prof_end(c);
    c->launches++;
    CKL(c);
    return FSIBE_OK;
}

static int advance(fsibe_ctx* c) {
    const AdvArgs a = adv_args(c);
    prof_begin(c, "advance");
    k_advance<<<1, 256, 0, c->stream>>>(a);
    prof_end(c);
    c->launches++;
    CKL(c);
    return FSIBE_OK;
}

// The fused step forms the pressure only on the forces' rows when it computes the forces
// (k_press_fin with srows); ensure_press forms the whole field before a reader sees it.
static bool press_rows_only(const fsibe_ctx* c) {
    return (c->P.iFLUSI == 1 || c->P.iSaveBeam > 0) && c->P.iBeam > 0;
}

template <typename R>
static int press_full_t(fsibe_ctx* c) {
    KArgs<R> a = kargs<R>(c);
    SizeKernels<R>& KX = kx_of<R>(c);
    launch_xv<R>(c, KX.xv[c->xv_fin].press_fin, KX.xv[c->xv_fin], 1, a, "press_fin");
    CKL(c);
    return FSIBE_OK;
}

static int ensure_press(fsibe_ctx* c) {
    if (!c->press_partial) return FSIBE_OK;
    c->press_partial = false;
    return c->fp32 ? press_full_t<float>(c) : press_full_t<double>(c);
}

// time_step.f90:178-228 (or :120-162 for the start-up step)
static int step_body(fsibe_ctx* c, int explicit_step) {
    const fsibe_params& P = c->P;
    int st;
    // time_step.f90:187: the mask is drawn every step for a moving beam, and while the mean flow
    // accelerates for the velocity sponge (iSponge = 4) and the frame (22)
    const bool moving = P.iFLUSI == 1 || P.iMotion > 0;
    const bool mask = moving || P.iSponge >= 4;
    const bool forces = P.iFLUSI == 1 || P.iSaveBeam > 0;
    // with a mask formed in the step, the advection part of the nonlinear term runs on the
    // second side stream beside the mask kernels; the forces' interpolation geometry, which
    // needs only the beam state, follows it there and runs beside the fluid step
    const bool split = mask && P.iBeam > 0 && c->nl_split;
    // the advection part is pipelined: each fused step launches the next step's beside its own
    // pressure and beam; a step that finds none ready (the first, or after the host changed the
    // state) launches its own first
    const bool adv_prev = split && c->adv_ready;
    const bool adv_next = split && c->adv_pipe;
    c->adv_ready = false;
    if (split || forces) {
        CK(c, cudaEventRecord(c->ev_geo, c->stream));
        CK(c, cudaStreamWaitEvent(c->side2, c->ev_geo, 0));
    }
    if (split && !adv_prev) {
        if (c->fp32) nl_advect_t<float>(c, explicit_step);
        else nl_advect_t<double>(c, explicit_step);
        CK(c, cudaEventRecord(c->ev_adv, c->side2));
    }
    if (forces) {
        forces_geo(c, c->side2);
        CK(c, cudaEventRecord(c->ev_geo, c->side2));
    }
    if (mask) { st = create_mask(c, !moving); if (st) return st; }
    st = fluid_step(c, explicit_step, split, forces, adv_prev, adv_next);
    if (st) return st;
    if (forces) { st = get_forces(c, true); if (st) return st; }
    bool advanced = false;
    if (P.iFLUSI == 1) { st = solid_step(c, true, &advanced); if (st) return st; }
    else if (P.iMotion > 0) {
        // the prescribed motion alone: integrate_position(time) (time_step.f90:211-216)
        launch_move_beam(beam_args(c), c->stream);
        c->launches++;
        CKL(c);
    }
    st = advanced ? FSIBE_OK : advance(c);
    if (st) return st;
    if (adv_next) {
        // join the next step's advection part: what follows on the main stream (the next step)
        // is ordered after it
        CK(c, cudaStreamWaitEvent(c->stream, c->ev_adv, 0));
        c->adv_ready = true;
    }
    return FSIBE_OK;
}

// The fused step pipelines the advection part (step_body): true when its graph expects the
// previous step to have launched it.
static bool adv_pipelined(const fsibe_ctx* c) {
    const fsibe_params& P = c->P;
    const bool mask = P.iFLUSI == 1 || P.iMotion > 0 || P.iSponge >= 4;
    return mask && P.iBeam > 0 && c->nl_split && c->adv_pipe;
}

static int do_step(fsibe_ctx* c) {
    if (!c->initialized) { c->err = "step before init_fields"; return FSIBE_ERR_STATE; }
    c->press_partial = press_rows_only(c);
    if (!c->startup_done) {
        int st = step_body(c, 1);
        if (st) return st;
        c->startup_done = true;
        return FSIBE_OK;
    }
    // the graph is the steady step: the previous step launched this one's advection part; a
    // step after the host changed the state runs directly once
    if (c->use_graph && (!adv_pipelined(c) || c->adv_ready)) {
        if (!c->graph_ready) {
            CK(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
            const int before = c->launches;
            int st = step_body(c, 0);
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaStreamEndCapture(c->stream, &g);
            if (st) return st;
            if (e != cudaSuccess) { c->err = std::string("capture: ") + cudaGetErrorString(e); return FSIBE_ERR_CUDA; }
            c->graph = g;
            CK(c, cudaGraphInstantiate(&c->gexec, g, cudaGraphInstantiateFlagUseNodePriority));
            c->graph_ready = true;
            c->launches = before;
        }
        CK(c, cudaGraphLaunch(c->gexec, c->stream));
        c->launches += 0;
        c->adv_ready = adv_pipelined(c);  // the graph launched the next step's advection part
        return FSIBE_OK;
    }
    return step_body(c, 0);
}

static void free_graph(fsibe_ctx* c) {
    if (c->gexec) cudaGraphExecDestroy(c->gexec);
    if (c->graph) cudaGraphDestroy(c->graph);
    c->gexec = nullptr;
    c->graph = nullptr;
    c->graph_ready = false;
}

// ---- transfers ----------------------------------------------------------------------
static int to_host(fsibe_ctx* c, const void* dev, size_t n, double* host, const double* offset = nullptr) {
    if (c->fp32) {
        k_convert<float><<<256, 256, 0, c->stream>>>(reinterpret_cast<const float*>(dev), c->dscratch, n, offset);
        CKL(c);
        CK(c, cudaMemcpyAsync(host, c->dscratch, n * 8, cudaMemcpyDeviceToHost, c->stream));
    } else {
        CK(c, cudaMemcpyAsync(host, dev, n * 8, cudaMemcpyDeviceToHost, c->stream));
    }
    CK(c, cudaStreamSynchronize(c->stream));
    return FSIBE_OK;
}

static int from_host(fsibe_ctx* c, const double* host, size_t n, void* dev, const double* offset = nullptr) {
    if (c->fp32) {
        CK(c, cudaMemcpyAsync(c->dscratch, host, n * 8, cudaMemcpyHostToDevice, c->stream));
        k_convert_in<float><<<256, 256, 0, c->stream>>>(c->dscratch, reinterpret_cast<float*>(dev), n, offset);
        CKL(c);
    } else {
        CK(c, cudaMemcpyAsync(dev, host, n * 8, cudaMemcpyHostToDevice, c->stream));
    }
    CK(c, cudaStreamSynchronize(c->stream));
    return FSIBE_OK;
}

static int spec_to_packed(fsibe_ctx* c, const void* H, double* host_fk, const void* Hlo = nullptr) {
    if (c->fp32) k_pack<float><<<c->g.hx, 256, 0, c->stream>>>(reinterpret_cast<const float2*>(H), reinterpret_cast<const float2*>(Hlo), c->dscratch, c->g.nx, c->g.ny);
    else k_pack<double><<<c->g.hx, 256, 0, c->stream>>>(reinterpret_cast<const double2*>(H), nullptr, c->dscratch, c->g.nx, c->g.ny);
    CKL(c);
    CK(c, cudaMemcpyAsync(host_fk, c->dscratch, 8 * (size_t)c->g.nx * c->g.ny, cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    return FSIBE_OK;
}

static int packed_to_spec(fsibe_ctx* c, const double* host_fk, void* H, void* Hlo = nullptr) {
    CK(c, cudaMemcpyAsync(c->dscratch, host_fk, 8 * (size_t)c->g.nx * c->g.ny, cudaMemcpyHostToDevice, c->stream));
    if (c->fp32) k_unpack<float><<<c->g.hx, 256, 0, c->stream>>>(c->dscratch, reinterpret_cast<float2*>(H), reinterpret_cast<float2*>(Hlo), c->g.nx, c->g.ny);
    else k_unpack<double><<<c->g.hx, 256, 0, c->stream>>>(c->dscratch, reinterpret_cast<double2*>(H), nullptr, c->g.nx, c->g.ny);
    CKL(c);
    CK(c, cudaStreamSynchronize(c->stream));
    return FSIBE_OK;
}

template <typename R>
static int fwd2d(fsibe_ctx* c, void* spec_out) {
    KArgs<R> a = kargs<R>(c);
    a.spec1 = reinterpret_cast<C2<R>*>(spec_out);
    launch_x<R>(c, kx_of<R>(c).xfwd, kx_of<R>(c).x_smem1, a);
    launch_y<R>(c, ky_of<R>(c).yfwd, ky_of<R>(c).y_smem1, a);
    CKL(c);
    return FSIBE_OK;
}

template <typename R>
static int inv_y(fsibe_ctx* c, const void* spec_in, void* t_out, int op) {
    KArgs<R> a = kargs<R>(c);
    a.spec1 = reinterpret_cast<C2<R>*>(const_cast<void*>(spec_in));
    a.spec0 = reinterpret_cast<C2<R>*>(t_out);
    a.op = op;
    launch_y<R>(c, ky_of<R>(c).yinv, ky_of<R>(c).y_smem1, a);
    CKL(c);
    return FSIBE_OK;
}

template <typename R>
static int inv_x(fsibe_ctx* c) {
    KArgs<R> a = kargs<R>(c);
    launch_x<R>(c, kx_of<R>(c).xinv, kx_of<R>(c).x_smem1, a);
    CKL(c);
    return FSIBE_OK;
}

// The sharp outflow sponge (iSponge = 10, NavierStokes.f90:103-122): du/dx of the state's
// velocity (i kx i ky psi from the vorticity spectrum, inverse y into the free spectrum SP_0,
// inverse x), then its integral along each row (k_sponge10), which the penalization part of
// k_nl_x adds to its x component.
template <typename R>
static int sponge10_term(fsibe_ctx* c) {
    int st;
    if ((st = inv_y<R>(c, c->spec[SP_W], c->spec[SP_0], OP_UX))) return st;
    KArgs<R> a = kargs<R>(c);
    a.spec0 = reinterpret_cast<C2<R>*>(c->spec[SP_0]);
    a.phys0 = reinterpret_cast<R*>(c->s10_dudx);
    launch_x<R>(c, kx_of<R>(c).xinv, kx_of<R>(c).x_smem1, a);
    k_sponge10<R><<<(c->g.ny + 127) / 128, 128, 0, c->stream>>>(reinterpret_cast<const R*>(c->s10_dudx),
                                                               reinterpret_cast<R*>(c->s10), c->g.nx, c->g.ny,
                                                               c->s10_ixmin, c->s10_ixmax, c->g.dx, 1.0 / c->P.eps_sponge);
    c->launches += 3;
    CKL(c);
    return FSIBE_OK;
}

// cal_velocity at time (init) : u, v and the velocity statistics for the first cal_nlk
template <typename R>
static int init_velocity(fsibe_ctx* c) {
    int st;
    if ((st = inv_y<R>(c, c->spec[SP_W], c->spec[SP_TU], OP_U))) return st;
    if ((st = inv_y<R>(c, c->spec[SP_W], c->spec[SP_TV], OP_V))) return st;
    if ((st = inv_y<R>(c, c->spec[SP_W], c->spec[SP_TDX], OP_DX))) return st;
    if ((st = inv_y<R>(c, c->spec[SP_W], c->spec[SP_TDY], OP_DY))) return st;
    if ((st = inv_y<R>(c, c->spec[SP_W], c->spec[SP_TW], OP_ID))) return st;  // the sponge's vorticity
    KArgs<R> a = kargs<R>(c);
    launch_x<R>(c, kx_of<R>(c).vel_x, kx_of<R>(c).x_smem2, a);
    CKL(c);
    return FSIBE_OK;
}

static double host_mean(const fsibe_params& P, double t, bool x) {
    const double pi = 4.0 * std::atan(1.0);
    double tf = 1.0;
    switch (P.iMeanVelocity) {
        case 1: tf = (t < P.T_fullspeed) ? (t * t * t) / (-0.5 * P.T_fullspeed * P.T_fullspeed * P.T_fullspeed) + 3.0 * (t * t) / (P.T_fullspeed * P.T_fullspeed) : 1.0; break;
        case 2: tf = (t < P.T_fullspeed) ? 0.5 * (1.0 - std::cos(0.5 * pi * t / P.T_fullspeed)) : 1.0; break;
        case 3: break;
        case 6: return x ? t : 0.0;
        case 22: return x ? 0.1 : 0.0;
        default: return 0.0;
    }
    return (x ? std::cos(P.theta_inf) : std::sin(P.theta_inf)) * tf;
}

// =====================================================================================
// C ABI
// =====================================================================================
// ---- ComputePressureSnapshot (NavierStokes.f90:598-665) ------------------------------
// u, v at `time` (the state's velocity plus the mean flow of the time), the penalization and
// the nonlinear term's divergence as two fields, forward 2-D, the Poisson divide, inverse 2-D,
// p = q - |u|^2 / 2.  Outside the time step; the state is not changed.
template <typename R>
__global__ void k_snap_terms(R* u, R* v, const R* w, const R* mask, const R* mvx, const R* mvy, R* px, R* py,
                             size_t n, double U, double V) {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
        const R uk = u[k] + (R)U, vk = -v[k] + (R)V, wk = w[k], m = mask[k];  // v = -d psi/dx + V
        u[k] = uk;
        v[k] = vk;
        px[k] = m * (uk - mvx[k]) + (-wk * vk);  // the penalization (positive here) and -omega v
        py[k] = m * (vk - mvy[k]) + wk * uk;     // and +omega u
    }
}
// q^ = (i kx P^x + i ky P^y) / k^2 (zero at k = 0 and ky = ny/2), in place of P^x
template <typename R>
__global__ void k_snap_poisson(C2<R>* sx, const C2<R>* sy, Geometry g) {
    const size_t n = (size_t)g.hx * g.ny;
    for (size_t o = blockIdx.x * (size_t)blockDim.x + threadIdx.x; o < n; o += (size_t)gridDim.x * blockDim.x) {
        const int kx = (int)(o / g.ny), ky = (int)(o % g.ny);
        const int ks = signed_k(ky, g.ny);
        const R kxs = (R)((double)kx * g.kxs), kys = (R)ks * (R)g.kys;
        const C2<R> Q = cadd<R>(cimul<R>(sx[o], kxs), cimul<R>(sy[o], kys));
        const R k2 = (R)(kx * kx) * (R)g.scalex + (R)(ks * ks) * (R)g.scaley;
        C2<R> q;
        if ((kx == 0 && ky == 0) || ky == g.ny / 2) q = mk<R>(0, 0);
        else if constexpr (kIsF32<R>) q = cscale<R>(Q, (R)1 / k2);
        else q = mk<R>(Q.x / k2, Q.y / k2);
        sx[o] = q;
    }
}
template <typename R>
__global__ void k_snap_fin(const R* q, const R* u, const R* v, double* out, size_t n) {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
        out[k] = (double)(q[k] - (R)0.5 * (u[k] * u[k] + v[k] * v[k]));
}

template <typename R>
static int pressure_snapshot_t(fsibe_ctx* c, double time, double* host_out) {
    const size_t NN = (size_t)c->g.nx * c->g.ny, rs = sizeof(R);
    if (!c->snap) CK(c, cudaMalloc(&c->snap, 7 * rs * NN));
    R* f = reinterpret_cast<R*>(c->snap);
    R *pu = f, *pv = f + NN, *pw = f + 2 * NN, *px = f + 3 * NN, *py = f + 4 * NN;
    C2<R>* s0 = reinterpret_cast<C2<R>*>(f + 5 * NN);
    C2<R>* s1 = reinterpret_cast<C2<R>*>(f + 6 * NN);
    C2<R>* T = reinterpret_cast<C2<R>*>(c->spec[SP_0]);
    const SizeKernels<R>& KX = kx_of<R>(c);
    const SizeKernels<R>& KY = ky_of<R>(c);
    auto to_phys = [&](const void* spec, int op, R* out) {
        int st = inv_y<R>(c, spec, T, op);
        if (st) return st;
        KArgs<R> a = kargs<R>(c);
        a.spec0 = T;
        a.phys0 = out;
        launch_x<R>(c, KX.xinv, KX.x_smem1, a);
        return FSIBE_OK;
    };
    auto to_spec = [&](R* in, C2<R>* out) {
        KArgs<R> a = kargs<R>(c);
        a.phys0 = in;
        a.spec0 = T;
        a.spec1 = out;
        launch_x<R>(c, KX.xfwd, KX.x_smem1, a);
        launch_y<R>(c, KY.yfwd, KY.y_smem1, a);
    };
    int st;
    if ((st = to_phys(c->spec[SP_W], OP_U, pu))) return st;
    if ((st = to_phys(c->spec[SP_W], OP_V, pv))) return st;
    if ((st = to_phys(c->spec[SP_W], OP_ID, pw))) return st;
    const double U = c->U_mean_true * host_mean(c->P, time, true), V = c->U_mean_true * host_mean(c->P, time, false);
    const int grid = 4 * c->nsm;
    k_snap_terms<R><<<grid, 256, 0, c->stream>>>(pu, pv, pw, reinterpret_cast<const R*>(c->phys[PH_MASK]),
                                                 reinterpret_cast<const R*>(c->phys[PH_MVX]),
                                                 reinterpret_cast<const R*>(c->phys[PH_MVY]), px, py, NN, U, V);
    to_spec(px, s0);
    to_spec(py, s1);
    k_snap_poisson<R><<<grid, 256, 0, c->stream>>>(s0, s1, c->g);
    if ((st = to_phys(s0, OP_ID, pw))) return st;
    double* out = c->dscratch;  // nx ny doubles
    k_snap_fin<R><<<grid, 256, 0, c->stream>>>(pw, pu, pv, out, NN);
    CKL(c);
    CK(c, cudaMemcpyAsync(host_out, out, 8 * NN, cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    return FSIBE_OK;
}

extern "C" {

const char* fsibe_strerror(int s) {
    switch (s) {
        case FSIBE_OK: return "ok";
        case FSIBE_ERR_PARAM: return "bad parameters";
        case FSIBE_ERR_CUDA: return "CUDA error";
        case FSIBE_ERR_NAN: return "NaN in the beam system";
        case FSIBE_ERR_NEWTON_MAXIT: return "Newton iteration limit";
        case FSIBE_ERR_SINGULAR: return "singular matrix";
        case FSIBE_ERR_INTERP_OOB: return "interpolation target outside the grid";
        case FSIBE_ERR_TIMEOUT: return "device wait timed out";
        case FSIBE_ERR_UNSUPPORTED: return "unsupported size or option";
        case FSIBE_ERR_MASK_OOB: return "beam point outside the domain";
        case FSIBE_ERR_BRAKE: return "emergency brake (continue_timestep = .false.)";
        case FSIBE_ERR_STATE: return "call out of order";
        default: return "unknown status";
    }
}

const char* fsibe_last_error(const fsibe_ctx* ctx) { return ctx ? ctx->err.c_str() : g_err.c_str(); }

}  // extern "C"

// ---- autotuner ----------------------------------------------------------------------
// The fused x kernels (k_nl_x, k_press_x, k_press_fin) come in three tile heights (rows of the
// grid per block).  A new context times each candidate on its own freshly allocated buffers
// (no state exists yet; fsibe_init_fields overwrites everything they touch) and keeps the
// fastest per kernel.  The choice is cached per (precision, nx, ny) for the process, so an
// ensemble of many runs of one size tunes once.  FSIBE_AUTOTUNE=0 keeps the default tiles.
template <typename R>
static float time_xv(fsibe_ctx* c, int kind, const typename SizeKernels<R>::XVariant& v) {
    KArgs<R> a = kargs<R>(c);
    void (*k)(KArgs<R>) = kind == 0 ? v.nl_x : (kind == 1 ? v.press_x : v.press_fin);
    const int smem = kind == 2 ? v.smem1 : v.smem3;
    const dim3 grid(c->g.ny / v.rows);
    for (int i = 0; i < 2; ++i) k<<<grid, v.threads, smem, c->stream>>>(a);
    // the best of three rounds of five launches (one round's mean moved by up to 10% between
    // processes at 4096^2 and flipped the choice)
    float best = 1e30f;
    for (int round = 0; round < 3; ++round) {
        cudaEventRecord(c->ev0, c->stream);
        for (int i = 0; i < 5; ++i) k<<<grid, v.threads, smem, c->stream>>>(a);
        cudaEventRecord(c->ev1, c->stream);
        if (cudaEventSynchronize(c->ev1) != cudaSuccess) return 1e30f;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev0, c->ev1);
        best = ms / 5.f < best ? ms / 5.f : best;
    }
    return best;
}

// One y-pass kernel over the kx rows, timed as time_xv times the x-pass candidates.
template <typename R>
static float time_y(fsibe_ctx* c, void (*k)(KArgs<R>), int smem, int threads) {
    KArgs<R> a = kargs<R>(c);
    const dim3 grid(c->g.hx);
    for (int i = 0; i < 2; ++i) k<<<grid, threads, smem, c->stream>>>(a);
    float best = 1e30f;
    for (int round = 0; round < 3; ++round) {
        cudaEventRecord(c->ev0, c->stream);
        for (int i = 0; i < 5; ++i) k<<<grid, threads, smem, c->stream>>>(a);
        cudaEventRecord(c->ev1, c->stream);
        if (cudaEventSynchronize(c->ev1) != cudaSuccess) return 1e30f;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev0, c->ev1);
        best = ms / 5.f < best ? ms / 5.f : best;
    }
    return best;
}

template <typename R>
static int autotune_x(fsibe_ctx* c) {
    static std::mutex mu;
    static std::vector<std::array<int, 7>> cache;  // fp32, nx, ny, nl, px, fin, press_y engine
    const char* env = std::getenv("FSIBE_AUTOTUNE");
    if (env && env[0] == '0') return FSIBE_OK;
    std::lock_guard<std::mutex> lock(mu);
    const int f32 = c->fp32 ? 1 : 0;
    for (const auto& e : cache)
        if (e[0] == f32 && e[1] == c->g.nx && e[2] == c->g.ny) {
            c->xv_nl = e[3]; c->xv_px = e[4]; c->xv_fin = e[5]; c->py_eng = e[6];
            return FSIBE_OK;
        }
    const SizeKernels<R>& K = kx_of<R>(c);
    int choice[3];
    for (int kind = 0; kind < 3; ++kind) {
        // the default first; a candidate must be faster by 3% to replace it
        int best = 1;
        float tbest = time_xv<R>(c, kind, K.xv[1]);
        for (int v : {0, 2, 3}) {
            if (K.xv[v].rows == K.xv[1].rows && K.xv[v].minb == K.xv[1].minb) continue;
            const float t = time_xv<R>(c, kind, K.xv[v]);
            if (t < 0.97f * tbest) { tbest = t; best = v; }
        }
        // FP32: the paired press_x (index 4), when its tile (128 threads: 128 / (H/16) rows)
        // divides the grid's rows
        if (kind == 1 && K.xp.press_x && c->g.ny % K.xp.rows == 0) {
            const float t = time_xv<R>(c, kind, K.xp);
            if (t < 0.97f * tbest) { tbest = t; best = 4; }
        }
        choice[kind] = best;
    }
    // k_press_y's transform engine (FP32): the paired one by default, the one-butterfly one when
    // it is faster by 3%
    int eng = 0;
    const SizeKernels<R>& KY = ky_of<R>(c);
    if (KY.press_y1) {
        const float t0 = time_y<R>(c, KY.press_y, KY.y_smem2, KY.press_y_threads);
        const float t1 = time_y<R>(c, KY.press_y1, KY.press_y1_smem, KY.y_threads);
        if (t1 < 0.97f * t0) eng = 1;
    }
    CKL(c);
    CK(c, cudaStreamSynchronize(c->stream));
    c->xv_nl = choice[0]; c->xv_px = choice[1]; c->xv_fin = choice[2]; c->py_eng = eng;
    cache.push_back({f32, c->g.nx, c->g.ny, choice[0], choice[1], choice[2], eng});
    return FSIBE_OK;
}

extern "C" {

static void adj_free(fsibe_ctx* c);

int fsibe_destroy(fsibe_ctx* c) {
    if (!c) return FSIBE_OK;
    free_graph(c);
    adj_free(c);
    for (void* p : c->phys) if (p) cudaFree(p);
    for (void* p : c->spec) if (p) cudaFree(p);
    for (double* p : c->beam) if (p) cudaFree(p);
    void* others[] = {c->twX, c->twR, c->twY, c->S, c->red, c->oo, c->ws, c->pred, c->minv, c->minv_rse, c->d1d, c->fgeo, c->fgij, c->clws, c->prims, c->primg, c->nprims,
                      c->rect, c->counter, c->fterm, c->rows, c->dscratch, c->dscratch2, c->etab, c->etabf, c->dcut, c->kxw,
                      c->bg, c->frame, c->spg, c->s10, c->s10_dudx, c->rect_full, c->snap};
    for (void* p : others) if (p) cudaFree(p);
    for (cudaEvent_t e : c->pool) cudaEventDestroy(e);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->side) { cudaStreamSynchronize(c->side); cudaStreamDestroy(c->side); }
    if (c->side2) { cudaStreamSynchronize(c->side2); cudaStreamDestroy(c->side2); }
    if (c->ev_ff) cudaEventDestroy(c->ev_ff);
    if (c->ev_ffj) cudaEventDestroy(c->ev_ffj);
    if (c->ev_sb0) cudaEventDestroy(c->ev_sb0);
    if (c->ev_geo) cudaEventDestroy(c->ev_geo);
    if (c->ev_adv) cudaEventDestroy(c->ev_adv);
    if (c->ev_ny) cudaEventDestroy(c->ev_ny);
    if (c->ev_sb) cudaEventDestroy(c->ev_sb);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return FSIBE_OK;
}

int fsibe_create(const fsibe_params* p, fsibe_ctx** out) {
    if (!p || !out) { g_err = "null argument"; return FSIBE_ERR_PARAM; }
    *out = nullptr;
    if (!pow2_ok(p->nx) || !pow2_ok(p->ny)) { g_err = "nx, ny must be powers of two in [32, 4096]"; return FSIBE_ERR_UNSUPPORTED; }
    if (p->iBeam > 0 && p->ns < 8) { g_err = "ns must be >= 8"; return FSIBE_ERR_PARAM; }
    if (p->iBeam > 1) { g_err = "one beam per run"; return FSIBE_ERR_UNSUPPORTED; }
    {
        // mouvement.f90:17-155: fixed (0), heaving (2), flapping (3), impulsive translation (4),
        // heaving with a soft start (201-213, 300-350), the Paraz heaving cases (401-413: the
        // reference indexes its 13 periods with iMotion - 400, so 400 and 414-450 read outside them)
        const int m = p->iMotion;
        const bool ok = m == 0 || m == 2 || m == 3 || m == 4 || (m >= 201 && m <= 213) || (m >= 300 && m <= 350) ||
                        (m >= 401 && m <= 413);
        if (!ok) { g_err = "iMotion in {0, 2, 3, 4, 201-213, 300-350, 401-413} (mouvement.f90)"; return FSIBE_ERR_PARAM; }
        if (m != 0 && p->iBeam != 1) { g_err = "a prescribed motion needs the beam (iBeam = 1)"; return FSIBE_ERR_UNSUPPORTED; }
    }
    if (p->precision != FSIBE_FP64 && p->precision != FSIBE_FP32C) { g_err = "precision"; return FSIBE_ERR_PARAM; }
    if (p->iMeanVelocity == 11) { g_err = "iMeanVelocity = 11 is not implemented"; return FSIBE_ERR_UNSUPPORTED; }
    {
        const int isp = p->iSponge;
        if (p->iWalls < 0 || p->iWalls > 1 || p->iCylinder < 0 || p->iCylinder > 1 ||
            !(isp == 0 || isp == 1 || isp == 2 || isp == 3 || isp == 4 || isp == 22 || isp == 10)) {
            g_err = "iWalls, iCylinder in {0, 1}; iSponge in {0, 1, 2, 3, 4, 10, 22}"; return FSIBE_ERR_PARAM;
        }
        if ((p->iWalls || p->iCylinder || isp) && p->iBeam != 1) {
            g_err = "walls, the cylinder and the sponges run with the beam (iBeam = 1)"; return FSIBE_ERR_UNSUPPORTED;
        }
        if (isp > 0 && isp != 4 && !(p->eps_sponge >= 1.0e-9)) { g_err = "eps_sponge (params.f90:185-188)"; return FSIBE_ERR_PARAM; }
        if (isp > 0 && !(p->SpongeSize > 0.0 && p->SpongeSize < std::min(p->xl, p->yl))) {
            g_err = "SpongeSize must lie in (0, min(xl, yl))"; return FSIBE_ERR_PARAM;
        }
        if (p->iWalls == 1 && p->theta_inf != 0.0) { g_err = "walls need theta_inf = 0 (params.f90:199-203)"; return FSIBE_ERR_PARAM; }
    }
    if (p->time_method_solid != FSIBE_BDF2 && p->time_method_solid != FSIBE_CRANK_NICHOLSON &&
        p->time_method_solid != FSIBE_EULER_IMPLICIT) { g_err = "time_method_solid"; return FSIBE_ERR_PARAM; }
    fsibe_ctx* c = new fsibe_ctx();
    c->P = *p;
    if (c->P.iMotion >= 401 && c->P.iMotion <= 413) {
        // mouvement.f90:102-104: these cases set the forces' soft start-up to one period
        static const double periods[13] = {0.51, 0.34, 0.25, 0.20, 0.17, 0.14, 0.13, 0.11, 0.10, 0.09, 0.08, 0.08, 0.07};
        c->P.tau = periods[c->P.iMotion - 401];
    }
    if (c->P.newton_tol <= 0.0) c->P.newton_tol = 1.0e-7;
    if (c->P.newton_maxit <= 0) c->P.newton_maxit = 50;
    c->fp32 = p->precision == FSIBE_FP32C;
    Geometry& g = c->g;
    g.nx = p->nx; g.ny = p->ny; g.hx = p->nx / 2; g.ns = p->ns;
    g.xl = p->xl; g.yl = p->yl;
    g.dx = p->xl / (double)p->nx;
    g.dy = p->yl / (double)p->ny;
    g.ds = p->length / (double)(p->ns - 1);
    g.pi = 4.0 * std::atan(1.0);
    g.kxs = 2.0 * g.pi / p->xl;
    g.kys = 2.0 * g.pi / p->yl;
    g.scalex = g.kxs * g.kxs;
    g.scaley = g.kys * g.kys;
    const double kxt = 2.0 / 3.0 * (double)(p->nx / 2 - 1), kyt = 2.0 / 3.0 * (double)(p->ny / 2 - 1);
    g.kx_trunc2 = kxt * kxt;
    g.ky_trunc2 = kyt * kyt;
    g.idealis = p->idealis;
    g.inv_nxny = 1.0 / ((double)p->nx * (double)p->ny);
    c->gerf = std::fabs((std::exp(-(2.0 * 1.0) * (2.0 * 1.0)) - 1.0) / std::sqrt(g.pi));
    SizeKernels<double> dx_, dy_;
    SizeKernels<float> fx_, fy_;
    if (!get_sizes(p->nx, dx_, fx_) || !get_sizes(p->ny, dy_, fy_)) { g_err = "size"; delete c; return FSIBE_ERR_UNSUPPORTED; }
    c->kxd = dx_; c->kxf = fx_; c->kyd = dy_; c->kyf = fy_;
    const size_t NN = (size_t)p->nx * p->ny;
    const size_t rs = c->fp32 ? 4 : 8;
#define ALLOC(ptr, bytes)                                                                       \
    do {                                                                                        \
        cudaError_t e_ = cudaMalloc((void**)&(ptr), (bytes));                                   \
        if (e_ != cudaSuccess) { g_err = std::string("cudaMalloc: ") + cudaGetErrorString(e_); \
                                 fsibe_destroy(c); return FSIBE_ERR_CUDA; }                     \
        cudaMemset((ptr), 0, (bytes));                                                          \
    } while (0)
    for (int i = 0; i < PH_N; ++i) ALLOC(c->phys[i], rs * NN);
    for (int i = 0; i < SP_N; ++i) ALLOC(c->spec[i], rs * NN);
    const int ns = p->ns > 8 ? p->ns : 8, n = 2 * ns + 4;
    for (int i = 0; i < B_N; ++i) ALLOC(c->beam[i], 8 * (size_t)ns);
    ALLOC(c->oo, 8 * (size_t)ns * 6);
    ALLOC(c->ws, 8 * beam_ws_doubles(ns));
    ALLOC(c->pred, 8 * beam_pred_doubles(ns));
    ALLOC(c->d1d, 8 * 96);
    ALLOC(c->fgeo, 8 * 76 * (size_t)ns);
    ALLOC(c->fgij, 4 * 8 * (size_t)ns);
    {
        double tab[96];
        beam_d1d_table(c->g.ds, tab);
        cudaMemcpy(c->d1d, tab, sizeof(tab), cudaMemcpyHostToDevice);
    }
    c->beam_smem = beam_smem_setup(ns);
    {
        // the beam's Newton step on a cluster of 16 (or 8) CTAs when the device places one;
        // FSIBE_BEAM_CLUSTER = 0 / 8 / 16 caps the size (0: the single-CTA kernel)
        const char* e = std::getenv("FSIBE_BEAM_CLUSTER");
        const int want = e ? std::atoi(e) : 16;
        c->beam_cl = (want >= 8) ? beam_cluster_setup(ns, want, &c->beam_cl_smem, &c->beam_cl_big) : 0;
        if (c->beam_cl) {
            ALLOC(c->minv, 4 * beam_cluster_minv_floats(ns, c->beam_cl));
            ALLOC(c->minv_rse, 4 * (size_t)(n + 16));
            if (c->beam_cl_big) ALLOC(c->clws, 4 * beam_cluster_fact_floats(ns, c->beam_cl));
        }
    }
    c->beam_pre_smem = beam_pre_smem_setup(ns);
    {
        const char* e = std::getenv("FSIBE_NL_SPLIT");
        c->nl_split = !(e && std::atoi(e) == 0);
        e = std::getenv("FSIBE_PDL");
        c->pdl = !(e && std::atoi(e) == 0);
        e = std::getenv("FSIBE_STRESS_SPLIT");
        c->stress_split = !(e && std::atoi(e) == 0);

    }
    ALLOC(c->prims, sizeof(Prim) * (size_t)(2 * ns + 8));
    if (c->fp32) ALLOC(c->primg, sizeof(PrimG) * (size_t)(2 * ns + 8));
    ALLOC(c->nprims, 16);
    ALLOC(c->rect, 64);
    {
        // previous box: none drawn yet (all cells zero); box accumulator: empty
        const int r0[16] = {0, 0, 0, 0, 0, 0, 0, 0, p->nx, -1, p->ny, -1, 0, 0, 0, 0};
        cudaMemcpy(c->rect, r0, sizeof(r0), cudaMemcpyHostToDevice);
    }
    ALLOC(c->counter, 16);
    ALLOC(c->fterm, 16 * (size_t)ns);
    ALLOC(c->S, sizeof(DevScalars));
    ALLOC(c->red, 8 * (size_t)p->ny * RED_NSLOTS);
    ALLOC(c->etab, 8 * (size_t)(p->nx / 2 + p->ny / 2 + 8));
    ALLOC(c->etabf, 8 * (size_t)(p->nx / 2 + p->ny / 2 + 8));
    ALLOC(c->dcut, 4 * (size_t)(p->nx / 2 + 8));
    ALLOC(c->kxw, 4 * (size_t)(p->nx / 2 + 8));
    {
        std::vector<float> kw(p->nx / 2 + 1);
        for (int kx = 0; kx <= p->nx / 2; ++kx) kw[kx] = (float)((double)kx * g.kxs);
        cudaMemcpy(c->kxw, kw.data(), 4 * kw.size(), cudaMemcpyHostToDevice);
    }
    {
        // 2/3 rule (dealiase_mask.f90:9-26), evaluated with the reference's FP64 expression:
        // dcut[kx] = smallest |ky| that is removed
        std::vector<int> cut(p->nx / 2);
        for (int kx = 0; kx < p->nx / 2; ++kx) {
            int k = 0;
            while (k < p->ny / 2 && !((double)kx * (double)kx / (kxt * kxt) + (double)k * (double)k / (kyt * kyt) >= 1.0)) ++k;
            cut[kx] = k;
        }
        cudaMemcpy(c->dcut, cut.data(), 4 * cut.size(), cudaMemcpyHostToDevice);
        c->kcut = p->nx / 2;
        if (p->idealis == 1)
            for (int kx = 0; kx < p->nx / 2; ++kx)
                if (cut[kx] == 0) { c->kcut = kx; break; }
    }
    ALLOC(c->dscratch, 8 * 2 * NN);
    ALLOC(c->dscratch2, 8 * NN);
    {
        // walls, cylinder and sponges (create_mask.f90:21-68, 120-204, 223-364): the static
        // fields, and every cell drawn each step
        const int isp = p->iSponge;
        c->full_mask = p->iWalls > 0 || p->iCylinder > 0 || isp == 4 || isp == 22;
        if (p->iWalls > 0 || p->iCylinder > 0) ALLOC(c->bg, 8 * NN);
        if (isp == 22) ALLOC(c->frame, 8 * NN);
        if (isp == 1 || isp == 2 || isp == 3 || isp == 22) ALLOC(c->spg, rs * NN);
        if (isp == 10) {
            // NavierStokes.f90:107-108: ixmin = nint((xl - SpongeSize)/dx), ixmax = nx - 1 - 15
            c->s10_ixmin = (int)std::lround((p->xl - p->SpongeSize) / c->g.dx);
            c->s10_ixmax = p->nx - 1 - 15;
            ALLOC(c->s10, rs * NN);
            ALLOC(c->s10_dudx, rs * NN);
            cudaMemset(c->s10, 0, rs * NN);
        }
        if (c->full_mask || isp == 10) {
            ALLOC(c->rect_full, 16);
            const int rf[4] = {0, p->nx - 1, 0, p->ny - 1};
            cudaMemcpy(c->rect_full, rf, sizeof(rf), cudaMemcpyHostToDevice);
        }
        if (c->bg || c->frame) {
            launch_static_masks(static_mask_args(c), c->gerf, 0);
            cudaError_t e_ = cudaGetLastError();
            if (e_ == cudaSuccess) e_ = cudaStreamSynchronize(0);  // the run's streams do not wait on stream 0
            if (e_ != cudaSuccess) { g_err = std::string("static masks: ") + cudaGetErrorString(e_); fsibe_destroy(c); return FSIBE_ERR_CUDA; }
        }
    }
    if (c->fp32) {
        std::vector<float2> tX, tR, tY;
        make_table(tX, p->nx / 2, p->nx / 2);
        make_table(tR, p->nx, p->nx / 2 + 1);
        make_table(tY, p->ny, p->ny);
        ALLOC(c->twX, 8 * tX.size()); ALLOC(c->twR, 8 * tR.size()); ALLOC(c->twY, 8 * tY.size());
        cudaMemcpy(c->twX, tX.data(), 8 * tX.size(), cudaMemcpyHostToDevice);
        cudaMemcpy(c->twR, tR.data(), 8 * tR.size(), cudaMemcpyHostToDevice);
        cudaMemcpy(c->twY, tY.data(), 8 * tY.size(), cudaMemcpyHostToDevice);
    } else {
        std::vector<double2> tX, tR, tY;
        make_table(tX, p->nx / 2, p->nx / 2);
        make_table(tR, p->nx, p->nx / 2 + 1);
        make_table(tY, p->ny, p->ny);
        ALLOC(c->twX, 16 * tX.size()); ALLOC(c->twR, 16 * tR.size()); ALLOC(c->twY, 16 * tY.size());
        cudaMemcpy(c->twX, tX.data(), 16 * tX.size(), cudaMemcpyHostToDevice);
        cudaMemcpy(c->twR, tR.data(), 16 * tR.size(), cudaMemcpyHostToDevice);
        cudaMemcpy(c->twY, tY.data(), 16 * tY.size(), cudaMemcpyHostToDevice);
    }
#undef ALLOC
    {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, dev);
        if (c->nsm <= 0) c->nsm = 152;
    }
    // with the advection part pipelined, the main stream has the greatest priority and the
    // second side stream the least: the next step's advection part then fills the SMs that the
    // pressure and beam kernels leave, without holding them back (the graph keeps the
    // priorities: cudaGraphInstantiateFlagUseNodePriority)
    int prio_lo = 0, prio_hi = 0;
    cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
    {
        // on by default from 2048^2 on, where the advection part outlasts the mask kernels it
        // otherwise runs beside (4096^2: the step 1.61 -> 1.46 ms); at 1024^2 it is hidden there
        // already and the pipelined form was 2.5% slower.  FSIBE_ADV_PIPE = 0 / 1 overrides.
        const char* pe = std::getenv("FSIBE_ADV_PIPE");
        c->adv_pipe = pe ? std::atoi(pe) != 0 : (long long)p->nx * p->ny >= 2048LL * 2048LL;
    }
    if (!c->adv_pipe) prio_lo = prio_hi = 0;
    cudaError_t e = cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, prio_hi);
    if (e != cudaSuccess) { g_err = cudaGetErrorString(e); fsibe_destroy(c); return FSIBE_ERR_CUDA; }
    c->own_stream = true;
    cudaEventCreate(&c->ev0);
    cudaEventCreate(&c->ev1);
    e = cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking);
    if (e != cudaSuccess) { g_err = cudaGetErrorString(e); fsibe_destroy(c); return FSIBE_ERR_CUDA; }
    cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming);
    e = cudaStreamCreateWithPriority(&c->side2, cudaStreamNonBlocking, prio_lo);
    if (e != cudaSuccess) { g_err = cudaGetErrorString(e); fsibe_destroy(c); return FSIBE_ERR_CUDA; }
    cudaEventCreateWithFlags(&c->ev_ff, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&c->ev_ffj, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&c->ev_sb0, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&c->ev_geo, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&c->ev_adv, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&c->ev_ny, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&c->ev_sb, cudaEventDisableTiming);
    {
        const int st = c->fp32 ? autotune_x<float>(c) : autotune_x<double>(c);
        if (st) { g_err = c->err; fsibe_destroy(c); return st; }
        // FSIBE_PX_PAIRED = 1 / 0 forces / forbids the paired FP32 press_x (tests of both forms)
        const char* pe = std::getenv("FSIBE_PX_PAIRED");
        if (pe && c->fp32) {
            if (pe[0] == '1' && c->g.ny % c->kxf.xp.rows == 0) c->xv_px = 4;
            else if (pe[0] == '0' && c->xv_px == 4) c->xv_px = 1;
        }
        // FSIBE_PY_ENG = 0 / 1 forces k_press_y's paired / one-butterfly engine (FP32)
        const char* ye = std::getenv("FSIBE_PY_ENG");
        if (ye && c->fp32) c->py_eng = (ye[0] == '1') ? 1 : 0;
    }
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess) { g_err = std::string("create: ") + cudaGetErrorString(e); fsibe_destroy(c); return FSIBE_ERR_CUDA; }
    *out = c;
    return FSIBE_OK;
}

int fsibe_set_stream(fsibe_ctx* c, void* stream) {
    if (!c) return FSIBE_ERR_PARAM;
    CK(c, cudaStreamSynchronize(c->stream));
    free_graph(c);
    if (c->own_stream) { cudaStreamDestroy(c->stream); c->own_stream = false; }
    c->stream = reinterpret_cast<cudaStream_t>(stream);
    return FSIBE_OK;
}

int fsibe_use_graph(fsibe_ctx* c, int enable) {
    if (!c) return FSIBE_ERR_PARAM;
    if (!enable) free_graph(c);
    c->use_graph = enable != 0;
    return FSIBE_OK;
}

// ---- spectral operators on packed arrays --------------------------------------------
int fsibe_fft_forward(fsibe_ctx* c, const double* f, double* fk) {
    if (!c || !f || !fk) return FSIBE_ERR_PARAM;
    int st = from_host(c, f, (size_t)c->g.nx * c->g.ny, c->phys[PH_0]);
    if (st) return st;
    st = c->fp32 ? fwd2d<float>(c, c->spec[SP_1]) : fwd2d<double>(c, c->spec[SP_1]);
    if (st) return st;
    return spec_to_packed(c, c->spec[SP_1], fk);
}

int fsibe_fft_inverse(fsibe_ctx* c, const double* fk, double* f) {
    if (!c || !f || !fk) return FSIBE_ERR_PARAM;
    int st = packed_to_spec(c, fk, c->spec[SP_1]);
    if (st) return st;
    if (c->fp32) {
        if ((st = inv_y<float>(c, c->spec[SP_1], c->spec[SP_0], OP_ID))) return st;
        if ((st = inv_x<float>(c))) return st;
    } else {
        if ((st = inv_y<double>(c, c->spec[SP_1], c->spec[SP_0], OP_ID))) return st;
        if ((st = inv_x<double>(c))) return st;
    }
    return to_host(c, c->phys[PH_0], (size_t)c->g.nx * c->g.ny, f);
}

static int packed_op(fsibe_ctx* c, const double* in, double* out, int op, double dt) {
    if (!c || !out) return FSIBE_ERR_PARAM;
    const size_t NN = (size_t)c->g.nx * c->g.ny;
    if (in) CK(c, cudaMemcpyAsync(c->dscratch, in, 8 * NN, cudaMemcpyHostToDevice, c->stream));
    k_packed_op<<<512, 256, 0, c->stream>>>(c->dscratch, c->dscratch2, op, c->g.nx, c->g.ny, c->P.xl, c->P.yl, c->g.pi,
                                            c->g.scalex, c->g.scaley, c->P.nu, dt, c->P.idealis);
    CKL(c);
    CK(c, cudaMemcpyAsync(out, c->dscratch2, 8 * NN, cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    return FSIBE_OK;
}

int fsibe_cofdx(fsibe_ctx* c, const double* a, double* b) { return packed_op(c, a, b, PK_DX, 0.0); }
int fsibe_cofdy(fsibe_ctx* c, const double* a, double* b) { return packed_op(c, a, b, PK_DY, 0.0); }
int fsibe_cofdxdx(fsibe_ctx* c, const double* a, double* b) { return packed_op(c, a, b, PK_DXDX, 0.0); }
int fsibe_cofdydy(fsibe_ctx* c, const double* a, double* b) { return packed_op(c, a, b, PK_DYDY, 0.0); }
int fsibe_cofdxdy(fsibe_ctx* c, const double* a, double* b) { return packed_op(c, a, b, PK_DXDY, 0.0); }
int fsibe_poisson(fsibe_ctx* c, const double* a, double* b) { return packed_op(c, a, b, PK_POISSON, 0.0); }
int fsibe_vis(fsibe_ctx* c, double dt, double* w) { return packed_op(c, nullptr, w, PK_VIS, dt); }
int fsibe_dealiase_mask(fsibe_ctx* c, double* d) { return packed_op(c, nullptr, d, PK_DEALIAS, 0.0); }

// ---- the time step ------------------------------------------------------------------
// init_fields (inicond=111): vorticity, velocity, scalars, beam start state; the mask is
// drawn unless keep_mask (a prescribed mask stays as it is).
static int init_state(fsibe_ctx* c, const double* vort, bool keep_mask) {
    const size_t NN = (size_t)c->g.nx * c->g.ny;
    const size_t rs = c->fp32 ? 4 : 8;
    free_graph(c);
    c->adv_ready = false;  // a new state: the next step forms its own advection part
    int st = from_host(c, vort, NN, c->phys[PH_0]);
    if (st) return st;
    for (int q : {SP_W, SP_M, SP_WLO}) CK(c, cudaMemsetAsync(c->spec[q], 0, rs * NN, c->stream));
    for (int q : {PH_VORMEAN, PH_PRESS, PH_SA, PH_SB}) CK(c, cudaMemsetAsync(c->phys[q], 0, rs * NN, c->stream));
    st = c->fp32 ? fwd2d<float>(c, c->spec[SP_W]) : fwd2d<double>(c, c->spec[SP_W]);
    if (st) return st;
    DevScalars h;
    std::memset(&h, 0, sizeof(h));
    h.startup_step = 1;
    h.method = c->P.time_method_solid;
    h.grav = c->P.grav;
    c->U_mean_true = (c->P.iWalls == 1) ? 1.0 - 2.0 * c->P.h_channel / c->P.yl : 1.0;  // time_step.f90:95-100
    h.mean_u_next = c->U_mean_true * host_mean(c->P, 0.0, true);
    h.mean_v_next = c->U_mean_true * host_mean(c->P, 0.0, false);
    h.mean_u_cur = h.mean_u_next;
    h.mean_v_cur = h.mean_v_next;
    CK(c, cudaMemcpyAsync(c->S, &h, sizeof(h), cudaMemcpyHostToDevice, c->stream));
    c->pre_launched = false;
    launch_init_beam(beam_args(c), c->stream);
    CKL(c);
    st = c->fp32 ? init_velocity<float>(c) : init_velocity<double>(c);
    if (st) return st;
    if (!keep_mask) {
        st = create_mask(c);
        if (st) return st;
        if ((st = sponge_mask(c))) return st;
    }
    CK(c, cudaStreamSynchronize(c->stream));
    c->initialized = true;
    c->startup_done = false;
    return FSIBE_OK;
}

static int read_status(fsibe_ctx* c);
static int set_time(fsibe_ctx* c, double time);

int fsibe_init_fields(fsibe_ctx* c, const double* vort) {
    if (!c || !vort) return FSIBE_ERR_PARAM;
    return init_state(c, vort, false);
}

int fsibe_create_mask(fsibe_ctx* c, double time) {
    if (!c) return FSIBE_ERR_PARAM;
    int st = set_time(c, time);  // the motion and the mean flow of the time
    if (st) return st;
    st = create_mask(c);
    if (st) return st;
    return read_status(c);  // a beam point below the domain: FSIBE_ERR_MASK_OOB
}

static int read_status(fsibe_ctx* c) {
    int32_t s = 0;
    CK(c, cudaMemcpyAsync(&s, &c->S->status, 4, cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    if (s) c->err = fsibe_strerror(s);
    return s;
}

int fsibe_fluid_step(fsibe_ctx* c, int explicit_step) {
    if (!c) return FSIBE_ERR_PARAM;
    if (!c->initialized) return FSIBE_ERR_STATE;
    c->adv_ready = false;  // the routine's fluid step forms its nonlinear term whole
    int st = fluid_step(c, explicit_step ? 1 : 0);
    if (st) return st;
    return read_status(c);
}

static int set_time(fsibe_ctx* c, double time) {
    CK(c, cudaMemcpyAsync(&c->S->time, &time, 8, cudaMemcpyHostToDevice, c->stream));
    return FSIBE_OK;
}

int fsibe_get_forces(fsibe_ctx* c, double time) {
    if (!c) return FSIBE_ERR_PARAM;
    int st = set_time(c, time);
    if (st) return st;
    st = get_forces(c);
    if (st) return st;
    return read_status(c);
}

int fsibe_solid_step(fsibe_ctx* c, double time) {
    if (!c) return FSIBE_ERR_PARAM;
    int st = set_time(c, time);
    if (st) return st;
    st = solid_step(c);
    if (st) return st;
    return read_status(c);
}

int fsibe_advance(fsibe_ctx* c) {
    if (!c) return FSIBE_ERR_PARAM;
    int st = advance(c);
    if (st) return st;
    if (!c->startup_done) c->startup_done = true;
    return read_status(c);
}

int fsibe_step(fsibe_ctx* c) {
    if (!c) return FSIBE_ERR_PARAM;
    return do_step(c);
}

// nsteps steps with the per-step records kept in the device ring (FSIBE_RECORD_COLS a step);
// cols = 21 copies the beam_data rows alone (a pitched copy of the ring's first columns)
static int run_steps(fsibe_ctx* c, int nsteps, double* out, int cols) {
    if (!c || nsteps < 0) return FSIBE_ERR_PARAM;
    if (out) {
        if (c->rows_cap < nsteps) {
            if (c->rows) cudaFree(c->rows);
            c->rows = nullptr;
            CK(c, cudaMalloc((void**)&c->rows, 8 * FSIBE_RECORD_COLS * (size_t)(nsteps > 0 ? nsteps : 1)));
            c->rows_cap = nsteps;
            free_graph(c);  // the graph captured the old ring pointer
        }
        int32_t z[2] = {0, nsteps};
        CK(c, cudaMemcpyAsync(&c->S->run_row, z, 8, cudaMemcpyHostToDevice, c->stream));
    } else {
        int32_t z[2] = {0, 0};
        CK(c, cudaMemcpyAsync(&c->S->run_row, z, 8, cudaMemcpyHostToDevice, c->stream));
    }
    for (int s = 0; s < nsteps; ++s) {
        int st = do_step(c);
        if (st) return st;
    }
    if (out && nsteps > 0)
        CK(c, cudaMemcpy2DAsync(out, 8 * (size_t)cols, c->rows, 8 * (size_t)FSIBE_RECORD_COLS, 8 * (size_t)cols,
                                (size_t)nsteps, cudaMemcpyDeviceToHost, c->stream));
    return read_status(c);
}

int fsibe_run(fsibe_ctx* c, int nsteps, double* rows) { return run_steps(c, nsteps, rows, 21); }

int fsibe_run_records(fsibe_ctx* c, int nsteps, double* records) {
    return run_steps(c, nsteps, records, FSIBE_RECORD_COLS);
}

// ---- state transfer -------------------------------------------------------------------
int fsibe_upload_vortk(fsibe_ctx* c, const double* v) {
    if (!c) return FSIBE_ERR_PARAM;
    c->adv_ready = false;
    return packed_to_spec(c, v, c->spec[SP_W], c->fp32 ? c->spec[SP_WLO] : nullptr);
}
int fsibe_download_vortk(fsibe_ctx* c, double* v) {
    return c ? spec_to_packed(c, c->spec[SP_W], v, c->fp32 ? c->spec[SP_WLO] : nullptr) : FSIBE_ERR_PARAM;
}
int fsibe_download_vort(fsibe_ctx* c, double* v) {
    if (!c) return FSIBE_ERR_PARAM;
    int st;
    if (c->fp32) {
        if ((st = inv_y<float>(c, c->spec[SP_W], c->spec[SP_0], OP_ID))) return st;
        if ((st = inv_x<float>(c))) return st;
    } else {
        if ((st = inv_y<double>(c, c->spec[SP_W], c->spec[SP_0], OP_ID))) return st;
        if ((st = inv_x<double>(c))) return st;
    }
    return to_host(c, c->phys[PH_0], (size_t)c->g.nx * c->g.ny, v);
}
// The FP32 form stores u - U (U = mean flow of that velocity, kept as FP64 scalars).
int fsibe_upload_u(fsibe_ctx* c, const double* u) {
    if (!c) return FSIBE_ERR_PARAM;
    c->adv_ready = false;
    const size_t NN = (size_t)c->g.nx * c->g.ny;
    const double* ou = c->fp32 ? &c->S->mean_u_cur : nullptr;
    const double* ov = c->fp32 ? &c->S->mean_v_cur : nullptr;
    int st = from_host(c, u, NN, c->phys[PH_U], ou);
    return st ? st : from_host(c, u + NN, NN, c->phys[PH_V], ov);
}
int fsibe_download_u(fsibe_ctx* c, double* u) {
    if (!c) return FSIBE_ERR_PARAM;
    const size_t NN = (size_t)c->g.nx * c->g.ny;
    const double* ou = c->fp32 ? &c->S->mean_u_cur : nullptr;
    const double* ov = c->fp32 ? &c->S->mean_v_cur : nullptr;
    int st = to_host(c, c->phys[PH_U], NN, u, ou);
    return st ? st : to_host(c, c->phys[PH_V], NN, u + NN, ov);
}
int fsibe_download_press(fsibe_ctx* c, double* p) {
    if (!c) return FSIBE_ERR_PARAM;
    const int st = ensure_press(c);
    return st ? st : to_host(c, c->phys[PH_PRESS], (size_t)c->g.nx * c->g.ny, p);
}
int fsibe_upload_press(fsibe_ctx* c, const double* p) {
    if (!c) return FSIBE_ERR_PARAM;
    c->press_partial = false;
    return from_host(c, p, (size_t)c->g.nx * c->g.ny, c->phys[PH_PRESS]);
}
int fsibe_download_vor_mean(fsibe_ctx* c, double* p) { return c ? to_host(c, c->phys[PH_VORMEAN], (size_t)c->g.nx * c->g.ny, p) : FSIBE_ERR_PARAM; }
int fsibe_upload_mask(fsibe_ctx* c, const double* m, const double* vx, const double* vy) {
    if (!c) return FSIBE_ERR_PARAM;
    const size_t NN = (size_t)c->g.nx * c->g.ny;
    int st = from_host(c, m, NN, c->phys[PH_MASK]);
    if (!st) st = from_host(c, vx, NN, c->phys[PH_MVX]);
    if (!st) st = from_host(c, vy, NN, c->phys[PH_MVY]);
    if (st) return st;
    // any cell may be non-zero now: the next raster pass clears the whole grid
    const int full[4] = {0, c->g.nx - 1, 0, c->g.ny - 1};
    CK(c, cudaMemcpyAsync(c->rect, full, sizeof(full), cudaMemcpyHostToDevice, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    return FSIBE_OK;
}
int fsibe_download_mask(fsibe_ctx* c, double* m, double* vx, double* vy) {
    if (!c) return FSIBE_ERR_PARAM;
    const size_t NN = (size_t)c->g.nx * c->g.ny;
    int st = to_host(c, c->phys[PH_MASK], NN, m);
    if (!st) st = to_host(c, c->phys[PH_MVX], NN, vx);
    if (!st) st = to_host(c, c->phys[PH_MVY], NN, vy);
    return st;
}
int fsibe_upload_beam(fsibe_ctx* c, const double* beam, const double* po, const double* pn, const double* to,
                      const double* tn) {
    if (!c) return FSIBE_ERR_PARAM;
    const size_t ns = (size_t)c->P.ns;
    if (beam) for (int q = 0; q < 6; ++q) CK(c, cudaMemcpyAsync(c->beam[q == 4 ? B_TH : (q == 5 ? B_THD : q)], beam + q * ns, 8 * ns, cudaMemcpyHostToDevice, c->stream));
    if (po) CK(c, cudaMemcpyAsync(c->beam[B_PO], po, 8 * ns, cudaMemcpyHostToDevice, c->stream));
    if (pn) CK(c, cudaMemcpyAsync(c->beam[B_PN], pn, 8 * ns, cudaMemcpyHostToDevice, c->stream));
    if (to) CK(c, cudaMemcpyAsync(c->beam[B_TO], to, 8 * ns, cudaMemcpyHostToDevice, c->stream));
    if (tn) CK(c, cudaMemcpyAsync(c->beam[B_TN], tn, 8 * ns, cudaMemcpyHostToDevice, c->stream));
    CK(c, cudaMemsetAsync(&c->S->beam_fact, 0, sizeof(int32_t), c->stream));  // a new state: refactor
    c->pre_launched = false;
    CK(c, cudaStreamSynchronize(c->stream));
    return FSIBE_OK;
}
int fsibe_download_beam(fsibe_ctx* c, double* beam, double* po, double* pn, double* to, double* tn) {
    if (!c) return FSIBE_ERR_PARAM;
    const size_t ns = (size_t)c->P.ns;
    if (beam) for (int q = 0; q < 6; ++q) CK(c, cudaMemcpyAsync(beam + q * ns, c->beam[q == 4 ? B_TH : (q == 5 ? B_THD : q)], 8 * ns, cudaMemcpyDeviceToHost, c->stream));
    if (po) CK(c, cudaMemcpyAsync(po, c->beam[B_PO], 8 * ns, cudaMemcpyDeviceToHost, c->stream));
    if (pn) CK(c, cudaMemcpyAsync(pn, c->beam[B_PN], 8 * ns, cudaMemcpyDeviceToHost, c->stream));
    if (to) CK(c, cudaMemcpyAsync(to, c->beam[B_TO], 8 * ns, cudaMemcpyDeviceToHost, c->stream));
    if (tn) CK(c, cudaMemcpyAsync(tn, c->beam[B_TN], 8 * ns, cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    return FSIBE_OK;
}

// ---- BeamSurfaceIntegral (BeamForces.f90:306-509) ---------------------------------------
// From the stresses and pressure of the last fluid step and the current beam: between
// GetForces and the solid step this is the reference's call (:129).
int fsibe_pressure_snapshot(fsibe_ctx* c, double time, double* press) {
    if (!c || !press) return FSIBE_ERR_PARAM;
    if (!c->initialized) { c->err = "pressure snapshot before init_fields"; return FSIBE_ERR_STATE; }
    return c->fp32 ? pressure_snapshot_t<float>(c, time, press) : pressure_snapshot_t<double>(c, time, press);
}

int fsibe_surface_integral(fsibe_ctx* c, double time, double* out) {
    if (!c || !out) return FSIBE_ERR_PARAM;
    if (!c->initialized) { c->err = "surface_integral before init_fields"; return FSIBE_ERR_STATE; }
    if (c->P.iViscous != 1 || c->P.iBeam <= 0) { c->err = "BeamSurfaceIntegral needs iViscous = 1 and a beam"; return FSIBE_ERR_PARAM; }
    // BeamForces.f90:331-336: no surface integral with the leading-edge cylinder
    if (c->P.iCylinder == 1) { c->err = "BeamSurfaceIntegral is not computed with a cylinder at the leading edge"; return FSIBE_ERR_UNSUPPORTED; }
    const int pst = ensure_press(c);  // the contour's stencils may reach rows the step left
    if (pst) return pst;
    double dxi, dyi;
    const ForceArgs f = force_args(c, dxi, dyi);
    SurfArgs s;
    s.nx = c->g.nx; s.ny = c->g.ny; s.fp32 = c->fp32 ? 1 : 0;
    s.nblk = 2 * c->nsm;
    s.u = c->phys[PH_U]; s.v = c->phys[PH_V];
    s.mask = c->phys[PH_MASK]; s.mvx = c->phys[PH_MVX]; s.mvy = c->phys[PH_MVY];
    static_assert(offsetof(DevScalars, mean_v_cur) == offsetof(DevScalars, mean_u_cur) + sizeof(double), "U, V adjacent");
    s.mean = &c->S->mean_u_cur;  // mean_u_cur, mean_v_cur
    s.part = c->dscratch;          // 2 nblk + 11 doubles of the nx ny scratch
    s.out = c->dscratch + 2 * s.nblk;
    launch_surface_integral(f, s, dxi, dyi, time, c->stream);
    CKL(c);
    CK(c, cudaMemcpyAsync(out, s.out, 8 * 11, cudaMemcpyDeviceToHost, c->stream));
    const int st = read_status(c);
    if (c->P.iWalls > 0) out[1] = out[2] = 0.0;  // with walls the file's drag and lift are 0 (BeamForces.f90:494-502)
    return st;
}

// ---- runtime backup (save_fields.f90:109-152, init_fields.f90:44-100) ------------------
// Fortran sequential unformatted records: a 4-byte length before and after each record;
// reals are 8 bytes, integers and logicals 4.
namespace {
struct BackupOut {
    FILE* f = nullptr;
    std::vector<char> rec;
    bool ok = true;
    void put(const void* p, size_t n) { const char* q = static_cast<const char*>(p); rec.insert(rec.end(), q, q + n); }
    void d(double v) { put(&v, 8); }
    void i(int32_t v) { put(&v, 4); }
    void dv(const double* p, size_t n) { put(p, 8 * n); }
    void end() {
        const int32_t n = (int32_t)rec.size();
        ok = ok && fwrite(&n, 4, 1, f) == 1 && (rec.empty() || fwrite(rec.data(), 1, rec.size(), f) == rec.size()) &&
             fwrite(&n, 4, 1, f) == 1;
        rec.clear();
    }
};
struct BackupIn {
    FILE* f = nullptr;
    std::vector<char> rec;
    size_t pos = 0;
    bool ok = true;
    void next() {
        int32_t n = -1, m = -2;
        ok = ok && fread(&n, 4, 1, f) == 1 && n >= 0;
        if (ok) rec.resize((size_t)n);
        ok = ok && (n == 0 || fread(rec.data(), 1, (size_t)n, f) == (size_t)n) && fread(&m, 4, 1, f) == 1 && m == n;
        pos = 0;
    }
    void get(void* p, size_t n) {
        ok = ok && pos + n <= rec.size();
        if (ok) std::memcpy(p, rec.data() + pos, n);
        pos += n;
    }
    double d() { double v = 0.0; get(&v, 8); return v; }
    int32_t i() { int32_t v = 0; get(&v, 4); return v; }
    void dv(double* p, size_t n) { get(p, 8 * n); }
};
}  // namespace

// The state between two steps as MakeRuntimeBackup writes it.  The AB2 history is stored as
// the product the next step forms first (nlk(n1) workvis(n0), NavierStokes.f90:480): nlk(n1)
// holds it and workvis(n0) is one, so the reference and this library both resume from the
// same history.
int fsibe_write_backup(fsibe_ctx* c, const char* path) {
    if (!c || !path) return FSIBE_ERR_PARAM;
    if (!c->initialized) { c->err = "write_backup before init_fields"; return FSIBE_ERR_STATE; }
    const size_t NN = (size_t)c->g.nx * c->g.ny, ns = (size_t)c->P.ns;
    std::vector<double> W(NN), M(NN), zero(NN, 0.0), one(NN, 1.0), mk(3 * NN), u(2 * NN), vm(NN);
    int st = spec_to_packed(c, c->spec[SP_W], W.data(), c->fp32 ? c->spec[SP_WLO] : nullptr);
    if (!st) st = spec_to_packed(c, c->spec[SP_M], M.data());
    if (!st) st = fsibe_download_mask(c, mk.data(), mk.data() + NN, mk.data() + 2 * NN);
    if (!st) st = fsibe_download_u(c, u.data());
    if (!st) st = fsibe_download_vor_mean(c, vm.data());
    if (st) return st;
    std::vector<double> bm(B_N * ns), oo(6 * ns);
    for (int q = 0; q < B_N; ++q) CK(c, cudaMemcpyAsync(bm.data() + q * ns, c->beam[q], 8 * ns, cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaMemcpyAsync(oo.data(), c->oo, 8 * 6 * ns, cudaMemcpyDeviceToHost, c->stream));
    DevScalars h;
    CK(c, cudaMemcpyAsync(&h, c->S, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    BackupOut o;
    o.f = std::fopen(path, "wb");
    if (!o.f) { c->err = "cannot open the backup file for writing"; return FSIBE_ERR_PARAM; }
    o.d(h.time); o.end();
    o.d(123.0); o.end();
    o.i(1); o.d(h.dt1);
    o.dv(W.data(), NN); o.dv(zero.data(), NN);   // vortk(n0 = 0) current, vortk(n1) unused
    o.dv(zero.data(), NN); o.dv(M.data(), NN);   // nlk(n0) unused, nlk(n1) the history
    o.dv(one.data(), NN); o.dv(zero.data(), NN); // workvis(n0) = 1
    o.dv(mk.data(), 3 * NN);
    o.i(1);  // ivideo
    o.dv(u.data(), 2 * NN);
    o.end();
    o.i(c->P.ns); o.end();
    o.d(0.0); o.i(0); o.end();  // colorscale, colorscale_done
    if (c->P.iBeam > 0) {
        for (int q : {B_X, B_Y, B_VX, B_VY, B_TH, B_THD}) o.dv(bm.data() + q * ns, ns);
        o.end();
        for (int q : {B_PN, B_PO, B_TN, B_TO}) o.dv(bm.data() + q * ns, ns);
        o.end();
        o.dv(h.force, 2); o.dv(h.force_unst, 2); o.dv(h.force_press, 2);
        o.d(h.e_kinetic); o.d(h.e_pot); o.d(h.e_elastic); o.d(c->P.x0); o.d(c->P.y0);
        o.end();
        o.d(c->P.angle_beam); o.i(c->P.iMotion);
        // drag_unst_new, _old, lift_unst_new, _old: cal_drag ends every step with old = new
        // (NavierStokes.f90:583-584), so between steps both slots hold the one tracked value
        o.d(h.drag_unst_old); o.d(h.drag_unst_old); o.d(h.lift_unst_old); o.d(h.lift_unst_old);
        o.end();
        o.i(h.unst_ready ? 1 : 0); o.d(h.dt_old); o.dv(oo.data(), 6 * ns);
        o.end();
        o.dv(bm.data() + B_AX * ns, ns); o.dv(bm.data() + B_AY * ns, ns); o.dv(h.inertial_force, 2);
        o.end();
    }
    o.dv(vm.data(), NN); o.end();
    const bool ok = (std::fclose(o.f) == 0) && o.ok;
    if (!ok) { c->err = "writing the backup file failed"; return FSIBE_ERR_PARAM; }
    return FSIBE_OK;
}

// Resume: init_beams and InitializeSolidSolver (the next solid step is a Crank-Nicolson
// start-up step), the records, n0 = 1 - n1, the start-up mask (time_step.f90:60-84); no Euler
// start-up step follows.  The velocity statistics of the first step come from the file's u.
int fsibe_read_backup(fsibe_ctx* c, const char* path) {
    if (!c || !path) return FSIBE_ERR_PARAM;
    c->adv_ready = false;
    const size_t NN = (size_t)c->g.nx * c->g.ny, ns = (size_t)c->P.ns;
    BackupIn in;
    in.f = std::fopen(path, "rb");
    if (!in.f) { c->err = "cannot open the backup file"; return FSIBE_ERR_PARAM; }
    std::vector<double> vortk(2 * NN), nlk(2 * NN), workvis(2 * NN), mk(3 * NN), u(2 * NN), vm(NN);
    std::vector<double> bm(B_N * ns, 0.0), oo(6 * ns, 0.0);
    double force[2] = {0, 0}, force_unst[2] = {0, 0}, force_press[2] = {0, 0}, inertial[2] = {0, 0};
    double ek = 0, ep = 0, ee = 0, dun = 0, duo = 0, lun = 0, luo = 0, dt_old = 0;
    int32_t ready = 0;
    in.next(); const double time = in.d();
    in.next(); const bool sum_ok = in.d() == 123.0;
    in.next();
    const int32_t n1 = in.i();
    const double dt1 = in.d();
    in.dv(vortk.data(), 2 * NN); in.dv(nlk.data(), 2 * NN); in.dv(workvis.data(), 2 * NN);
    in.dv(mk.data(), 3 * NN);
    (void)in.i();  // ivideo
    in.dv(u.data(), 2 * NN);
    in.next(); const bool ns_ok = in.i() == c->P.ns;
    in.next(); (void)in.d(); (void)in.i();  // colorscale, colorscale_done
    if (in.ok && ns_ok && c->P.iBeam > 0) {
        in.next();
        for (int q : {B_X, B_Y, B_VX, B_VY, B_TH, B_THD}) in.dv(bm.data() + q * ns, ns);
        in.next();
        for (int q : {B_PN, B_PO, B_TN, B_TO}) in.dv(bm.data() + q * ns, ns);
        in.next();
        in.dv(force, 2); in.dv(force_unst, 2); in.dv(force_press, 2);
        ek = in.d(); ep = in.d(); ee = in.d(); (void)in.d(); (void)in.d();  // x0, y0 come from the parameters
        in.next();
        (void)in.d(); (void)in.i();  // AngleBeam, iMouvement come from the parameters
        dun = in.d(); duo = in.d(); lun = in.d(); luo = in.d();
        in.next();
        ready = in.i(); dt_old = in.d(); in.dv(oo.data(), 6 * ns);
        in.next();
        in.dv(bm.data() + B_AX * ns, ns); in.dv(bm.data() + B_AY * ns, ns); in.dv(inertial, 2);
    }
    in.next(); in.dv(vm.data(), NN);
    std::fclose(in.f);
    (void)dun; (void)lun;
    if (!in.ok || !sum_ok || !ns_ok || (n1 != 0 && n1 != 1)) {
        c->err = "not a runtime backup of this configuration (record, checksum or ns)";
        return FSIBE_ERR_PARAM;
    }
    const int n0 = 1 - n1;
    // the AB2 history nlk(n1) workvis(n0), formed as the next step would
    std::vector<double> M(NN);
    for (size_t i = 0; i < NN; ++i) M[i] = nlk[n1 * NN + i] * workvis[n0 * NN + i];
    free_graph(c);
    const size_t rs = c->fp32 ? 4 : 8;
    int st = packed_to_spec(c, vortk.data() + n0 * NN, c->spec[SP_W], c->fp32 ? c->spec[SP_WLO] : nullptr);
    if (!st) st = packed_to_spec(c, M.data(), c->spec[SP_M]);
    if (st) return st;
    for (int q : {PH_PRESS, PH_SA, PH_SB}) CK(c, cudaMemsetAsync(c->phys[q], 0, rs * NN, c->stream));
    if ((st = from_host(c, vm.data(), NN, c->phys[PH_VORMEAN]))) return st;
    DevScalars h;
    std::memset(&h, 0, sizeof(h));
    h.time = time; h.dt1 = dt1; h.dt0 = dt1; h.dt_old = dt_old;
    h.startup_step = 1;
    h.method = c->P.time_method_solid;
    h.grav = c->P.grav;
    h.unst_ready = ready ? 1 : 0;
    h.drag_unst_old = duo; h.lift_unst_old = luo;
    for (int k = 0; k < 2; ++k) {
        h.force[k] = force[k]; h.force_unst[k] = force_unst[k]; h.force_press[k] = force_press[k]; h.inertial_force[k] = inertial[k];
    }
    h.e_kinetic = ek; h.e_pot = ep; h.e_elastic = ee;
    c->U_mean_true = (c->P.iWalls == 1) ? 1.0 - 2.0 * c->P.h_channel / c->P.yl : 1.0;
    h.mean_u_next = h.mean_u_cur = c->U_mean_true * host_mean(c->P, time, true);
    h.mean_v_next = h.mean_v_cur = c->U_mean_true * host_mean(c->P, time, false);
    CK(c, cudaMemcpyAsync(c->S, &h, sizeof(h), cudaMemcpyHostToDevice, c->stream));
    c->pre_launched = false;
    if (c->P.iBeam > 0) {
        for (int q = 0; q < B_N; ++q) CK(c, cudaMemcpyAsync(c->beam[q], bm.data() + q * ns, 8 * ns, cudaMemcpyHostToDevice, c->stream));
        CK(c, cudaMemcpyAsync(c->oo, oo.data(), 8 * 6 * ns, cudaMemcpyHostToDevice, c->stream));
    }
    // the spectra the first step's x-pass reads, then the file's velocity over the one formed here
    st = c->fp32 ? init_velocity<float>(c) : init_velocity<double>(c);
    if (!st) st = fsibe_upload_u(c, u.data());
    if (st) return st;
    // the first step's dt and mean velocity (cal_nlk's statistics of u) from the file's u
    std::vector<double> red(RED_NSLOTS, 0.0);
    for (size_t i = 0; i < NN; ++i) {
        red[RED_UMAX2] = std::max(red[RED_UMAX2], u[i] * u[i] + u[NN + i] * u[NN + i]);
        red[RED_SUM_U] += u[i];
        red[RED_SUM_V] += u[NN + i];
    }
    const int32_t one_block = 1;
    CK(c, cudaMemcpyAsync(c->red, red.data(), 8 * RED_NSLOTS, cudaMemcpyHostToDevice, c->stream));
    CK(c, cudaMemcpyAsync(&c->S->nred, &one_block, 4, cudaMemcpyHostToDevice, c->stream));
    if ((st = create_mask(c))) return st;
    if ((st = sponge_mask(c))) return st;
    CK(c, cudaStreamSynchronize(c->stream));
    c->initialized = true;
    c->startup_done = true;
    return FSIBE_OK;
}

int fsibe_get_scalars(fsibe_ctx* c, fsibe_scalars* o) {
    if (!c || !o) return FSIBE_ERR_PARAM;
    DevScalars h;
    CK(c, cudaMemcpyAsync(&h, c->S, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    std::memset(o, 0, sizeof(*o));
    o->time = h.time; o->dt0 = h.dt0; o->dt1 = h.dt1;
    o->u_max = h.u_max; o->mean_ux = h.mean_ux; o->mean_uy = h.mean_uy;
    o->vor_rms = h.vor_rms; o->kinetic = h.kinetic; o->dissipation = h.dissipation;
    o->porous_diss = h.porous_diss; o->inflow_solid = h.inflow_solid; o->inflow_mean = h.inflow_mean;
    for (int q = 0; q < 2; ++q) {
        o->force[q] = h.force[q]; o->force_unst[q] = h.force_unst[q];
        o->force_press[q] = h.force_press[q]; o->inertial_force[q] = h.inertial_force[q];
    }
    o->e_kinetic = h.e_kinetic; o->e_elastic = h.e_elastic; o->e_pot = h.e_pot;
    for (int q = 0; q < 21; ++q) o->beam_data[q] = h.row[q];
    o->newton_iters = h.newton_iters;
    o->status = h.status;
    o->step = h.step;
    return FSIBE_OK;
}

int fsibe_time_steps(fsibe_ctx* c, int nsteps, float* ms) {
    if (!c || !ms) return FSIBE_ERR_PARAM;
    CK(c, cudaEventRecord(c->ev0, c->stream));
    for (int s = 0; s < nsteps; ++s) {
        int st = do_step(c);
        if (st) return st;
    }
    CK(c, cudaEventRecord(c->ev1, c->stream));
    CK(c, cudaEventSynchronize(c->ev1));
    CK(c, cudaEventElapsedTime(ms, c->ev0, c->ev1));
    return read_status(c);
}

int fsibe_kernel_times(fsibe_ctx* c, int nsteps, fsibe_kernel_time* out, int cap, int* count) {
    if (!c || !out || !count || cap <= 0) return FSIBE_ERR_PARAM;
    CK(c, cudaStreamSynchronize(c->stream));
    const bool graph = c->use_graph;
    c->use_graph = false;
    c->profiling = true;
    c->prof.clear();
    c->pool_used = 0;
    int st = FSIBE_OK;
    for (int s = 0; s < nsteps && !st; ++s) st = do_step(c);
    c->profiling = false;
    c->use_graph = graph;
    if (st) return st;
    CK(c, cudaStreamSynchronize(c->stream));
    int n = 0;
    for (auto& r : c->prof) {
        float ms = 0.f;
        CK(c, cudaEventElapsedTime(&ms, c->pool[r.second], c->pool[r.second + 1]));
        int k = 0;
        while (k < n && std::strncmp(out[k].name, r.first, sizeof(out[k].name)) != 0) ++k;
        if (k == n) {
            if (n == cap) continue;
            std::memset(&out[n], 0, sizeof(out[n]));
            std::strncpy(out[n].name, r.first, sizeof(out[n].name) - 1);
            ++n;
        }
        out[k].ms_total += ms;
        out[k].launches += 1;
    }
    *count = n;
    c->prof.clear();
    return read_status(c);
}

int fsibe_beam_phase_cycles(fsibe_ctx* c, long long* out32, int reset) {
    if (!c || !out32) return FSIBE_ERR_PARAM;
    CK(c, cudaMemcpyAsync(out32, c->S->phase, 32 * sizeof(long long), cudaMemcpyDeviceToHost, c->stream));
    if (reset) CK(c, cudaMemsetAsync(c->S->phase, 0, 32 * sizeof(long long), c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    return FSIBE_OK;
}

int fsibe_press_y_engine(fsibe_ctx* c, int32_t* eng) {
    if (!c || !eng) return FSIBE_ERR_PARAM;
    *eng = c->fp32 ? c->py_eng : 1;
    return FSIBE_OK;
}

int fsibe_tile_config(fsibe_ctx* c, int32_t* out6) {
    if (!c || !out6) return FSIBE_ERR_PARAM;
    const int idx[3] = {c->xv_nl, c->xv_px, c->xv_fin};
    for (int q = 0; q < 3; ++q) {
        const auto& vf = idx[q] == 4 ? c->kxf.xp : c->kxf.xv[idx[q]];
        const auto& vd = c->kxd.xv[idx[q] < 4 ? idx[q] : 1];
        out6[2 * q] = c->fp32 ? vf.rows : vd.rows;
        out6[2 * q + 1] = c->fp32 ? vf.minb : vd.minb;
    }
    return FSIBE_OK;
}

int fsibe_tiles(fsibe_ctx* c, int32_t* rows3) {
    if (!c || !rows3) return FSIBE_ERR_PARAM;
    if (c->fp32) {
        rows3[0] = c->kxf.xv[c->xv_nl].rows; rows3[1] = c->xv_px == 4 ? c->kxf.xp.rows : c->kxf.xv[c->xv_px].rows;
        rows3[2] = c->kxf.xv[c->xv_fin].rows;
    } else {
        rows3[0] = c->kxd.xv[c->xv_nl].rows; rows3[1] = c->kxd.xv[c->xv_px].rows; rows3[2] = c->kxd.xv[c->xv_fin].rows;
    }
    return FSIBE_OK;
}

int fsibe_beam_cluster(fsibe_ctx* c, int32_t* ctas) {
    if (!c || !ctas) return FSIBE_ERR_PARAM;
    *ctas = c->beam_cl;
    return FSIBE_OK;
}

int fsibe_launches_per_step(fsibe_ctx* c, int* n) {
    if (!c || !n) return FSIBE_ERR_PARAM;
    const fsibe_params& P = c->P;
    int k = 6;  // step_begin, nl_x, nl_y, press_x, fluid_finish, advance
    if (P.iViscous == 1 && c->stress_split) k += 1;  // k_stress_x
    if (P.iFLUSI == 1 || P.iSaveBeam > 0) k += 2 + 2;  // press_y, press_fin, forces geometry, forces
    // mask prep + raster, and nl_x split into its advection and penalization parts
    if ((P.iFLUSI == 1 || P.iMotion > 0 || P.iSponge >= 4) && P.iBeam > 0) k += c->nl_split ? 3 : 2;
    if (c->s10) k += 3;  // du/dx (inverse y, inverse x) and the outflow sponge's integral
    if (P.iFLUSI == 1) k += 2;  // beam predictor + beam
    if (P.iFLUSI == 0 && P.iMotion > 0) k += 1;  // k_move_beam
    if (P.iFLUSI == 1 && c->beam_cl) k -= 1;  // the cluster beam kernel ends the step itself
    *n = k;
    return FSIBE_OK;
}

}  // extern "C"

// =====================================================================================
// Adjoint of the fluid step on a prescribed rigid mask, with binomial checkpointing
// =====================================================================================
// Objective: J = mean over the steps n in [avg_from, nsteps] of the drag after step n (the
// first step is the Euler start-up step).  Gradients of J with respect to the initial
// vorticity field, the mask field (the reference's `mask` array, chi / eta) and nu.  The
// forward states (W, M, u, v, scalars) are kept in snapshot slots; the reverse sweep follows
// the schedule that minimises recomputed forward steps for the given number of slots
// (binomial checkpointing: C(t, s) = min_j j + C(t - j, s - 1) + C(j, s)).
// A snapshot holds everything the next step reads: the state W, M, the velocity u, v, the
// inverse-y derivative spectra Tdx, Tdy that k_nl_x transforms, and the scalars.
struct AdjSlot {
    void *W = nullptr, *M = nullptr, *u = nullptr, *v = nullptr, *Tdx = nullptr, *Tdy = nullptr;
    DevScalars* S = nullptr;
};
struct AdjWork {
    std::vector<void*> spec, phys;  // spectral / physical buffers (FP64)
    std::vector<AdjSlot> slots;
    double* part = nullptr;         // block partials
    double* acc = nullptr;          // [0] J, [1] d J / d nu
    int nparts = 0;
    // schedule
    std::vector<long long> cost;
    std::vector<int> split;
    int T = 0, S = 0;
    // run state
    int reached = 0, nsteps = 0, avg_from = 0;
    int comp = 0;                   // objective: 0 mean drag, 1 mean lift
    double dt = 0.0, b10 = 0.0, b11 = 0.0, cobj = 0.0;
    int win[4] = {0, 0, 0, 0};
    long long fwd_steps = 0, adj_steps = 0;
};
// buffers (fields of nx*ny doubles); the blocks X (X0, X1, X2), G (G1..G4), T (transform
// scratch), P (lnl, lp2, lp1) and L (lwx, lwy, lu, lv) are contiguous, so that one launch
// transforms all of their fields
enum AdjSpec { AS_LW = 0, AS_LM, AS_LN, AS_Q, AS_X, AS_G, AS_GD, AS_WN, AS_MN, AS_T, AS_N };
enum AdjPhys { AP_WX = 0, AP_WY, AP_P, AP_L, AP_GMASK, AP_UBAR, AP_N };
static int adj_spec_fields(int i) { return i == AS_X ? 3 : (i == AS_G || i == AS_T) ? 4 : 1; }
static int adj_phys_fields(int i) { return i == AP_P ? 3 : i == AP_L ? 4 : 1; }

static void adj_free(fsibe_ctx* c) {
    AdjWork* w = c->adj;
    if (!w) return;
    for (void* p : w->spec) if (p) cudaFree(p);
    for (void* p : w->phys) if (p) cudaFree(p);
    for (AdjSlot& sl : w->slots) {
        for (void* p : {sl.W, sl.M, sl.u, sl.v, sl.Tdx, sl.Tdy}) if (p) cudaFree(p);
        if (sl.S) cudaFree(sl.S);
    }
    if (w->part) cudaFree(w->part);
    if (w->acc) cudaFree(w->acc);
    delete w;
    c->adj = nullptr;
}

static size_t adj_field_bytes(fsibe_ctx* c) { return 8 * (size_t)c->g.nx * c->g.ny; }

static int adj_alloc(fsibe_ctx* c, int nslots) {
    if (!c->adj) {
        c->adj = new AdjWork;
        AdjWork* w = c->adj;
        const size_t b = adj_field_bytes(c);
        w->spec.assign(AS_N, nullptr);
        w->phys.assign(AP_N, nullptr);
        for (int i = 0; i < AS_N; ++i) CK(c, cudaMalloc(&w->spec[i], b * adj_spec_fields(i)));
        for (int i = 0; i < AP_N; ++i) CK(c, cudaMalloc(&w->phys[i], b * adj_phys_fields(i)));
        w->nparts = 2 * c->nsm;
        CK(c, cudaMalloc((void**)&w->part, 8 * (size_t)w->nparts));
        CK(c, cudaMalloc((void**)&w->acc, 64));
    }
    AdjWork* w = c->adj;
    const size_t b = adj_field_bytes(c);
    while ((int)w->slots.size() < nslots) {
        AdjSlot sl;
        CK(c, cudaMalloc(&sl.W, b));
        CK(c, cudaMalloc(&sl.M, b));
        CK(c, cudaMalloc(&sl.u, b));
        CK(c, cudaMalloc(&sl.v, b));
        CK(c, cudaMalloc(&sl.Tdx, b));
        CK(c, cudaMalloc(&sl.Tdy, b));
        CK(c, cudaMalloc((void**)&sl.S, sizeof(DevScalars)));
        w->slots.push_back(sl);
    }
    return FSIBE_OK;
}

static AdjArgs adj_args(fsibe_ctx* c) {
    AdjWork* w = c->adj;
    AdjArgs a;
    std::memset(&a, 0, sizeof(a));
    a.g = c->g;
    a.etab = c->etab;
    a.dcut = c->dcut;
    a.b10 = w->b10; a.b11 = w->b11; a.dt = w->dt;
    auto sp = [&](int i) { return reinterpret_cast<C2<double>*>(w->spec[i]); };
    auto ph = [&](int i) { return reinterpret_cast<double*>(w->phys[i]); };
    const size_t F = (size_t)c->g.hx * c->g.ny, N = (size_t)c->g.nx * c->g.ny;
    a.lW = sp(AS_LW); a.lM = sp(AS_LM); a.lN = sp(AS_LN); a.q = sp(AS_Q);
    a.X0 = sp(AS_X); a.X1 = sp(AS_X) + F; a.X2 = sp(AS_X) + 2 * F;
    a.G1 = sp(AS_G); a.G2 = sp(AS_G) + F; a.G3 = sp(AS_G) + 2 * F; a.G4 = sp(AS_G) + 3 * F;
    a.Gd = sp(AS_GD);
    a.Wn = sp(AS_WN); a.Mn = sp(AS_MN);
    a.u = reinterpret_cast<const double*>(c->phys[PH_U]);
    a.v = reinterpret_cast<const double*>(c->phys[PH_V]);
    a.mask = reinterpret_cast<const double*>(c->phys[PH_MASK]);
    a.wx = ph(AP_WX); a.wy = ph(AP_WY);
    a.lnl = ph(AP_P); a.lp2 = ph(AP_P) + N; a.lp1 = ph(AP_P) + 2 * N;
    a.lwx = ph(AP_L); a.lwy = ph(AP_L) + N; a.lu = ph(AP_L) + 2 * N; a.lv = ph(AP_L) + 3 * N;
    a.gmask = ph(AP_GMASK); a.ubar = ph(AP_UBAR);
    a.part = w->part;
    a.S = c->S;
    a.J = w->acc;
    a.comp = w->comp;
    return a;
}

// inverse 2D transforms of nf consecutive half spectra into nf consecutive physical fields,
// x inverses of given y-inverted spectra, and forward 2D transforms of nf consecutive physical
// fields (the ordinary transform kernels, FP64, one launch per pass for all fields)
static int adj_inv2d(fsibe_ctx* c, const void* spec, int nf, void* phys) {
    KArgs<double> a = kargs<double>(c);
    a.bstride = (size_t)c->g.hx * c->g.ny;
    a.spec1 = reinterpret_cast<C2<double>*>(const_cast<void*>(spec));
    a.spec0 = reinterpret_cast<C2<double>*>(c->adj->spec[AS_T]);
    a.op = OP_ID;
    launch_y<double>(c, ky_of<double>(c).yinv, ky_of<double>(c).y_smem1, a, "adj_yinv", nf);
    a.phys0 = reinterpret_cast<double*>(phys);
    launch_x<double>(c, kx_of<double>(c).xinv, kx_of<double>(c).x_smem1, a, "adj_xinv", nf);
    CKL(c);
    return FSIBE_OK;
}
static int adj_invx(fsibe_ctx* c, const void* T, void* phys) {
    KArgs<double> a = kargs<double>(c);
    a.spec0 = reinterpret_cast<C2<double>*>(const_cast<void*>(T));
    a.phys0 = reinterpret_cast<double*>(phys);
    launch_x<double>(c, kx_of<double>(c).xinv, kx_of<double>(c).x_smem1, a, "adj_xinv");
    CKL(c);
    return FSIBE_OK;
}
static int adj_fwd2d(fsibe_ctx* c, const void* phys, int nf, void* spec) {
    KArgs<double> a = kargs<double>(c);
    a.bstride = (size_t)c->g.hx * c->g.ny;
    a.phys0 = reinterpret_cast<double*>(const_cast<void*>(phys));
    a.spec0 = reinterpret_cast<C2<double>*>(c->adj->spec[AS_T]);
    a.spec1 = reinterpret_cast<C2<double>*>(spec);
    launch_x<double>(c, kx_of<double>(c).xfwd, kx_of<double>(c).x_smem1, a, "adj_xfwd", nf);
    launch_y<double>(c, ky_of<double>(c).yfwd, ky_of<double>(c).y_smem1, a, "adj_yfwd", nf);
    CKL(c);
    return FSIBE_OK;
}

static int adj_grid(fsibe_ctx* c) { return 4 * c->nsm; }

static int adj_save(fsibe_ctx* c, int slot) {
    AdjSlot& sl = c->adj->slots[slot];
    const size_t b = adj_field_bytes(c);
    CK(c, cudaMemcpyAsync(sl.W, c->spec[SP_W], b, cudaMemcpyDeviceToDevice, c->stream));
    CK(c, cudaMemcpyAsync(sl.M, c->spec[SP_M], b, cudaMemcpyDeviceToDevice, c->stream));
    CK(c, cudaMemcpyAsync(sl.u, c->phys[PH_U], b, cudaMemcpyDeviceToDevice, c->stream));
    CK(c, cudaMemcpyAsync(sl.v, c->phys[PH_V], b, cudaMemcpyDeviceToDevice, c->stream));
    CK(c, cudaMemcpyAsync(sl.Tdx, c->spec[SP_TDX], b, cudaMemcpyDeviceToDevice, c->stream));
    CK(c, cudaMemcpyAsync(sl.Tdy, c->spec[SP_TDY], b, cudaMemcpyDeviceToDevice, c->stream));
    CK(c, cudaMemcpyAsync(sl.S, c->S, sizeof(DevScalars), cudaMemcpyDeviceToDevice, c->stream));
    return FSIBE_OK;
}
static int adj_restore(fsibe_ctx* c, int slot, int k) {
    AdjSlot& sl = c->adj->slots[slot];
    const size_t b = adj_field_bytes(c);
    CK(c, cudaMemcpyAsync(c->spec[SP_W], sl.W, b, cudaMemcpyDeviceToDevice, c->stream));
    CK(c, cudaMemcpyAsync(c->spec[SP_M], sl.M, b, cudaMemcpyDeviceToDevice, c->stream));
    CK(c, cudaMemcpyAsync(c->phys[PH_U], sl.u, b, cudaMemcpyDeviceToDevice, c->stream));
    CK(c, cudaMemcpyAsync(c->phys[PH_V], sl.v, b, cudaMemcpyDeviceToDevice, c->stream));
    CK(c, cudaMemcpyAsync(c->spec[SP_TDX], sl.Tdx, b, cudaMemcpyDeviceToDevice, c->stream));
    CK(c, cudaMemcpyAsync(c->spec[SP_TDY], sl.Tdy, b, cudaMemcpyDeviceToDevice, c->stream));
    CK(c, cudaMemcpyAsync(c->S, sl.S, sizeof(DevScalars), cudaMemcpyDeviceToDevice, c->stream));
    c->startup_done = k > 0;
    return FSIBE_OK;
}

// objective weight of the drag after step n
static double adj_weight(const AdjWork* w, int n) {
    return (n >= w->avg_from && n <= w->nsteps && n >= 1) ? w->cobj : 0.0;
}

// one forward step from state k; the first time a state is reached its drag (and velocity,
// for the mask gradient's direct term) enters the objective sums; the final state is kept
// for the viscosity term of the last step
static int adj_advance(fsibe_ctx* c, int k, bool gradient) {
    AdjWork* w = c->adj;
    int st = do_step(c);
    if (st) return st;
    w->fwd_steps++;
    const int n = k + 1;
    if (n > w->reached) {
        w->reached = n;
        const double cw = adj_weight(w, n);
        if (cw != 0.0) {
            AdjArgs a = adj_args(c);
            a.c_obj = cw;
            k_adj_accum<<<adj_grid(c), 256, 0, c->stream>>>(a, (size_t)c->g.nx * c->g.ny);
            CKL(c);
        }
        if (gradient && n == w->nsteps) {
            const size_t b = adj_field_bytes(c);
            CK(c, cudaMemcpyAsync(w->spec[AS_WN], c->spec[SP_W], b, cudaMemcpyDeviceToDevice, c->stream));
            CK(c, cudaMemcpyAsync(w->spec[AS_MN], c->spec[SP_M], b, cudaMemcpyDeviceToDevice, c->stream));
        }
    }
    return FSIBE_OK;
}

// the adjoint of step k (state k loaded): cotangents of state k+1 -> state k
static int adj_step(fsibe_ctx* c, int k) {
    AdjWork* w = c->adj;
    AdjArgs a = adj_args(c);
    const int G = adj_grid(c);
    const size_t ncell = (size_t)c->g.nx * c->g.ny;
    int st;
    // viscosity term of step k: d W'/d nu = -dt |k|^2 W', d M'/d nu = -dt |k|^2 M'
    k_adj_nu<<<w->nparts, 256, 0, c->stream>>>(a);
    k_adj_reduce<<<1, 32, 0, c->stream>>>(w->part, w->nparts, -w->dt, w->acc + 1);
    // linearisation point of step k: u, v and omega_x, omega_y exactly as k_nl_x forms them
    // (the x inverse of the state's Tdx, Tdy)
    if ((st = adj_invx(c, c->spec[SP_TDX], w->phys[AP_WX]))) return st;
    if ((st = adj_invx(c, c->spec[SP_TDY], w->phys[AP_WY]))) return st;
    a.euler = (k == 0);
    k_adj_q<<<G, 256, 0, c->stream>>>(a);
    k_adj_w3<<<G, 256, 0, c->stream>>>(a);
    // (X0, X1, X2) -> (lnl, lp2, lp1); then (lwx, lwy, lu, lv) -> (G1, G2, G3, G4)
    if ((st = adj_inv2d(c, w->spec[AS_X], 3, w->phys[AP_P]))) return st;
    k_adj_phys<<<G, 256, 0, c->stream>>>(a, ncell);
    if ((st = adj_fwd2d(c, w->phys[AP_L], 4, w->spec[AS_G]))) return st;
    a.c_obj = adj_weight(w, k);
    k_adj_combine<<<G, 256, 0, c->stream>>>(a);
    CKL(c);
    // state k for the viscosity term of step k-1
    const size_t b = adj_field_bytes(c);
    CK(c, cudaMemcpyAsync(w->spec[AS_WN], c->spec[SP_W], b, cudaMemcpyDeviceToDevice, c->stream));
    CK(c, cudaMemcpyAsync(w->spec[AS_MN], c->spec[SP_M], b, cudaMemcpyDeviceToDevice, c->stream));
    w->adj_steps++;
    return FSIBE_OK;
}

// binomial schedule: cost[t][s] forward steps to reverse t steps from a stored state with s
// free slots; split[t][s] the steps to advance before the next snapshot
static constexpr int kAdjMaxSched = 64;  // slots the schedule table covers (more: a slot per step)
static void adj_schedule(AdjWork* w, int T, int S) {
    S = S < kAdjMaxSched ? S : kAdjMaxSched;
    if (w->T == T && w->S == S) return;
    w->T = T;
    w->S = S;
    const size_t W = (size_t)S + 1;
    w->cost.assign((size_t)(T + 1) * W, 0);
    w->split.assign((size_t)(T + 1) * W, 1);
    for (int t = 1; t <= T; ++t) w->cost[(size_t)t * W] = (long long)t * (t - 1) / 2;
    for (int s = 1; s <= S; ++s)
        for (int t = 2; t <= T; ++t) {
            long long best = -1;
            int bj = 1;
            for (int j = 1; j < t; ++j) {
                const long long v = j + w->cost[(size_t)(t - j) * W + s - 1] + w->cost[(size_t)j * W + s];
                if (best < 0 || v < best) { best = v; bj = j; }
            }
            w->cost[(size_t)t * W + s] = best;
            w->split[(size_t)t * W + s] = bj;
        }
}

// reverse steps [a, a + t) with state a in slot `slot` and s free slots above it
static int adj_reverse(fsibe_ctx* c, int a, int t, int s, int slot) {
    AdjWork* w = c->adj;
    int st;
    if ((t == 1 || s == 0) && a + t == w->nsteps && w->reached < w->nsteps) {
        // the last stretch of the first sweep: the final state's drag and fields come first
        if ((st = adj_restore(c, slot, a))) return st;
        for (int k = a; k < a + t; ++k)
            if ((st = adj_advance(c, k, true))) return st;
    }
    if (t == 1) {
        if ((st = adj_restore(c, slot, a))) return st;
        return adj_step(c, a);
    }
    if (s == 0) {
        for (int k = a + t - 1; k >= a; --k) {
            if ((st = adj_restore(c, slot, a))) return st;
            for (int i = a; i < k; ++i)
                if ((st = adj_advance(c, i, true))) return st;
            if ((st = adj_step(c, k))) return st;
        }
        return FSIBE_OK;
    }
    // a slot for every remaining step: advance one step at a time; else the schedule's split
    const int j = (s >= t - 1) ? 1 : w->split[(size_t)t * (w->S + 1) + (s < w->S ? s : w->S)];
    if ((st = adj_restore(c, slot, a))) return st;
    for (int i = a; i < a + j; ++i)
        if ((st = adj_advance(c, i, true))) return st;
    if ((st = adj_save(c, slot + 1))) return st;
    if ((st = adj_reverse(c, a + j, t - j, s - 1, slot + 1))) return st;
    return adj_reverse(c, a, j, s, slot);
}

static int adj_check(fsibe_ctx* c, int nsteps, int avg_from) {
    if (c->fp32) { c->err = "the adjoint runs in the FP64 form"; return FSIBE_ERR_UNSUPPORTED; }
    if (c->P.iFLUSI != 0 || c->P.iMotion != 0 || c->P.iBeam <= 0) {
        c->err = "the adjoint needs a prescribed rigid mask (iFLUSI = 0, iMotion = 0, iBeam > 0)";
        return FSIBE_ERR_UNSUPPORTED;
    }
    if (c->spg || c->full_mask || c->s10) { c->err = "the adjoint runs without walls, cylinder and sponges"; return FSIBE_ERR_UNSUPPORTED; }
    if (nsteps < 1 || avg_from < 1 || avg_from > nsteps) { c->err = "need 1 <= avg_from <= nsteps"; return FSIBE_ERR_PARAM; }
    return FSIBE_OK;
}

// state 0 from vort0 (the mask kept), nu set, the drag window known
static int adj_begin(fsibe_ctx* c, int comp, const double* vort0, double nu, int nsteps, int avg_from, int nslots) {
    c->adv_ready = false;  // the adjoint's runs replace the state
    int st = adj_alloc(c, nslots);
    if (st) return st;
    AdjWork* w = c->adj;
    w->comp = comp;
    if (nu > 0.0 && nu != c->P.nu) {
        c->P.nu = nu;
        free_graph(c);
    }
    if ((st = init_state(c, vort0, true))) return st;
    w->nsteps = nsteps;
    w->avg_from = avg_from;
    w->cobj = 1.0 / (double)(nsteps - avg_from + 1);
    w->reached = 0;
    w->fwd_steps = w->adj_steps = 0;
    CK(c, cudaMemsetAsync(w->acc, 0, 64, c->stream));
    CK(c, cudaMemsetAsync(w->phys[AP_UBAR], 0, adj_field_bytes(c), c->stream));
    CK(c, cudaMemsetAsync(w->phys[AP_GMASK], 0, adj_field_bytes(c), c->stream));
    return adj_save(c, 0);
}

extern "C" {

int fsibe_force_objective(fsibe_ctx* c, int component, const double* vort0, double nu, int nsteps, int avg_from,
                          double* J) {
    if (!c || !vort0 || !J) return FSIBE_ERR_PARAM;
    if (component != 0 && component != 1) { c->err = "component: 0 (drag) or 1 (lift)"; return FSIBE_ERR_PARAM; }
    int st = adj_check(c, nsteps, avg_from);
    if (st) return st;
    if ((st = adj_begin(c, component, vort0, nu, nsteps, avg_from, 1))) return st;
    for (int k = 0; k < nsteps; ++k)
        if ((st = adj_advance(c, k, false))) return st;
    CK(c, cudaMemcpyAsync(J, c->adj->acc, 8, cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    return read_status(c);
}

int fsibe_drag_objective(fsibe_ctx* c, const double* vort0, double nu, int nsteps, int avg_from, double* J) {
    return fsibe_force_objective(c, 0, vort0, nu, nsteps, avg_from, J);
}

int fsibe_force_gradient(fsibe_ctx* c, int component, const double* vort0, double nu, int nsteps, int avg_from,
                         int snapshots, double* J, double* g_vort0, double* g_mask, double* g_nu,
                         fsibe_adjoint_info* info) {
    if (!c || !vort0) return FSIBE_ERR_PARAM;
    if (component != 0 && component != 1) { c->err = "component: 0 (drag) or 1 (lift)"; return FSIBE_ERR_PARAM; }
    int st = adj_check(c, nsteps, avg_from);
    if (st) return st;
    if (snapshots < 1) snapshots = 1;
    if (snapshots > nsteps) snapshots = nsteps;
    CK(c, cudaEventRecord(c->ev0, c->stream));
    if ((st = adj_begin(c, component, vort0, nu, nsteps, avg_from, snapshots + 1))) return st;
    AdjWork* w = c->adj;
    // time step and AB2 weights (fixed dt), the drag window: from one start-up step
    if ((st = adj_advance(c, 0, true))) return st;
    DevScalars h;
    CK(c, cudaMemcpyAsync(&h, c->S, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    w->dt = h.dt1;
    w->b10 = 1.5 * h.dt1;
    w->b11 = -0.5 * h.dt1;
    for (int q = 0; q < 4; ++q) w->win[q] = h.win[q];
    // d drag / d W (constant: the mask and the window are fixed)
    AdjArgs a = adj_args(c);
    const int G = adj_grid(c);
    k_adj_window<<<G, 256, 0, c->stream>>>(a, w->win[0], w->win[1], w->win[2], w->win[3], 0);
    if ((st = adj_fwd2d(c, a.lu, 1, a.G3))) return st;
    k_adj_gdrag<<<G, 256, 0, c->stream>>>(a);
    CKL(c);
    // the reverse sweep from the cotangents of the final state
    if (snapshots < nsteps - 1) adj_schedule(w, nsteps, snapshots);
    const size_t b = adj_field_bytes(c);
    CK(c, cudaMemsetAsync(w->spec[AS_LW], 0, b, c->stream));
    CK(c, cudaMemsetAsync(w->spec[AS_LM], 0, b, c->stream));
    {
        // lW(T) = c_T d drag / d W: q <- 0, G1..G4 <- 0 and one combine
        CK(c, cudaMemsetAsync(w->spec[AS_Q], 0, b, c->stream));
        CK(c, cudaMemsetAsync(w->spec[AS_G], 0, 4 * b, c->stream));
        a.c_obj = adj_weight(w, nsteps);
        k_adj_combine<<<G, 256, 0, c->stream>>>(a);
        CKL(c);
    }
    if ((st = adj_reverse(c, 0, nsteps, snapshots, 0))) return st;
    // the direct term of the mask gradient, then the outputs
    k_adj_window<<<G, 256, 0, c->stream>>>(a, w->win[0], w->win[1], w->win[2], w->win[3], 1);
    CKL(c);
    CK(c, cudaEventRecord(c->ev1, c->stream));
    double acc[2];
    CK(c, cudaMemcpyAsync(acc, w->acc, 16, cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    if ((st = read_status(c))) return st;
    if (J) *J = acc[0];
    if (g_nu) *g_nu = acc[1];
    const size_t NN = (size_t)c->g.nx * c->g.ny;
    if (g_mask) {
        if ((st = to_host(c, w->phys[AP_GMASK], NN, g_mask))) return st;
    }
    if (g_vort0) {
        // W0 = F(omega0): d J / d omega0 = F^T lW(0) = Phi(w lW(0)) / (nx ny)
        CK(c, cudaMemcpyAsync(w->spec[AS_LN], w->spec[AS_LW], b, cudaMemcpyDeviceToDevice, c->stream));
        k_adj_w3<<<G, 256, 0, c->stream>>>(a);
        CKL(c);
        if ((st = adj_inv2d(c, w->spec[AS_X], 1, w->phys[AP_P]))) return st;
        if ((st = to_host(c, w->phys[AP_P], NN, g_vort0))) return st;
    }
    if (info) {
        info->forward_steps = (int32_t)w->fwd_steps;
        info->adjoint_steps = (int32_t)w->adj_steps;
        info->snapshots = snapshots;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev0, c->ev1);
        info->ms_total = ms;
    }
    return FSIBE_OK;
}

int fsibe_drag_gradient(fsibe_ctx* c, const double* vort0, double nu, int nsteps, int avg_from, int snapshots,
                        double* J, double* g_vort0, double* g_mask, double* g_nu, fsibe_adjoint_info* info) {
    return fsibe_force_gradient(c, 0, vort0, nu, nsteps, avg_from, snapshots, J, g_vort0, g_mask, g_nu, info);
}

}  // extern "C"

// =====================================================================================
// Ensembles: independent runs advanced together, one graph launch per step
// =====================================================================================
// Every run keeps its own context (fields, streams, beam workspace).  One step of the
// ensemble is captured once as a CUDA graph: a fork from the ensemble's stream, each run's
// whole step on its own stream (with its own predictor fork), and a join.  The runs' kernels
// of different grid sizes then share the GPU in one launch; the single-CTA beam kernels of
// many runs fill separate SMs at the same time.
struct fsibe_ensemble {
    std::vector<fsibe_ctx*> runs;
    cudaStream_t master = nullptr;
    cudaEvent_t fork = nullptr, ev0 = nullptr, ev1 = nullptr;
    std::vector<cudaEvent_t> done;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    std::string err;
};

static void ens_free(fsibe_ensemble* e) {
    if (e->gexec) cudaGraphExecDestroy(e->gexec);
    if (e->graph) cudaGraphDestroy(e->graph);
    for (cudaEvent_t ev : e->done) if (ev) cudaEventDestroy(ev);
    if (e->fork) cudaEventDestroy(e->fork);
    if (e->ev0) cudaEventDestroy(e->ev0);
    if (e->ev1) cudaEventDestroy(e->ev1);
    if (e->master) cudaStreamDestroy(e->master);
    for (fsibe_ctx* c : e->runs) fsibe_destroy(c);
    delete e;
}

#define CKE(ens, call)                                                                  \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) {                                                        \
            (ens)->err = std::string(#call) + ": " + cudaGetErrorString(e_);            \
            g_err = (ens)->err;                                                         \
            return FSIBE_ERR_CUDA;                                                      \
        }                                                                               \
    } while (0)

// the ensemble's stream waits for every run's stream (work issued on the runs directly), or
// every run's stream waits for the ensemble's stream
static int ens_join_runs(fsibe_ensemble* e, bool runs_first) {
    if (!runs_first) CKE(e, cudaEventRecord(e->fork, e->master));
    for (size_t i = 0; i < e->runs.size(); ++i) {
        fsibe_ctx* c = e->runs[i];
        if (runs_first) {
            CKE(e, cudaEventRecord(e->done[i], c->stream));
            CKE(e, cudaStreamWaitEvent(e->master, e->done[i], 0));
        } else {
            CKE(e, cudaStreamWaitEvent(c->stream, e->fork, 0));
        }
    }
    return FSIBE_OK;
}

static int ens_step(fsibe_ensemble* e) {
    bool started = true;
    for (fsibe_ctx* c : e->runs) {
        if (!c->initialized) { e->err = "ensemble step before init_fields of every run"; g_err = e->err; return FSIBE_ERR_STATE; }
        // a run whose next advection part is not in place steps directly once (do_step's rule)
        started = started && c->startup_done && (!adv_pipelined(c) || c->adv_ready);
    }
    if (!started) {
        // the Euler start-up steps, each run on its own stream
        int st = ens_join_runs(e, false);
        if (st) return st;
        for (fsibe_ctx* c : e->runs) {
            st = c->startup_done ? step_body(c, 0) : step_body(c, 1);
            if (st) { e->err = c->err; g_err = e->err; return st; }
            c->startup_done = true;
            c->press_partial = press_rows_only(c);
        }
        return ens_join_runs(e, true);
    }
    if (!e->gexec) {
        CKE(e, cudaStreamBeginCapture(e->master, cudaStreamCaptureModeThreadLocal));
        CKE(e, cudaEventRecord(e->fork, e->master));
        int st = FSIBE_OK;
        for (size_t i = 0; i < e->runs.size() && !st; ++i) {
            fsibe_ctx* c = e->runs[i];
            if (cudaStreamWaitEvent(c->stream, e->fork, 0) != cudaSuccess) { st = FSIBE_ERR_CUDA; break; }
            const int before = c->launches;
            st = step_body(c, 0);
            c->launches = before;
            if (st) { e->err = c->err; break; }
            if (cudaEventRecord(e->done[i], c->stream) != cudaSuccess ||
                cudaStreamWaitEvent(e->master, e->done[i], 0) != cudaSuccess) st = FSIBE_ERR_CUDA;
        }
        cudaGraph_t g = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(e->master, &g);
        if (st) { if (g) cudaGraphDestroy(g); g_err = e->err; return st; }
        if (ce != cudaSuccess) { e->err = std::string("ensemble capture: ") + cudaGetErrorString(ce); g_err = e->err; return FSIBE_ERR_CUDA; }
        e->graph = g;
        CKE(e, cudaGraphInstantiate(&e->gexec, g, cudaGraphInstantiateFlagUseNodePriority));
    }
    CKE(e, cudaGraphLaunch(e->gexec, e->master));
    for (fsibe_ctx* c : e->runs) {
        c->press_partial = press_rows_only(c);
        c->adv_ready = adv_pipelined(c);
    }
    return FSIBE_OK;
}

extern "C" {

int fsibe_ensemble_create(const fsibe_params* params, int nruns, fsibe_ensemble** out) {
    if (!params || nruns <= 0 || !out) { g_err = "null argument or nruns <= 0"; return FSIBE_ERR_PARAM; }
    auto* e = new fsibe_ensemble;
    for (int i = 0; i < nruns; ++i) {
        fsibe_ctx* c = nullptr;
        const int st = fsibe_create(&params[i], &c);
        if (st) { ens_free(e); return st; }
        e->runs.push_back(c);
    }
    // Many concurrent runs fill the GPU by themselves: the single-CTA beam kernel then gives
    // more throughput than 16-SM clusters, which wait for whole free GPCs (measured with the
    // 64-run batch: 6276 against 4854 Mcell-steps/s).  FSIBE_BEAM_CLUSTER, when set, decides.
    if (nruns >= 8 && !std::getenv("FSIBE_BEAM_CLUSTER"))
        for (fsibe_ctx* c : e->runs) c->beam_cl = 0;
    // For the same reason the launches that take work off one run's critical path (the split
    // nonlinear term, the stresses beside k_press_x) only add graph nodes here (64-run batch:
    // 6350 against 6220 Mcell-steps/s without them).  FSIBE_NL_SPLIT / FSIBE_STRESS_SPLIT decide
    // when set.
    if (nruns >= 8) {
        for (fsibe_ctx* c : e->runs) {
            if (!std::getenv("FSIBE_NL_SPLIT")) c->nl_split = false;
            if (!std::getenv("FSIBE_STRESS_SPLIT")) c->stress_split = false;
        }
    }
    cudaError_t ce = cudaStreamCreateWithFlags(&e->master, cudaStreamNonBlocking);
    if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming);
    if (ce == cudaSuccess) ce = cudaEventCreate(&e->ev0);
    if (ce == cudaSuccess) ce = cudaEventCreate(&e->ev1);
    e->done.assign(nruns, nullptr);
    for (int i = 0; i < nruns && ce == cudaSuccess; ++i) ce = cudaEventCreateWithFlags(&e->done[i], cudaEventDisableTiming);
    if (ce != cudaSuccess) { g_err = cudaGetErrorString(ce); ens_free(e); return FSIBE_ERR_CUDA; }
    *out = e;
    return FSIBE_OK;
}

int fsibe_ensemble_destroy(fsibe_ensemble* e) {
    if (!e) return FSIBE_OK;
    cudaStreamSynchronize(e->master);
    ens_free(e);
    return FSIBE_OK;
}

int fsibe_ensemble_size(fsibe_ensemble* e, int* nruns) {
    if (!e || !nruns) return FSIBE_ERR_PARAM;
    *nruns = (int)e->runs.size();
    return FSIBE_OK;
}

int fsibe_ensemble_get(fsibe_ensemble* e, int run, fsibe_ctx** ctx) {
    if (!e || !ctx || run < 0 || run >= (int)e->runs.size()) return FSIBE_ERR_PARAM;
    *ctx = e->runs[run];
    return FSIBE_OK;
}

int fsibe_ensemble_step(fsibe_ensemble* e, int nsteps) {
    if (!e || nsteps < 0) return FSIBE_ERR_PARAM;
    int st = ens_join_runs(e, true);
    for (int s = 0; s < nsteps && !st; ++s) st = ens_step(e);
    if (!st) st = ens_join_runs(e, false);
    if (st) return st;
    CKE(e, cudaStreamSynchronize(e->master));
    for (fsibe_ctx* c : e->runs) {
        const int rs = read_status(c);
        if (rs) return rs;
    }
    return FSIBE_OK;
}

int fsibe_ensemble_time_steps(fsibe_ensemble* e, int nsteps, float* ms) {
    if (!e || !ms || nsteps < 0) return FSIBE_ERR_PARAM;
    int st = ens_join_runs(e, true);
    if (st) return st;
    CKE(e, cudaEventRecord(e->ev0, e->master));
    for (int s = 0; s < nsteps && !st; ++s) st = ens_step(e);
    if (st) return st;
    CKE(e, cudaEventRecord(e->ev1, e->master));
    CKE(e, cudaEventSynchronize(e->ev1));
    CKE(e, cudaEventElapsedTime(ms, e->ev0, e->ev1));
    st = ens_join_runs(e, false);
    if (st) return st;
    for (fsibe_ctx* c : e->runs) {
        const int rs = read_status(c);
        if (rs) return rs;
    }
    return FSIBE_OK;
}

const char* fsibe_ensemble_last_error(fsibe_ensemble* e) { return e ? e->err.c_str() : g_err.c_str(); }

}  // extern "C"

// =====================================================================================
// coftxy on caller-owned device buffers with file-scope scratch (allocates nothing)
// =====================================================================================
// Scratch for one forward transform: the x-transformed half spectrum T and the result S
// (nx*ny doubles each) and the twiddle tables (ny + nx/2 + nx/2+1 complex values).
#define FSIBE_STATIC_MAX_CELLS 65536
#define FSIBE_STATIC_MAX_DIM 2048
#define FSIBE_STATIC_TABLES (2 * (FSIBE_STATIC_MAX_DIM + FSIBE_STATIC_MAX_DIM / 2 + FSIBE_STATIC_MAX_DIM / 2 + 1))
static __device__ __align__(256) double g_static_scratch[2 * FSIBE_STATIC_MAX_CELLS + FSIBE_STATIC_TABLES];

namespace {
// Device address of g_static_scratch per device (host code may not use the symbol itself: on
// the host it names a stand-in, not device memory), and the transform kernels per
// (device, length), filled on first use.  The address is looked up again on every call made
// outside a stream capture, so a device reset or another context made current since the last
// call cannot leave a stale address behind; during a capture the last looked-up address of
// the device is used.
constexpr int kStaticDevs = 128;
double* g_static_dev[kStaticDevs] = {};
SizeKernels<double> g_static_k[kStaticDevs][7];  // lengths 32 .. 2048
bool g_static_k_ok[kStaticDevs][7] = {};
std::mutex g_static_mu;

int static_log2_index(int n) { int i = 0; while ((32 << i) < n) ++i; return i; }

__global__ void k_static_twiddles(double2* twY, int ny, double2* twX, int hx, double2* twR, int nx) {
    const int total = ny + hx + hx + 1;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        double s, c;
        if (i < ny) {
            sincospi(2.0 * (double)i / (double)ny, &s, &c);
            twY[i] = make_double2(c, -s);
        } else if (i < ny + hx) {
            const int m = i - ny;
            sincospi(2.0 * (double)m / (double)hx, &s, &c);
            twX[m] = make_double2(c, -s);
        } else {
            const int m = i - ny - hx;
            sincospi(2.0 * (double)m / (double)nx, &s, &c);
            twR[m] = make_double2(c, -s);
        }
    }
}
}  // namespace

// The beam kernels' running sums on the caller's terms (host arrays of 4 n doubles):
// out[q n + k] = s_k of row q, and *nserial the rows the step check sent to the serial loop.
extern "C" int fsibe_running_sums(const double* terms, int32_t n, double* out, int32_t* nserial) {
    if (!terms || !out || !nserial) { g_err = "fsibe_running_sums: null argument"; return FSIBE_ERR_PARAM; }
    if (n < 1 || n > (1 << 20)) { g_err = "fsibe_running_sums: n must be in [1, 2^20]"; return FSIBE_ERR_PARAM; }
    const size_t bytes = (size_t)4 * n * sizeof(double);
    double *d_in = nullptr, *d_out = nullptr;
    int* d_ns = nullptr;
    cudaError_t e = cudaMalloc(&d_in, 2 * bytes + 16);
    if (e == cudaSuccess) {
        d_out = d_in + 4 * (size_t)n;
        d_ns = reinterpret_cast<int*>(d_out + 4 * (size_t)n);
        e = cudaMemcpy(d_in, terms, bytes, cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = launch_running_sums(d_in, d_out, n, d_ns, 0);
    if (e == cudaSuccess) e = cudaMemcpy(out, d_out, bytes, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(nserial, d_ns, sizeof(int32_t), cudaMemcpyDeviceToHost);
    if (d_in) cudaFree(d_in);
    if (e != cudaSuccess) { g_err = std::string("fsibe_running_sums: ") + cudaGetErrorString(e); return FSIBE_ERR_CUDA; }
    return FSIBE_OK;
}

extern "C" int fsibe_coftxy_static(const double* f_dev, double* fk_dev, int32_t nx, int32_t ny, void* stream) {
    if (!f_dev || !fk_dev) { g_err = "fsibe_coftxy_static: null buffer"; return FSIBE_ERR_PARAM; }
    if (!pow2_ok(nx) || !pow2_ok(ny) || nx > FSIBE_STATIC_MAX_DIM || ny > FSIBE_STATIC_MAX_DIM ||
        (long)nx * (long)ny > FSIBE_STATIC_MAX_CELLS) {
        g_err = "fsibe_coftxy_static: nx, ny must be powers of two in [32, 2048] with nx*ny <= 65536 "
                "(the size of its static scratch)";
        return FSIBE_ERR_UNSUPPORTED;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kStaticDevs) { g_err = "fsibe_coftxy_static: cudaGetDevice failed"; return FSIBE_ERR_CUDA; }
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(st, &cap);
    if (e != cudaSuccess) { g_err = std::string("fsibe_coftxy_static: cudaStreamIsCapturing: ") + cudaGetErrorString(e); return FSIBE_ERR_CUDA; }
    double* base;
    SizeKernels<double> kx, ky;
    {
        std::lock_guard<std::mutex> lk(g_static_mu);
        if (cap == cudaStreamCaptureStatusNone) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_static_scratch);
            if (e != cudaSuccess || !p) {
                g_err = std::string("fsibe_coftxy_static: cudaGetSymbolAddress: ") + cudaGetErrorString(e);
                return FSIBE_ERR_CUDA;
            }
            g_static_dev[dev] = static_cast<double*>(p);
        } else if (!g_static_dev[dev]) {
            g_err = "fsibe_coftxy_static: the first call on a device must come before any stream capture";
            return FSIBE_ERR_STATE;
        }
        base = g_static_dev[dev];
        for (int n : {nx, ny}) {
            const int li = static_log2_index(n);
            if (!g_static_k_ok[dev][li]) {
                SizeKernels<float> unused;
                if (!get_sizes(n, g_static_k[dev][li], unused)) { g_err = "fsibe_coftxy_static: size"; return FSIBE_ERR_UNSUPPORTED; }
                g_static_k_ok[dev][li] = true;
            }
        }
        kx = g_static_k[dev][static_log2_index(nx)];
        ky = g_static_k[dev][static_log2_index(ny)];
    }
    const int hx = nx / 2;
    double2* T = reinterpret_cast<double2*>(base);
    double2* Sx = reinterpret_cast<double2*>(base + FSIBE_STATIC_MAX_CELLS);
    double2* twY = reinterpret_cast<double2*>(base + 2 * FSIBE_STATIC_MAX_CELLS);
    double2* twX = twY + ny;
    double2* twR = twX + hx;
    k_static_twiddles<<<16, 256, 0, st>>>(twY, ny, twX, hx, twR, nx);
    KArgs<double> a;
    std::memset(&a, 0, sizeof(a));
    a.g.nx = nx; a.g.ny = ny; a.g.hx = hx;
    a.g.inv_nxny = 1.0 / ((double)nx * (double)ny);
    a.phys0 = const_cast<double*>(f_dev);
    a.spec0 = T;
    a.spec1 = Sx;
    a.twX = twX; a.twR = twR; a.twY = twY;
    kx.xfwd<<<ny / kx.x_rows, kx.x_threads, kx.x_smem1, st>>>(a);
    ky.yfwd<<<hx, ky.y_threads, ky.y_smem1, st>>>(a);
    k_pack<double><<<hx, 256, 0, st>>>(Sx, nullptr, fk_dev, nx, ny);
    e = cudaGetLastError();
    if (e != cudaSuccess) { g_err = std::string("fsibe_coftxy_static: ") + cudaGetErrorString(e); return FSIBE_ERR_CUDA; }
    return FSIBE_OK;
}
