// solid.cuh -- mask rasterisation, beam-force interpolation and the IBES beam solver (FP64).
#pragma once
#include "common.cuh"

namespace fsibe {

// The leading edge's prescribed motion (mouvement.f90:5-200).  alpha0 = angle_deg pi / 180 and
// its cosine and sine come from the host; every case but flapping (3) keeps alpha = alpha0.
struct MotionArgs {
    int iMotion;
    double x0, y0, alpha0, cos0, sin0, phase, pi;
};
struct Motion {
    double alpha, alpha_t, alpha_tt, ca, sa;
    double le[6];  // x, y, vx, vy, ax, ay of the leading edge
};

__device__ __forceinline__ Motion motion_at(const MotionArgs& m, double time) {
    Motion o;
    const double pi = m.pi;
    const int k = m.iMotion;
    o.alpha = m.alpha0; o.alpha_t = 0.0; o.alpha_tt = 0.0; o.ca = m.cos0; o.sa = m.sin0;
    o.le[0] = m.x0; o.le[1] = m.y0;
    o.le[2] = 0.0; o.le[3] = 0.0; o.le[4] = 0.0; o.le[5] = 0.0;
    if ((k >= 201 && k <= 213) || (k >= 300 && k <= 350)) {
        // heaving with the soft start k(t) = -20 t^7 + 70 t^6 - 84 t^5 + 35 t^4 over t <= 1
        const double periods[13] = {1.0, 1.09, 1.20, 1.29, 1.33, 1.4, 1.5, 1.71, 2.0, 2.4, 3.0, 4.0, 1.62};
        const double y_max = 0.5, t_max = (k < 300) ? periods[k - 201] : 1.62;
        double s = 1.0, st = 0.0, stt = 0.0;
        if (time <= 1.0) {
            const double t = time, t2 = t * t, t3 = t2 * t, t4 = t3 * t, t5 = t4 * t, t6 = t5 * t, t7 = t6 * t;
            s = -20.0 * t7 + 70.0 * t6 + -84.0 * t5 + 35.0 * t4;
            st = 7.0 * -20.0 * t6 + 6.0 * 70.0 * t5 + 5.0 * -84.0 * t4 + 4.0 * 35.0 * t3;
            stt = 42. * -20.0 * t5 + 30. * 70.0 * t4 + 20. * -84.0 * t3 + 12. * 35.0 * t2;
        }
        const double w = 2.0 * pi / t_max, arg = 2.0 * pi * time / t_max + pi / 2. + m.phase;
        const double sn = sin(arg), cn = cos(arg);
        const double y = y_max * sn, yt = y_max * w * cn, ytt = -y_max * (w * w) * sn;
        o.le[1] = m.y0 + s * y;
        o.le[3] = st * y + yt * s;
        o.le[5] = stt * y + ytt * s + 2. * st * yt;
    } else if ((k >= 401 && k <= 413) || k == 2) {
        // heaving without a soft start (2) and the cases compared with experiments (401-413)
        const double periods[13] = {0.51, 0.34, 0.25, 0.20, 0.17, 0.14, 0.13, 0.11, 0.10, 0.09, 0.08, 0.08, 0.07};
        const double y_max = (k == 2) ? 0.5 : 0.0333, t_max = (k == 2) ? 2.5 : periods[k - 401];
        const double w = 2.0 * pi / t_max, arg = 2.0 * pi * time / t_max + pi / 2;
        const double sn = sin(arg), cn = cos(arg);
        o.le[1] = m.y0 + y_max * sn;
        o.le[3] = y_max * w * cn;
        o.le[5] = -y_max * (w * w) * sn;
    } else if (k == 3) {
        // flapping: alpha = 80 deg sin(2 pi f t), f = 0.5
        const double amax = 80.0 * pi / 180.0, w = 2.0 * pi * 0.5;
        const double sn = sin(w * time), cn = cos(w * time);
        o.alpha = amax * sn;
        o.alpha_t = amax * cn * w;
        o.alpha_tt = -1.0 * amax * sn * (w * w);
        o.ca = cos(o.alpha);
        o.sa = sin(o.alpha);
    } else if (k == 4) {
        // impulsive translation at u0 = -1
        o.le[0] = m.x0 + -1.0 * time;
        o.le[2] = -1.0;
    }
    return o;
}

// One drawing primitive of create_mask (create_mask.f90:91-117), in drawing order.
enum PrimType { PRIM_SEGMENT = 0, PRIM_SHARP = 1, PRIM_HINGE = 2, PRIM_DOT = 3 };
struct Prim {
    int type;
    int box[4];   // ixmin, ixmax, iymin, iymax (inclusive, clipped to the grid)
    double p[12];
};

// The FP32 form's per-primitive data, relative to a raster tile's origin (x0, y0) so that every
// coordinate is small and FP32 keeps it to ~1e-9:
//   segment: a = (cos, sin, p1x - x0, p1y - y0), b = (length along the axis, lower bound of the
//            normal offset, -, -), c = (v1x, v1y, (v2x - v1x)/ds, (v2y - v1y)/ds)
//   hinge / dot: a = (px - x0, py - y0, R^2 limit, -), b = (beta1, beta2, -, -), c = (vx, vy, -, -)
// k_mask_prep forms everything but the tile-relative offsets (zero there) once per primitive.
struct PrimG {
    float4 a, b, c;
};

struct MaskArgs {
    DevScalars* S;
    int until_full;  // 1: keep the previous mask once the time reaches T_fullspeed (the step's
                     // redraw for the velocity sponge and the frame, time_step.f90:187)
    int nx, ny, ns, sharp_trailing, sharp;
    double dx, dy, ds, t_beam, N_smooth, eps, pi, angle_deg;
    const double *x, *y, *vx, *vy, *th;
    Prim* prims;
    PrimG* primg;  // the FP32 form's data of prims (k_mask_prep), or null
    int* nprims;
    int* rect;    // [0..3] union of this step's primitive boxes (x0, x1, y0, y1), [4..7] its union
                  // with the previous step's box (every cell outside [0..3] is zero), [8..11] the
                  // accumulator of the next box (empty between steps), [12] blocks done
    double rdx, rdy, rpi;  // 1/dx, 1/dy, 1/pi (correctly rounded)
    double inv_delta, inv_ds, inv_eps;  // 1 / (N_smooth max(dx, dy) gerf), 1 / ds, 1 / eps (host quotients)
    MotionArgs mo;         // the leading edge's motion (alpha of the time)
    int nsm;      // SMs of the device (raster grid size)
    void *mask, *mvx, *mvy;  // R*[ny][nx]
    // the parts of the mask that are not the beam (create_mask.f90:21-68, 120-204); with `full`
    // set every cell is drawn each step (the box is the grid)
    int full;
    const double* bg;        // walls and the leading-edge cylinder (unscaled, velocity 0), or null
    const double* frame;     // iSponge = 22: the smoothed frame around the domain, or null
    double frame_c;          // its weight eps / max(1e-3, eps)
    int sponge4;             // iSponge = 4: the velocity sponge at the inflow
    int s4_l1, s4_r0, s4_r1; // its columns: [0, s4_l1] (left half), [s4_r0, s4_r1] (right half)
    double s4_star, s4_size, h_channel, H_eff;
    int iMeanVelocity;       // Mean_ux / Mean_uy of the time (mean_velocity.f90:4-84)
    double T_fullspeed, cos_ti, sin_ti;
};

// Mean_ux / Mean_uy (mean_velocity.f90:4-84) for iMeanVelocity 1, 2, 3, 4, 6, 22.
__device__ __forceinline__ double mean_flow_x(int mode, double time, double cos_ti, double Tf, double pi) {
    switch (mode) {
        case 1: return cos_ti * ((time < Tf) ? (time * time * time) / (-0.5 * Tf * Tf * Tf) + 3.0 * (time * time) / (Tf * Tf) : 1.0);
        case 2: return cos_ti * ((time < Tf) ? 0.5 * (1.0 - cos(0.5 * pi * time / Tf)) : 1.0);
        case 3: return cos_ti;
        case 6: return time;
        case 22: return 0.1;
        default: return 0.0;
    }
}
__device__ __forceinline__ double mean_flow_y(int mode, double time, double sin_ti, double Tf, double pi) {
    switch (mode) {
        case 1: return sin_ti * ((time < Tf) ? (time * time * time) / (-0.5 * Tf * Tf * Tf) + 3.0 * (time * time) / (Tf * Tf) : 1.0);
        case 2: return sin_ti * ((time < Tf) ? 0.5 * (1.0 - cos(0.5 * pi * time / Tf)) : 1.0);
        case 3: return sin_ti;
        default: return 0.0;
    }
}

// The static fields of the walls, cylinder, frame and vorticity sponge (solid.cu).
struct StaticMaskArgs {
    int nx, ny, sharp, iWalls, iCylinder, iSponge;
    double dx, dy, xl, yl, N, pi, h_channel, R_cylinder, x0, y0, t_beam, SpongeSize, eps, eps_sponge;
    double* bg;              // out: walls + cylinder
    double* frame;           // out: iSponge = 22
    void* spg;               // out: R*[ny][nx] the vorticity sponge / eps_sponge
    const void* mask;        // in (sponge): the start-up mask (R, divided by eps)
    int fp32;
};

struct ForceArgs {
    DevScalars* S;
    int nx, ny, ns, viscous;
    double xl, yl, dx, dy, ds, t_beam, N_smooth, pi, angle_deg, t_release, tau;
    double rdxi, rdyi;  // RN(1/dxi), RN(1/dyi) (host)
    MotionArgs mo;      // the leading edge's motion (alpha of the time)
    double* geo;     // per node: trig[4], phi4* weights dl[4][18] (k_forces_geo)
    int* gij;        // per node: the four surface points' cells ij[4][2]
    const double *x, *y, *th;
    const void *press, *sa, *sb;   // R*[ny][nx]
    double *p_new, *tau_new;
    unsigned int* counter;  // blocks done (last block computes the force integral)
    double* fterm;          // 2*ns per-node terms of the force integral
    int fp32;
};

// BeamSurfaceIntegral's grid sums (BeamForces.f90:483-486) and its output.
struct SurfArgs {
    int nx, ny, nblk, fp32;
    const void *u, *v, *mask, *mvx, *mvy;  // R*[ny][nx]; the FP32 form stores u - U
    const double* mean;                     // U, V of the stored velocity (FP32 form)
    double* part;                           // 2 nblk block partials
    double* out;                            // 11 values
};

// The end of a time step (time_step.f90:152-161 / :222-236): old <- new beam loads, time +=
// dt1, the step count and the beam_data row (BeamIO.f90:193-216), kept in the scalars and, when
// a ring is given, appended to it as one record of FSIBE_RECORD_COLS values: the beam_data row,
// then the step's u_max row (NavierStokes.f90:80-82), energies row (:259-261) and IBES_iter row
// (SolidSolver.f90:392-394), which the reference writes with the time before the step.  Run by
// one block after everything else of the step.
struct AdvArgs {
    DevScalars* S;
    int ns;
    MotionArgs mo;   // the leading edge's motion, for the record's mouvement row
    double *x, *y, *vx, *vy, *th, *thd, *p_old, *p_new, *tau_old, *tau_new;
    double* rows;
};

// tip: x, y, vx, vy, theta, theta_dot of the last node when the caller has them (else read).
__device__ __forceinline__ void advance_state(const AdvArgs& a, const double* tip = nullptr) {
    for (int i = threadIdx.x; i < a.ns; i += blockDim.x) {
        a.p_old[i] = a.p_new[i];
        a.tau_old[i] = a.tau_new[i];
    }
    if (threadIdx.x == 0) {
        DevScalars* S = a.S;
        const int ns = a.ns;
        const double t_before = S->time;
        S->time = S->time + S->dt1;
        S->step += 1;
        const double t0 = tip ? tip[0] : a.x[ns - 1], t1 = tip ? tip[1] : a.y[ns - 1], t2 = tip ? tip[2] : a.vx[ns - 1],
                     t3 = tip ? tip[3] : a.vy[ns - 1], t4 = tip ? tip[4] : a.th[ns - 1], t5 = tip ? tip[5] : a.thd[ns - 1];
        const double row[21] = {S->time, a.p_new[ns - 1], a.p_new[3 * ns / 4], a.p_new[ns / 2], t0, t1,
                                t2, t3, t4, t5, S->force[0], S->force[1],
                                S->force_unst[0], S->force_unst[1], S->force_press[0], S->force_press[1],
                                S->inertial_force[0], S->inertial_force[1], S->e_kinetic, S->e_elastic, S->e_pot};
        for (int c = 0; c < 21; ++c) S->row[c] = row[c];
        if (a.rows && S->run_row < S->run_cap) {
            double* rec = a.rows + (size_t)S->run_row * FSIBE_RECORD_COLS;
            for (int c = 0; c < 21; ++c) rec[c] = row[c];
            const Motion m = motion_at(a.mo, S->time);
            const double tail[FSIBE_RECORD_COLS - 21] = {
                t_before, S->dt1, S->u_max, S->mean_ux, S->mean_uy,
                t_before, S->dt1, S->vor_rms, S->kinetic, S->dissipation, S->porous_diss, S->inflow_solid, S->inflow_mean,
                t_before, (double)S->newton_iters,
                S->time, m.alpha, m.alpha_t, m.alpha_tt, m.le[0], m.le[1], m.le[2], m.le[3], m.le[4], m.le[5]};
            for (int c = 21; c < FSIBE_RECORD_COLS; ++c) rec[c] = tail[c - 21];
            S->run_row += 1;
        }
    }
}

// Reciprocal constants of the beam's grid spacing ds (formed on the host).
struct BeamConsts {
    double ids, i2ds, ids2, i2ds2, ids4, e2ds3, eds4, e2ds4;
};

struct BeamArgs {
    DevScalars* S;
    int ns, iImpulse, maxit, iFLUSI;
    double ds, eta, mue, sigma, t_release, tau, tol, pi, x0, y0, angle_deg;
    MotionArgs mo;        // the leading edge's motion
    BeamConsts k;
    double *x, *y, *vx, *vy, *th, *thd, *ax, *ay, *p_old, *p_new, *tau_old, *tau_new, *oo;
    double* ws;      // global workspace (used when the shared-memory workspace does not fit)
    int use_smem;    // workspace parts in shared memory: bit 1 << part of beam_part_bytes' parts
    double* pred;    // predictor output (beam_pred_doubles)
    const double* d1d;  // Differentiate1D table (4 x 3 x 8 doubles, beam_d1d_table)
    double* rows;    // beam_data ring (21 per step) or nullptr
    int row_cap;
    float* minv;     // cluster form: the rows of the preconditioner inverse, one slice per CTA
    int* minv_rse;   // cluster form: the row-scale exponents of those rows
    int cl_big;      // cluster form for large beams: the factor and M^-1 in global memory
    float* clws;     // its per-CTA factor copies (beam_cluster_fact_floats)
    int fuse_adv;    // cluster form: 1 = also end the time step (advance_state with adv)
    AdvArgs adv;
};

}  // namespace fsibe
