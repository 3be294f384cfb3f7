// beam.cu -- FP64 device code of the flexible beam (IBES_solver, SolidSolver.f90:13-414) on
// one CTA per kernel:
//   * k_beam_pre: gravity, the EE1 predictor with the tension solve (an FP32 tridiagonal
//     elimination preconditioning an FP64 iterative refinement), the initial guess and the
//     Crank-Nicolson right-hand side -- beside the fluid step, on a side stream,
//   * k_beam: Newton with the analytic Jacobian as a band (interleaved theta/T ordering,
//     kl = ku = 7); J dx = -F by FP64 iterative refinement preconditioned by an FP32 banded LU
//     with partial pivoting whose triangular solves run in chunks in parallel; positions and
//     energies (the single-CTA form; beam_cluster.cu holds the cluster form),
//   * k_init_beam.
// The routines they share are in beam_impl.cuh.
#include <mutex>

#include "beam_impl.cuh"
#include "running_sum.cuh"

namespace fsibe {

// Workspace length (doubles) of the global copy of the beam workspace for ns nodes.
__host__ size_t beam_ws_doubles(int ns) {
    return beam_vec_doubles(ns) + beam_band_doubles(ns) +
           (beam_lu_floats(ns) + beam_fact_floats(ns) + beam_scr_floats(ns) + beam_bulk_floats(ns) + 1) / 2;
}

// Doubles of the predictor's output: the initial guess x (n), the Crank-Nicolson right-hand
// side old_rhs, the EE1 angles g5 and the EE1 tension T (ns each).
__host__ size_t beam_pred_doubles(int ns) { return pred_consts(ns) + 16; }

// The Differentiate1D table for spacing ds (create_diff_matrices' rows over 2ds / ds^2 /
// 2ds^3 / ds^4), in the layout of D1DTab.
__host__ void beam_d1d_table(double ds, double* out) {
    static const double D1[3][3] = {{-3., 4., -1.}, {1., -4., 3.}, {-1., 0., 1.}};
    static const double D2[3][4] = {{2., -5., 4., -1.}, {-1., 4., -5., 2.}, {1., -2., 1., 0.}};
    static const double D3[3][6] = {{-17.0 / 2., 71.0 / 2., -59., 49., -41.0 / 2., 7.0 / 2.},
                                    {-7.0 / 2., 41.0 / 2., -49., 59., -71.0 / 2., 17.0 / 2.},
                                    {-1., 2., 0., -2., 1., 0.}};
    static const double D4[3][7] = {{35.0 / 6., -31., 137.0 / 2., -242.0 / 3., 107.0 / 2., -19.0, 17.0 / 6.},
                                    {17.0 / 6.0, -19.0, 107.0 / 2.0, -242.0 / 3.0, 137.0 / 2.0, -31.0, 35.0 / 6.0},
                                    {1., -4., 6., -4., 1., 0., 0.}};
    const double dx = ds;
    const double den[4] = {2.0 * dx, dx * dx, 2.0 * (dx * dx * dx), (dx * dx) * (dx * dx)};
    for (int o = 0; o < 4; ++o)
        for (int r = 0; r < 3; ++r)
            for (int q = 0; q < 8; ++q) {
                double v = 0.0;
                if (o == 0 && q < 3) v = D1[r][q];
                else if (o == 1 && q < 4) v = D2[r][q];
                else if (o == 2 && q < 6) v = D3[r][q];
                else if (o == 3 && q < 7) v = D4[r][q];
                out[(o * 3 + r) * 8 + q] = v / den[o];
            }
}

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
    d1d_load(&dtab, b.d1d);
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
    const Motion mo = motion_at(b.mo, time);  // mouvement(time) of EE1 and the CN right-hand side
    int st = rhs_beameqn(b, w, w.th1, w.td1, b.p_old, w.T, b.tau_old, grav, mo);
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
        st = rhs_beameqn(b, w, w.th1, w.old_rhs, b.p_old, w.T, b.tau_old, grav, mo);
        if (st) { if (threadIdx.x == 0) set_status(S, FSIBE_ERR_SINGULAR); return; }
        for (int i = threadIdx.x; i < ns; i += blockDim.x) p_old_rhs[i] = w.old_rhs[i];
    }
    // the step constants with divisions, for the Newton kernel (off its critical path)
    if (threadIdx.x == 0) {
        double* K = b.pred + pred_consts(ns);
        NewtonCtx cc;
        cc.dt = dt;
        solid_coeffs(method, dt, S->dt_old, cc.C1, cc.C2, cc.C3, cc.C4);
        newton_consts(cc, b);
        K[0] = cc.C1; K[1] = cc.C2; K[2] = cc.C3; K[3] = cc.C4; K[4] = cc.C1 / dt;
        K[5] = cc.g; K[6] = cc.gds2; K[7] = cc.gds4e;
        const double den0 = (3.0 * b.eta / (ds * ds)) - pT[0];
        K[8] = den0;
        K[9] = 1.0 / den0;
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
    d1d_load(&dtab, b.d1d);
    w.dtab = &dtab;
    const double grav = S->grav;
    for (int i = threadIdx.x; i < ns; i += blockDim.x) {
        w.bo3[i] = b.vx[i]; w.bo4[i] = b.vy[i]; w.bo5[i] = b.th[i]; w.bo6[i] = b.thd[i];
        w.oo5[i] = b.oo[4 * ns + i]; w.oo6[i] = b.oo[5 * ns + i];
    }
    __syncthreads();

    bool released = time > b.t_release;
    const Motion mo = motion_at(b.mo, time + dt);  // mouvement(time + dt) of the new level
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
            const double K2 = b.p_new[0] + mue * (mo.le[5] * mo.ca - mo.le[4] * mo.sa + grav * mo.ca);
            const double C2v = 2.0 * ds * K2 - T[0] * g5[1] + (eta / ds2) * (10.0 * g5[0] - 12.0 * g5[1] + 6.0 * g5[2] - g5[3]);
            w.x[xi_th(-1)] = C2v / ((3.0 * eta / ds2) - T[0]);
            const double K1 = mue * (mo.le[4] * mo.ca + mo.le[5] * mo.sa + grav * mo.sa) - b.tau_new[0];
            const double th_ss0 = (2.0 * g5[0] - 5.0 * g5[1] + 4.0 * g5[2] - 1.0 * g5[3]) * b.k.ids2;
            const double th_s0 = (-1.5 * g5[0] + 2.0 * g5[1] - 0.5 * g5[2]) * b.k.ids;
            const double T_s0 = -eta * th_ss0 * th_s0 + K1;
            w.x[xi_T(ns, -1)] = T[1] - 2.0 * ds * T_s0;
        }
        __syncthreads();
        // the step's Newton constants, evaluated once (divisions are long FP64 sequences here)
        __shared__ NewtonCtx cs;
        if (threadIdx.x == 0) {
            cs.time = time; cs.dt = dt; cs.dt_old = dt_old; cs.alpha_t = mo.alpha_t; cs.alpha_tt = mo.alpha_tt; cs.grav = grav;
            solid_coeffs(method, dt, dt_old, cs.C1, cs.C2, cs.C3, cs.C4);
            cs.D = cs.C1 / dt;
            newton_consts(cs, b);
            cs.K1 = mue * (mo.le[4] * mo.ca + mo.le[5] * mo.sa + grav * mo.sa) - b.tau_new[0];
            cs.K2 = b.p_new[0] + mue * (mo.le[5] * mo.ca - mo.le[4] * mo.sa + grav * mo.ca);
        }
        __syncthreads();
        const NewtonCtx& c = cs;
        // the FP32 factor of an earlier step, when one is stored
        bool need_factor = (S->beam_fact == 0), factored = false;
        if (!need_factor && (mode & (2 | 16))) {
            // the global copy holds [lu | fact] at its place
            const float* g = reinterpret_cast<const float*>(b.ws + beam_vec_doubles(ns) + beam_band_doubles(ns));
            if (mode & 16) copy_f4(reinterpret_cast<float4*>(w.Uf), reinterpret_cast<const float4*>(g), beam_lu_floats(ns) / 4);
            if (mode & 2)
                copy_f4(reinterpret_cast<float4*>(w.rse), reinterpret_cast<const float4*>(g + beam_lu_floats(ns)),
                        beam_fact_floats(ns) / 4);
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
                if (jac_row(b, w, c, k, w.band + (size_t)row_of(ns, k) * 16)) flag = FSIBE_ERR_NAN;
            };
            for (int r = threadIdx.x; r < n - 8; r += blockDim.x) assemble(9 + r);
            for (int q = threadIdx.x >> 5; q < 8; q += blockDim.x >> 5)
                if ((threadIdx.x & 31) == 0) assemble(1 + q);
            __syncthreads();
            if (flag) { if (threadIdx.x == 0) set_status(S, flag); return; }
            PH(4);
            // J dx = -F: FP32 LU of the row-scaled band as the preconditioner of an FP64
            // iterative refinement, run to 2^-30 of the correction (refine_step).  The factor is
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
                    const int rs = refine_step(w.xdi, w.yf, n, pass, cprev, &red[2][0], 0x1p-30);
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
            float* g = reinterpret_cast<float*>(b.ws + beam_vec_doubles(ns) + beam_band_doubles(ns));
            if (mode & 16) copy_f4(reinterpret_cast<float4*>(g), reinterpret_cast<const float4*>(w.Uf), beam_lu_floats(ns) / 4);
            if (mode & 2)
                copy_f4(reinterpret_cast<float4*>(g + beam_lu_floats(ns)), reinterpret_cast<const float4*>(w.rse),
                        beam_fact_floats(ns) / 4);
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
        w.cs[2 * (ns + 8) + i] = -(td * sn * ds);  // the third sum subtracts: s - a == s + (-a)
        w.cs[3 * (ns + 8) + i] = td * cn * ds;
    }
    __syncthreads();
    // the four running sums in the reference's order: the positions decide grid-aligned
    // boxes (mask, drag window), so their roundings must be the reference's (one lane a sum in
    // integer arithmetic, checked step by step: running_sum.cuh)
    {
        __shared__ int rs_flags[4];
        const int nser = running_sums4(w.cs, ns + 8, w.pre, ns + 8, ns, rs_flags, NoIdle());
        if (threadIdx.x == 0 && nser) S->phase[30] += nser;
    }
    // positions and velocities, and in the same pass each thread's terms of the emergency brake
    // (SolidSolver.f90:370-380) and of SolidEnergies (SolidSolver.f90:76-92); then block
    // reductions (per-thread partials, a shuffle tree, one warp over the warps' results), since
    // a serial FP64 loop costs a full warp issue slot per addition on this chip.  (The cluster
    // kernel sums columns in shared memory instead; here those 12 KB would push the LU factor
    // out of shared memory at ns = 1024.)
    {
        __shared__ double esum[6][8];
        const double ca = mo.ca, sa = mo.sa, alpha_t = mo.alpha_t, idt = 1.0 / dt;
        double sk = 0, sp = 0, se = 0, sax = 0, say = 0, mx = 0;
        for (int i = threadIdx.x; i < ns; i += blockDim.x) {
            const double xrel = w.pre[i], yrel = w.pre[(ns + 8) + i];
            const double vxrel = w.pre[2 * (ns + 8) + i], vyrel = w.pre[3 * (ns + 8) + i];
            const double yi = mo.le[1] + yrel * ca + xrel * sa;
            b.x[i] = mo.le[0] + xrel * ca - yrel * sa;
            b.y[i] = yi;
            const double vx = mo.le[2] + ca * (vxrel - alpha_t * yrel) - sa * (vyrel + alpha_t * xrel);
            const double vy = mo.le[3] + ca * (vyrel + alpha_t * xrel) + sa * (vxrel - alpha_t * yrel);
            b.vx[i] = vx;
            b.vy[i] = vy;
            double ax, ay;
            if (released) {
                ax = (vx - w.bo3[i]) * idt;
                ay = (vy - w.bo4[i]) * idt;
                b.ax[i] = ax;
                b.ay[i] = ay;
                mx = fmax(mx, fabs(b.thd[i] - w.bo6[i]));
            } else {
                ax = b.ax[i];
                ay = b.ay[i];
            }
            const double th_s = d1d(w.dtab, b.th, ns, 1, i);
            sk += vx * vx + vy * vy;
            sp += yi - b.y0;
            se += th_s * th_s;
            sax += ax;
            say += ay;
        }
        for (int o = 16; o > 0; o >>= 1) {
            sk += __shfl_xor_sync(0xffffffffu, sk, o);
            sp += __shfl_xor_sync(0xffffffffu, sp, o);
            se += __shfl_xor_sync(0xffffffffu, se, o);
            sax += __shfl_xor_sync(0xffffffffu, sax, o);
            say += __shfl_xor_sync(0xffffffffu, say, o);
            mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        }
        const int wv = threadIdx.x >> 5, ln = lane_id();
        if (ln == 0) {
            esum[0][wv] = sk; esum[1][wv] = sp; esum[2][wv] = se; esum[3][wv] = sax; esum[4][wv] = say; esum[5][wv] = mx;
        }
        __syncthreads();
        PH(8);
        if (threadIdx.x < 32) {
            const int nw = blockDim.x >> 5;
            double v[6];
#pragma unroll
            for (int q = 0; q < 6; ++q) v[q] = (ln < nw) ? esum[q][ln] : 0.0;
#pragma unroll
            for (int o = 4; o > 0; o >>= 1) {
#pragma unroll
                for (int q = 0; q < 5; ++q) v[q] += __shfl_xor_sync(0xffffffffu, v[q], o);
                v[5] = fmax(v[5], __shfl_xor_sync(0xffffffffu, v[5], o));
            }
            if (threadIdx.x == 0) {
                S->e_kinetic = mue * 0.5 * ds * v[0];
                S->e_pot = mue * grav * ds * v[1];
                S->e_elastic = eta * 0.5 * ds * v[2];
                S->inertial_force[0] = mue * ds * v[3];
                S->inertial_force[1] = mue * ds * v[4];
                if (released && v[5] > 100.0) set_status(S, FSIBE_ERR_BRAKE);
            }
        }
    }
    PH(9);
    if (threadIdx.x == 0)
        for (int k = 4; k < 24; ++k) S->phase[k] += ph[k];
}

// integrate_position (integrate_position.f90:14-44) by one thread: the four running sums in the
// reference's order and the positions and velocities of the motion mo.
__device__ void integrate_position_seq(const BeamArgs& b, const Motion& mo) {
    const int ns = b.ns;
    const double ds = b.ds, ca = mo.ca, sa = mo.sa, alpha_t = mo.alpha_t;
    double xrel = 0.0, yrel = 0.0, vxrel = 0.0, vyrel = 0.0;
    for (int s = 0; s < ns; ++s) {
        if (s > 0) {
            double sn, cn;
            sincos(b.th[s - 1], &sn, &cn);
            const double td = b.thd[s - 1];
            xrel = xrel + cn * ds;
            yrel = yrel + sn * ds;
            vxrel = vxrel - td * sn * ds;
            vyrel = vyrel + td * cn * ds;
        }
        b.x[s] = mo.le[0] + xrel * ca - yrel * sa;
        b.y[s] = mo.le[1] + yrel * ca + xrel * sa;
        b.vx[s] = mo.le[2] + ca * (vxrel - alpha_t * yrel) - sa * (vyrel + alpha_t * xrel);
        b.vy[s] = mo.le[3] + ca * (vyrel + alpha_t * xrel) + sa * (vxrel - alpha_t * yrel);
    }
}

// Beam start state (init_beam.f90:83-120): straight beam at the leading edge, at rest relative
// to it, placed by integrate_position(0).
__global__ void k_init_beam(BeamArgs b) {
    const int ns = b.ns;
    if (threadIdx.x == 0) b.S->beam_fact = 0;
    for (int i = threadIdx.x; i < ns; i += blockDim.x) {
        b.th[i] = 0.0; b.thd[i] = 0.0; b.ax[i] = 0.0; b.ay[i] = 0.0;
        b.p_old[i] = 0.0; b.p_new[i] = 0.0; b.tau_old[i] = 0.0; b.tau_new[i] = 0.0;
        for (int q = 0; q < 6; ++q) b.oo[q * ns + i] = 0.0;
        b.vx[i] = 0.0; b.vy[i] = 0.0;
    }
    __syncthreads();
    if (threadIdx.x == 0) integrate_position_seq(b, motion_at(b.mo, 0.0));
}

// A prescribed motion without the beam solver (iFLUSI = 0, iMotion > 0; time_step.f90:211-216):
// integrate_position at the step's time.
__global__ void k_move_beam(BeamArgs b) {
    pdl_wait();     // the previous kernel of the stream has completed
    if (threadIdx.x == 0) integrate_position_seq(b, motion_at(b.mo, b.S->time));
}

// ===================================================================================
// Host launchers
// ===================================================================================
static size_t beam_smem_bytes(int ns, int mask) {
    size_t bytes = 0;
    for (int part = 0; part < BEAM_PARTS; ++part)
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
// Shared-memory placement of the beam workspace: parts taken in beam_part_at order (scratch,
// LU factor, rest of the factor, FP64 vectors, band), each one kept when it still fits beside
// the kernel's static shared memory (at ns = 1024 the 198 KB LU factor fits, so the chunk
// sweeps' dependent loads come from shared memory).
int beam_smem_setup(int ns) {
    int dev = 0, optin = 0;
    cudaFuncAttributes fa;
    size_t budget = 216 * 1024;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) == cudaSuccess &&
        cudaFuncGetAttributes(&fa, (const void*)k_beam) == cudaSuccess && (size_t)optin > fa.sharedSizeBytes + 1024)
        budget = (size_t)optin - fa.sharedSizeBytes - 1024;
    cudaGetLastError();
    int mask = 0;
    size_t bytes = 0;
    for (int o = 0; o < BEAM_PARTS; ++o) {
        const int part = beam_part_at(o);
        const size_t pb = beam_part_bytes(ns, part);
        if (bytes + pb <= budget) { mask |= 1 << part; bytes += pb; }
    }
    if (mask && !raise_smem_limit((const void*)k_beam, bytes, &g_beam_smem)) mask = 0;
    return mask;
}
void launch_init_beam(const BeamArgs& b, cudaStream_t st) { k_init_beam<<<1, 256, 0, st>>>(b); }
void launch_move_beam(const BeamArgs& b, cudaStream_t st) { k_move_beam<<<1, 32, 0, st>>>(b); }

}  // namespace fsibe
