/*
 * fsibe.h -- C ABI of the GB300 (sm_103a) implementation of the FSIBE_2D hot path:
 * the pseudo-spectral vorticity step with volume penalization, coupled to the
 * inextensible flexible-beam (IBES) solver.
 *
 * Every entry point replaces one Fortran routine of the reference (cited per
 * function as file:line of tommy-engels/FSIBE_2D).  All entry points return an
 * int status (FSIBE_OK == 0).  The reference has no status returns: it calls
 * `stop`, or sets `continue_timestep=.false.`; the Fortran shim in
 * fortran/fsibe_iso_c.f90 maps non-zero codes back onto that behaviour.
 *
 * Conventions shared with the reference:
 *   - physical fields are (0:nx-1, 0:ny-1) column-major, x fastest, FP64 on the
 *     host side of the ABI: element (ix,iy) sits at f[iy*nx + ix];
 *   - spectral fields at the ABI are in the reference's packed "Temperton"
 *     bicomplex real layout produced by coftxy (cof_fftw33.f90:142-193), scaled
 *     by 1/(nx*ny), Nyquist row and column dropped;
 *   - u is (0:nx-1, 0:ny-1, 1:2): u[c*nx*ny + iy*nx + ix], c = 0 (x), 1 (y);
 *   - a beam is (0:ns-1, 1:6): beam[c*ns + n], columns x, y, vx, vy, theta,
 *     theta_dot (create_mask.f90:12).
 * Device state lives inside the opaque context in HBM; the host sees it only
 * through the fsibe_upload_* / fsibe_download_* calls.
 */
#ifndef FSIBE_H
#define FSIBE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define FSIBE_OK                 0
#define FSIBE_ERR_PARAM          1  /* bad parameters (params.f90:152-233 checks) */
#define FSIBE_ERR_CUDA           2  /* a CUDA runtime call failed                   */
#define FSIBE_ERR_NAN            3  /* NaN in the beam system (SolidSolver.f90:539-546,854-857) */
#define FSIBE_ERR_NEWTON_MAXIT   4  /* Newton did not converge (SolidSolver.f90:298-301) */
#define FSIBE_ERR_SINGULAR       5  /* zero pivot in an LU (SolidSolver.f90:515-525,1074-1077) */
#define FSIBE_ERR_INTERP_OOB     6  /* delta-interpolation target or stencil off the grid (Interpolation.f90:19-24) */
#define FSIBE_ERR_TIMEOUT        7  /* a bounded device-side wait gave up              */
#define FSIBE_ERR_UNSUPPORTED    8  /* size or option the library does not implement    */
#define FSIBE_ERR_MASK_OOB       9  /* beam point below the domain (create_mask.f90:685-688) */
#define FSIBE_ERR_BRAKE         10  /* emergency brake |d theta_dot| > 100 (SolidSolver.f90:370-380);
                                       soft: the reference sets continue_timestep=.false. */
#define FSIBE_ERR_STATE         11  /* call out of order (e.g. step before init_fields) */

/* ---- precision forms ------------------------------------------------- */
#define FSIBE_FP64    0  /* plain form: FP64 everywhere (the reference's arithmetic)          */
#define FSIBE_FP32C   1  /* FP32 transforms / derivatives / products; FP64 k=0 mode, vorticity
                            state (compensated hi+lo), reductions, forces and beam Newton   */

/* ---- solid time methods (share_vars.f90:43) ----------------------------- */
#define FSIBE_EULER_IMPLICIT   1
#define FSIBE_CRANK_NICHOLSON  2
#define FSIBE_BDF2             5

/*
 * Run parameters.  Mirrors the module globals of share_vars.f90:8-37 that the
 * hot path reads, in the units the reference uses after params.f90 ran
 * (nu = 1/Re already inverted; theta_inf in radians).
 */
typedef struct fsibe_params {
    int32_t nx, ny, ns;          /* grid and beam nodes (share_vars.f90:8)                   */
    int32_t precision;           /* FSIBE_FP64 or FSIBE_FP32C                                 */
    double  xl, yl;              /* box size                                                  */
    double  nu;                  /* kinematic viscosity = 1/Re                                */
    double  eps;                 /* penalization parameter (often written eta)               */
    double  cfl, dt_fixed, time_end;
    double  eta;                 /* beam stiffness EI                                         */
    double  mue;                 /* beam inertia (density ratio)                              */
    double  t_release, tau;      /* release time, soft-startup duration                       */
    double  angle_beam;          /* static beam angle, degrees (mouvement.f90:26)             */
    double  grav, sigma;         /* gravity, beam damping                                     */
    int32_t iImpulse;            /* GravityImpulse mode (SolidSolver.f90:874-911)             */
    int32_t time_method_solid;   /* FSIBE_BDF2 / FSIBE_CRANK_NICHOLSON / FSIBE_EULER_IMPLICIT */
    int32_t iFLUSI, iMotion, iViscous, iSaveBeam;
    int32_t iBeam, iSharpTrailing, iMeanVelocity, idealis;
    double  T_fullspeed, theta_inf;
    double  x0, y0, length;      /* leading edge and beam length                              */
    double  t_beam;              /* HALF thickness                                            */
    double  N_smooth;            /* half smoothing-layer width in grid points                 */
    double  newton_tol;          /* reference hard-codes 1e-7 (SolidSolver.f90:126)           */
    int32_t newton_maxit;        /* reference stops after iteration 49 (SolidSolver.f90:298)  */
    int32_t reserved;
    /* channel walls, a cylinder at the leading edge and sponges (share_vars.f90:11-21, read by
     * params.f90:32-78); all zero leaves the beam alone in the periodic box */
    int32_t iWalls;              /* 1: walls of half thickness h_channel at y = 0 and y = yl   */
    int32_t iCylinder;           /* 1: a cylinder of radius R_cylinder touching the leading edge */
    int32_t iSponge;             /* 1, 2, 3, 22: vorticity sponges; 4: velocity sponge (inflow)  */
    int32_t reserved2;
    double  h_channel, R_cylinder, SpongeSize, eps_sponge;
} fsibe_params;

/* Per-step scalar outputs: the columns of beam_data (BeamIO.f90:193-216),
 * u_max (NavierStokes.f90:80-82), energies (NavierStokes.f90:259-261) and
 * IBES_iter (SolidSolver.f90:392-394). */
typedef struct fsibe_scalars {
    double time, dt0, dt1;
    double u_max, mean_ux, mean_uy;                    /* u_max file, columns 3..5 */
    double vor_rms, kinetic, dissipation, porous_diss, inflow_solid, inflow_mean;
    double force[2], force_unst[2], force_press[2], inertial_force[2];
    double e_kinetic, e_elastic, e_pot;
    double beam_data[21];                              /* one beam_data row        */
    int32_t newton_iters;
    int32_t status;
    int32_t step;
    int32_t reserved;
} fsibe_scalars;

typedef struct fsibe_ctx fsibe_ctx;

/* ---- lifecycle (replaces dns.f90:170-207 StartSimulation set-up) ------------ */
/* Allocates every device field of one run, builds the dealiasing predicate
 * (dealiase_mask.f90:1-33) and the transform tables (fft_initialize,
 * cof_fftw33.f90:18-66).  Device-resident from here on. */
int fsibe_create(const fsibe_params* p, fsibe_ctx** out);
/* fft_free (cof_fftw33.f90:119-137) plus release of every field. */
int fsibe_destroy(fsibe_ctx* ctx);
/* Run all kernels of ctx on this cudaStream_t (NULL = the legacy stream). */
int fsibe_set_stream(fsibe_ctx* ctx, void* cuda_stream);
const char* fsibe_strerror(int status);
/* Last error message recorded by ctx (or the library when ctx is NULL). */
const char* fsibe_last_error(const fsibe_ctx* ctx);

/* ---- spectral operators on packed arrays (host in, host out) ------------------ */
int fsibe_fft_forward(fsibe_ctx* ctx, const double* f, double* fk);      /* coftxy  cof_fftw33.f90:142-193 */
int fsibe_fft_inverse(fsibe_ctx* ctx, const double* fk, double* f);      /* cofitxy cof_fftw33.f90:197-243 */
int fsibe_cofdx(fsibe_ctx* ctx, const double* fk, double* out);          /* cofdx.f90:1-29   */
int fsibe_cofdy(fsibe_ctx* ctx, const double* fk, double* out);          /* cofdy.f90:1-30   */
int fsibe_cofdxdx(fsibe_ctx* ctx, const double* fk, double* out);        /* cofdxdx.f90:1-27 */
int fsibe_cofdydy(fsibe_ctx* ctx, const double* fk, double* out);        /* cofdydy.f90:1-27 */
int fsibe_cofdxdy(fsibe_ctx* ctx, const double* fk, double* out);        /* cofdxdy.f90:1-32 */
int fsibe_poisson(fsibe_ctx* ctx, const double* f, double* ans);         /* poisson.f90:1-30 */
int fsibe_vis(fsibe_ctx* ctx, double dt, double* work);                  /* cal_vis.f90:1-36 */
int fsibe_dealiase_mask(fsibe_ctx* ctx, double* dealiase);               /* dealiase_mask.f90:1-33 */

/* ---- the time step ------------------------------------------------------ */
/* init_fields with inicond=111 (init_fields.f90:110-130) followed by the rest of
 * time_step's set-up (time_step.f90:60-100): init_beams, InitializeSolidSolver,
 * the zero state, then cal_velocity at t=0. vort is the physical vorticity. */
int fsibe_init_fields(fsibe_ctx* ctx, const double* vort);
/* create_mask(time, beams) (create_mask.f90:2-218): beam segments, sharp end,
 * hinges, leading/trailing dots, then mask /= eps. */
int fsibe_create_mask(fsibe_ctx* ctx, double time);
/* EvolveFluidExplicit (NavierStokes.f90:422-459) when explicit_step != 0, else
 * EvolveFluidAB2 (NavierStokes.f90:463-508); both end with pressure()
 * (NavierStokes.f90:273-403): velocity at n+1, drag/lift, energies, vor_mean,
 * pressure. */
int fsibe_fluid_step(fsibe_ctx* ctx, int explicit_step);
/* GetForces(time, beams, press, u, "new") (BeamForces.f90:6-51) with SPL=3. */
int fsibe_get_forces(fsibe_ctx* ctx, double time);
/* GravityImpulse(time) + SolidSolverWrapper(time, dt1, beams)
 * (SolidSolver.f90:874-911, 13-44). */
int fsibe_solid_step(fsibe_ctx* ctx, double time);
/* Time-level swap, time += dt1, pressure_old = pressure_new, tau_old = tau_new
 * (time_step.f90:152-159, 222-228). */
int fsibe_advance(fsibe_ctx* ctx);
/* One whole step in the reference order (time_step.f90:120-162 when the
 * startup step is due, else :178-228).  The same results as the five calls above, in fewer
 * dependent launches: cal_nlk's advection part runs beside the mask kernels and its
 * penalization part covers only the rows of the mask's box (FSIBE_NL_SPLIT=0: one kernel),
 * the viscous stresses run beside the pressure kernels on the rows the forces' stencils reach
 * (FSIBE_STRESS_SPLIT=0: inside the pressure kernel, every row), and the main stream's kernels
 * are programmatic dependent launches (FSIBE_PDL=0: plain launches). */
int fsibe_step(fsibe_ctx* ctx);
/* nsteps calls of fsibe_step; when rows != NULL writes one 21-column beam_data
 * row per step (rows[s*21 + c]). Stops early on a non-zero status. */
int fsibe_run(fsibe_ctx* ctx, int nsteps, double* rows);

/* Per-step records of fsibe_run_records: everything the reference appends to its
 * per-step text files in one time step, FSIBE_RECORD_COLS values a step.  The device keeps
 * them in a ring during the run; one copy to the host at the end.
 *   [0..20]  the beam_data row, written after the step (BeamIO.f90:193-216, SaveBeamData)
 *   [21..25] the u_max row: time, dt1, u_max, mean u, mean v (NavierStokes.f90:80-82)
 *   [26..33] the energies row: time, dt1, vor_rms, kinetic, dissipation, porous_diss,
 *            inflow_solid, inflow_mean (NavierStokes.f90:259-261)
 *   [34..35] the IBES_iter row: time, Newton iterations (SolidSolver.f90:392-394)
 *   [36..45] the mouvement row: time, alpha, alpha_t, alpha_tt, the leading edge's x, y, vx,
 *            vy, ax, ay (BeamIO.f90:229-238, SaveBeamData)
 * The u_max, energies and IBES_iter rows carry the time before the step, as the reference
 * writes them during it; beam_data and mouvement the time after it. */
#define FSIBE_RECORD_COLS 46
/* nsteps calls of fsibe_step with one record per step (records[s*FSIBE_RECORD_COLS + c]);
 * the time loop of time_step.f90:178-236 with its per-step output. */
int fsibe_run_records(fsibe_ctx* ctx, int nsteps, double* records);

/* ---- state transfer (host <-> HBM) --------------------------------------- */
int fsibe_upload_vortk(fsibe_ctx* ctx, const double* vortk_packed);
int fsibe_download_vortk(fsibe_ctx* ctx, double* vortk_packed);
int fsibe_download_vort(fsibe_ctx* ctx, double* vort);   /* cofitxy of vortk(n0) */
int fsibe_upload_u(fsibe_ctx* ctx, const double* u);
int fsibe_download_u(fsibe_ctx* ctx, double* u);
int fsibe_download_press(fsibe_ctx* ctx, double* press);
int fsibe_download_vor_mean(fsibe_ctx* ctx, double* vor_mean);
int fsibe_upload_mask(fsibe_ctx* ctx, const double* mask, const double* maskvx, const double* maskvy);
int fsibe_download_mask(fsibe_ctx* ctx, double* mask, double* maskvx, double* maskvy);
int fsibe_upload_press(fsibe_ctx* ctx, const double* press);
/* beam (ns,6) plus pressure_old/new, tau_old/new (ns each) */
int fsibe_upload_beam(fsibe_ctx* ctx, const double* beam, const double* p_old, const double* p_new,
                      const double* tau_old, const double* tau_new);
int fsibe_download_beam(fsibe_ctx* ctx, double* beam, double* p_old, double* p_new,
                        double* tau_old, double* tau_new);
int fsibe_get_scalars(fsibe_ctx* ctx, fsibe_scalars* out);

/* BeamSurfaceIntegral (BeamForces.f90:306-509): the stresses and pressure of the last fluid
 * step, phi4*-interpolated on the contour around the beam (half circles of 128 points at the
 * ends, the top and bottom lines), and the penalization drag/lift over the grid.
 * out[11] = time, drag, lift, drag_surf, lift_surf, Ft(1), Fn(1), Fp(1), Ft(2), Fn(2), Fp(2),
 * the columns of the reference's 'surface' file.  Replaces the call of BeamForces.f90:129; called
 * between fsibe_get_forces and fsibe_solid_step it sees the reference's state.  Needs
 * iViscous = 1 and a beam (else FSIBE_ERR_PARAM).  `time` fills column 0 and the soft
 * start-up factor; the contour follows the device's current beam (angle and positions of the
 * step) and the leading edge's angle mouvement(time).  With the leading-edge cylinder the
 * reference computes no surface integral (FSIBE_ERR_UNSUPPORTED); with walls its drag and lift
 * columns are zero (BeamForces.f90:331-336, 494-502). */
int fsibe_surface_integral(fsibe_ctx* ctx, double time, double* out);

/* ComputePressureSnapshot (NavierStokes.f90:598-665): the static pressure of the current
 * vorticity, with the velocity at `time` (the state's velocity plus the mean flow of the
 * time) and the current mask: p = q - |u|^2/2, q from the Poisson equation of the divergence
 * of the penalization and of the nonlinear term.  press: (0:nx-1, 0:ny-1) column-major FP64.
 * Outside the time step; the state is not changed.  After a step at the context's time it
 * equals that step's pressure up to rounding. */
int fsibe_pressure_snapshot(fsibe_ctx* ctx, double time, double* press);

/* ---- runtime backup ----------------------------------------------------------
 * The file runtime_backup<n>.in of MakeRuntimeBackup (save_fields.f90:109-152): Fortran
 * sequential unformatted records (a 4-byte record length before and after each record),
 * reals 8 bytes, integers and logicals 4; one beam.
 *
 * fsibe_write_backup: the state between two steps (after fsibe_step / fsibe_run / advance).
 *   Replaces the MakeRuntimeBackup call of time_step.f90:249.  The AB2 history is stored as
 *   nlk(n1) = the product nlk workvis that the next step forms first, with workvis(n0) = 1.
 * fsibe_read_backup: resume, as inicond = 2 (init_fields.f90:44-100) with the init_beams /
 *   InitializeSolidSolver / create_mask around it (time_step.f90:60-84).  The next fsibe_step
 *   is an AB2 step with a Crank-Nicolson solid step.  Reads files of either writer.
 * Both return FSIBE_ERR_PARAM on an I/O error, a wrong checksum or a different ns. */
int fsibe_write_backup(fsibe_ctx* ctx, const char* path);
int fsibe_read_backup(fsibe_ctx* ctx, const char* path);

/* ---- measurement helpers ---------------------------------------------------- */
/* Device time (ms, CUDA events on ctx's stream) of nsteps whole steps. */
int fsibe_time_steps(fsibe_ctx* ctx, int nsteps, float* ms);
/* Device time of each kernel of the step: runs nsteps whole steps (no graph) with CUDA events
 * around every launch on ctx's stream; out[k] = {name, summed ms, launches}. */
typedef struct fsibe_kernel_time {
    char name[32];
    float ms_total;
    int32_t launches;
} fsibe_kernel_time;
int fsibe_kernel_times(fsibe_ctx* ctx, int nsteps, fsibe_kernel_time* out, int cap, int* count);
/* Accumulated SM cycles of the beam kernels' phases since the last reset.  Predictor kernel
 * (runs beside the fluid step): [0] set-up, [1] EE1 predictor (tension solve), [2] initial
 * guess, [3] Crank-Nicolson right-hand side.  Newton kernel: [4] Newton F + Jacobian (with
 * the previous iteration's update and norms), [5] FP32 band factorisation, [6] the rest of
 * the refinement, [7] set-up, last Newton update and bookkeeping, [8] positions,
 * [9] energies, [11] FP64 residuals, [12] FP32 chunked solves, [13] correction updates;
 * [10] is the number of refinement solves (a count, not cycles).  Parts of [12]: [16] local
 * forward eliminations, [17] window carry, [18] forward correction, [19] local back
 * substitutions, [20] state carry, [21] back correction.  Parts of [7]: [22] set-up before
 * the Newton loop.  Parts of [4]: [23] Newton update and norms.  The cluster form of the
 * Newton kernel (fsibe_beam_cluster > 0) records, on its first CTA: [22] set-up, [4] F +
 * Jacobian, [5] row scaling, exchange, factorisation and inverse rows, [19] residuals (with the
 * previous pass's decision), [20] the push and [16] the barrier of the right-hand side's
 * all-gather, [17] inverse products and solution updates, [21] the push and [18] the barrier
 * of the solution rows' all-gather, [6] the refinement's decisions, [23] Newton update and
 * norms, [7] saving the inverse, [24] the angles' increments to the first CTA, [25] the
 * cluster barrier after them, [8] position sums, [26] positions and the terms of the brake
 * and the energies, [9] their reduction, [27] the end of the time step, [10] the solve count;
 * [30] the running sums that failed their step check (a count, see fsibe_running_sums).
 * out32 receives 32 values; reset != 0 zeroes them after reading. */
int fsibe_beam_phase_cycles(fsibe_ctx* ctx, long long* out32, int reset);
/* The beam kernels' running sums of integrate_position (integrate_position.f90:14-44) on the
 * caller's terms, a diagnostic of their exactness: terms and out are host arrays of 4 n doubles
 * (four rows of n); out[q n + k] = s_k with s_0 = +0 and s_(k+1) = s_k + terms[q n + k], bit
 * for bit the serial FP64 loop.  The kernels add the terms as integers on the grid of the
 * running value's binade, check every step with the FP64 addition and form a row that fails
 * the check by the serial loop; *nserial receives how many rows did (the Newton kernels count
 * them in fsibe_beam_phase_cycles' [30]).  n in [1, 2^20]; runs on the current device's
 * legacy stream. */
int fsibe_running_sums(const double* terms, int32_t n, double* out, int32_t* nserial);
/* Rows per block chosen by the autotuner for the fused x-pass kernels (nl_x, press_x,
 * press_fin).  fsibe_create times four candidates per kernel on the new context's buffers --
 * half, the default and twice the default tile height, and the default tile with its
 * registers capped for two resident blocks an SM -- and, for press_x in the FP32 form, the
 * paired kernel (two adjacent butterflies a thread) -- and keeps the fastest (cached per
 * precision and grid size for the process; FSIBE_AUTOTUNE=0 in the environment keeps the
 * defaults; FSIBE_PX_PAIRED=1 / 0 forces / forbids the paired press_x).  fsibe_tile_config
 * gives the rows and the blocks-per-SM bound (0: the kernel's default; 16 marks the paired
 * press_x) of each: out6 = {rows, bound} for nl_x, press_x, press_fin. */
int fsibe_tiles(fsibe_ctx* ctx, int32_t* rows3);
int fsibe_tile_config(fsibe_ctx* ctx, int32_t* out6);
/* The transform engine the autotuner chose for k_press_y: 0 the paired FP32 engine (two
 * adjacent butterflies a thread), 1 the one-butterfly engine (always in the FP64 form).
 * fsibe_create times both in the FP32 form and keeps the paired one unless the other is 3%
 * faster; FSIBE_PY_ENG = 0 / 1 forces one. */
int fsibe_press_y_engine(fsibe_ctx* ctx, int32_t* eng);

/* CTAs of the thread-block cluster that runs the beam's Newton step (16 or 8; 0 when the
 * single-CTA kernel runs it).  Chosen at fsibe_create from what the device can place;
 * the environment variable FSIBE_BEAM_CLUSTER = 0, 8 or 16 caps it. */
int fsibe_beam_cluster(fsibe_ctx* ctx, int32_t* ctas);
/* Number of kernel launches one fsibe_step issues (for the bench's gpu_launches). */
int fsibe_launches_per_step(fsibe_ctx* ctx, int* launches);
/* Capture one fsibe_step in a CUDA graph and replay it for later steps (1) or
 * launch kernels directly (0, default). */
int fsibe_use_graph(fsibe_ctx* ctx, int enable);

/* ---- adjoint of the fluid step on a prescribed rigid mask --------------------------------
 * No counterpart in the reference.  For a context with a prescribed rigid mask (iFLUSI = 0,
 * iMotion = 0, iBeam > 0, FP64 form; the mask is drawn by fsibe_init_fields or set with
 * fsibe_upload_mask and is kept by these calls):
 *   J = mean of the drag (Force(1), cal_drag NavierStokes.f90:567) after the steps
 *       avg_from .. nsteps, the first step being the Euler start-up step, starting from the
 *       physical vorticity vort0 ((0:nx-1,0:ny-1) column-major) with viscosity nu (nu <= 0:
 *       the context's).  fsibe_drag_objective returns J alone.
 *   fsibe_drag_gradient also returns dJ/d vort0 (nx*ny), dJ/d mask (nx*ny, the reference's
 *       `mask` array, chi/eta) and dJ/d nu, by the discrete adjoint of the step (transposed
 *       transforms, linearised advection and penalization).  Forward states are kept in
 *       `snapshots` slots and recomputed between them on the binomial schedule; with
 *       snapshots >= nsteps - 1 every state is kept.  Any output pointer may be NULL. */
typedef struct fsibe_adjoint_info {
    int32_t forward_steps;   /* forward steps taken, recomputation included               */
    int32_t adjoint_steps;
    int32_t snapshots;
    float   ms_total;        /* device time of the whole gradient computation            */
} fsibe_adjoint_info;
int fsibe_drag_objective(fsibe_ctx* ctx, const double* vort0, double nu, int nsteps, int avg_from, double* J);
int fsibe_drag_gradient(fsibe_ctx* ctx, const double* vort0, double nu, int nsteps, int avg_from, int snapshots,
                        double* J, double* g_vort0, double* g_mask, double* g_nu, fsibe_adjoint_info* info);
/* The same for either force component: component 0 is the drag above, 1 the lift, the mean of
 * Force(2) (cal_drag NavierStokes.f90:568, the window sum of chi (v - v_s)).  The drag calls
 * are these with component 0. */
int fsibe_force_objective(fsibe_ctx* ctx, int component, const double* vort0, double nu, int nsteps, int avg_from,
                          double* J);
int fsibe_force_gradient(fsibe_ctx* ctx, int component, const double* vort0, double nu, int nsteps, int avg_from,
                         int snapshots, double* J, double* g_vort0, double* g_mask, double* g_nu,
                         fsibe_adjoint_info* info);

/* ---- ensembles: independent runs advanced together (batched configuration) -------------
 * No counterpart in the reference (its batch mode, dns.f90:76-100, runs the parameter sets
 * one after another).  The runs may differ in grid size, beam size, parameters and precision.
 * Each run is an ordinary context (fsibe_ensemble_get), initialised and read with the
 * functions above.  fsibe_ensemble_step advances every run by nsteps; after the first step
 * (every run's Euler start-up step) one step of all runs is one CUDA graph launch, with each
 * run's step on its own stream.  Work issued on a run's context directly is ordered before
 * and after the ensemble's steps.  Ensembles of 8 runs or more run each beam on one CTA
 * (fsibe_beam_cluster reports 0) unless FSIBE_BEAM_CLUSTER is set: many runs fill the GPU by
 * themselves, and the single-CTA kernel then gives the higher throughput.  For the same reason
 * their steps form the nonlinear term and the stresses in the fused kernels (the split launches
 * of a single run, see fsibe_step, would only add graph nodes) unless FSIBE_NL_SPLIT or
 * FSIBE_STRESS_SPLIT is set. */
typedef struct fsibe_ensemble fsibe_ensemble;
int fsibe_ensemble_create(const fsibe_params* params, int nruns, fsibe_ensemble** out);
int fsibe_ensemble_destroy(fsibe_ensemble* ens);
int fsibe_ensemble_size(fsibe_ensemble* ens, int* nruns);
int fsibe_ensemble_get(fsibe_ensemble* ens, int run, fsibe_ctx** ctx);
int fsibe_ensemble_step(fsibe_ensemble* ens, int nsteps);
/* Device milliseconds (CUDA events on the ensemble's stream) for nsteps ensemble steps. */
int fsibe_ensemble_time_steps(fsibe_ensemble* ens, int nsteps, float* ms);
const char* fsibe_ensemble_last_error(fsibe_ensemble* ens);

/* ---- forward transform without any device allocation ------------------------------
 * No counterpart in the reference.  coftxy (the packed forward transform, same result as
 * fsibe_fft_forward) of a device field f_dev (nx*ny FP64, (0:nx-1,0:ny-1) column-major,
 * 16-byte aligned) into the device array fk_dev (nx*ny FP64, packed layout), on
 * cuda_stream (NULL = the legacy stream).  It needs no context and calls no cudaMalloc,
 * cudaFree or allocating library routine: its scratch is one file-scope device array of
 * about 1.1 MB that every GPU loading this library holds until the process exits.
 *
 * Why: some callers must not allocate device memory.  A host code whose device memory is
 * owned by a pool (a framework's caching allocator, a Fortran code that sizes every array
 * at start-up) cannot take extra cudaMalloc'd buffers outside that budget; and a per-step
 * loop cannot afford cudaFree, which synchronises the whole device.
 *
 * Limits: nx and ny powers of two in [32, 2048] with nx*ny <= 65536; larger sizes return
 * FSIBE_ERR_UNSUPPORTED (message in fsibe_last_error(NULL)) without launching anything.
 * The first call on a device looks up the scratch's device address
 * (cudaGetSymbolAddress) with that device current; make that first call before any stream
 * capture.  Every later call made outside a capture looks the address up again, so a
 * device reset or another context made current in between leaves no stale address; a call
 * made during a capture uses the address of the device's last uncaptured call (a capture
 * on a device with no earlier call returns FSIBE_ERR_STATE).
 * All calls share the one scratch array, so calls that overlap on the GPU
 * (different streams, or different host threads) race; every call rewrites all the
 * scratch it reads, so nothing carries over from the previous call. */
int fsibe_coftxy_static(const double* f_dev, double* fk_dev, int32_t nx, int32_t ny, void* cuda_stream);

#ifdef __cplusplus
}
#endif
#endif /* FSIBE_H */
