// common.cuh -- shared types, the device-resident run state and small helpers.
//
// Device layouts (all in HBM, one allocation per field):
//   physical field   R[ny][nx]         x fastest, identical to the reference's (0:nx-1,0:ny-1)
//   half spectrum    C2<R>[nx/2][ny]   one contiguous row of ny complex values per kx;
//                                      after the x pass it holds T(kx, iy), after the y pass
//                                      S(kx, ky).  kx = nx/2 (Nyquist) is never stored and
//                                      ky = ny/2 is kept at zero ("filtering" of coftxy).
// S(kx,ky) equals the reference's complex coefficient ft(kx,ky)/(nx*ny) of coftxy
// (cof_fftw33.f90:142-193); the packed Temperton layout exists only at the ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <type_traits>

#include "../../include/fsibe.h"

namespace fsibe {

// Programmatic dependent launch (PTX griddepcontrol).  A kernel launched with
// cudaLaunchAttributeProgrammaticStreamSerialization may start while the previous kernel of its
// stream still runs; pdl_wait() returns once that kernel has completed and its memory is
// visible (at once for a kernel launched without the attribute), so it comes before the first
// read of anything an earlier kernel wrote.  pdl_trigger() lets the next kernel of the stream
// launch: its blocks become resident and wait in their own pdl_wait().
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Launch k<<<g, b, smem, st>>>(args...), as a programmatic dependent launch when pdl is set.
template <typename... P, typename... A>
inline cudaError_t launch_k(void (*k)(P...), dim3 g, dim3 b, size_t smem, cudaStream_t st, bool pdl, A&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = g;
    cfg.blockDim = b;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k, static_cast<A&&>(args)...);
}

template <typename R> struct C2T;
template <> struct C2T<double> { typedef double2 type; };
template <> struct C2T<float> { typedef float2 type; };
template <typename R> using C2 = typename C2T<R>::type;

template <typename R> __host__ __device__ __forceinline__ C2<R> mk(R x, R y) { C2<R> r; r.x = x; r.y = y; return r; }
template <typename R> __device__ __forceinline__ C2<R> cadd(C2<R> a, C2<R> b) { return mk<R>(a.x + b.x, a.y + b.y); }
template <typename R> __device__ __forceinline__ C2<R> csub(C2<R> a, C2<R> b) { return mk<R>(a.x - b.x, a.y - b.y); }
template <typename R> __device__ __forceinline__ C2<R> cmul(C2<R> a, C2<R> b) {
    return mk<R>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename R> __device__ __forceinline__ C2<R> cconj(C2<R> a) { return mk<R>(a.x, -a.y); }
template <typename R> __device__ __forceinline__ C2<R> cscale(C2<R> a, R s) { return mk<R>(a.x * s, a.y * s); }
// (i * s) * a
template <typename R> __device__ __forceinline__ C2<R> cimul(C2<R> a, R s) { return mk<R>(-a.y * s, a.x * s); }

// Shared-memory index padding: one slot every 8 complex values keeps the strided
// Stockham writes free of bank conflicts for both float2 and double2.
__host__ __device__ __forceinline__ int pad8(int i) { return i + (i >> 3); }
__host__ __device__ constexpr int padded_len(int n) { return n + (n >> 3); }

// Scalars shared by all kernels of a step; lives in device memory so that a whole step can
// run (and be captured in a CUDA graph) without host round trips.
struct DevScalars {
    double time, dt0, dt1;
    double b10, b11;                 // AB2 coefficients of the current step
    double umax2, mean_ux, mean_uy;  // from the velocity at time n (CFL, u_max file)
    double u_max;
    double vor_rms, kinetic, dissipation, porous_diss, inflow_solid, inflow_mean;
    double force[2], force_unst[2], force_press[2], inertial_force[2];
    double drag_unst_old, lift_unst_old;
    double e_kinetic, e_elastic, e_pot;
    double grav;                     // GravityImpulse state
    double mean_u_next, mean_v_next; // Mean_Ux/Uy(time+dt1) used by the velocity kernel
    double mean_u_cur, mean_v_cur;   // mean flow of the stored velocity (FP32 form stores u - U)
    int32_t unst_ready;
    int32_t startup_step;            // beam StartupStep
    int32_t method;                  // current TimeMethodSolid
    int32_t actually_bdf2;
    int32_t newton_iters;
    int32_t status;                  // first non-zero FSIBE_ERR_* raised on the device
    int32_t step;
    int32_t explicit_step;           // 1 on the Euler start-up step
    int32_t win[4];                  // drag window ixmin, ixmax, iymin, iymax
    double dt_old;                   // beam dt_old
    double row[21];                  // last beam_data row (BeamIO.f90:193-216)
    int32_t run_row, run_cap;        // beam_data ring position / capacity of fsibe_run
    long long phase[32];             // beam kernel phase cycle counters (measurement)
    int32_t beam_fact;               // 1: the global copy of the beam's FP32 band factor is usable
    int32_t etab_valid;              // 1: the integrating-factor tables hold exp of etab_cx, etab_cy
    int32_t nred;                    // per-block partial sums written by the last x-pass kernel
    double etab_cx, etab_cy;
    int32_t srow[2];                 // rows the forces' stencils can reach this step (k_step_begin)
};

// Reduction slots written per block by the velocity/pressure kernel.
enum RedSlot {
    RED_OMEGA2 = 0, RED_KIN, RED_POROUS, RED_INFLOW_SOLID, RED_INFLOW_MEAN,
    RED_SUM_U, RED_SUM_V, RED_DRAG_X, RED_DRAG_Y, RED_UNST_X, RED_UNST_Y, RED_UMAX2,
    RED_NSLOTS
};

struct Geometry {
    int nx, ny, hx, ns;
    double xl, yl, dx, dy, ds;
    double pi, scalex, scaley;  // (2 pi / L)^2
    double kxs, kys;            // 2 pi / L
    double kx_trunc2, ky_trunc2;
    int idealis;
    double inv_nxny;            // 1 / (nx ny), the transforms' normalisation (exact: powers of two)
};

// q / b correctly rounded from rb = RN(1/b): q0 = RN(q rb), then one FMA correction
// (Markstein, IBM J. Res. Dev. 34 (1990) 111-119); three FP64 instructions instead of a
// division sequence.  Valid away from overflow and underflow.
__device__ __forceinline__ double div_cr(double q, double b, double rb) {
    const double q0 = q * rb;
    const double r = fma(-b, q0, q);
    return fma(r, rb, q0);
}

__device__ __forceinline__ void set_status(DevScalars* S, int code) {
    atomicCAS(&S->status, 0, code);
}

}  // namespace fsibe
