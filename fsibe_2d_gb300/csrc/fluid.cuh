// fluid.cuh -- fused pseudo-spectral kernels of the vorticity step (templates).
//
// x pass ("X" kernels): a block owns TR physical rows; each row is a length-H=nx/2 complex
//   FFT (real-to-complex split) done by G = H/8 threads.  Spectral intermediates are read /
//   written transposed, T[kx][iy], through shared memory, so both sides stay coalesced.
// y pass ("Y" kernels): a block owns one kx row of ny complex values (contiguous), does the
//   y FFTs and all pointwise spectral work for that row.
//
// Kernel map onto the reference (NavierStokes.f90):
//   k_nl_x     cal_nlk :40-52 and :88-132  inverse-x of dw/dx, dw/dy; -u.grad(w); the
//              penalization -chi(u-us); forward-x of all three; A = X(w) + i kx X(pen_y),
//              B = X(pen_x)
//   k_nl_y     cal_nlk's forward-y + curl (:169-173), EvolveFluidAB2/Explicit (:478-498, :446-450)
//              with vis (cal_vis.f90) and dealiasing, then the inverse-y transforms
//              that cal_velocity (:194-202), pressure (:331), GetForces' stresses
//              (BeamForces.f90:105-124) and the next cal_nlk (:40-44) need.
//   k_press_x  pressure :305-338 and :354-370: velocity at n+1 (+ mean flow), penalty term,
//              drag window sums, energies, time_avg_vort, the Poisson right-hand side and its
//              forward-x transform; viscous stresses to physical space.
//   k_press_y  pressure :366-383: forward-y, divergence, poisson, inverse-y
//   k_press_fin pressure :383-392: inverse-x, p = q - |u|^2/2
#pragma once
#include <algorithm>

#include "fft.cuh"

namespace fsibe {

template <typename R>
struct KArgs {
    Geometry g;
    double nu, eps;
    // physical fields R[ny][nx]
    R *u, *v, *mask, *mvx, *mvy, *vor_mean, *press, *sa, *sb, *phys0;
    // half spectra C2<R>[hx][ny]
    C2<R> *W, *M, *Wlo, *A, *B, *Tu, *Tv, *Tw, *Tsa, *Tsb, *Tdx, *Tdy, *P1, *P2, *Tq, *spec0, *spec1;
    const C2<R> *twX, *twR, *twY;
    DevScalars* S;
    double* red;
    const double* etab;   // integrating factor per direction: exp(coefx kx^2) [hx], exp(coefy ky^2) [ny/2+1]
    const float2* etabf;  // the same split hi + lo (FP32-compensated form)
    const int* dcut;      // 2/3-rule: modes with |ky| >= dcut[kx] are removed (dealiase_mask.f90:9-26)
    const float* kxw;     // FP32 form: (float)(kx kxs) for kx in [0, hx], formed on the host (the
                          // kernels' FP64 product and conversion per element, without the FP64 pipe)
    int kcut;             // rows kx >= kcut hold no dealiased mode (dcut = 0): exact zeros after the update
    int viscous, pressure_on, penalize, op;
    int explicit_step;    // 1 on the Euler start-up step (the host's flag: nl_x runs beside k_step_begin)
    const int* rect;      // the mask's box (rect[2..3]: its rows), written by k_mask_prep
    // the viscous stresses in their own kernel (k_stress_x) instead of k_press_x; with srows
    // set, only on the rows that the forces' stencils at the beam can reach (S->srow)
    int stress_split;
    int srows;
    const R* spg;         // the vorticity sponge / eps_sponge (NavierStokes.f90:142-160), or null
    const R* s10;         // iSponge = 10: the integral added to the x penalization (:103-122), or null
    size_t bstride;       // generic transforms over several fields at once: blockIdx.y selects the
                          // field, bstride complex values (= nx ny / 2) apart in every buffer
};

template <typename R> constexpr bool kIsF32 = std::is_same<R, float>::value;

// One warp reduces a column of n FP32 partials: their sum in float-float (Knuth's TwoSum at each
// addition; the parts added in FP64 at the end: within a few FP64 roundings of the FP64 sum of
// the partials, at FP32 speed -- an FP64 instruction takes its SMSP's FP64 pipe for some 64
// cycles on this chip), or their maximum (mx).
__device__ __forceinline__ double col_reduce_ff(const float* col, int n, bool mx) {
    const int l = threadIdx.x & 31;
    float s = 0.f, c = 0.f;
    for (int i = l; i < n; i += 32) {
        const float x = col[i];
        if (mx) { s = fmaxf(s, x); continue; }
        const float t = __fadd_rn(s, x), bb = __fsub_rn(t, s);
        c = __fadd_rn(c, __fadd_rn(__fsub_rn(s, __fsub_rn(t, bb)), __fsub_rn(x, bb)));
        s = t;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float so = __shfl_xor_sync(0xffffffffu, s, o), co = __shfl_xor_sync(0xffffffffu, c, o);
        if (mx) { s = fmaxf(s, so); continue; }
        const float t = __fadd_rn(s, so), bb = __fsub_rn(t, s);
        c = __fadd_rn(__fadd_rn(c, co), __fadd_rn(__fsub_rn(s, __fsub_rn(t, bb)), __fsub_rn(so, bb)));
        s = t;
    }
    return mx ? (double)s : (double)s + (double)c;
}

// kx 2 pi / xl in the kernels' type: FP32 from the host's table, FP64 as the product
template <typename R> __device__ __forceinline__ R kx_wave(const KArgs<R>& a, int kx) {
    if constexpr (kIsF32<R>) return a.kxw[kx];
    else return (double)kx * a.g.kxs;
}

// k_nl_x's parts.  The advection part needs no mask, so it can run beside the mask kernels;
// the penalization part then adds the mask's term on the rows of the mask's box alone
// (outside it the mask and the penalization are zero).
enum { NL_WHOLE = 0, NL_ADVECT = 1, NL_PENAL = 2 };
// shared-memory row buffers of k_nl_y: in FP32 two for the forward transforms and three for the
// prefetched state, then all five for the inverse transforms; two in FP64
template <typename R> constexpr int nl_y_bufs() { return kIsF32<R> ? 5 : 2; }

// 16-byte asynchronous global -> shared copies (the copy engine fills shared memory while the
// threads compute); completed by cp_async_wait before use
__device__ __forceinline__ void cp_async16_f(void* s, const void* g) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(s);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(g) : "memory");
}
__device__ __forceinline__ void cp_async_wait_f() {
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}
// one complex value global -> shared without a register round trip (8 bytes in FP32 through
// L1, 16 in FP64 bypassing it): a thread issues all of a tile's copies before waiting
template <typename R>
__device__ __forceinline__ void cp_async_el(C2<R>* s, const C2<R>* g) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(s);
    if constexpr (sizeof(C2<R>) == 8) asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sa), "l"(g) : "memory");
    else asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(g) : "memory");
}

// Error-free transformations for the compensated (hi + lo) vorticity state of the FP32 form.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}
// (h + l) = ((wh + wl) + d) * (Eh + El), all floats, ~1e-14 relative
__device__ __forceinline__ void ff_update(float wh, float wl, float d, float Eh, float El, float& oh, float& ol) {
    float s, e, sh, sl;
    two_sum(wh, d, s, e);
    fast_two_sum(s, __fadd_rn(e, wl), sh, sl);
    const float ph = __fmul_rn(sh, Eh);
    const float pe = __fmaf_rn(sh, Eh, -ph);
    const float pl = __fadd_rn(pe, __fmaf_rn(sh, El, __fmul_rn(sl, Eh)));
    fast_two_sum(ph, pl, oh, ol);
}

// Operators the generic inverse-y kernel applies before the transform.
enum SpecOp { OP_ID = 0, OP_DX = 1, OP_DY = 2, OP_U = 3, OP_V = 4, OP_UX = 5 };  // OP_UX: du/dx

__device__ __forceinline__ int signed_k(int k, int n) { return (k <= n / 2) ? k : k - n; }

template <typename R, int H, int TRV = 0>
struct XRows {
    static constexpr int G = H / 8;
    // rows per block: keep the transposed chunks >= 32 bytes while bounding shared memory
    static constexpr int TR0 = (sizeof(R) == 8) ? (H <= 512 ? 4 : 2) : (H <= 256 ? 8 : (H <= 1024 ? 4 : 2));
    // at least one full warp per block (the block reductions use full-warp shuffles)
    static constexpr int TRD = (G * TR0 >= 32) ? TR0 : 32 / G;
    // TRV > 0: an explicit tile height (the autotuner's candidates)
    static constexpr int TR = TRV > 0 ? TRV : TRD;
    static constexpr int PL = padded_len(H) + 1;  // row stride (complex) in shared memory
    static constexpr int THREADS = G * TR;
    // blocks per SM that keep a thread at <= 128 registers
    static constexpr int MINB128 = (65536 / (THREADS * 128)) > 0 ? 65536 / (THREADS * 128) : 1;
};

// A tile height for the fused x-pass kernels: tr when it is valid (a full warp, at most 1024
// threads, at most 200 KB of shared memory for three row buffers), else the default.
template <typename R, int H>
constexpr int xrows_valid(int tr) {
    using X = XRows<R, H>;
    return (tr >= 1 && X::G * tr >= 32 && X::G * tr <= 1024 &&
            3 * tr * X::PL * (int)(2 * sizeof(R)) <= 200 * 1024) ? tr : X::TRD;
}

// ---- x-pass helpers -------------------------------------------------------------------
// Rows kx >= kmax are known to be zero and are not read.
template <typename R, int H, int TR, int PL>
// Asynchronous: the caller completes the copies (cp_async_wait_f) before its __syncthreads.
__device__ __forceinline__ void load_tileT(C2<R>* buf, const C2<R>* __restrict__ T, int ny, int iy0, int kmax = H) {
    for (int i = threadIdx.x; i < H * TR; i += blockDim.x) {
        const int r = i % TR, kx = i / TR;
        if (kx < kmax) cp_async_el<R>(&buf[r * PL + pad8(kx)], &T[(size_t)kx * ny + iy0 + r]);
        else buf[r * PL + pad8(kx)] = mk<R>(0, 0);
    }
}

// load_tileT of i kx T (kx's wavenumber kx kxs0 as k_nl_y forms it, in R): the FP32 form keeps
// only T and forms the x derivative as it loads (cofdx of omega from Tw, du/dx from Tu)
template <typename R, int H, int TR, int PL>
__device__ __forceinline__ void load_tileT_dx(C2<R>* buf, const C2<R>* __restrict__ T, int ny, int iy0, int kmax,
                                              double kxs0) {
    for (int i = threadIdx.x; i < H * TR; i += blockDim.x) {
        const int r = i % TR, kx = i / TR;
        buf[r * PL + pad8(kx)] = (kx < kmax) ? cimul<R>(T[(size_t)kx * ny + iy0 + r], (R)kx * (R)kxs0) : mk<R>(0, 0);
    }
}

// inverse x transform of one row buffer (after load + __syncthreads)
template <typename R, int H>
__device__ __forceinline__ void row_c2r(C2<R>* rb, const C2<R>* __restrict__ twR, const C2<R>* __restrict__ twX, int t) {
    c2r_merge<R, H>(rb, twR, t);
    block_fft<R, H, true>(rb, twX, t);
}

template <typename R, int H>
__device__ __forceinline__ void row_r2c(C2<R>* rb, const C2<R>* __restrict__ twR, const C2<R>* __restrict__ twX, int t) {
    block_fft<R, H, false>(rb, twX, t);
    r2c_split<R, H>(rb, twR, t);
}

// NB rows at rb + b * bstride at once (their stages share synchronisations and twiddles)
template <typename R, int H, int NB>
__device__ __forceinline__ void row_c2r_m(C2<R>* rb, int bstride, const C2<R>* __restrict__ twR,
                                          const C2<R>* __restrict__ twX, int t) {
    c2r_merge_m<R, H, NB>(rb, bstride, twR, t);
    block_fft_m<R, H, true, NB>(rb, bstride, twX, t);
}
template <typename R, int H, int NB>
__device__ __forceinline__ void row_r2c_m(C2<R>* rb, int bstride, const C2<R>* __restrict__ twR,
                                          const C2<R>* __restrict__ twX, int t) {
    block_fft_m<R, H, false, NB>(rb, bstride, twX, t);
    r2c_split_m<R, H, NB>(rb, bstride, twR, t);
}

// row_c2r_m with the transform's output in registers: v[b][q] = element t + q (H/8) of row b
// (the row buffers are free on return).  The merge runs in shared memory, the transform's
// stages exchange through it; the arithmetic is row_c2r_m's.
template <typename R, int H, int NB, int NBA>
__device__ __forceinline__ void row_c2r_reg(C2<R>* rb, int bstride, const C2<R>* __restrict__ twR,
                                            const C2<R>* __restrict__ twX, int t, C2<R> (&v)[NBA][8]) {
    constexpr int G = H / 8;
    c2r_merge_m<R, H, NB>(rb, bstride, twR, t);
#pragma unroll
    for (int b = 0; b < NB; ++b)
#pragma unroll
        for (int q = 0; q < 8; ++q) v[b][q] = rb[b * bstride + pad8(t + q * G)];
    __syncthreads();
    block_fft_reg_m<R, H, true, NB>(v, rb, bstride, twX, t);
}
// row_r2c_m of rows given in registers (v[b][q] = element t + q (H/8)); the rows must be free
// (synchronised after their last use).  The result is in the row buffers, as from row_r2c_m.
template <typename R, int H, int NB, int NBA>
__device__ __forceinline__ void row_r2c_reg(C2<R> (&v)[NBA][8], C2<R>* rb, int bstride, const C2<R>* __restrict__ twR,
                                            const C2<R>* __restrict__ twX, int t) {
    constexpr int G = H / 8;
    block_fft_reg_m<R, H, false, NB>(v, rb, bstride, twX, t);
#pragma unroll
    for (int b = 0; b < NB; ++b)
#pragma unroll
        for (int q = 0; q < 8; ++q) rb[b * bstride + pad8(t + q * G)] = v[b][q];
    __syncthreads();
    r2c_split_m<R, H, NB>(rb, bstride, twR, t);
}

template <typename R>
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// ======================================================================================
// Generic transforms (used by the ABI's coftxy/cofitxy and by the start-up path)
// ======================================================================================

// real field (phys0) -> T (spec0): forward x
template <typename R, int H>
__global__ void __launch_bounds__(XRows<R, H>::THREADS) k_xfwd(KArgs<R> a) {
    using X = XRows<R, H>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C2<R>* buf = reinterpret_cast<C2<R>*>(smem_raw);
    const int r = threadIdx.x / X::G, t = threadIdx.x % X::G;
    const int iy0 = blockIdx.x * X::TR, ny = a.g.ny;
    C2<R>* rb = buf + r * X::PL;
    const size_t boff = blockIdx.y * a.bstride;
    const C2<R>* f2 = reinterpret_cast<const C2<R>*>(a.phys0) + boff + (size_t)(iy0 + r) * H;
#pragma unroll
    for (int q = 0; q < 8; ++q) rb[pad8(t + q * X::G)] = f2[t + q * X::G];
    __syncthreads();
    row_r2c<R, H>(rb, a.twR, a.twX, t);
    C2<R>* T = a.spec0 + boff;
    for (int i = threadIdx.x; i < H * X::TR; i += blockDim.x) {
        const int rr = i % X::TR, kx = i / X::TR;
        T[(size_t)kx * ny + iy0 + rr] = buf[rr * X::PL + pad8(kx)];
    }
}

// T (spec0) -> real field (phys0): inverse x (unnormalised)
template <typename R, int H>
__global__ void __launch_bounds__(XRows<R, H>::THREADS) k_xinv(KArgs<R> a) {
    using X = XRows<R, H>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C2<R>* buf = reinterpret_cast<C2<R>*>(smem_raw);
    const int r = threadIdx.x / X::G, t = threadIdx.x % X::G;
    const int iy0 = blockIdx.x * X::TR, ny = a.g.ny;
    C2<R>* rb = buf + r * X::PL;
    const size_t boff = blockIdx.y * a.bstride;
    load_tileT<R, H, X::TR, X::PL>(buf, a.spec0 + boff, ny, iy0);
    cp_async_wait_f();
    __syncthreads();
    row_c2r<R, H>(rb, a.twR, a.twX, t);
    C2<R>* f2 = reinterpret_cast<C2<R>*>(a.phys0) + boff + (size_t)(iy0 + r) * H;
#pragma unroll
    for (int q = 0; q < 8; ++q) f2[t + q * X::G] = rb[pad8(t + q * X::G)];
}

// forward y of spec0 (T) -> spec1 (S), scaled by 1/(nx ny), ky = ny/2 zeroed
template <typename R, int NY>
__global__ void __launch_bounds__(NY / 8) k_yfwd(KArgs<R> a) {
    constexpr int G = NY / 8;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C2<R>* buf = reinterpret_cast<C2<R>*>(smem_raw);
    const int kx = blockIdx.x, t = threadIdx.x;
    const size_t boff = blockIdx.y * a.bstride;
    const C2<R>* in = a.spec0 + boff + (size_t)kx * NY;
#pragma unroll
    for (int q = 0; q < 8; ++q) buf[pad8(t + q * G)] = in[t + q * G];
    __syncthreads();
    block_fft<R, NY, false>(buf, a.twY, t);
    const R norm = (R)a.g.inv_nxny;
    C2<R>* out = a.spec1 + boff + (size_t)kx * NY;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int ky = t + q * G;
        C2<R> z = buf[pad8(ky)];
        out[ky] = (ky == NY / 2) ? mk<R>(0, 0) : cscale<R>(z, norm);
    }
}

// inverse y of op(spec1) -> spec0 (T)
template <typename R, int NY>
__global__ void __launch_bounds__(NY / 8) k_yinv(KArgs<R> a) {
    constexpr int G = NY / 8;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C2<R>* buf = reinterpret_cast<C2<R>*>(smem_raw);
    const int kx = blockIdx.x, t = threadIdx.x;
    const size_t boff = blockIdx.y * a.bstride;
    const C2<R>* in = a.spec1 + boff + (size_t)kx * NY;
    const Geometry& g = a.g;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int ky = t + q * G;
        const int ks = signed_k(ky, NY);
        C2<R> s = in[ky];
        C2<R> o = s;
        if (a.op != OP_ID) {
            const double k2 = (double)(kx * kx) * g.scalex + (double)(ks * ks) * g.scaley;
            const R kxs = (R)((double)kx * g.kxs), kys = (R)((double)ks * g.kys);
            if (a.op == OP_DX) o = cimul<R>(s, kxs);
            else if (a.op == OP_DY) o = cimul<R>(s, kys);
            else {
                C2<R> psi = (kx == 0 && ky == 0) ? mk<R>(0, 0) : cscale<R>(s, (R)(1.0 / k2));
                o = (a.op == OP_U) ? cimul<R>(psi, kys) : (a.op == OP_V) ? cimul<R>(psi, kxs) : cimul<R>(cimul<R>(psi, kys), kxs);
            }
        }
        if (ky == NY / 2) o = mk<R>(0, 0);
        buf[pad8(ky)] = o;
    }
    __syncthreads();
    block_fft<R, NY, true>(buf, a.twY, t);
    C2<R>* out = a.spec0 + boff + (size_t)kx * NY;
#pragma unroll
    for (int q = 0; q < 8; ++q) out[t + q * G] = buf[pad8(t + q * G)];
}

// ======================================================================================
// Start-up velocity: from Tu, Tv (inverse-y done) to u, v at `time` (cal_velocity) plus the
// statistics cal_nlk needs (max |u|^2, mean u, mean v).
// ======================================================================================
template <typename R, int H>
__global__ void __launch_bounds__(XRows<R, H>::THREADS) k_vel_x(KArgs<R> a) {
    using X = XRows<R, H>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C2<R>* bufA = reinterpret_cast<C2<R>*>(smem_raw);
    C2<R>* bufB = bufA + X::TR * X::PL;
    __shared__ double red_s[3][X::THREADS / 32];
    const int r = threadIdx.x / X::G, t = threadIdx.x % X::G;
    const int iy0 = blockIdx.x * X::TR, ny = a.g.ny;
    load_tileT<R, H, X::TR, X::PL>(bufA, a.Tu, ny, iy0);
    load_tileT<R, H, X::TR, X::PL>(bufB, a.Tv, ny, iy0);
    cp_async_wait_f();
    __syncthreads();
    row_c2r<R, H>(bufA + r * X::PL, a.twR, a.twX, t);
    row_c2r<R, H>(bufB + r * X::PL, a.twR, a.twX, t);
    const R U = (R)a.S->mean_u_next, V = (R)a.S->mean_v_next;
    const int iy = iy0 + r;
    C2<R>* u2 = reinterpret_cast<C2<R>*>(a.u) + (size_t)iy * H;
    C2<R>* v2 = reinterpret_cast<C2<R>*>(a.v) + (size_t)iy * H;
    double mx = 0.0, su = 0.0, sv = 0.0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int m = t + q * X::G;
        C2<R> ur = bufA[r * X::PL + pad8(m)], vr = bufB[r * X::PL + pad8(m)];
        C2<R> uu = mk<R>(ur.x + U, ur.y + U);
        C2<R> vv = mk<R>(-vr.x + V, -vr.y + V);
        if constexpr (kIsF32<R>) {  // FP32 form keeps the k=0 mean flow out of the stored field
            u2[m] = ur;
            v2[m] = mk<R>(-vr.x, -vr.y);
        } else {
            u2[m] = uu;
            v2[m] = vv;
        }
        mx = fmax(mx, fmax((double)(uu.x * uu.x + vv.x * vv.x), (double)(uu.y * uu.y + vv.y * vv.y)));
        su += (double)uu.x + (double)uu.y;
        sv += (double)vv.x + (double)vv.y;
    }
    mx = warp_max(mx);
    su = warp_sum<R>(su);
    sv = warp_sum<R>(sv);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { red_s[0][w] = mx; red_s[1][w] = su; red_s[2][w] = sv; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double m0 = 0.0, s0 = 0.0, s1 = 0.0;
        for (int i = 0; i < X::THREADS / 32; ++i) { m0 = fmax(m0, red_s[0][i]); s0 += red_s[1][i]; s1 += red_s[2][i]; }
        double* out = a.red + (size_t)blockIdx.x * RED_NSLOTS;
        if (blockIdx.x == 0) a.S->nred = (int)gridDim.x;
        for (int s = 0; s < RED_NSLOTS; ++s) out[s] = 0.0;
        out[RED_UMAX2] = m0;
        out[RED_SUM_U] = s0;
        out[RED_SUM_V] = s1;
    }
}

// ======================================================================================
// K2: nonlinear term and penalization in physical space (cal_nlk)
// ======================================================================================
// One tile of TR rows from iy0 (the whole kernel's work for one block)
// SPG: 1 the run has a vorticity sponge, 2 the sharp outflow sponge's integral (separate
// instantiations, so that the plain step keeps its registers)
template <typename R, int H, int TRV, int PART, int SPG>
__device__ __forceinline__ void nl_x_tile(const KArgs<R>& a, const int iy0) {
    using X = XRows<R, H, TRV>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C2<R>* bufA = reinterpret_cast<C2<R>*>(smem_raw);
    constexpr int BS = X::TR * X::PL;  // one row buffer (TR rows)
    C2<R>* bufB = bufA + BS;
    C2<R>* bufC = bufB + BS;
    const int r = threadIdx.x / X::G, t = threadIdx.x % X::G;
    const int ny = a.g.ny;
    constexpr int part = PART;
    // the penalization part: only the rows of the mask's box carry a non-zero term
    if (part == NL_PENAL && (iy0 + X::TR - 1 < a.rect[2] || iy0 > a.rect[3])) return;
    C2<R>* ra = bufA + r * X::PL;
    C2<R>* rb = bufB + r * X::PL;
    C2<R>* rc = bufC + r * X::PL;
    // the penalization part adds to the advection part's A: its values (kx < kcut <= H, at
    // most H / G per thread) are loaded first, to arrive while the transforms run
    static_assert(H % X::G == 0 && X::THREADS == X::TR * X::G, "one block: TR rows of G threads");
    constexpr int NLA = H / X::G;
    const int nout = a.kcut * X::TR;
    C2<R> av[NLA];
    if (part == NL_PENAL) {
#pragma unroll
        for (int u = 0; u < NLA; ++u) {
            const int i = threadIdx.x + u * blockDim.x;
            if (i < nout) av[u] = a.A[(size_t)(i / X::TR) * ny + iy0 + i % X::TR];
        }
    }
    C2<R> dxy[2][8];  // the vorticity's x and y derivatives at this thread's elements
    if (part != NL_PENAL) {
        // after the first AB2/Euler update the vorticity is dealiased: rows kx >= kcut are zero
        const int kin = a.explicit_step ? H : a.kcut;
        if constexpr (kIsF32<R>) load_tileT_dx<R, H, X::TR, X::PL>(bufA, a.Tw, ny, iy0, kin, a.g.kxs);
        else load_tileT<R, H, X::TR, X::PL>(bufA, a.Tdx, ny, iy0, kin);
        load_tileT<R, H, X::TR, X::PL>(bufB, a.Tdy, ny, iy0, kin);
        cp_async_wait_f();
        __syncthreads();
        row_c2r_reg<R, H, 2>(ra, BS, a.twR, a.twX, t, dxy);  // both together, to registers
    }
    // the vorticity sponge: the vorticity itself (x inverse of Tw, the inverse-y transform of the
    // state that k_nl_y left), for the term -F(mask_sponge omega) of cal_nlk
    C2<R> om[1][8];
    if constexpr (SPG == 1 && PART != NL_PENAL) {
        const int kin = a.explicit_step ? H : a.kcut;
        load_tileT<R, H, X::TR, X::PL>(bufA, a.Tw, ny, iy0, kin);
        cp_async_wait_f();
        __syncthreads();
        row_c2r_reg<R, H, 1>(ra, BS, a.twR, a.twX, t, om);
    }
    const int iy = iy0 + r;
    const size_t roff = (size_t)iy * H;
    const C2<R>* u2 = reinterpret_cast<const C2<R>*>(a.u) + roff;
    const C2<R>* v2 = reinterpret_cast<const C2<R>*>(a.v) + roff;
    const C2<R>* k2 = reinterpret_cast<const C2<R>*>(a.mask) + roff;
    const C2<R>* x2 = reinterpret_cast<const C2<R>*>(a.mvx) + roff;
    const C2<R>* y2 = reinterpret_cast<const C2<R>*>(a.mvy) + roff;
    const bool adv = part != NL_PENAL, pen = part != NL_ADVECT && a.penalize;
    // the rows to forward-transform: WHOLE w, pen_y, pen_x; ADVECT w; PENAL pen_y, pen_x
    C2<R> fw[3][8];
    C2<R> wv[8], pyv[8], pxv[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int m = t + q * X::G;
        C2<R> uu = u2[m], vv = v2[m];
        if constexpr (kIsF32<R>) {
            const R Uc = (R)a.S->mean_u_cur, Vc = (R)a.S->mean_v_cur;
            uu = mk<R>(uu.x + Uc, uu.y + Uc);
            vv = mk<R>(vv.x + Vc, vv.y + Vc);
        }
        if (adv) {
            const C2<R> dx = dxy[0][q], dy = dxy[1][q];
            wv[q] = mk<R>(-uu.x * dx.x - vv.x * dy.x, -uu.y * dx.y - vv.y * dy.y);
            if constexpr (SPG == 1) {
                const C2<R> sg = reinterpret_cast<const C2<R>*>(a.spg)[roff + m], w = om[0][q];
                wv[q] = mk<R>(wv[q].x - sg.x * w.x, wv[q].y - sg.y * w.y);
            }
        }
        if (pen) {
            const C2<R> kk = k2[m], mx = x2[m], my = y2[m];
            pxv[q] = mk<R>(-kk.x * (uu.x - mx.x), -kk.y * (uu.y - mx.y));
            pyv[q] = mk<R>(-kk.x * (vv.x - my.x), -kk.y * (vv.y - my.y));
            if constexpr (SPG == 2) {
                const C2<R> si = reinterpret_cast<const C2<R>*>(a.s10)[roff + m];
                pxv[q] = mk<R>(pxv[q].x + si.x, pxv[q].y + si.y);
            }
        } else {
            pxv[q] = mk<R>(0, 0);
            pyv[q] = mk<R>(0, 0);
        }
    }
    // the row buffers are free (the inverse transform returned them so; the penalization part
    // used none)
    if constexpr (PART == NL_WHOLE) {
#pragma unroll
        for (int q = 0; q < 8; ++q) { fw[0][q] = wv[q]; fw[1][q] = pyv[q]; fw[2][q] = pxv[q]; }
        row_r2c_reg<R, H, 3>(fw, ra, BS, a.twR, a.twX, t);  // into buffers A, B and C together
    } else if constexpr (PART == NL_ADVECT) {
#pragma unroll
        for (int q = 0; q < 8; ++q) fw[0][q] = wv[q];
        row_r2c_reg<R, H, 1>(fw, ra, BS, a.twR, a.twX, t);
    } else {
        // the penalization's y and x components into the buffers A and B (the whole kernel's
        // B and C)
#pragma unroll
        for (int q = 0; q < 8; ++q) { fw[0][q] = pyv[q]; fw[1][q] = pxv[q]; }
        row_r2c_reg<R, H, 2>(fw, ra, BS, a.twR, a.twX, t);
    }
    // the right-hand side only matters where the update keeps modes (kx < kcut):
    // A = X(w) + i kx X(pen_y), B = X(pen_x); the advection part writes X(w) and a zero B,
    // the penalization part adds its terms to that
    if constexpr (PART == NL_PENAL) {
#pragma unroll
        for (int u = 0; u < NLA; ++u) {
            const int i = threadIdx.x + u * blockDim.x;
            if (i < nout) {
                const int rr = i % X::TR, kx = i / X::TR;
                const size_t o = (size_t)kx * ny + iy0 + rr;
                const R kxs = kx_wave<R>(a, kx);
                a.A[o] = cadd<R>(av[u], cimul<R>(bufA[rr * X::PL + pad8(kx)], kxs));
                a.B[o] = bufB[rr * X::PL + pad8(kx)];
            }
        }
    } else {
        for (int i = threadIdx.x; i < nout; i += blockDim.x) {
            const int rr = i % X::TR, kx = i / X::TR;
            const size_t o = (size_t)kx * ny + iy0 + rr;
            const C2<R> xa = bufA[rr * X::PL + pad8(kx)];
            if constexpr (PART == NL_WHOLE) {
                const R kxs = kx_wave<R>(a, kx);
                a.A[o] = cadd<R>(xa, cimul<R>(bufB[rr * X::PL + pad8(kx)], kxs));
                a.B[o] = bufC[rr * X::PL + pad8(kx)];
            } else {
                a.A[o] = xa;
                a.B[o] = mk<R>(0, 0);
            }
        }
    }
}

// Blocks per SM that the fused x kernels' launch bounds ask for: MB > 0 an explicit count (the
// autotuner's "two blocks an SM" candidates cap the registers for it), else the kernel's default.
template <int MB, int DEF>
constexpr int xminb() { return MB > 0 ? MB : DEF; }

template <typename R, int H, int TRV, int PART = NL_WHOLE, int MB = 0, int SPG = 0>
__global__ void __launch_bounds__(XRows<R, H, TRV>::THREADS, (xminb<MB, 1>())) k_nl_x(KArgs<R> a) {
    pdl_wait();     // the previous kernel of the stream has completed
    using X = XRows<R, H, TRV>;
    if constexpr (PART == NL_ADVECT) {
        // the advection part runs beside the mask kernels on fewer blocks than tiles (the
        // launch gives one a SM), each taking tiles in turn, so that the raster launched after
        // it still finds room on every SM
        const int ntile = a.g.ny / X::TR;
        for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
            nl_x_tile<R, H, TRV, PART, SPG>(a, tile * X::TR);
            __syncthreads();  // the next tile reuses the row buffers
        }
    } else {
        nl_x_tile<R, H, TRV, PART, SPG>(a, blockIdx.x * X::TR);
    }
}

// The sharp outflow sponge (iSponge = 10, NavierStokes.f90:103-122): per row iy, the term added
// to the x penalization at ix in [ixmin, ixmax] is the trapezoid integral from ixmin to ix of
// w = -mask_sponge du/dx, mask_sponge = 1 / eps_sponge there.  One thread a row sums in the
// reference's order (the running sum adds the same terms as its sum from ixmin for every ix);
// the rest of the output stays zero.
template <typename R>
__global__ void __launch_bounds__(128) k_sponge10(const R* __restrict__ dudx, R* __restrict__ out, int nx, int ny,
                                                  int ixmin, int ixmax, double dx, double inv_eps) {
    const int iy = blockIdx.x * blockDim.x + threadIdx.x;
    if (iy >= ny || ixmin < 0 || ixmax >= nx) return;
    const R* d = dudx + (size_t)iy * nx;
    R* o = out + (size_t)iy * nx;
    double summe = 0.0, wprev = 0.0;
    for (int ix = ixmin; ix <= ixmax; ++ix) {
        const double w = -(inv_eps * (double)d[ix]);
        if (ix > ixmin) summe = summe + 0.5 * (wprev + w) * dx;
        o[ix] = (R)summe;
        wprev = w;
    }
}

// ======================================================================================
// K3: forward-y of the right-hand side, AB2 / Euler integrating-factor update, and the
// inverse-y transforms of everything the velocity/pressure/force kernels need.
// ======================================================================================
// Blocks per SM that k_nl_y's launch bounds ask for: in FP32 as many as 128 registers a thread
// allow (four at NY = 1024, so that its 512 rows run in one wave; one at NY = 4096), never
// fewer registers than that (fewer spill the transforms' state)
template <typename R, int NY>
constexpr int nl_y_minb() {
    return !kIsF32<R> ? 1 : (65536 / ((NY / 8) * 128) >= 4 ? 4 : (65536 / ((NY / 8) * 128) >= 1 ? 65536 / ((NY / 8) * 128) : 1));
}

template <typename R, int NY>
__global__ void __launch_bounds__(NY / 8, (nl_y_minb<R, NY>())) k_nl_y(KArgs<R> a) {
    pdl_wait();     // the previous kernel of the stream has completed
    constexpr int G = NY / 8;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C2<R>* bufA = reinterpret_cast<C2<R>*>(smem_raw);
    C2<R>* bufB = bufA + padded_len(NY);
    const int kx = blockIdx.x, t = threadIdx.x;
    const Geometry& g = a.g;
    const size_t row = (size_t)kx * NY;
    if (kx >= a.kcut) {
        // every mode of this row is removed by the 2/3 rule: the new state is exactly zero and
        // none of the inverse transforms is read (the x pass treats rows >= kcut as zero)
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            a.W[row + t + q * G] = mk<R>(0, 0);
            a.M[row + t + q * G] = mk<R>(0, 0);
            if constexpr (kIsF32<R>) a.Wlo[row + t + q * G] = mk<R>(0, 0);
        }
        return;
    }
    // FP32 form: the row's state (W, Wlo, M) flows into the spare buffers C, D, E while the
    // forward transforms run (unpadded rows of NY complex values)
    C2<R>* preW = bufA + 2 * padded_len(NY);
    C2<R>* preWl = bufA + 3 * padded_len(NY);
    C2<R>* preM = bufA + 4 * padded_len(NY);
    if constexpr (kIsF32<R>) {
        for (int e = t; e < NY / 2; e += G) {  // 16 bytes = two complex values per copy
            cp_async16_f(preW + 2 * e, a.W + row + 2 * e);
            cp_async16_f(preWl + 2 * e, a.Wlo + row + 2 * e);
            cp_async16_f(preM + 2 * e, a.M + row + 2 * e);
        }
    }
    // forward-y of A and B from registers (this thread's elements ky = t + q G) to registers
    C2<R> fab[2][8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        fab[0][q] = a.A[row + t + q * G];
        fab[1][q] = a.B[row + t + q * G];
    }
    block_fft_reg_m<R, NY, false, 2>(fab, bufA, padded_len(NY), a.twY, t);  // A and B together
    if constexpr (kIsF32<R>) {
        cp_async_wait_f();
        __syncthreads();
    }
    const DevScalars* S = a.S;
    const double dt1 = S->dt1, b10 = S->b10, b11 = S->b11;
    const bool expl = S->explicit_step != 0;
    const double norm = g.inv_nxny;
    const int cut = a.dcut[kx];
    C2<R> wn[8], ps[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int ky = t + q * G;
        const int ks = signed_k(ky, NY);
        const int ka = ks < 0 ? -ks : ks;
        const bool nyq = (ky == NY / 2);
        const R kys = (R)ks * (R)g.kys;
        const C2<R> fa = fab[0][q], fb = fab[1][q];
        C2<R> N = csub<R>(fa, cimul<R>(fb, kys));
        N = cscale<R>(N, (R)norm);
        if (nyq) N = mk<R>(0, 0);
        const bool keep = (g.idealis != 1) || (ka < cut);
        C2<R> Wn, Mn;
        if constexpr (kIsF32<R>) {
            const float2 ex = a.etabf[kx], ey = a.etabf[g.hx + ka];
            const float Eh = __fmul_rn(ex.x, ey.x);
            const float El = __fadd_rn(__fmaf_rn(ex.x, ey.x, -Eh), __fmaf_rn(ex.x, ey.y, __fmul_rn(ex.y, ey.x)));
            const C2<R> Wo = preW[ky], Wl = preWl[ky];
            float dx_, dy_;
            if (expl) {
                dx_ = (float)dt1 * N.x;
                dy_ = (float)dt1 * N.y;
            } else {
                const C2<R> Mo = preM[ky];
                dx_ = fmaf((float)b10, N.x, (float)b11 * Mo.x);
                dy_ = fmaf((float)b10, N.y, (float)b11 * Mo.y);
            }
            float h0, l0, h1, l1;
            ff_update(Wo.x, Wl.x, dx_, Eh, El, h0, l0);
            ff_update(Wo.y, Wl.y, dy_, Eh, El, h1, l1);
            if (!keep || nyq) { h0 = l0 = h1 = l1 = 0.f; }
            Wn = mk<R>(h0, h1);
            a.Wlo[row + ky] = mk<R>(l0, l1);
            Mn = cscale<R>(N, Eh);
        } else {
            const R E1 = a.etab[kx] * a.etab[g.hx + ka];
            const R D = keep ? (R)1 : (R)0;
            const C2<R> Wo = a.W[row + ky];
            if (expl) {
                Wn = mk<R>((Wo.x + (R)dt1 * N.x) * E1 * D, (Wo.y + (R)dt1 * N.y) * E1 * D);
            } else {
                const C2<R> Mo = a.M[row + ky];
                Wn = mk<R>(((Wo.x + (R)b10 * N.x) + (R)b11 * Mo.x) * E1 * D, ((Wo.y + (R)b10 * N.y) + (R)b11 * Mo.y) * E1 * D);
            }
            if (nyq) Wn = mk<R>(0, 0);
            Mn = cscale<R>(N, E1);
        }
        a.W[row + ky] = Wn;
        a.M[row + ky] = Mn;
        wn[q] = Wn;
        const R k2 = (R)(kx * kx) * (R)g.scalex + (R)(ks * ks) * (R)g.scaley;
        if (kx == 0 && ky == 0) ps[q] = mk<R>(0, 0);
        else if constexpr (kIsF32<R>) ps[q] = cscale<R>(Wn, (R)1 / k2);
        else ps[q] = mk<R>(Wn.x / k2, Wn.y / k2);   // poisson.f90:159-162 divides
    }
    // inverse-y outputs, NBO at a time: their transforms share the stages' synchronisations and
    // twiddle loads (NBO buffers of shared memory).  In the FP32 form the factor i kx, constant
    // along a kx row, is applied after the transform where that saves one: cofdx(omega) =
    // i kx T(omega) and d2psi/dxdy = i kx T(cofdy psi), so five spectra are transformed (cofdy
    // psi, cofdx psi, omega, cofdy omega, (kx^2 - ky^2) psi).  The FP64 form transforms all seven
    // in the reference's order (cofdx, then cofitxy), which keeps its roundings those of the
    // operators its adjoint transposes.
    // transforms at a time: the five FP32 buffers (the prefetched state they held is consumed),
    // so the FP32 form's five spectra take one round; two in FP64
    constexpr int NBO = kIsF32<R> ? 5 : 2;
    static_assert(NBO <= nl_y_bufs<R>(), "one shared-memory row buffer per transform");
    constexpr int PLY = padded_len(NY);
    const R kxs = (R)kx * (R)g.kxs;
    // spectra: 0 cofdy psi, 1 cofdx psi, 2 omega, 3 cofdy omega, 4 (kx^2 - ky^2) psi, and in
    // the FP64 form 5 cofdx omega, 6 d2psi/dxdy
    const int ntr = kIsF32<R> ? (a.viscous ? 5 : 4) : (a.viscous ? 7 : 5);
    for (int s0 = 0; s0 < ntr; s0 += NBO) {
        const int cnt = (ntr - s0 < NBO) ? ntr - s0 : NBO;
        // the spectra in registers (this thread's ky = t + q G), transformed with the
        // shared-memory rows as exchange buffers, stored from registers
        C2<R> ov[NBO][8];
#pragma unroll
        for (int b = 0; b < NBO; ++b) {
            const int sp = s0 + b;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int ky = t + q * G;
                const int ks = signed_k(ky, NY);
                const R kys = (R)ks * (R)g.kys;
                C2<R> val;
                // (FP64 without the stresses: spectra 0..3 and 5; sp 4 stands for 5 there)
                const int spk = (!kIsF32<R> && !a.viscous && sp == 4) ? 5 : sp;
                switch (spk) {
                    case 0: val = cimul<R>(ps[q], kys); break;                 // cofdy(psi)   -> u
                    case 1: val = cimul<R>(ps[q], kxs); break;                 // cofdx(psi)   -> -v
                    case 2: val = wn[q]; break;                                // omega
                    case 3: val = cimul<R>(wn[q], kys); break;                 // cofdy(omega)
                    case 4: val = cscale<R>(ps[q], kxs * kxs - kys * kys); break;  // du/dy + dv/dx
                    case 5: val = cimul<R>(wn[q], kxs); break;                 // cofdx(omega)
                    default: val = cscale<R>(ps[q], -(kxs * kys)); break;      // d2psi/dxdy = du/dx
                }
                if (ky == NY / 2) val = mk<R>(0, 0);
                ov[b][q] = val;
            }
        }
        // the buffers are free: the state loop above read the prefetched rows (buffers C..E),
        // and a previous round's transform ended synchronised
        __syncthreads();
        if (cnt == 5) {
            if constexpr (NBO >= 5) block_fft_reg_m<R, NY, true, 5>(ov, bufA, PLY, a.twY, t);
        } else if (cnt == 4) {
            if constexpr (NBO >= 4) block_fft_reg_m<R, NY, true, 4>(ov, bufA, PLY, a.twY, t);
        } else if (cnt == 3) {
            if constexpr (NBO >= 3) block_fft_reg_m<R, NY, true, 3>(ov, bufA, PLY, a.twY, t);
        } else if (cnt == 2) {
            block_fft_reg_m<R, NY, true, 2>(ov, bufA, PLY, a.twY, t);
        } else {
            block_fft_reg_m<R, NY, true, 1>(ov, bufA, PLY, a.twY, t);
        }
        for (int b = 0; b < cnt; ++b) {
            const int sp = s0 + b;
            const int spk = (!kIsF32<R> && !a.viscous && sp == 4) ? 5 : sp;
            C2<R>* dst = (spk == 0) ? a.Tu : (spk == 1) ? a.Tv : (spk == 2) ? a.Tw : (spk == 3) ? a.Tdy
                       : (spk == 4) ? a.Tsb : (spk == 5) ? a.Tdx : a.Tsa;
            // (FP32: cofdx(omega) = i kx Tw and du/dx = i kx Tu are formed by their readers as
            // they load Tw and Tu, load_tileT_dx)
#pragma unroll
            for (int q = 0; q < 8; ++q) dst[row + t + q * G] = ov[b][q];
        }
    }
}

// ======================================================================================
// K4: velocity at n+1, penalty, drag/energy reductions, vor_mean, Poisson RHS (forward-x),
// stresses to physical space.
// ======================================================================================
template <typename R, int H, int TRV, int MB = 0>
// (FP32: at most 128 registers a thread, so that two 256-thread blocks share an SM and the
// 1024^2 grid runs in one wave; FP64 is bound by its arithmetic and keeps its registers)
__global__ void __launch_bounds__(XRows<R, H, TRV>::THREADS,
                                  (xminb<MB, (sizeof(R) == 4) ? XRows<R, H, TRV>::MINB128 : 1>())) k_press_x(KArgs<R> a) {
    pdl_wait();     // the previous kernel of the stream has completed
    using X = XRows<R, H, TRV>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C2<R>* bufA = reinterpret_cast<C2<R>*>(smem_raw);
    constexpr int BS = X::TR * X::PL;  // one row buffer (TR rows)
    C2<R>* bufB = bufA + BS;
    C2<R>* bufC = bufB + BS;
    __shared__ double red_s[RED_NSLOTS][X::THREADS / 32 > 2 ? X::THREADS / 32 : 2];
    static_assert((kIsF32<R> ? (RED_NSLOTS + 1) * 4 : RED_NSLOTS * 8) * X::THREADS <= X::TR * X::PL * (int)sizeof(C2<R>),
                  "the reduction columns fit the spare row buffer");
    const int r = threadIdx.x / X::G, t = threadIdx.x % X::G;
    const int iy0 = blockIdx.x * X::TR, ny = a.g.ny;
    C2<R>* ra = bufA + r * X::PL;
    C2<R>* rb = bufB + r * X::PL;
    C2<R>* rc = bufC + r * X::PL;
    const DevScalars* S = a.S;
    const double time = S->time, dt1 = S->dt1;
    const R U = (R)S->mean_u_next, V = (R)S->mean_v_next;
    const int ixmin = S->win[0], ixmax = S->win[1], iymin = S->win[2], iymax = S->win[3];
    // FP32 form: time_avg_vort's weights time / (time + dt) and dt / (time + dt), once a block
    __shared__ float vm_w[2];
    if (kIsF32<R> && threadIdx.x == 0) { vm_w[0] = (float)(time / (time + dt1)); vm_w[1] = (float)(dt1 / (time + dt1)); }

    load_tileT<R, H, X::TR, X::PL>(bufA, a.Tu, ny, iy0, a.kcut);
    load_tileT<R, H, X::TR, X::PL>(bufB, a.Tv, ny, iy0, a.kcut);
    load_tileT<R, H, X::TR, X::PL>(bufC, a.Tw, ny, iy0, a.kcut);
    cp_async_wait_f();
    __syncthreads();
    // u, v and omega together, this thread's elements m = t + q G to registers (the row buffers
    // are free afterwards)
    C2<R> uvw[3][8];
    row_c2r_reg<R, H, 3>(ra, BS, a.twR, a.twX, t, uvw);
    C2<R> uv[8], vv[8], wv[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const C2<R> ur = uvw[0][q], vr = uvw[1][q];
        if constexpr (kIsF32<R>) {   // keep the raw perturbation; the mean is added in the FP32 path
            uv[q] = ur;
            vv[q] = mk<R>(-vr.x, -vr.y);
        } else {
            uv[q] = mk<R>(ur.x + U, ur.y + U);
            vv[q] = mk<R>(-vr.x + V, -vr.y + V);
        }
        wv[q] = uvw[2][q];
    }
    C2<R> pxy[2][8];  // the pressure right-hand side's x and y parts, for the forward transform

    const int iy = iy0 + r;
    const size_t roff = (size_t)iy * H;
    C2<R>* u2 = reinterpret_cast<C2<R>*>(a.u) + roff;
    C2<R>* v2 = reinterpret_cast<C2<R>*>(a.v) + roff;
    C2<R>* vm2 = reinterpret_cast<C2<R>*>(a.vor_mean) + roff;
    const C2<R>* k2 = reinterpret_cast<const C2<R>*>(a.mask) + roff;
    const C2<R>* x2 = reinterpret_cast<const C2<R>*>(a.mvx) + roff;
    const C2<R>* y2 = reinterpret_cast<const C2<R>*>(a.mvy) + roff;
    const bool in_rows = (iy >= iymin && iy <= iymax);
    double acc[RED_NSLOTS];
#pragma unroll
    for (int s = 0; s < RED_NSLOTS; ++s) acc[s] = 0.0;
    const double Ud = S->mean_u_next, Vd = S->mean_v_next;
    if constexpr (kIsF32<R>) {
        // FP32 form: stored velocity is the perturbation u' (mean flow U,V kept in FP64 scalars);
        // per-thread partial sums in FP32 over 16 cells, FP64 across threads and blocks.
        float f[RED_NSLOTS];
#pragma unroll
        for (int s = 0; s < RED_NSLOTS; ++s) f[s] = 0.f;
        float spx = 0.f, spy = 0.f;
        const float Uf = (float)Ud, Vf = (float)Vd;
        const float ca = vm_w[0], cb = vm_w[1];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int m = t + q * X::G;
            const C2<R> up = uv[q], vp = vv[q];
            u2[m] = up;
            v2[m] = vp;
            const C2<R> kk = k2[m], mx = x2[m], my = y2[m], w = wv[q], vmo = vm2[m];
            const float upc[2] = {up.x, up.y}, vpc[2] = {vp.x, vp.y}, wc[2] = {w.x, w.y};
            const float kc[2] = {kk.x, kk.y}, xc[2] = {mx.x, mx.y}, yc[2] = {my.x, my.y}, vmc[2] = {vmo.x, vmo.y};
            float px[2], py[2], vmn[2];
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int ix = 2 * m + e;
                const float uc = upc[e] + Uf, vc = vpc[e] + Vf;
                const float rx = uc - xc[e], ry = vc - yc[e];
                const float penx = kc[e] * rx, peny = kc[e] * ry;
                f[RED_OMEGA2] += wc[e] * wc[e];
                f[RED_KIN] += upc[e] * upc[e] + vpc[e] * vpc[e];
                f[RED_POROUS] += kc[e] * (rx * rx + ry * ry);
                f[RED_INFLOW_SOLID] += kc[e] * (xc[e] * rx + yc[e] * ry);
                spx += penx;
                spy += peny;
                f[RED_SUM_U] += uc;
                f[RED_SUM_V] += vc;
                f[RED_UMAX2] = fmaxf(f[RED_UMAX2], uc * uc + vc * vc);
                if (in_rows && ix >= ixmin && ix <= ixmax) {
                    f[RED_DRAG_X] += penx;
                    f[RED_DRAG_Y] += peny;
                    f[RED_UNST_X] += xc[e] * kc[e];
                    f[RED_UNST_Y] += yc[e] * kc[e];
                }
                vmn[e] = vmc[e] * ca + wc[e] * cb;
                px[e] = penx - wc[e] * vc;
                py[e] = peny + wc[e] * uc;
            }
            vm2[m] = mk<R>(vmn[0], vmn[1]);
            pxy[0][q] = mk<R>(px[0], px[1]);
            pxy[1][q] = mk<R>(py[0], py[1]);
        }
        // the FP32 partials go to the spare row buffer; the block reduces them in FP64 below
        float* cols = reinterpret_cast<float*>(bufC);
#pragma unroll
        for (int s = 0; s < RED_NSLOTS; ++s)
            cols[s * X::THREADS + threadIdx.x] = (s == RED_INFLOW_MEAN) ? spx : f[s];
        cols[RED_NSLOTS * X::THREADS + threadIdx.x] = spy;
    } else {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int m = t + q * X::G;
        const C2<R> uu = uv[q], vq = vv[q], w = wv[q];
        u2[m] = uu;
        v2[m] = vq;
        const C2<R> kk = k2[m], mx = x2[m], my = y2[m];
        const C2<R> vmo = vm2[m];
        R px[2], py[2];
        const R uc[2] = {uu.x, uu.y}, vc[2] = {vq.x, vq.y}, wc[2] = {w.x, w.y};
        const R kc[2] = {kk.x, kk.y}, xc[2] = {mx.x, mx.y}, yc[2] = {my.x, my.y}, vmc[2] = {vmo.x, vmo.y};
        R vmn[2];
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const int ix = 2 * m + e;
            const R rx = uc[e] - xc[e], ry = vc[e] - yc[e];
            const R penx = kc[e] * rx, peny = kc[e] * ry;
            acc[RED_OMEGA2] += (double)(wc[e] * wc[e]);
            const double du = (double)uc[e] - Ud, dv = (double)vc[e] - Vd;
            acc[RED_KIN] += du * du + dv * dv;
            acc[RED_POROUS] += (double)(kc[e] * (rx * rx + ry * ry));
            acc[RED_INFLOW_SOLID] += (double)(kc[e] * (xc[e] * rx + yc[e] * ry));
            acc[RED_INFLOW_MEAN] += Ud * (double)penx + Vd * (double)peny;
            acc[RED_SUM_U] += (double)uc[e];
            acc[RED_SUM_V] += (double)vc[e];
            acc[RED_UMAX2] = fmax(acc[RED_UMAX2], (double)(uc[e] * uc[e] + vc[e] * vc[e]));
            if (in_rows && ix >= ixmin && ix <= ixmax) {
                acc[RED_DRAG_X] += (double)penx;
                acc[RED_DRAG_Y] += (double)peny;
                acc[RED_UNST_X] += (double)(xc[e] * kc[e]);
                acc[RED_UNST_Y] += (double)(yc[e] * kc[e]);
            }
            vmn[e] = (R)(((double)vmc[e] * time + dt1 * (double)wc[e]) / (time + dt1));
            px[e] = penx - wc[e] * vc[e];
            py[e] = peny + wc[e] * uc[e];
        }
        vm2[m] = mk<R>(vmn[0], vmn[1]);
        pxy[0][q] = mk<R>(px[0], px[1]);
        pxy[1][q] = mk<R>(py[0], py[1]);
    }
    }
    // block reduction in a fixed order: every thread's partials go to the spare row buffer as
    // columns; one warp per column sums it in FP64 (its lanes over the column, then a shuffle
    // tree), far fewer FP64 warp instructions than a shuffle tree per warp and column
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    constexpr int NW = X::THREADS / 32;
    if constexpr (!kIsF32<R>) {
        double* cols = reinterpret_cast<double*>(bufC);
#pragma unroll
        for (int s = 0; s < RED_NSLOTS; ++s) cols[s * X::THREADS + threadIdx.x] = acc[s];
    }
    __syncthreads();
    constexpr int NCOL = kIsF32<R> ? RED_NSLOTS + 1 : RED_NSLOTS;  // FP32: spx and spy for INFLOW_MEAN
    for (int cidx = w; cidx < NCOL; cidx += NW) {
        const bool mx = cidx == RED_UMAX2;
        double v = 0.0;
        if constexpr (kIsF32<R>) {
            v = col_reduce_ff(reinterpret_cast<const float*>(bufC) + cidx * X::THREADS, X::THREADS, mx);
        } else {
            for (int i = l; i < X::THREADS; i += 32) {
                const double x = reinterpret_cast<const double*>(bufC)[cidx * X::THREADS + i];
                v = mx ? fmax(v, x) : v + x;
            }
            v = mx ? warp_max(v) : warp_sum<R>(v);
        }
        if (l == 0) {
            if (cidx < RED_NSLOTS) red_s[cidx][0] = v;
            else red_s[RED_INFLOW_MEAN][1] = v;  // FP32: the sum of spy (spx is in column INFLOW_MEAN)
        }
    }
    __syncthreads();
    if (threadIdx.x < RED_NSLOTS) {
        const int s = threadIdx.x;
        double v = red_s[s][0];
        if constexpr (kIsF32<R>)
            if (s == RED_INFLOW_MEAN) v = Ud * red_s[s][0] + Vd * red_s[s][1];
        a.red[(size_t)blockIdx.x * RED_NSLOTS + s] = v;
        if (blockIdx.x == 0 && s == 0) a.S->nred = (int)gridDim.x;
    }
    if (a.pressure_on) {
        row_r2c_reg<R, H, 2>(pxy, ra, BS, a.twR, a.twX, t);  // x and y parts together
        for (int i = threadIdx.x; i < H * X::TR; i += blockDim.x) {
            const int rr = i % X::TR, kx = i / X::TR;
            const R kxs = kx_wave<R>(a, kx);
            const size_t o = (size_t)kx * ny + iy0 + rr;
            a.P1[o] = cimul<R>(bufA[rr * X::PL + pad8(kx)], kxs);
            a.P2[o] = bufB[rr * X::PL + pad8(kx)];
        }
    }
    if (a.viscous && !a.stress_split) {
        __syncthreads();
        if constexpr (kIsF32<R>) load_tileT_dx<R, H, X::TR, X::PL>(bufA, a.Tu, ny, iy0, a.kcut, a.g.kxs);
        else load_tileT<R, H, X::TR, X::PL>(bufA, a.Tsa, ny, iy0, a.kcut);
        load_tileT<R, H, X::TR, X::PL>(bufB, a.Tsb, ny, iy0, a.kcut);
        cp_async_wait_f();
        __syncthreads();
        row_c2r_m<R, H, 2>(ra, BS, a.twR, a.twX, t);  // ra and rb together
        C2<R>* sa2 = reinterpret_cast<C2<R>*>(a.sa) + roff;
        C2<R>* sb2 = reinterpret_cast<C2<R>*>(a.sb) + roff;
        const R c2 = (R)(2.0 * a.nu), c1 = (R)a.nu;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int m = t + q * X::G;
            const C2<R> x = ra[pad8(m)], y = rb[pad8(m)];
            sa2[m] = mk<R>(c2 * x.x, c2 * x.y);
            sb2[m] = mk<R>(c1 * y.x, c1 * y.y);
        }
    }
}

// ---- k_press_x on paired rows (FP32) ---------------------------------------------------------
// The same work as k_press_x's FP32 form (the stresses in their own kernel), with the row
// transforms of the paired engine: H/16 threads a row, each holding two adjacent butterflies,
// 16-byte exchanges between the stages.  Rows of pair_slots(H) float4 slots; element e of a row
// sits at half e & 1 of slot padp(e >> 1).
template <int H, int TR>
struct XPairs {
    static constexpr int U = H / 16;                 // threads a row
    static constexpr int THREADS = U * TR;
    static constexpr int PS = pair_slots(H);         // float4 slots a row
    // three 128-thread blocks an SM: up to 170 registers a thread (the pairs' transforms of two
    // rows and the elementwise state need about 160)
    static constexpr int MINB = 3;
};
// The tile height of the paired kernel: 128 threads a block (H / 16 a row), at least one row.
template <int H>
constexpr int xpairs_rows() {
    return (128 / (H / 16)) > 0 ? 128 / (H / 16) : 1;
}

template <int H, int TR>
__device__ __forceinline__ void load_tileP(float4* buf, const float2* __restrict__ T, int ny, int iy0, int kmax) {
    constexpr int PS = pair_slots(H);
    for (int i = threadIdx.x; i < H * TR; i += blockDim.x) {  // asynchronous, as load_tileT
        const int r = i % TR, kx = i / TR;
        if (kx < kmax) cp_async_el<float>(&pel(buf + r * PS, kx), &T[(size_t)kx * ny + iy0 + r]);
        else pel(buf + r * PS, kx) = make_float2(0.f, 0.f);
    }
}

template <int H, int TR>
__global__ void __launch_bounds__(XPairs<H, TR>::THREADS, XPairs<H, TR>::MINB) k_press_x2(KArgs<float> a) {
    pdl_wait();     // the previous kernel of the stream has completed
    using X = XPairs<H, TR>;
    constexpr int G = H / 8, HG = X::U;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float4* bufA = reinterpret_cast<float4*>(smem_raw);
    constexpr int BS = TR * X::PS;  // one row buffer (TR rows)
    float4* bufB = bufA + BS;
    float4* bufC = bufB + BS;
    __shared__ double red_s[RED_NSLOTS][X::THREADS / 32 > 2 ? X::THREADS / 32 : 2];
    static_assert((RED_NSLOTS + 1) * 4 * X::THREADS <= BS * 16, "the reduction columns fit the spare row buffer");
    const int r = threadIdx.x / HG, u = threadIdx.x % HG;
    const int iy0 = blockIdx.x * TR, ny = a.g.ny;
    float4* ra = bufA + r * X::PS;
    const DevScalars* S = a.S;
    const double time = S->time, dt1 = S->dt1;
    const int ixmin = S->win[0], ixmax = S->win[1], iymin = S->win[2], iymax = S->win[3];
    // time_avg_vort's weights time / (time + dt) and dt / (time + dt), once a block
    __shared__ float vm_w[2];
    if (threadIdx.x == 0) { vm_w[0] = (float)(time / (time + dt1)); vm_w[1] = (float)(dt1 / (time + dt1)); }

    load_tileP<H, TR>(bufA, a.Tu, ny, iy0, a.kcut);
    load_tileP<H, TR>(bufB, a.Tv, ny, iy0, a.kcut);
    load_tileP<H, TR>(bufC, a.Tw, ny, iy0, a.kcut);
    cp_async_wait_f();
    __syncthreads();
    // u and v together, then omega (three rows at once would not fit 128 registers):
    // v[f][2m + h] = element 2u + h + m G (the rows are free afterwards)
    float2 uvw[2][16], ww[1][16];
    row_c2r_reg2<H, 2>(ra, BS, a.twR, a.twX, u, uvw);
    row_c2r_reg2<H, 1>(ra + 2 * BS, BS, a.twR, a.twX, u, ww);
    float2 pxy[2][16];  // the pressure right-hand side's x and y parts, for the forward transform

    const int iy = iy0 + r;
    const size_t roff = (size_t)iy * H;
    float2* u2 = reinterpret_cast<float2*>(a.u) + roff;
    float2* v2 = reinterpret_cast<float2*>(a.v) + roff;
    float2* vm2 = reinterpret_cast<float2*>(a.vor_mean) + roff;
    const float2* k2 = reinterpret_cast<const float2*>(a.mask) + roff;
    const float2* x2 = reinterpret_cast<const float2*>(a.mvx) + roff;
    const float2* y2 = reinterpret_cast<const float2*>(a.mvy) + roff;
    const bool in_rows = (iy >= iymin && iy <= iymax);
    const double Ud = S->mean_u_next, Vd = S->mean_v_next;
    // stored velocity is the perturbation u' (the mean flow U, V kept in FP64 scalars); per-thread
    // partial sums in FP32 over 32 cells, FP64 across threads and blocks
    float f[RED_NSLOTS];
#pragma unroll
    for (int s = 0; s < RED_NSLOTS; ++s) f[s] = 0.f;
    float spx = 0.f, spy = 0.f;
    const float Uf = (float)Ud, Vf = (float)Vd;
    const float ca = vm_w[0], cb = vm_w[1];
#pragma unroll
    for (int m = 0; m < 8; ++m) {
        const int e0 = 2 * u + m * G;  // elements e0 and e0 + 1: 16-byte accesses of the rows
        const float4 kk4 = *reinterpret_cast<const float4*>(k2 + e0), mx4 = *reinterpret_cast<const float4*>(x2 + e0);
        const float4 my4 = *reinterpret_cast<const float4*>(y2 + e0), vm4 = *reinterpret_cast<const float4*>(vm2 + e0);
        float out_u[4], out_v[4], out_vm[4];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const float2 ur = uvw[0][2 * m + h], vr = uvw[1][2 * m + h], w = ww[0][2 * m + h];
            const float upc[2] = {ur.x, ur.y}, vpc[2] = {-vr.x, -vr.y}, wc[2] = {w.x, w.y};
            const float kc[2] = {h ? kk4.z : kk4.x, h ? kk4.w : kk4.y};
            const float xc[2] = {h ? mx4.z : mx4.x, h ? mx4.w : mx4.y};
            const float yc[2] = {h ? my4.z : my4.x, h ? my4.w : my4.y};
            const float vmc[2] = {h ? vm4.z : vm4.x, h ? vm4.w : vm4.y};
            float px[2], py[2];
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int ix = 2 * (e0 + h) + e;
                const float uc = upc[e] + Uf, vc = vpc[e] + Vf;
                const float rx = uc - xc[e], ry = vc - yc[e];
                const float penx = kc[e] * rx, peny = kc[e] * ry;
                f[RED_OMEGA2] += wc[e] * wc[e];
                f[RED_KIN] += upc[e] * upc[e] + vpc[e] * vpc[e];
                f[RED_POROUS] += kc[e] * (rx * rx + ry * ry);
                f[RED_INFLOW_SOLID] += kc[e] * (xc[e] * rx + yc[e] * ry);
                spx += penx;
                spy += peny;
                f[RED_SUM_U] += uc;
                f[RED_SUM_V] += vc;
                f[RED_UMAX2] = fmaxf(f[RED_UMAX2], uc * uc + vc * vc);
                if (in_rows && ix >= ixmin && ix <= ixmax) {
                    f[RED_DRAG_X] += penx;
                    f[RED_DRAG_Y] += peny;
                    f[RED_UNST_X] += xc[e] * kc[e];
                    f[RED_UNST_Y] += yc[e] * kc[e];
                }
                out_u[2 * h + e] = upc[e];
                out_v[2 * h + e] = vpc[e];
                out_vm[2 * h + e] = vmc[e] * ca + wc[e] * cb;
                px[e] = penx - wc[e] * vc;
                py[e] = peny + wc[e] * uc;
            }
            pxy[0][2 * m + h] = make_float2(px[0], px[1]);
            pxy[1][2 * m + h] = make_float2(py[0], py[1]);
        }
        *reinterpret_cast<float4*>(u2 + e0) = make_float4(out_u[0], out_u[1], out_u[2], out_u[3]);
        *reinterpret_cast<float4*>(v2 + e0) = make_float4(out_v[0], out_v[1], out_v[2], out_v[3]);
        *reinterpret_cast<float4*>(vm2 + e0) = make_float4(out_vm[0], out_vm[1], out_vm[2], out_vm[3]);
    }
    // the FP32 partials go to the spare row buffer; the block reduces them in FP64 in a fixed
    // order (one warp a column)
    float* cols = reinterpret_cast<float*>(bufC);
#pragma unroll
    for (int s = 0; s < RED_NSLOTS; ++s) cols[s * X::THREADS + threadIdx.x] = (s == RED_INFLOW_MEAN) ? spx : f[s];
    cols[RED_NSLOTS * X::THREADS + threadIdx.x] = spy;
    __syncthreads();
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    constexpr int NW = X::THREADS / 32;
    for (int cidx = w; cidx < RED_NSLOTS + 1; cidx += NW) {
        const bool mx = cidx == RED_UMAX2;
        const double v = col_reduce_ff(cols + cidx * X::THREADS, X::THREADS, mx);
        if (l == 0) {
            if (cidx < RED_NSLOTS) red_s[cidx][0] = v;
            else red_s[RED_INFLOW_MEAN][1] = v;  // the sum of spy (spx is in column INFLOW_MEAN)
        }
    }
    __syncthreads();
    if (threadIdx.x < RED_NSLOTS) {
        const int s = threadIdx.x;
        double v = red_s[s][0];
        if (s == RED_INFLOW_MEAN) v = Ud * red_s[s][0] + Vd * red_s[s][1];
        a.red[(size_t)blockIdx.x * RED_NSLOTS + s] = v;
        if (blockIdx.x == 0 && s == 0) a.S->nred = (int)gridDim.x;
    }
    if (a.pressure_on) {
        row_r2c_reg2<H, 2>(pxy, ra, BS, a.twR, a.twX, u);  // x and y parts together (buffers A and B)
        for (int i = threadIdx.x; i < H * TR; i += blockDim.x) {
            const int rr = i % TR, kx = i / TR;
            const float kxs = a.kxw[kx];
            const size_t o = (size_t)kx * ny + iy0 + rr;
            a.P1[o] = cimul<float>(pel(bufA + rr * X::PS, kx), kxs);
            a.P2[o] = pel(bufB + rr * X::PS, kx);
        }
    }
}

// The viscous stresses (NavierStokes.f90:354-370: 2 nu d2psi/dxdy, nu (d2psi/dy2 - d2psi/dx2))
// to physical space, beside k_press_x on another stream: only GetForces reads them.  With
// a.srows set, a block whose rows no stencil of the forces reaches (rows j - 4 .. j + 4 of the
// stress points' cells j, BeamForces.f90:105-124, which lie within the stress points' offset
// of the beam's y range; k_step_begin forms the range into S->srow) leaves them.
template <typename R, int H, int TRV, int MB = 0>
__global__ void __launch_bounds__(XRows<R, H, TRV>::THREADS, (xminb<MB, 1>())) k_stress_x(KArgs<R> a) {
    using X = XRows<R, H, TRV>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C2<R>* bufA = reinterpret_cast<C2<R>*>(smem_raw);
    constexpr int BS = X::TR * X::PL;
    C2<R>* bufB = bufA + BS;
    const int r = threadIdx.x / X::G, t = threadIdx.x % X::G;
    const int iy0 = blockIdx.x * X::TR, ny = a.g.ny;
    if (a.srows) {
        const int j0 = a.S->srow[0], j1 = a.S->srow[1];
        if (iy0 + X::TR - 1 < j0 || iy0 > j1) return;
    }
    C2<R>* ra = bufA + r * X::PL;
    C2<R>* rb = bufB + r * X::PL;
    if constexpr (kIsF32<R>) load_tileT_dx<R, H, X::TR, X::PL>(bufA, a.Tu, ny, iy0, a.kcut, a.g.kxs);  // du/dx
    else load_tileT<R, H, X::TR, X::PL>(bufA, a.Tsa, ny, iy0, a.kcut);
    load_tileT<R, H, X::TR, X::PL>(bufB, a.Tsb, ny, iy0, a.kcut);
    cp_async_wait_f();
    __syncthreads();
    C2<R> sv[2][8];
    row_c2r_reg<R, H, 2>(ra, BS, a.twR, a.twX, t, sv);  // both together, to registers
    const size_t roff = (size_t)(iy0 + r) * H;
    C2<R>* sa2 = reinterpret_cast<C2<R>*>(a.sa) + roff;
    C2<R>* sb2 = reinterpret_cast<C2<R>*>(a.sb) + roff;
    const R c2 = (R)(2.0 * a.nu), c1 = (R)a.nu;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int m = t + q * X::G;
        const C2<R> x = sv[0][q], y = sv[1][q];
        sa2[m] = mk<R>(c2 * x.x, c2 * x.y);
        sb2[m] = mk<R>(c1 * y.x, c1 * y.y);
    }
}

// Threads of k_press_y: the paired FP32 engine (two butterflies a thread) or the one-butterfly
// engine (FP64).
// ENG = 1 forces the one-butterfly engine in FP32 (the autotuner's other candidate).
template <typename R, int NY, int ENG = 0> constexpr int press_y_threads() { return (kIsF32<R> && ENG == 0) ? NY / 16 : NY / 8; }

// K5, FP32: the paired engine.  Thread u holds the row's elements 2u + h + m (NY/8) as v[2m + h];
// the pairs are loaded from and stored to global memory as 16-byte accesses.  The arithmetic of
// each element is that of the one-butterfly form below.
template <int NY>
__device__ __forceinline__ void press_y_paired(const KArgs<float>& a) {
    constexpr int G = NY / 8, HG = G / 2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float4* buf = reinterpret_cast<float4*>(smem_raw);
    const int kx = blockIdx.x, u = threadIdx.x;
    const Geometry& g = a.g;
    const size_t row = (size_t)kx * NY;
    const float4* p1 = reinterpret_cast<const float4*>(a.P1 + row);
    const float4* p2 = reinterpret_cast<const float4*>(a.P2 + row);
    float2 fp[2][16];
#pragma unroll
    for (int m = 0; m < 8; ++m) {
        const float4 x = p1[u + m * HG], y = p2[u + m * HG];
        fp[0][2 * m] = make_float2(x.x, x.y); fp[0][2 * m + 1] = make_float2(x.z, x.w);
        fp[1][2 * m] = make_float2(y.x, y.y); fp[1][2 * m + 1] = make_float2(y.z, y.w);
    }
    block_fft2_m<NY, false, 2>(fp, buf, pair_slots(NY), a.twY, u);  // P1 and P2 together
    const float norm = (float)g.inv_nxny;
    float2 qv[1][16];
#pragma unroll
    for (int m = 0; m < 8; ++m)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int ky = 2 * u + h + m * G;
            const int ks = signed_k(ky, NY);
            const float kys = (float)ks * (float)g.kys;
            const float2 Q = cadd<float>(cscale<float>(fp[0][2 * m + h], norm), cimul<float>(cscale<float>(fp[1][2 * m + h], norm), kys));
            const float k2 = (float)(kx * kx) * (float)g.scalex + (float)(ks * ks) * (float)g.scaley;
            float2 qh = (kx == 0 && ky == 0) ? mk<float>(0, 0) : cscale<float>(Q, 1.0f / k2);
            if (ky == NY / 2) qh = mk<float>(0, 0);
            qv[0][2 * m + h] = qh;
        }
    block_fft2_m<NY, true, 1>(qv, buf, pair_slots(NY), a.twY, u);  // the forward transform left the rows free
    float4* tq = reinterpret_cast<float4*>(a.Tq + row);
#pragma unroll
    for (int m = 0; m < 8; ++m)
        tq[u + m * HG] = make_float4(qv[0][2 * m].x, qv[0][2 * m].y, qv[0][2 * m + 1].x, qv[0][2 * m + 1].y);
}

// K5: forward-y of the Poisson right-hand side, divergence, poisson, inverse-y -> Tq
template <typename R, int NY, int ENG = 0>
__global__ void __launch_bounds__(press_y_threads<R, NY, ENG>(), (kIsF32<R> && NY >= 4096) ? 2 : 1) k_press_y(KArgs<R> a) {
    pdl_wait();     // the previous kernel of the stream has completed
    if constexpr (kIsF32<R> && ENG == 0) {
        press_y_paired<NY>(a);
        return;
    }
    constexpr int G = NY / 8;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C2<R>* bufA = reinterpret_cast<C2<R>*>(smem_raw);
    C2<R>* bufB = bufA + padded_len(NY);
    const int kx = blockIdx.x, t = threadIdx.x;
    const Geometry& g = a.g;
    const size_t row = (size_t)kx * NY;
    // forward-y of P1 and P2 from registers (this thread's ky = t + q G) to registers
    C2<R> fp[2][8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        fp[0][q] = a.P1[row + t + q * G];
        fp[1][q] = a.P2[row + t + q * G];
    }
    block_fft_reg_m<R, NY, false, 2>(fp, bufA, padded_len(NY), a.twY, t);  // P1 and P2 together
    const R norm = (R)g.inv_nxny;
    C2<R> qv[1][8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int ky = t + q * G;
        const int ks = signed_k(ky, NY);
        const R kys = (R)ks * (R)g.kys;
        C2<R> Q = cadd<R>(cscale<R>(fp[0][q], norm), cimul<R>(cscale<R>(fp[1][q], norm), kys));
        const R k2 = (R)(kx * kx) * (R)g.scalex + (R)(ks * ks) * (R)g.scaley;
        C2<R> qh;
        if (kx == 0 && ky == 0) qh = mk<R>(0, 0);
        else if constexpr (kIsF32<R>) qh = cscale<R>(Q, (R)1 / k2);
        else qh = mk<R>(Q.x / k2, Q.y / k2);
        if (ky == NY / 2) qh = mk<R>(0, 0);
        qv[0][q] = qh;
    }
    // inverse-y of q from registers to registers (the forward transform left bufA free)
    block_fft_reg_m<R, NY, true, 1>(qv, bufA, padded_len(NY), a.twY, t);
#pragma unroll
    for (int q = 0; q < 8; ++q) a.Tq[row + t + q * G] = qv[0][q];
}

// K6: inverse-x of q, p = q - |u|^2/2
template <typename R, int H, int TRV, int MB = 0>
__global__ void __launch_bounds__(XRows<R, H, TRV>::THREADS, (xminb<MB, 1>())) k_press_fin(KArgs<R> a) {
    pdl_wait();     // the previous kernel of the stream has completed
    using X = XRows<R, H, TRV>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C2<R>* buf = reinterpret_cast<C2<R>*>(smem_raw);
    const int r = threadIdx.x / X::G, t = threadIdx.x % X::G;
    const int iy0 = blockIdx.x * X::TR, ny = a.g.ny;
    // in the fused step only the rows the forces' stencils reach (k_step_begin's S->srow, as
    // in k_stress_x); the host forms the other rows when the whole field is read
    if (a.srows) {
        const int j0 = a.S->srow[0], j1 = a.S->srow[1];
        if (iy0 + X::TR - 1 < j0 || iy0 > j1) return;
    }
    C2<R>* rb = buf + r * X::PL;
    const size_t roff = (size_t)(iy0 + r) * H;
    const C2<R>* u2 = reinterpret_cast<const C2<R>*>(a.u) + roff;
    const C2<R>* v2 = reinterpret_cast<const C2<R>*>(a.v) + roff;
    C2<R>* p2 = reinterpret_cast<C2<R>*>(a.press) + roff;
    // the velocity loads are issued before the transform, which hides their latency
    C2<R> ul[8], vl[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) { ul[q] = u2[t + q * X::G]; vl[q] = v2[t + q * X::G]; }
    load_tileT<R, H, X::TR, X::PL>(buf, a.Tq, ny, iy0);
    cp_async_wait_f();
    __syncthreads();
    C2<R> qv[1][8];
    row_c2r_reg<R, H, 1>(rb, X::PL, a.twR, a.twX, t, qv);  // to registers
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int m = t + q * X::G;
        const C2<R> qq = qv[0][q];
        C2<R> uu = ul[q], vq = vl[q];
        if constexpr (kIsF32<R>) {
            // the velocity press_x stored holds the mean flow at time + dt1 (mean_u_next; the
            // fluid step's last scalar kernel copies it to mean_u_cur, beside this kernel)
            const R Uc = (R)a.S->mean_u_next, Vc = (R)a.S->mean_v_next;
            uu = mk<R>(uu.x + Uc, uu.y + Uc);
            vq = mk<R>(vq.x + Vc, vq.y + Vc);
        }
        p2[m] = mk<R>(qq.x - (R)0.5 * (uu.x * uu.x + vq.x * vq.x), qq.y - (R)0.5 * (uu.y * uu.y + vq.y * vq.y));
    }
}

// ======================================================================================
// Dispatch table: one entry per supported length, filled by the inst_*.cu units.
// ======================================================================================
template <typename R>
struct SizeKernels {
    // x-pass kernels for H = nx/2
    void (*xfwd)(KArgs<R>);
    void (*xinv)(KArgs<R>);
    void (*vel_x)(KArgs<R>);
    void (*nl_x)(KArgs<R>);
    void (*press_x)(KArgs<R>);
    void (*press_fin)(KArgs<R>);
    int x_threads, x_rows, x_smem1, x_smem2;
    // tile-height candidates of the fused x kernels (index 1 is the default)
    struct XVariant {
        int rows, threads, smem1, smem3;  // smem3: the three row buffers of nl_x / press_x
        int minb;                         // blocks per SM asked of the launch bounds (0: default)
        void (*nl_x)(KArgs<R>);
        void (*nl_adv)(KArgs<R>);  // k_nl_x's advection and penalization parts (two buffers)
        void (*nl_pen)(KArgs<R>);
        void (*nl_x_spg)(KArgs<R>);   // nl_x and its advection part with the vorticity sponge,
        void (*nl_adv_spg)(KArgs<R>); // nl_x and its penalization part with the sharp outflow
        void (*nl_x_s10)(KArgs<R>);   // sponge's integral (the default tile only; null
        void (*nl_pen_s10)(KArgs<R>); // elsewhere)
        void (*stress_x)(KArgs<R>);  // two buffers
        void (*press_x)(KArgs<R>);
        void (*press_fin)(KArgs<R>);
    } xv[4];  // [0..2]: half, the default and twice the default tile height; [3]: the default, two blocks an SM
    XVariant xp;  // FP32: k_press_x on paired rows (press_x only; null in the FP64 form)
    // y-pass kernels for NY
    void (*yfwd)(KArgs<R>);
    void (*yinv)(KArgs<R>);
    void (*nl_y)(KArgs<R>);
    void (*press_y)(KArgs<R>);
    int y_threads, y_smem1, y_smem2, y_smem_nl;
    int press_y_threads;  // the paired FP32 engine runs NY/16 threads
    void (*press_y1)(KArgs<R>);  // FP32: k_press_y on the one-butterfly engine (NY/8 threads), or null
    int press_y1_smem;
};

template <typename R, int H, int TR, int MB = 0, bool SPG = false>
inline void fill_xvariant(typename SizeKernels<R>::XVariant& v) {
    using X = XRows<R, H, TR>;
    v.rows = TR;
    v.minb = MB;
    v.threads = X::THREADS;
    v.smem1 = (int)(TR * X::PL * sizeof(C2<R>));
    v.smem3 = 3 * v.smem1;
    v.nl_x = k_nl_x<R, H, TR, NL_WHOLE, MB>;
    v.nl_adv = k_nl_x<R, H, TR, NL_ADVECT, MB>;
    v.nl_pen = k_nl_x<R, H, TR, NL_PENAL, MB>;
    v.nl_x_spg = v.nl_adv_spg = v.nl_x_s10 = v.nl_pen_s10 = nullptr;
    if constexpr (SPG) {
        v.nl_x_spg = k_nl_x<R, H, TR, NL_WHOLE, MB, 1>;
        v.nl_adv_spg = k_nl_x<R, H, TR, NL_ADVECT, MB, 1>;
        v.nl_x_s10 = k_nl_x<R, H, TR, NL_WHOLE, MB, 2>;
        v.nl_pen_s10 = k_nl_x<R, H, TR, NL_PENAL, MB, 2>;
        cudaFuncSetAttribute(k_nl_x<R, H, TR, NL_WHOLE, MB, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, v.smem3);
        cudaFuncSetAttribute(k_nl_x<R, H, TR, NL_ADVECT, MB, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * v.smem1);
        cudaFuncSetAttribute(k_nl_x<R, H, TR, NL_WHOLE, MB, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, v.smem3);
        cudaFuncSetAttribute(k_nl_x<R, H, TR, NL_PENAL, MB, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * v.smem1);
    }
    v.stress_x = k_stress_x<R, H, TR, MB>;
    cudaFuncSetAttribute(k_stress_x<R, H, TR, MB>, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * v.smem1);
    cudaFuncSetAttribute(k_nl_x<R, H, TR, NL_ADVECT, MB>, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * v.smem1);
    cudaFuncSetAttribute(k_nl_x<R, H, TR, NL_PENAL, MB>, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * v.smem1);
    v.press_x = k_press_x<R, H, TR, MB>;
    v.press_fin = k_press_fin<R, H, TR, MB>;
    cudaFuncSetAttribute(k_nl_x<R, H, TR, NL_WHOLE, MB>, cudaFuncAttributeMaxDynamicSharedMemorySize, v.smem3);
    cudaFuncSetAttribute(k_press_x<R, H, TR, MB>, cudaFuncAttributeMaxDynamicSharedMemorySize, v.smem3);
    cudaFuncSetAttribute(k_press_fin<R, H, TR, MB>, cudaFuncAttributeMaxDynamicSharedMemorySize, v.smem1);
}

template <typename R, int N>
inline void fill_size_kernels(SizeKernels<R>& k) {
    constexpr int H = N / 2;
    using X = XRows<R, H>;
    k.xfwd = k_xfwd<R, H>;
    k.xinv = k_xinv<R, H>;
    k.vel_x = k_vel_x<R, H>;
    k.x_threads = X::THREADS;
    k.x_rows = X::TR;
    k.x_smem1 = (int)(X::TR * X::PL * sizeof(C2<R>));
    k.x_smem2 = 2 * k.x_smem1;
    cudaFuncSetAttribute(k_xfwd<R, H>, cudaFuncAttributeMaxDynamicSharedMemorySize, k.x_smem1);
    cudaFuncSetAttribute(k_xinv<R, H>, cudaFuncAttributeMaxDynamicSharedMemorySize, k.x_smem1);
    cudaFuncSetAttribute(k_vel_x<R, H>, cudaFuncAttributeMaxDynamicSharedMemorySize, k.x_smem2);
    constexpr int T0 = xrows_valid<R, H>(X::TRD / 2), T1 = X::TRD, T2 = xrows_valid<R, H>(X::TRD * 2);
    fill_xvariant<R, H, T0>(k.xv[0]);
    fill_xvariant<R, H, T1, 0, true>(k.xv[1]);
    fill_xvariant<R, H, T2>(k.xv[2]);
    // the default tile with the registers capped for two resident blocks (when two fit an SM)
    constexpr int MB2 = (2 * XRows<R, H, T1>::THREADS <= 2048) ? 2 : 1;
    fill_xvariant<R, H, T1, MB2>(k.xv[3]);
    k.xp = typename SizeKernels<R>::XVariant{};
    if constexpr (kIsF32<R>) {
        constexpr int TP = xpairs_rows<H>();
        k.xp.rows = TP;
        k.xp.threads = XPairs<H, TP>::THREADS;
        k.xp.smem3 = 3 * TP * pair_slots(H) * 16;
        k.xp.smem1 = k.xp.smem3 / 3;
        k.xp.minb = 16;  // the marker of the paired kernel in fsibe_tile_config
        k.xp.press_x = k_press_x2<H, TP>;
        cudaFuncSetAttribute(k_press_x2<H, TP>, cudaFuncAttributeMaxDynamicSharedMemorySize, k.xp.smem3);
    }
    k.nl_x = k.xv[1].nl_x;
    k.press_x = k.xv[1].press_x;
    k.press_fin = k.xv[1].press_fin;
    k.yfwd = k_yfwd<R, N>;
    k.yinv = k_yinv<R, N>;
    k.nl_y = k_nl_y<R, N>;
    k.press_y = k_press_y<R, N>;
    k.y_threads = N / 8;
    k.y_smem1 = (int)(padded_len(N) * sizeof(C2<R>));
    k.y_smem2 = 2 * k.y_smem1;
    if (kIsF32<R>) k.y_smem2 = std::max(k.y_smem2, 2 * pair_slots(N) * 16);
    k.press_y_threads = press_y_threads<R, N>();
    k.y_smem_nl = nl_y_bufs<R>() * k.y_smem1;
    cudaFuncSetAttribute(k_yfwd<R, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, k.y_smem1);
    cudaFuncSetAttribute(k_yinv<R, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, k.y_smem1);
    cudaFuncSetAttribute(k_nl_y<R, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, k.y_smem_nl);
    cudaFuncSetAttribute(k_press_y<R, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, k.y_smem2);
    k.press_y1 = nullptr;
    k.press_y1_smem = 2 * k.y_smem1;
    if constexpr (kIsF32<R>) {
        k.press_y1 = k_press_y<R, N, 1>;
        cudaFuncSetAttribute(k_press_y<R, N, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, k.press_y1_smem);
    }
}

}  // namespace fsibe
