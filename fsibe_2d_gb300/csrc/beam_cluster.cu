// beam_cluster.cu -- the Newton step of the beam (the work of k_beam: IBES_solver after the
// step's loads are known, SolidSolver.f90:197-414, with integrate_position and SolidEnergies)
// on one thread-block cluster of R CTAs (R = 16, or 8 where 16 cannot be placed).
//
// Why a cluster: FP64 issue limits the beam (one FP64 warp instruction per SMSP every ~64
// cycles on this chip) and one CTA has four SMSPs.  Spreading F, the Jacobian rows and the
// residuals over R SMs divides that work by R; the cluster's hardware barrier and distributed
// shared memory (DSMEM) keep every exchange between the SMs on chip.
//
// Layout: CTA r owns the interleaved rows [r n / R, (r+1) n / R) of the Newton system
// (n = 2 ns + 4): their F values, their FP64 Jacobian band rows, and the same rows of M^-1,
// the inverse of the row-scaled FP32 LU factor that preconditions the FP64 iterative
// refinement.  Every CTA keeps a full copy of the iterate x and of the refinement solution.
// One refinement pass:
//   FP64 residual of the own rows -> all-gather of the FP32 right-hand side -> barrier ->
//   own rows of M^-1 y (FP32) -> FP64 update of the own solution rows -> all-gather of those
//   rows and of the pass's maxima -> barrier -> the same convergence decision in every CTA.
// A new factor: each CTA scales its band rows and all-gathers them; every CTA runs the same
// FP32 band LU (the routine of the single-CTA kernel, so every copy is bitwise identical) and
// computes its own rows of M^-1 by transposed solves.  M^-1 persists between steps in global
// memory under the single-CTA kernel's reuse rule (kept while <= 5 passes per Newton step).
// The iterate update, the norms and the stopping test run redundantly in every CTA on
// identical data, so they need no exchange.
// Large beams (ns >= 512: M^-1's rows and the factor exceed a CTA's shared memory) run the
// same algorithm with both in global memory, where they stay L2-resident: each CTA reads its
// rows of M^-1 from its slice of the persistent copy, and factors its own copy of the band
// (the all-gather of the scaled rows writes every CTA's copy directly; the cluster barrier's
// release/acquire orders those global stores as it orders the DSMEM ones).
#include <math.h>

#include <mutex>

#include "beam_impl.cuh"
#include "running_sum.cuh"

namespace fsibe {
namespace {

// ---- cluster primitives (PTX) --------------------------------------------------------
__device__ __forceinline__ unsigned cl_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned cl_nrank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}
// Cluster-wide barrier of all threads; release/acquire orders the DSMEM writes before it
// against the reads after it.
__device__ __forceinline__ void cl_sync() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// The generic address of the same shared-memory location in CTA `rank` of the cluster.
template <typename T>
__device__ __forceinline__ T* cl_map(T* p, unsigned rank) {
    unsigned long long out;
    asm volatile("mapa.u64 %0, %1, %2;" : "=l"(out) : "l"(reinterpret_cast<unsigned long long>(p)), "r"(rank));
    return reinterpret_cast<T*>(out);
}
__device__ __forceinline__ void cp_async16(void* s, const void* g) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(s);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(g) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// ---- shared-memory layout (the same function sizes the launch on the host) ------------
// Row stride of M^-1: >= n, 16-byte rows, = 4 (mod 32) words.
__host__ __device__ inline int cl_mld(int n) { return ((n + 27) / 32) * 32 + 4; }
__host__ __device__ inline size_t al16(size_t v) { return (v + 15) & ~(size_t)15; }
constexpr int CL_NODE = 9;  // per-node FP64 arrays: tdn, bo3, bo4, bo5, bo6, oo5, oo6, old_rhs, taun_s

struct ClLayout {
    int n, L, R, rmax, mld;
    size_t x, xdi, node, bvec, band, part, slots, yf, fact, minv, total;  // byte offsets
};

// Floats of one CTA's global copy of the factor area in the large-beam form (the factor, or
// after the Newton loop the position sums, as in shared memory), a multiple of 4.
__host__ __device__ inline size_t cl_fact_floats(int ns) {
    const int n = 2 * ns + 4, L = ns + 8;
    const size_t fact = 25 * (size_t)(n + 16), post = 20 * (size_t)L;
    return ((fact > post ? fact : post) + 3) & ~(size_t)3;
}

// big: the factor area and M^-1 live in global memory (not in the shared-memory layout)
__host__ __device__ inline void cl_layout(int ns, int R, ClLayout& Y, bool big = false) {
    Y.n = 2 * ns + 4;
    Y.L = ns + 8;
    Y.R = R;
    Y.rmax = 4 * (((Y.n + 3) / 4 + R - 1) / R);  // rows are dealt in quads (cl_rows)
    Y.mld = cl_mld(Y.n);
    size_t o = 0;
    Y.x = o;     o = al16(o + 8 * (size_t)(Y.n + 8));
    Y.xdi = o;   o = al16(o + 8 * (size_t)(Y.n + 8));
    Y.node = o;  o = al16(o + 8 * (size_t)CL_NODE * Y.L);
    Y.bvec = o;  o = al16(o + 8 * (size_t)Y.rmax);
    Y.band = o;  o = al16(o + 8 * 16 * (size_t)Y.rmax);
    Y.part = o;  o = al16(o + 8 * 4 * (size_t)Y.rmax);
    Y.slots = o; o = al16(o + 8 * 4 * (size_t)R);
    Y.yf = o;    o = al16(o + 4 * (size_t)(Y.mld + 16));
    if (big) { Y.fact = Y.minv = Y.total = o; return; }
    Y.fact = o;
    // the factor (U 16, L 8 floats and a row-scale exponent per row); after the Newton loop
    // CTA 0 reuses it for the position sums (cs, pre: 4 L each) and th, thd (L each)
    const size_t fact = 4 * 25 * (size_t)(Y.n + 16), post = 8 * 10 * (size_t)Y.L;
    o = al16(o + (fact > post ? fact : post));
    Y.minv = o;  o = al16(o + 4 * (size_t)Y.rmax * Y.mld);
    Y.total = o;
}

// The rows [lo, hi) of CTA r: quads of rows dealt evenly, so that every CTA's slice of the FP32
// right-hand side (and of the FP64 solution) starts on a 16-byte boundary.
__host__ __device__ inline void cl_rows(int n, int R, int r, int& lo, int& hi) {
    const int nq = (n + 3) / 4;
    lo = 4 * (int)(((long long)r * nq) / R);
    hi = 4 * (int)(((long long)(r + 1) * nq) / R);
    lo = lo < n ? lo : n;
    hi = hi < n ? hi : n;
}

// Fortran equation (1-based) of interleaved row r: the inverse of row_of.
__device__ __forceinline__ int k_of_row(int ns, int r) {
    if (r <= 3) return (r == 3) ? 7 : r + 1;
    if (r >= 2 * ns) { const int q = r - 2 * ns; return (q == 0) ? 8 : 7 - q; }
    if ((r & 1) == 0) return 8 + (r / 2 - 1);
    return 8 + (ns - 2) + ((r - 1) / 2 - 1);
}

// Row i of M^-1 = (P L U)^-1 of the FP32 factor (band_factor_f32's U and L rows):
// z = U^-T e_i by forward substitution, then the transposed elimination steps in reverse
// order -- step k: v_k -= sum_r l_(k,r) v_(k+r), then the interchange of v_k and v_(k+p_k).
// Written to out[0 .. mld) (zeros from n on).
__device__ void inv_row(const float* __restrict__ U, const float* __restrict__ Lm, int n, int mld, int i,
                        float* __restrict__ out) {
    for (int k = 0; k < i; ++k) out[k] = 0.f;
    float zw[15];
#pragma unroll
    for (int j = 0; j < 15; ++j) zw[j] = 0.f;
    for (int k = i; k < n; ++k) {
        float acc = (k == i) ? 1.f : 0.f;
#pragma unroll
        for (int j = 14; j >= 2; --j) {
            const int m = (k - j) > 0 ? (k - j) : 0;  // rows before 0 meet zw[j] == 0
            acc = __fmaf_rn(-U[(size_t)m * 16 + j], zw[j], acc);
        }
        acc = __fmaf_rn(-U[(size_t)((k - 1) > 0 ? (k - 1) : 0) * 16 + 1], zw[1], acc);
        const float zk = __fmul_rn(acc, U[(size_t)k * 16]);
        out[k] = zk;
#pragma unroll
        for (int j = 14; j >= 2; --j) zw[j] = zw[j - 1];
        zw[1] = zk;
    }
    float wv[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) wv[r] = 0.f;
    for (int k = n - 1; k >= 0; --k) {
        if (k + 8 < n) out[k + 8] = wv[7];  // v_(k+8) is final: later steps reach k+6 at most
#pragma unroll
        for (int r = 7; r >= 1; --r) wv[r] = wv[r - 1];
        const float4 la = *reinterpret_cast<const float4*>(Lm + (size_t)k * 8);
        const float4 lb = *reinterpret_cast<const float4*>(Lm + (size_t)k * 8 + 4);
        float t = out[k];
        t = __fmaf_rn(-la.y, wv[1], t);
        t = __fmaf_rn(-la.z, wv[2], t);
        t = __fmaf_rn(-la.w, wv[3], t);
        t = __fmaf_rn(-lb.x, wv[4], t);
        t = __fmaf_rn(-lb.y, wv[5], t);
        t = __fmaf_rn(-lb.z, wv[6], t);
        t = __fmaf_rn(-lb.w, wv[7], t);
        wv[0] = t;
        const int p = __float_as_int(la.x);
        if (p != 0) {
#pragma unroll
            for (int r = 1; r <= 7; ++r)
                if (r == p) { wv[0] = wv[r]; wv[r] = t; }
        }
    }
#pragma unroll
    for (int r = 0; r < 8; ++r)
        if (r < n) out[r] = wv[r];
    for (int k = n; k < mld; ++k) out[k] = 0.f;
}

}  // namespace

#define PH(k) do { const long long t_ = clock64(); ph[k] += t_ - ph_t; ph_t = t_; } while (0)

// The cluster form of k_beam (one cluster of R CTAs of 256 threads; R from the launch).
// k_beam_pre of the same step ran before it and left the step's constants in b.pred.
// k_forces lets it start early (pdl_trigger): the set-up that reads only what earlier kernels
// wrote (the beam state, the predictor's output, the stored inverse rows) runs before its
// pdl_wait, which precedes every read of the forces' loads and of the status.
__global__ void __launch_bounds__(256, 1) k_beam_cl(BeamArgs b) {
    extern __shared__ __align__(16) unsigned char cl_smem[];
    DevScalars* S = b.S;
    const unsigned rank = cl_rank(), R = cl_nrank();
    const int ns = b.ns, n = 2 * ns + 4;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nthr = blockDim.x, nwarp = nthr >> 5;
    const bool big = b.cl_big != 0;
    const size_t fstride = cl_fact_floats(ns);
    ClLayout Y;
    cl_layout(ns, (int)R, Y, big);
    const int L = Y.L, mld = Y.mld, rmax = Y.rmax;
    int lo, hi;
    cl_rows(n, (int)R, (int)rank, lo, hi);
    const int nr = hi - lo;
    double* x = reinterpret_cast<double*>(cl_smem + Y.x);
    double* xdi = reinterpret_cast<double*>(cl_smem + Y.xdi);
    double* nd = reinterpret_cast<double*>(cl_smem + Y.node);
    double *tdn = nd, *bo3 = nd + L, *bo4 = nd + 2 * L, *bo5 = nd + 3 * L, *bo6 = nd + 4 * L, *oo5 = nd + 5 * L,
           *oo6 = nd + 6 * L, *old_rhs = nd + 7 * L, *taun_s = nd + 8 * L;
    double* bvec = reinterpret_cast<double*>(cl_smem + Y.bvec);
    double* band = reinterpret_cast<double*>(cl_smem + Y.band);
    double* part = reinterpret_cast<double*>(cl_smem + Y.part);
    // exchange words, written by every CTA into every CTA: [0, R) the passes' max |c| (FP32
    // bits), [R, 2R) max |x| (FP64 bits), [2R, 3R) the flags sent with the right-hand side,
    // [3R, 4R) the flags sent with the factor rows
    unsigned long long* slots = reinterpret_cast<unsigned long long*>(cl_smem + Y.slots);
    float* yf = reinterpret_cast<float*>(cl_smem + Y.yf);
    float* Uf = big ? b.clws + (size_t)rank * fstride : reinterpret_cast<float*>(cl_smem + Y.fact);
    float* Lf = Uf + (size_t)16 * (n + 16);
    int* rse = reinterpret_cast<int*>(Lf + (size_t)8 * (n + 16));
    float* minv = big ? b.minv + (size_t)rank * rmax * mld : reinterpret_cast<float*>(cl_smem + Y.minv);
    __shared__ D1DTab dtab;
    __shared__ NewtonCtx cs;
    __shared__ double red[2][8];
    __shared__ unsigned long long redu[2][8];
    __shared__ int flag_s, stop_s, info_s, dec_s;
    __shared__ float cprev_s;

    BeamWS w;
    memset(&w, 0, sizeof(w));
    w.x = x; w.tdn = tdn; w.bo5 = bo5; w.bo6 = bo6; w.oo5 = oo5; w.oo6 = oo6;
    w.old_rhs = old_rhs; w.taun_s = taun_s; w.dtab = &dtab; w.Uf = Uf; w.Lf = Lf; w.rse = rse;

    long long ph_t = clock64(), ph[28] = {};
    // the cluster barrier that guarantees every CTA runs before the first DSMEM access comes
    // just before that access (cl_up), so the set-up overlaps the CTAs' start
    bool cl_up = false;
    d1d_load(&dtab, b.d1d);
    const double time = S->time, dt = S->dt1, grav = S->grav;
    const double ds = b.ds, mue = b.mue, eta = b.eta;
    for (int i = tid; i < ns; i += nthr) {
        bo3[i] = b.vx[i]; bo4[i] = b.vy[i]; bo5[i] = b.th[i]; bo6[i] = b.thd[i];
        oo5[i] = b.oo[4 * ns + i]; oo6[i] = b.oo[5 * ns + i];
    }
    for (int i = n + tid; i < mld + 16; i += nthr) yf[i] = 0.f;
    if (tid == 0) flag_s = 0;
    __syncthreads();

    const bool released = time > b.t_release;
    const Motion mo = motion_at(b.mo, time + dt);  // mouvement(time + dt) of the new level
    int iter = 0;
    const bool have_inv = released && S->beam_fact != 0;
    if (released) {
        if (have_inv) {
            // this CTA's rows of M^-1 and their row-scale exponents, kept from an earlier step
            const float* g = b.minv + (size_t)rank * rmax * mld;
            const int nv = nr * mld / 4;
            if (!big)  // the large-beam form reads its rows where they are
                for (int q = tid; q < nv; q += nthr) cp_async16(minv + 4 * q, g + 4 * q);
            for (int k = lo + tid; k < hi; k += nthr) rse[k] = b.minv_rse[k];
        }
        for (int i = tid; i < n; i += nthr)
            if (i != xi_th(-1) && i != xi_T(ns, -1)) x[i] = b.pred[i];
    }
    pdl_wait();     // k_forces has completed: its loads and any status it raised are visible
    if (S->status != 0) {  // the same value in every CTA: they all return here
        cp_async_wait_all();
        return;
    }
    if (released) {
        const double* K = b.pred + pred_consts(ns);
        for (int i = tid; i < ns; i += nthr) {
            old_rhs[i] = b.pred[n + i];
            taun_s[i] = d1d(&dtab, b.tau_new, ns, 1, i);
        }
        // initial guess ghost values from the new loads (SolidSolver.f90:175-187, 197-202)
        // on warp 0, the Newton constants (divisions done by the predictor) on warp 1
        if (tid == 0) {
            const double* g5 = b.pred + n + ns;
            const double* T = g5 + ns;
            const double ds2 = ds * ds;
            const double K2 = b.p_new[0] + mue * (mo.le[5] * mo.ca - mo.le[4] * mo.sa + grav * mo.ca);
            const double C2v = 2.0 * ds * K2 - T[0] * g5[1] + (eta / ds2) * (10.0 * g5[0] - 12.0 * g5[1] + 6.0 * g5[2] - g5[3]);
            x[xi_th(-1)] = div_cr(C2v, K[8], K[9]);  // C2v / (3 eta/ds^2 - T_0), correctly rounded
            const double K1 = mue * (mo.le[4] * mo.ca + mo.le[5] * mo.sa + grav * mo.sa) - b.tau_new[0];
            const double th_ss0 = (2.0 * g5[0] - 5.0 * g5[1] + 4.0 * g5[2] - 1.0 * g5[3]) * b.k.ids2;
            const double th_s0 = (-1.5 * g5[0] + 2.0 * g5[1] - 0.5 * g5[2]) * b.k.ids;
            const double T_s0 = -eta * th_ss0 * th_s0 + K1;
            x[xi_T(ns, -1)] = T[1] - 2.0 * ds * T_s0;
        }
        if (tid == 32) {
            cs.time = time; cs.dt = dt; cs.dt_old = S->dt_old; cs.alpha_t = mo.alpha_t; cs.alpha_tt = mo.alpha_tt; cs.grav = grav;
            newton_consts_pre(cs, b, K);
            cs.K1 = mue * (mo.le[4] * mo.ca + mo.le[5] * mo.sa + grav * mo.sa) - b.tau_new[0];
            cs.K2 = b.p_new[0] + mue * (mo.le[5] * mo.ca - mo.le[4] * mo.sa + grav * mo.ca);
        }
        __syncthreads();
        const NewtonCtx& c = cs;
        bool inv_pending = have_inv && !big;  // the stored inverse rows are still arriving (cp.async)
        bool need_factor = !have_inv, factored = false;
        // own rows: generic ones [glo, ghi); the boundary equations (rows 0..3: k = 1, 2, 3, 7;
        // rows 2ns..2ns+3: k = 8, 6, 5, 4) sit in the first and last CTA and take warps 4..7,
        // one F or J evaluation per lane, so that their separate code paths do not serialise
        // a warp of generic rows
        const int glo = lo > 4 ? lo : 4, ghi = hi < 2 * ns ? hi : 2 * ns;
        const int ngen = ghi > glo ? ghi - glo : 0;
        const bool has_sp = (lo < 4) || (hi > 2 * ns);
        const int npairs = has_sp ? 2 : (nwarp >> 1);
        PH(22);
        for (;;) {
            for (int i = tid; i < ns; i += nthr)
                tdn[i] = c.D * (x[xi_th(i)] - c.C3 * bo5[i] - c.C4 * oo5[i]) - c.C2 * bo6[i];
            __syncthreads();
            // F (even warps) and the Jacobian rows (odd warps: another SMSP), 32 rows a pair
            if ((warp >> 1) < npairs) {
                for (int g = warp >> 1; g * 32 < ngen; g += npairs) {
                    const int r = glo + g * 32 + lane;
                    if (r < ghi) {
                        const int k = k_of_row(ns, r);
                        if ((warp & 1) == 0) {
                            const double f = f_eq(b, w, c, k);
                            if (isnan(f)) flag_s = FSIBE_ERR_NAN;
                            bvec[r - lo] = -1.0 * f;
                        } else if (jac_row(b, w, c, k, band + (size_t)(r - lo) * 16)) {
                            flag_s = FSIBE_ERR_NAN;
                        }
                    }
                }
            } else if (has_sp && warp >= 4) {
                // special s (0..3 in row order) -> F on warp 4 + 2 (s & 1), J on warp 5 + 2 (s & 1)
                const int s = 2 * lane + ((warp >> 1) & 1);
                const int base = (lo < 4) ? 0 : 2 * ns;
                const int r = base + s;
                if (lane < 2 && r >= lo && r < hi) {
                    const int k = k_of_row(ns, r);
                    if ((warp & 1) == 0) {
                        const double f = f_eq(b, w, c, k);
                        if (isnan(f)) flag_s = FSIBE_ERR_NAN;
                        bvec[r - lo] = -1.0 * f;
                    } else if (jac_row(b, w, c, k, band + (size_t)(r - lo) * 16)) {
                        flag_s = FSIBE_ERR_NAN;
                    }
                }
            }
            __syncthreads();
            PH(4);
            if (inv_pending) {
                cp_async_wait_all();
                inv_pending = false;
            }
            if (!cl_up) { cl_sync(); cl_up = true; }
            int solves = 0;
            for (int attempt = 0; attempt < 2; ++attempt) {
                const bool fresh = need_factor;
                if (need_factor) {
                    // the scaled FP32 rows: own copy first, then every other CTA's
                    for (int r = lo + tid; r < hi; r += nthr)
                        scale_band_row(band + (size_t)(r - lo) * 16, Uf + (size_t)r * 16, rse + r);
                    __syncthreads();
                    for (int e = tid; e < nr * 5 * ((int)R - 1); e += nthr) {
                        const unsigned dst = (rank + 1 + (unsigned)(e / (nr * 5))) % R;
                        const int q = e % (nr * 5), r = lo + q / 5, part5 = q % 5;
                        float* Ud = big ? b.clws + (size_t)dst * fstride : nullptr;  // dst's global copy
                        if (part5 < 4) {
                            float4* s4 = reinterpret_cast<float4*>(Uf + (size_t)r * 16) + part5;
                            if (big) reinterpret_cast<float4*>(Ud + (size_t)r * 16)[part5] = *s4;
                            else *cl_map(s4, dst) = *s4;
                        } else {
                            if (big) reinterpret_cast<int*>(Ud + (size_t)24 * (n + 16))[r] = rse[r];
                            else *cl_map(rse + r, dst) = rse[r];
                        }
                    }
                    if (tid < (int)R) *cl_map(slots + 3 * R + rank, (unsigned)tid) = (unsigned long long)flag_s;
                    cl_sync();
                    int fl = 0;
                    for (unsigned q = 0; q < R; ++q) fl = fl ? fl : (int)slots[3 * R + q];
                    if (fl) { if (rank == 0 && tid == 0) set_status(S, fl); return; }
                    if (warp == 0) {
                        const int info = band_factor_f32(w, n);
                        if (tid == 0) info_s = info;
                    }
                    __syncthreads();
                    if (info_s) { if (rank == 0 && tid == 0) set_status(S, FSIBE_ERR_SINGULAR); return; }
                    for (int t = tid; t < nr; t += nthr) inv_row(Uf, Lf, n, mld, lo + t, minv + (size_t)t * mld);
                    __syncthreads();
                    need_factor = false;
                    factored = true;
                }
                PH(5);
                bool ok = false;
                for (int pass = 0;; ++pass) {
                    // FP32 right-hand side of the own rows: -F, or the FP64 residual, its 15
                    // band products split in four column chunks over four warps (SMSPs)
                    if (pass > 0) {
                        const int ch = warp & 3;
                        for (int g = warp >> 2; g * 32 < nr; g += nwarp >> 2) {
                            const int t = g * 32 + lane;
                            if (t < nr) {
                                const int k = lo + t;
                                const double* Bk = band + (size_t)t * 16;
                                double acc = 0.0;
#pragma unroll
                                for (int u = 0; u < 4; ++u) {
                                    const int ci = 4 * ch + u, j = k - KL + ci;
                                    if (ci < BW && j >= 0 && j < n) acc = fma(Bk[ci], xdi[j], acc);
                                }
                                part[ch * rmax + t] = acc;
                            }
                        }
                        __syncthreads();
                    }
                    for (int t = tid; t < nr; t += nthr) {
                        const int k = lo + t;
                        double acc = bvec[t];
                        if (pass > 0) acc = acc - ((part[t] + part[rmax + t]) + (part[2 * rmax + t] + part[3 * rmax + t]));
                        yf[k] = __double2float_rn(acc * row_scale(rse[k]));
                    }
                    __syncthreads();
                    PH(19);
                    // the own rows to every other CTA, 16 bytes a store (slices start on quads)
                    {
                        const int nq4 = (nr + 3) / 4;
                        for (int e = tid; e < nq4 * ((int)R - 1); e += nthr) {
                            const unsigned dst = (rank + 1 + (unsigned)(e / nq4)) % R;
                            float4* p4 = reinterpret_cast<float4*>(yf + lo + 4 * (e % nq4));
                            *cl_map(p4, dst) = *p4;
                        }
                    }
                    if (tid < (int)R) *cl_map(slots + 2 * R + rank, (unsigned)tid) = (unsigned long long)flag_s;
                    PH(20);
                    cl_sync();
                    PH(16);
                    {
                        int fl = 0;
#pragma unroll
                        for (int q = 0; q < 16; ++q)
                            if (q < (int)R) fl = fl ? fl : (int)slots[2 * R + q];
                        if (fl) { if (rank == 0 && tid == 0) set_status(S, fl); return; }
                    }
                    // own rows of M^-1 y, eight rows per warp: lanes split the columns (float4),
                    // a transposing butterfly leaves the sum of row
                    // 4 ((l >> 4) & 1) + 2 ((l >> 3) & 1) + ((l >> 2) & 1) in lanes l = 0 (mod 4);
                    // those lanes update the FP64 solution rows
                    unsigned cm = 0;
                    unsigned long long xm = 0;
                    const float4* y4 = reinterpret_cast<const float4*>(yf);
                    for (int g = warp; g * 8 < nr; g += nwarp) {
                        const int t0 = g * 8;
                        const float4* mr[8];
#pragma unroll
                        for (int j = 0; j < 8; ++j) {
                            const int t = (t0 + j < nr) ? t0 + j : nr - 1;  // rows past nr: repeat the last
                            mr[j] = reinterpret_cast<const float4*>(minv + (size_t)t * mld);
                        }
                        float acc[8];
#pragma unroll
                        for (int j = 0; j < 8; ++j) acc[j] = 0.f;
                        for (int q = lane; q < (mld >> 2); q += 32) {
                            const float4 v = y4[q];
#pragma unroll
                            for (int j = 0; j < 8; ++j) {
                                const float4 m = mr[j][q];
                                acc[j] = __fmaf_rn(m.x, v.x, acc[j]);
                                acc[j] = __fmaf_rn(m.y, v.y, acc[j]);
                                acc[j] = __fmaf_rn(m.z, v.z, acc[j]);
                                acc[j] = __fmaf_rn(m.w, v.w, acc[j]);
                            }
                        }
                        {
                            const bool up = (lane & 16) != 0;
#pragma unroll
                            for (int j = 0; j < 4; ++j) {
                                const float send = up ? acc[j] : acc[j + 4], keep = up ? acc[j + 4] : acc[j];
                                acc[j] = __fadd_rn(keep, __shfl_xor_sync(0xffffffffu, send, 16));
                            }
                            const bool b8 = (lane & 8) != 0;
#pragma unroll
                            for (int j = 0; j < 2; ++j) {
                                const float send = b8 ? acc[j] : acc[j + 2], keep = b8 ? acc[j + 2] : acc[j];
                                acc[j] = __fadd_rn(keep, __shfl_xor_sync(0xffffffffu, send, 8));
                            }
                            const bool b4 = (lane & 4) != 0;
                            const float send = b4 ? acc[0] : acc[1], keep = b4 ? acc[1] : acc[0];
                            acc[0] = __fadd_rn(keep, __shfl_xor_sync(0xffffffffu, send, 4));
                            acc[0] = __fadd_rn(acc[0], __shfl_xor_sync(0xffffffffu, acc[0], 2));
                            acc[0] = __fadd_rn(acc[0], __shfl_xor_sync(0xffffffffu, acc[0], 1));
                        }
                        const int t = t0 + 4 * ((lane >> 4) & 1) + 2 * ((lane >> 3) & 1) + ((lane >> 2) & 1);
                        if ((lane & 3) == 0 && t < nr) {
                            const float s = acc[0];
                            const int k = lo + t;
                            const double xn = (pass == 0) ? (double)s : xdi[k] + (double)s;
                            xdi[k] = xn;
                            const unsigned a = __float_as_uint(s) & 0x7fffffffu;
                            const unsigned long long ax = (unsigned long long)__double_as_longlong(xn) & 0x7fffffffffffffffull;
                            cm = (a > cm) ? a : cm;
                            xm = (ax > xm) ? ax : xm;
                        }
                    }
#pragma unroll
                    for (int o = 16; o >= 4; o >>= 1) {
                        const unsigned c2 = __shfl_xor_sync(0xffffffffu, cm, o);
                        const unsigned long long x2 = __shfl_xor_sync(0xffffffffu, xm, o);
                        cm = (c2 > cm) ? c2 : cm;
                        xm = (x2 > xm) ? x2 : xm;
                    }
                    if (lane == 0) { redu[0][warp] = cm; redu[1][warp] = xm; }
                    __syncthreads();
                    PH(17);
                    if (tid < (int)R) {
                        unsigned long long c2 = 0, x2 = 0;
                        for (int q = 0; q < nwarp; ++q) {
                            c2 = (redu[0][q] > c2) ? redu[0][q] : c2;
                            x2 = (redu[1][q] > x2) ? redu[1][q] : x2;
                        }
                        *cl_map(slots + rank, (unsigned)tid) = c2;
                        *cl_map(slots + R + rank, (unsigned)tid) = x2;
                    }
                    // the own solution rows to every other CTA, 16 bytes a store
                    {
                        const int nq2 = (nr + 1) / 2;
                        for (int e = tid; e < nq2 * ((int)R - 1); e += nthr) {
                            const unsigned dst = (rank + 1 + (unsigned)(e / nq2)) % R;
                            double2* p2 = reinterpret_cast<double2*>(xdi + lo + 2 * (e % nq2));
                            *cl_map(p2, dst) = *p2;
                        }
                    }
                    PH(21);
                    cl_sync();
                    PH(18);
                    ++solves;
                    // the convergence decision of refine_step from the cluster's maxima, on one
                    // thread (FP64 issue is per warp)
                    if (tid == 0) {
                        unsigned long long c2 = 0, x2 = 0;
                        for (int q = 0; q < (int)R; ++q) {
                            c2 = (slots[q] > c2) ? slots[q] : c2;
                            x2 = (slots[R + q] > x2) ? slots[R + q] : x2;
                        }
                        const float cpf = (pass == 0) ? 0.f : cprev_s;
                        const double cmd = (double)__uint_as_float((unsigned)c2), cpd = (double)cpf;
                        const double xmd = __longlong_as_double((long long)x2);
                        // 2^-30 of the correction (refine_step says why that suffices)
                        const double tol = 0x1p-30 * xmd;
                        const bool conv = !(cmd > tol) || (pass >= 1 && cmd * cmd <= tol * cpd);
                        const bool stall = pass >= 2 && cmd > 0.5 * cpd;
                        cprev_s = __uint_as_float((unsigned)c2);
                        dec_s = (conv || (stall && cmd <= 0x1p-30 * xmd)) ? 1 : ((stall || pass >= 9) ? -1 : 0);
                    }
                    __syncthreads();
                    const int dec = dec_s;
                    if (dec > 0) { ok = true; break; }
                    if (dec < 0) break;
                }
                if (ok || fresh) break;
                need_factor = true;
            }
            if (solves > 5) need_factor = true;
            if (tid == 0) ph[10] += solves;
            PH(6);
            // x += dx in Fortran order, the norms and the stopping test: the same data in every
            // CTA, so the same decisions without an exchange
            // the stopping test needs iter > 2: before that the norms are not formed
            const bool test = iter + 1 > 2;
            double sd = 0.0, sx = 0.0;
            for (int l = tid; l < n; l += nthr) {
                const double d = xdi[col_of(ns, l + 1)];
                if (isnan(d)) flag_s = FSIBE_ERR_NAN;
                const double xn = x[l] + d;
                x[l] = xn;
                if (test) {
                    sd += d * d;
                    sx += xn * xn;
                }
            }
            if (test) {
                for (int o = 16; o > 0; o >>= 1) {
                    sd += __shfl_xor_sync(0xffffffffu, sd, o);
                    sx += __shfl_xor_sync(0xffffffffu, sx, o);
                }
                if (lane == 0) { red[0][warp] = sd; red[1][warp] = sx; }
            }
            __syncthreads();
            if (flag_s) { if (rank == 0 && tid == 0) set_status(S, flag_s); return; }
            iter = iter + 1;
            if (test) {
                if (tid < 32) {
                    double tsd = (lane < nwarp) ? red[0][lane] : 0.0, tsx = (lane < nwarp) ? red[1][lane] : 0.0;
                    for (int o = 4; o > 0; o >>= 1) {
                        tsd += __shfl_xor_sync(0xffffffffu, tsd, o);
                        tsx += __shfl_xor_sync(0xffffffffu, tsx, o);
                    }
                    if (lane == 0) stop_s = newton_stop(tsd, tsx, b.tol);
                }
                __syncthreads();
            } else if (tid == 0) {
                stop_s = 0;
            }
            __syncthreads();
            PH(23);
            const bool stop = stop_s != 0;
            if (iter > b.maxit - 1) {
                if (rank == 0 && tid == 0) set_status(S, FSIBE_ERR_NEWTON_MAXIT);
                return;
            }
            if (stop) break;
            __syncthreads();
        }
        if (factored) {
            float* g = b.minv + (size_t)rank * rmax * mld;
            const int nv = nr * mld / 4;
            if (!big)  // the large-beam form formed its rows in place
                for (int q = tid; q < nv; q += nthr)
                    reinterpret_cast<float4*>(g)[q] = reinterpret_cast<const float4*>(minv)[q];
            for (int k = lo + tid; k < hi; k += nthr) b.minv_rse[k] = rse[k];
            if (rank == 0 && tid == 0) S->beam_fact = 1;
        }
    }
    PH(7);
    // integrate_position (integrate_position.f90:14-44): each CTA evaluates theta, theta_dot
    // and the four position increments of its nodes into CTA 0; CTA 0 runs the sums in order.
    // They go to the start of CTA 0's factor area (cs[4][L], pre[4][L], th[L], thd[L]: 80 L
    // bytes), which its factor no longer needs; its row exponents, which it may still be
    // saving, start 96 (n + 16) > 80 L bytes in.  The third sum subtracts: its terms are
    // stored negated and added (s - a and s + (-a) round the same).
    double* pcs = big ? reinterpret_cast<double*>(b.clws) : reinterpret_cast<double*>(cl_smem + Y.fact);
    if (!cl_up) { cl_sync(); cl_up = true; }
    {
        const int q0 = (int)(((long long)rank * ns) / R), q1 = (int)(((long long)(rank + 1) * ns) / R);
        double* dst = big ? pcs : cl_map(pcs, 0u);  // CTA 0's area (its global copy when big)
        for (int i = q0 + tid; i < q1; i += nthr) {
            double th, td;
            if (released) {
                th = x[xi_th(i)];
                td = cs.D * (th - cs.C3 * bo5[i] - cs.C4 * oo5[i]) - cs.C2 * bo6[i];
            } else {
                th = b.th[i];
                td = b.thd[i];
            }
            double sn, cn;
            sincos(th, &sn, &cn);
            dst[i] = cn * ds;
            dst[L + i] = sn * ds;
            dst[2 * L + i] = -(td * sn * ds);
            dst[3 * L + i] = td * cn * ds;
            dst[8 * L + i] = th;
            dst[9 * L + i] = td;
        }
    }
    PH(24);
    cl_sync();  // the last DSMEM traffic; CTAs other than 0 are done
    if (rank != 0) return;
    PH(25);
    const double* thv = pcs + 8 * L;
    const double* tdv = pcs + 9 * L;
    // the new angles and rates, and beam_oldold = beam_old (the state at entry); done by the
    // threads that the running sums leave idle
    auto copies = [&](int i0, int stride) {
        if (!released) return;
        for (int i = i0; i < ns; i += stride) { b.th[i] = thv[i]; b.thd[i] = tdv[i]; }
        for (int i = i0; i < ns; i += stride) {
            b.oo[0 * ns + i] = b.x[i]; b.oo[1 * ns + i] = b.y[i]; b.oo[2 * ns + i] = bo3[i];
            b.oo[3 * ns + i] = bo4[i]; b.oo[4 * ns + i] = bo5[i]; b.oo[5 * ns + i] = bo6[i];
        }
    };
    if (released && tid == 0) {
        S->newton_iters = iter;
        if (S->actually_bdf2) { S->method = FSIBE_BDF2; S->actually_bdf2 = 0; }
        S->dt_old = dt;
    }
    // the four running sums in the reference's order (the positions decide grid-aligned boxes
    // of the mask and the drag window, so their roundings must be the reference's): one lane a
    // sum in integer arithmetic, checked step by step (running_sum.cuh), while the other warps
    // copy.  The large-beam form first stages the terms into the shared memory of the solution
    // vectors x and xdi (32 ns + 192 bytes, at least the 32 ns needed), which the Newton loop
    // is done with.
    const double* src0 = pcs;
    if (big) {
        double* st = x;  // x, then xdi: contiguous
        for (int i = tid; i < ns; i += nthr) {
            st[i] = pcs[i]; st[ns + i] = pcs[L + i]; st[2 * ns + i] = pcs[2 * L + i]; st[3 * ns + i] = pcs[3 * L + i];
        }
        src0 = st;
        __syncthreads();
    }
    {
        __shared__ int rs_flags[4];
        const int nser = running_sums4(src0, big ? ns : L, pcs + 4 * L, L, ns, rs_flags, copies);
        if (tid == 0 && nser) S->phase[30] += nser;
    }
    PH(8);
    // positions and velocities, and in the same pass each thread's terms of the emergency brake
    // (SolidSolver.f90:370-380) and of SolidEnergies (SolidSolver.f90:76-92); the block then
    // reduces the six columns in FP64, one warp a column
    {
        __shared__ double ecol[6][256];
        static_assert(256 >= 32 * 6, "one warp a column");
        const double* pre = pcs + 4 * L;
        const double ca = mo.ca, sa = mo.sa, alpha_t = mo.alpha_t, idt = 1.0 / dt;
        double sk = 0, sp = 0, se = 0, sax = 0, say = 0, mx = 0;
        for (int i = tid; i < ns; i += nthr) {
            const double xrel = pre[i], yrel = pre[L + i];
            const double vxrel = pre[2 * L + i], vyrel = pre[3 * L + i];
            const double yi = mo.le[1] + yrel * ca + xrel * sa;
            b.x[i] = mo.le[0] + xrel * ca - yrel * sa;
            b.y[i] = yi;
            const double vx = mo.le[2] + ca * (vxrel - alpha_t * yrel) - sa * (vyrel + alpha_t * xrel);
            const double vy = mo.le[3] + ca * (vyrel + alpha_t * xrel) + sa * (vxrel - alpha_t * yrel);
            b.vx[i] = vx;
            b.vy[i] = vy;
            double ax, ay;
            if (released) {
                ax = (vx - bo3[i]) * idt;
                ay = (vy - bo4[i]) * idt;
                b.ax[i] = ax;
                b.ay[i] = ay;
                mx = fmax(mx, fabs(tdv[i] - bo6[i]));
            } else {
                ax = b.ax[i];
                ay = b.ay[i];
            }
            const double th_s = d1d(&dtab, thv, ns, 1, i);
            sk += vx * vx + vy * vy;
            sp += yi - b.y0;
            se += th_s * th_s;
            sax += ax;
            say += ay;
        }
        ecol[0][tid] = sk; ecol[1][tid] = sp; ecol[2][tid] = se;
        ecol[3][tid] = sax; ecol[4][tid] = say; ecol[5][tid] = mx;
        __syncthreads();
        PH(26);
        if (warp < 6) {
            double v = 0.0;
            for (int k = lane; k < nthr; k += 32) v = (warp == 5) ? fmax(v, ecol[5][k]) : v + ecol[warp][k];
            for (int o = 16; o > 0; o >>= 1) {
                const double u = __shfl_xor_sync(0xffffffffu, v, o);
                v = (warp == 5) ? fmax(v, u) : v + u;
            }
            if (lane == 0) {
                if (warp == 0) S->e_kinetic = mue * 0.5 * ds * v;
                else if (warp == 1) S->e_pot = mue * grav * ds * v;
                else if (warp == 2) S->e_elastic = eta * 0.5 * ds * v;
                else if (warp == 3) S->inertial_force[0] = mue * ds * v;
                else if (warp == 4) S->inertial_force[1] = mue * ds * v;
                else if (released && v > 100.0) set_status(S, FSIBE_ERR_BRAKE);
            }
        }
    }
    PH(9);
    if (b.fuse_adv) {
        // the end of the time step, which the host would otherwise launch next (k_advance)
        __syncthreads();
        advance_state(b.adv);
    }
    PH(27);
    if (tid == 0)
        for (int k = 4; k < 28; ++k) S->phase[k] += ph[k];
}

// ---- host side ------------------------------------------------------------------------
// Floats of the global copy of M^-1 (R slices of rmax rows) and ints of its row exponents.
size_t beam_cluster_minv_floats(int ns, int R) {
    ClLayout Y;
    cl_layout(ns, R, Y);
    return (size_t)R * Y.rmax * Y.mld;
}

// The cluster size for a beam of ns nodes: 16 when the device places a 16-CTA cluster with
// this kernel's shared memory and every CTA gets at least 8 rows, else 8 under the same
// conditions, else 0 (the single-CTA kernel).  want caps it.  *big_out = 1 when only the
// large-beam form (factor and M^-1 in global memory) fits.
int beam_cluster_setup(int ns, int want, size_t* smem_out, int* big_out) {
    static std::mutex mu;
    std::lock_guard<std::mutex> lock(mu);
    int dev = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, (const void*)k_beam_cl) != cudaSuccess) return 0;
    static size_t cur = 0;
    for (int R = 16; R >= 8; R /= 2) {
        if (R > want || 2 * ns + 4 < 8 * R) continue;  // at least 8 rows per CTA
        for (int big = 0; big <= 1; ++big) {
            ClLayout Y;
            cl_layout(ns, R, Y, big != 0);
            if (Y.total + fa.sharedSizeBytes > (size_t)optin) continue;
            if (Y.total > cur) {
                if (cudaFuncSetAttribute((const void*)k_beam_cl, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Y.total) != cudaSuccess) continue;
                cur = Y.total;
            }
            if (R > 8 && cudaFuncSetAttribute((const void*)k_beam_cl, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) continue;
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(R);
            cfg.blockDim = dim3(256);
            cfg.dynamicSmemBytes = Y.total;
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = R;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            int nclusters = 0;
            if (cudaOccupancyMaxActiveClusters(&nclusters, (const void*)k_beam_cl, &cfg) != cudaSuccess || nclusters < 1) {
                cudaGetLastError();
                continue;
            }
            *smem_out = Y.total;
            *big_out = big;
            return R;
        }
    }
    cudaGetLastError();
    return 0;
}

// Floats of the large-beam form's global factor copies (one a CTA).
size_t beam_cluster_fact_floats(int ns, int R) { return (size_t)R * cl_fact_floats(ns); }

// The running sums on arbitrary terms (a diagnostic of their exactness): one 256-thread block,
// the terms and sums in global memory.
__global__ void __launch_bounds__(256, 1) k_running_sums(const double* src, double* dst, int n, int* nserial) {
    __shared__ int flags[4];
    const int r = running_sums4(src, n, dst, n, n, flags, NoIdle());
    if (threadIdx.x == 0) *nserial = r;
}
cudaError_t launch_running_sums(const double* src, double* dst, int n, int* nserial, cudaStream_t st) {
    k_running_sums<<<1, 256, 0, st>>>(src, dst, n, nserial);
    return cudaGetLastError();
}

void launch_beam_cluster(const BeamArgs& b, int R, size_t smem, cudaStream_t st, bool pdl) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(R);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[2];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = R;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 2 : 1;
    cudaLaunchKernelEx(&cfg, k_beam_cl, b);
}

}  // namespace fsibe
