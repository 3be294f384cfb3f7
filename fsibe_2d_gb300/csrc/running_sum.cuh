// The four running sums of integrate_position (integrate_position.f90:14-44), bit for bit the
// sequential FP64 loop s_0 = +0, s_(k+1) = s_k + a_k (round to nearest even), mostly in integer
// arithmetic.
//
// A dependent FP64 addition costs about 75 cycles on this chip.  While s_k and s_(k+1) stay in
// one binade [2^e, 2^(e+1)), the FP64 sum is an integer sum on that binade's grid 2^g
// (g = e - 52): with s_k = m 2^g,
//     s_(k+1) = (m + RN(a_k / 2^g)) 2^g,
// where RN rounds to the nearest integer and a tie towards the even m + RN.  The result is in
// the binade exactly when 2^52 < |m + RN| < 2^53 (at 2^52 the exact sum may lie below the
// binade, where the grid is finer).  So a warp per sum takes 32 steps at a time as a prefix sum
// of the rounded terms, up to the first step that leaves the binade, which is done by the FP64
// addition; its result gives the next binade.  Afterwards every step is checked in parallel by
// the FP64 addition, bits(s_k + a_k) == bits(s_(k+1)), and a sum with any mismatch is formed
// again by the plain serial loop: the result is that loop's in every case.
#pragma once
#include "common.cuh"

namespace fsibe {

// a / 2^g rounded to the nearest integer, for a term that allows an integer step (ok): zero, or
// finite and below the grid's unit.  A tie (tie) returns its lower candidate; its rounding
// depends on the running value's parity.
__device__ __forceinline__ long long term_inc(double a, int g, bool& ok, bool& tie) {
    const unsigned long long TWO52 = 1ull << 52, FRAC = TWO52 - 1ull;
    const unsigned long long ab = (unsigned long long)__double_as_longlong(a);
    const int ex = (int)((ab >> 52) & 0x7FF);
    const unsigned long long ma = (ab & FRAC) | (ex ? TWO52 : 0ull);
    const int sh = g - (ex ? ex - 1075 : -1074);      // a = ma 2^(g - sh)
    const int shc = sh < 1 ? 1 : (sh > 63 ? 63 : sh);  // for sh >= 63 the quotient rounds to 0 all the same
    const unsigned long long q = ma >> shc, rem = ma & ((1ull << shc) - 1ull), half = 1ull << (shc - 1);
    const bool neg = (ab >> 63) != 0;
    const long long r = (long long)(q + (rem > half ? 1ull : 0ull));
    ok = ma == 0ull || (sh > 0 && ex != 0x7FF);
    tie = ma != 0ull && rem == half;
    if (ma == 0ull) return 0;
    if (tie) return neg ? -(long long)q - 1 : (long long)q;
    return neg ? -r : r;
}

// One sum on one warp (all 32 lanes, the same arguments): dst[k] = s_k for k < n.  After an
// FP64 step, batches of 32 integer steps on the grid of its result's binade: lane t rounds term
// k + t (a tie by the parity of s_(k+t), from a scan of the steps' parity maps), a warp scan of
// the increments gives every s_(k+t+1), and the first step whose result leaves the binade (or
// whose term does not allow an integer step) ends the batch and is the next FP64 step.
__device__ __forceinline__ void running_sum_warp(const double* __restrict__ src, double* __restrict__ dst, int n) {
    const unsigned long long TWO52 = 1ull << 52, TWO53 = 1ull << 53, FRAC = TWO52 - 1ull;
    const int lane = threadIdx.x & 31;
    double cur = 0.0;  // s_k, the same in every lane
    int k = 0;
    while (k < n) {
        // the FP64 step k, then the binade of its result
        if (lane == 0) dst[k] = cur;
        cur = cur + src[k];
        ++k;
        const unsigned long long cb = (unsigned long long)__double_as_longlong(cur);
        const int ex = (int)((cb >> 52) & 0x7FF);
        if (ex == 0 || ex == 0x7FF) continue;  // zero, subnormal or non-finite: FP64 steps
        const bool negs = (cb >> 63) != 0;
        const long long mc = (long long)((cb & FRAC) | TWO52);
        long long m = negs ? -mc : mc;  // s_k = m 2^g, 2^52 <= |m| < 2^53
        const int g = ex - 1075;
        const unsigned long long hi = cb & ~FRAC;
        const long long blo = negs ? -(long long)TWO53 : (long long)TWO52;  // blo < s_(k+1) / 2^g < bhi
        const long long bhi = negs ? -(long long)TWO52 : (long long)TWO53;
        while (k < n) {
            const int j = k + lane;
            bool ok, tie;
            long long inc = term_inc(j < n ? src[j] : 0.0, g, ok, tie);
            // the parity of the running value before each step, by a scan of parity maps: a tie
            // makes the value even (bit 1: reset), any other step flips it by inc's low bit (bit 0)
            if (__any_sync(0xffffffffu, tie && ok)) {
                unsigned f = tie ? 2u : (unsigned)(inc & 1);
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const unsigned e = __shfl_up_sync(0xffffffffu, f, o);  // the earlier steps' map
                    if (lane >= o) f = (f & 2u) ? f : ((e & 2u) | ((e ^ f) & 1u));
                }
                unsigned fe = __shfl_up_sync(0xffffffffu, f, 1);
                if (lane == 0) fe = 0u;
                const long long par = (fe & 2u) ? (long long)(fe & 1u) : ((m ^ (long long)fe) & 1);
                if (tie) inc += (par ^ inc) & 1;  // the even of the two candidates
            }
            long long p = inc;  // inclusive scan of the increments
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const long long v = __shfl_up_sync(0xffffffffu, p, o);
                if (lane >= o) p += v;
            }
            const long long m1 = m + p;  // s_(j+1) / 2^g while the steps before it hold
            ok = ok && j < n && m1 > blo && m1 < bhi;
            const unsigned bad = __ballot_sync(0xffffffffu, !ok);
            const int nok = bad ? __ffs((int)bad) - 1 : 32;  // steps k .. k + nok - 1 hold
            if (lane < nok) {
                const long long mv = m + p - inc;  // s_j / 2^g
                dst[j] = __longlong_as_double((long long)(hi | ((unsigned long long)(mv < 0 ? -mv : mv) & FRAC)));
            }
            if (nok > 0) {
                m = __shfl_sync(0xffffffffu, m1, nok - 1);
                cur = __longlong_as_double((long long)(hi | ((unsigned long long)(m < 0 ? -m : m) & FRAC)));
            }
            k += nok;
            if (nok < 32) break;  // step k (if any) is an FP64 step
        }
    }
}

// The four sums of rows src + q sld into dst + q dld (q < 4), each by warp q, then checked by
// all threads of the (256-thread) block.  idle(i, m) runs on
// warps 4..7 (i < m) meanwhile.  flags: 4 ints of shared memory.  Returns the number of sums the
// check sent to the plain serial loop.  Ends with a barrier.
template <typename Idle>
__device__ int running_sums4(const double* src, int sld, double* dst, int dld, int n, int* flags, Idle idle) {
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (warp < 4) {
        if (lane == 0) flags[warp] = 0;
        running_sum_warp(src + (size_t)warp * sld, dst + (size_t)warp * dld, n);
    } else {
        idle(tid - 128, blockDim.x - 128);
    }
    __syncthreads();
    for (int j = tid; j < 4 * n; j += blockDim.x) {
        const int q = j / n, k = j - q * n;
        if (k + 1 < n) {
            const double* s = src + (size_t)q * sld;
            const double* d = dst + (size_t)q * dld;
            if (__double_as_longlong(d[k] + s[k]) != __double_as_longlong(d[k + 1])) flags[q] = 1;
        }
    }
    __syncthreads();
    const int bad = (flags[0] != 0) + (flags[1] != 0) + (flags[2] != 0) + (flags[3] != 0);
    if (lane == 0 && warp < 4 && flags[warp]) {
        const double* s = src + (size_t)warp * sld;
        double* d = dst + (size_t)warp * dld;
        double v = 0.0;
        for (int k = 0; k < n; ++k) { d[k] = v; v = v + s[k]; }
    }
    __syncthreads();
    return bad;
}

struct NoIdle {
    __device__ void operator()(int, int) const {}
};

}  // namespace fsibe
