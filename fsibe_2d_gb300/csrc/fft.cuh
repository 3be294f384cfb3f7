// fft.cuh -- block-level Stockham FFT engine for power-of-two lengths.
//
// A length-N complex sequence lives in shared memory (padded with pad8) and is transformed
// in place by a group of G = N/8 threads.  Each stage is a radix-8 Stockham pass (radix 4
// or 2 for the last stage when log2 N is not a multiple of 3): every thread loads its
// butterfly inputs into registers, the block synchronises, and the outputs are written to
// their autosorted positions.  Twiddles come from a table W_N^m = exp(-2 pi i m/N) computed
// on the host in long double and rounded once to the storage type.
//
// Forward = exp(-i..), inverse = exp(+i..), both unnormalised (like FFTW).
#pragma once
#include "common.cuh"

namespace fsibe {

template <typename R, bool INV>
__device__ __forceinline__ void dft2(C2<R>* v) {
    C2<R> a = v[0];
    v[0] = cadd<R>(a, v[1]);
    v[1] = csub<R>(a, v[1]);
}

template <typename R, bool INV>
__device__ __forceinline__ void dft4(C2<R>* v) {
    C2<R> a = cadd<R>(v[0], v[2]), b = csub<R>(v[0], v[2]);
    C2<R> c = cadd<R>(v[1], v[3]), d = csub<R>(v[1], v[3]);
    C2<R> sd = INV ? mk<R>(-d.y, d.x) : mk<R>(d.y, -d.x);  // (+-i) * d
    v[0] = cadd<R>(a, c);
    v[2] = csub<R>(a, c);
    v[1] = cadd<R>(b, sd);
    v[3] = csub<R>(b, sd);
}

template <typename R, bool INV>
__device__ __forceinline__ void dft8(C2<R>* v) {
    const R h = (R)0.70710678118654752440084436210485;
    C2<R> e[4], o[4];
    e[0] = cadd<R>(v[0], v[4]); o[0] = csub<R>(v[0], v[4]);
    e[1] = cadd<R>(v[1], v[5]); C2<R> t1 = csub<R>(v[1], v[5]);
    e[2] = cadd<R>(v[2], v[6]); C2<R> t2 = csub<R>(v[2], v[6]);
    e[3] = cadd<R>(v[3], v[7]); C2<R> t3 = csub<R>(v[3], v[7]);
    if (!INV) {
        o[1] = mk<R>((t1.x + t1.y) * h, (t1.y - t1.x) * h);    // * (1-i)/sqrt2
        o[2] = mk<R>(t2.y, -t2.x);                              // * -i
        o[3] = mk<R>((t3.y - t3.x) * h, -(t3.x + t3.y) * h);   // * (-1-i)/sqrt2
    } else {
        o[1] = mk<R>((t1.x - t1.y) * h, (t1.x + t1.y) * h);    // * (1+i)/sqrt2
        o[2] = mk<R>(-t2.y, t2.x);                              // * +i
        o[3] = mk<R>(-(t3.x + t3.y) * h, (t3.x - t3.y) * h);   // * (-1+i)/sqrt2
    }
    dft4<R, INV>(e);
    dft4<R, INV>(o);
    v[0] = e[0]; v[2] = e[1]; v[4] = e[2]; v[6] = e[3];
    v[1] = o[0]; v[3] = o[1]; v[5] = o[2]; v[7] = o[3];
}

template <typename R, int P, bool INV>
__device__ __forceinline__ void dftp(C2<R>* v) {
    if constexpr (P == 8) dft8<R, INV>(v);
    else if constexpr (P == 4) dft4<R, INV>(v);
    else dft2<R, INV>(v);
}

// One Stockham stage of radix P; NS = product of the radices already applied.
template <typename R, int N, int P, int NS, bool INV>
__device__ __forceinline__ void fft_stage(C2<R>* buf, const C2<R>* __restrict__ tw, int t) {
    constexpr int G = N / 8, B = N / P, PER = 8 / P;
    C2<R> v[8];
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int j = t + q * G;
#pragma unroll
        for (int r = 0; r < P; ++r) v[q * P + r] = buf[pad8(j + r * B)];
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int j = t + q * G;
        const int k = j & (NS - 1);
        if constexpr (NS > 1) {
#pragma unroll
            for (int r = 1; r < P; ++r) {
                C2<R> w = __ldg(&tw[r * k * (N / (NS * P))]);
                if (INV) w.y = -w.y;
                v[q * P + r] = cmul<R>(v[q * P + r], w);
            }
        }
        dftp<R, P, INV>(v + q * P);
        const int base = (j - k) * P + k;
#pragma unroll
        for (int r = 0; r < P; ++r) buf[pad8(base + r * NS)] = v[q * P + r];
    }
    __syncthreads();
}

template <typename R, int N, bool INV, int NS = 1>
__device__ __forceinline__ void fft_run(C2<R>* buf, const C2<R>* __restrict__ tw, int t) {
    if constexpr (NS * 8 <= N) {
        fft_stage<R, N, 8, NS, INV>(buf, tw, t);
        fft_run<R, N, INV, NS * 8>(buf, tw, t);
    } else if constexpr (NS * 4 == N) {
        fft_stage<R, N, 4, NS, INV>(buf, tw, t);
    } else if constexpr (NS * 2 == N) {
        fft_stage<R, N, 2, NS, INV>(buf, tw, t);
    }
}

// In-place transform of buf (padded, natural order). All threads of the block must call it;
// the caller synchronises before (data written by other threads) -- the routine ends synced.
template <typename R, int N, bool INV>
__device__ __forceinline__ void block_fft(C2<R>* buf, const C2<R>* __restrict__ tw, int t) {
    static_assert(N >= 16 && (N & (N - 1)) == 0, "power-of-two length >= 16");
    fft_run<R, N, INV>(buf, tw, t);
}

// NB independent transforms of the same length at buf + b * bstride, b < NB, stage by stage:
// each stage loads all NB butterflies, synchronises once, and shares its twiddles between the
// NB transforms.  Each transform's arithmetic is exactly that of block_fft.
template <typename R, int N, int P, int NS, bool INV, int NB>
__device__ __forceinline__ void fft_stage_m(C2<R>* buf, int bstride, const C2<R>* __restrict__ tw, int t) {
    constexpr int G = N / 8, B = N / P, PER = 8 / P;
    C2<R> v[NB][8];
#pragma unroll
    for (int b = 0; b < NB; ++b)
#pragma unroll
        for (int q = 0; q < PER; ++q) {
            const int j = t + q * G;
#pragma unroll
            for (int r = 0; r < P; ++r) v[b][q * P + r] = buf[b * bstride + pad8(j + r * B)];
        }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int j = t + q * G;
        const int k = j & (NS - 1);
        if constexpr (NS > 1) {
#pragma unroll
            for (int r = 1; r < P; ++r) {
                C2<R> w = __ldg(&tw[r * k * (N / (NS * P))]);
                if (INV) w.y = -w.y;
#pragma unroll
                for (int b = 0; b < NB; ++b) v[b][q * P + r] = cmul<R>(v[b][q * P + r], w);
            }
        }
        const int base = (j - k) * P + k;
#pragma unroll
        for (int b = 0; b < NB; ++b) {
            dftp<R, P, INV>(v[b] + q * P);
#pragma unroll
            for (int r = 0; r < P; ++r) buf[b * bstride + pad8(base + r * NS)] = v[b][q * P + r];
        }
    }
    __syncthreads();
}

template <typename R, int N, bool INV, int NB, int NS = 1>
__device__ __forceinline__ void fft_run_m(C2<R>* buf, int bstride, const C2<R>* __restrict__ tw, int t) {
    if constexpr (NS * 8 <= N) {
        fft_stage_m<R, N, 8, NS, INV, NB>(buf, bstride, tw, t);
        fft_run_m<R, N, INV, NB, NS * 8>(buf, bstride, tw, t);
    } else if constexpr (NS * 4 == N) {
        fft_stage_m<R, N, 4, NS, INV, NB>(buf, bstride, tw, t);
    } else if constexpr (NS * 2 == N) {
        fft_stage_m<R, N, 2, NS, INV, NB>(buf, bstride, tw, t);
    }
}

// NB in-place transforms (padded, natural order) at buf + b * bstride; the same contract as
// block_fft.
template <typename R, int N, bool INV, int NB>
__device__ __forceinline__ void block_fft_m(C2<R>* buf, int bstride, const C2<R>* __restrict__ tw, int t) {
    static_assert(N >= 16 && (N & (N - 1)) == 0, "power-of-two length >= 16");
    fft_run_m<R, N, INV, NB>(buf, bstride, tw, t);
}

// ---- transforms of values held in registers ------------------------------------------------
// A thread of the G = N/8 owns elements t + m G (m < 8) of each of the NB sequences.  These are
// exactly the inputs of its first-stage butterfly and the outputs of its last-stage
// butterflies, so a transform whose inputs are computed in registers and whose outputs go to
// registers needs shared memory only between stages: stages - 1 exchanges instead of a load and
// a store per stage plus the staging in and out.  Each stage's arithmetic (twiddles, radix-P
// butterfly, operation order) is that of fft_stage_m, so the results are bitwise the same.

// The butterflies of one stage on v[b][q P + r] (input r of butterfly q, j = t + q G), b < NB
// of the NBA rows of v.
template <typename R, int N, int P, int NS, bool INV, int NB, int NBA>
__device__ __forceinline__ void fft_reg_compute(C2<R> (&v)[NBA][8], const C2<R>* __restrict__ tw, int t) {
    constexpr int G = N / 8, PER = 8 / P;
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int j = t + q * G;
        const int k = j & (NS - 1);
        if constexpr (NS > 1) {
#pragma unroll
            for (int r = 1; r < P; ++r) {
                C2<R> w = __ldg(&tw[r * k * (N / (NS * P))]);
                if (INV) w.y = -w.y;
#pragma unroll
                for (int b = 0; b < NB; ++b) v[b][q * P + r] = cmul<R>(v[b][q * P + r], w);
            }
        }
#pragma unroll
        for (int b = 0; b < NB; ++b) dftp<R, P, INV>(v[b] + q * P);
    }
}

template <typename R, int N, bool INV, int NB, int NS, int NBA>
__device__ __forceinline__ void fft_reg_run(C2<R> (&v)[NBA][8], C2<R>* buf, int bstride, const C2<R>* __restrict__ tw,
                                            int t) {
    constexpr int G = N / 8;
    constexpr int P = (NS * 8 <= N) ? 8 : ((NS * 4 == N) ? 4 : 2), PER = 8 / P;
    fft_reg_compute<R, N, P, NS, INV, NB, NBA>(v, tw, t);
    if constexpr (NS * P < N) {
        // outputs to their autosorted positions, then the next stage's inputs
#pragma unroll
        for (int q = 0; q < PER; ++q) {
            const int j = t + q * G;
            const int k = j & (NS - 1);
            const int base = (j - k) * P + k;
#pragma unroll
            for (int b = 0; b < NB; ++b)
#pragma unroll
                for (int r = 0; r < P; ++r) buf[b * bstride + pad8(base + r * NS)] = v[b][q * P + r];
        }
        __syncthreads();
        constexpr int NS2 = NS * P;
        constexpr int P2 = (NS2 * 8 <= N) ? 8 : ((NS2 * 4 == N) ? 4 : 2), PER2 = 8 / P2, B2 = N / P2;
#pragma unroll
        for (int b = 0; b < NB; ++b)
#pragma unroll
            for (int q = 0; q < PER2; ++q)
#pragma unroll
                for (int r = 0; r < P2; ++r) v[b][q * P2 + r] = buf[b * bstride + pad8(t + q * G + r * B2)];
        __syncthreads();  // every thread has its inputs before the buffer is written again
        fft_reg_run<R, N, INV, NB, NS2, NBA>(v, buf, bstride, tw, t);
    } else if constexpr (PER > 1) {
        // the last stage's butterfly q, output r is element t + (q + PER r) G: element order
#pragma unroll
        for (int b = 0; b < NB; ++b) {
            C2<R> o[8];
#pragma unroll
            for (int q = 0; q < PER; ++q)
#pragma unroll
                for (int r = 0; r < P; ++r) o[q + PER * r] = v[b][q * P + r];
#pragma unroll
            for (int m = 0; m < 8; ++m) v[b][m] = o[m];
        }
    }
}

// NB transforms of the sequences v[b][m] = element t + m (N/8), b < NB (of the NBA rows of v);
// buf + b * bstride are NB padded shared-memory rows for the exchanges, free when this is
// called (the caller synchronises after their last use); they are free again on return.  All
// threads of the block call it.
template <typename R, int N, bool INV, int NB, int NBA>
__device__ __forceinline__ void block_fft_reg_m(C2<R> (&v)[NBA][8], C2<R>* buf, int bstride,
                                                const C2<R>* __restrict__ tw, int t) {
    static_assert(N >= 16 && (N & (N - 1)) == 0, "power-of-two length >= 16");
    static_assert(NB >= 1 && NB <= NBA, "NB of the NBA rows");
    fft_reg_run<R, N, INV, NB, 1, NBA>(v, buf, bstride, tw, t);
}

// ---- paired transforms (FP32): a thread owns two adjacent butterflies -----------------------
// A length-N transform runs on N/16 threads.  Thread u owns the elements 2u + h + m G (G = N/8,
// h < 2, m < 8), held as v[2m + h]: the inputs of its two first-stage butterflies j = 2u and
// 2u + 1, and the outputs of its last-stage butterflies.  The two butterflies of a stage have
// adjacent outputs (k and k + 1 of the same group), so between stages every exchange moves a
// pair (2p, 2p + 1) as one 16-byte shared-memory access, half the accesses of one butterfly a
// thread.  With one pad slot after every eight pairs, the eight 16-byte accesses of every
// quarter warp fall in distinct bank groups in every stage, for every length 16..4096.  A radix-8
// butterfly loads the twiddles w, w^2, w^3, w^4 and forms w^5 = w w^4, w^6 = w^2 w^4,
// w^7 = w^3 w^4 (a product of two correctly rounded FP32 twiddles: within 2 ulp).
__host__ __device__ constexpr int pair_slots(int n) { return n / 2 + n / 16 + 1; }  // float4 slots of a row
__device__ __forceinline__ int padp(int p) { return p + (p >> 3); }

template <int P, bool INV>
__device__ __forceinline__ void tw_powers(float2 (&w)[8], const float2* __restrict__ tw, int e) {
    if constexpr (P == 8) {
        w[1] = __ldg(&tw[e]); w[2] = __ldg(&tw[2 * e]); w[3] = __ldg(&tw[3 * e]); w[4] = __ldg(&tw[4 * e]);
        w[5] = cmul<float>(w[1], w[4]); w[6] = cmul<float>(w[2], w[4]); w[7] = cmul<float>(w[3], w[4]);
    } else {
#pragma unroll
        for (int r = 1; r < P; ++r) w[r] = __ldg(&tw[r * e]);
    }
    if (INV) {
#pragma unroll
        for (int r = 1; r < P; ++r) w[r].y = -w[r].y;
    }
}

// The butterflies of one stage (radix P, NS = product of the radices applied) on v[b][..],
// b < NB of the NBA rows.  Butterfly (q, h) takes its inputs from, and leaves its outputs in,
// v[b][2 (q + r PER) + h], r < P.
template <int N, int P, int NS, bool INV, int NB, int NBA>
__device__ __forceinline__ void fft2_compute(float2 (&v)[NBA][16], const float2* __restrict__ tw, int u) {
    constexpr int G = N / 8, PER = 8 / P;
#pragma unroll
    for (int q = 0; q < PER; ++q) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if constexpr (NS > 1) {
                const int j = 2 * u + h + q * G;
                const int k = j & (NS - 1);
                float2 w[8];
                tw_powers<P, INV>(w, tw, k * (N / (NS * P)));
#pragma unroll
                for (int r = 1; r < P; ++r)
#pragma unroll
                    for (int b = 0; b < NB; ++b) v[b][2 * (q + r * PER) + h] = cmul<float>(v[b][2 * (q + r * PER) + h], w[r]);
            }
#pragma unroll
            for (int b = 0; b < NB; ++b) {
                float2 x[P];
#pragma unroll
                for (int r = 0; r < P; ++r) x[r] = v[b][2 * (q + r * PER) + h];
                dftp<float, P, INV>(x);
#pragma unroll
                for (int r = 0; r < P; ++r) v[b][2 * (q + r * PER) + h] = x[r];
            }
        }
    }
}

template <int N, bool INV, int NB, int NS, int NBA>
__device__ __forceinline__ void fft2_run(float2 (&v)[NBA][16], float4* buf, int bstride, const float2* __restrict__ tw,
                                         int u) {
    constexpr int G = N / 8;
    constexpr int P = (NS * 8 <= N) ? 8 : ((NS * 4 == N) ? 4 : 2);
    fft2_compute<N, P, NS, INV, NB, NBA>(v, tw, u);
    if constexpr (NS * P < N) {
        static_assert(P == 8, "only the last stage has a radix below 8");
        // outputs r of butterfly h at base_h + r NS: with NS = 1 a butterfly's eight outputs are
        // contiguous (base_h = 8 (2u + h)); else base_1 = base_0 + 1 (k and k + 1)
#pragma unroll
        for (int b = 0; b < NB; ++b) {
            float4* rb = buf + b * bstride;
            if constexpr (NS == 1) {
#pragma unroll
                for (int h = 0; h < 2; ++h)
#pragma unroll
                    for (int r = 0; r < 8; r += 2) {
                        const float2 a = v[b][2 * r + h], c = v[b][2 * (r + 1) + h];
                        rb[padp(8 * u + 4 * h + r / 2)] = make_float4(a.x, a.y, c.x, c.y);
                    }
            } else {
                const int j0 = 2 * u, k0 = j0 & (NS - 1), base0 = (j0 - k0) * 8 + k0;
#pragma unroll
                for (int r = 0; r < 8; ++r) {
                    const float2 a = v[b][2 * r], c = v[b][2 * r + 1];
                    rb[padp((base0 + r * NS) >> 1)] = make_float4(a.x, a.y, c.x, c.y);
                }
            }
        }
        __syncthreads();
        // the next stage's inputs: elements 2u + h + m G, the pair u + m G / 2
#pragma unroll
        for (int b = 0; b < NB; ++b)
#pragma unroll
            for (int m = 0; m < 8; ++m) {
                const float4 t = buf[b * bstride + padp(u + m * (G / 2))];
                v[b][2 * m] = make_float2(t.x, t.y);
                v[b][2 * m + 1] = make_float2(t.z, t.w);
            }
        __syncthreads();  // every thread has its inputs before the rows are written again
        fft2_run<N, INV, NB, NS * 8, NBA>(v, buf, bstride, tw, u);
    }
}

// NB paired transforms (FP32) of v[b][2m + h] = element 2u + h + m (N/8), b < NB of NBA; buf +
// b * bstride are NB exchange rows of pair_slots(N) float4, free when called (the caller
// synchronises after their last use) and free again on return.  All N/16 threads call it.
template <int N, bool INV, int NB, int NBA>
__device__ __forceinline__ void block_fft2_m(float2 (&v)[NBA][16], float4* buf, int bstride,
                                             const float2* __restrict__ tw, int u) {
    static_assert(N >= 16 && (N & (N - 1)) == 0, "power-of-two length >= 16");
    static_assert(NB >= 1 && NB <= NBA, "NB of the NBA rows");
    fft2_run<N, INV, NB, 1, NBA>(v, buf, bstride, tw, u);
}

// ---- real <-> half-length complex split steps (x direction) -------------------------------
// A real row x[0..2H) is handled as z[m] = x[2m] + i x[2m+1], m < H, transformed with a
// length-H complex FFT.  twr[k] = exp(-2 pi i k / 2H), k <= H.

// After the forward length-H FFT of z (in buf): X[k], k in [0,H), in place.  The Nyquist bin
// X[H] is dropped (the reference's filtering).  Pairs (k, H-k) handled by the same thread.
template <typename R, int H>
__device__ __forceinline__ void r2c_split(C2<R>* buf, const C2<R>* __restrict__ twr, int t) {
    constexpr int G = H / 8;
    // pairs k = 1 .. H/2-1, plus k = 0 and k = H/2 handled by thread 0
    for (int k = 1 + t; k < H / 2; k += G) {
        const C2<R> zk = buf[pad8(k)], zm = buf[pad8(H - k)];
        const C2<R> wk = __ldg(&twr[k]), wm = __ldg(&twr[H - k]);
        // X[k] = 1/2 (zk + conj zm) + w^k (zk - conj zm)/(2i)
        C2<R> e = mk<R>((R)0.5 * (zk.x + zm.x), (R)0.5 * (zk.y - zm.y));
        C2<R> d = mk<R>(zk.x - zm.x, zk.y + zm.y);           // zk - conj zm
        C2<R> o = mk<R>((R)0.5 * d.y, (R)-0.5 * d.x);         // d / (2i)
        C2<R> Xk = cadd<R>(e, cmul<R>(wk, o));
        // X[H-k] = 1/2 (zm + conj zk) + w^(H-k) (zm - conj zk)/(2i)
        C2<R> e2 = mk<R>((R)0.5 * (zm.x + zk.x), (R)0.5 * (zm.y - zk.y));
        C2<R> d2 = mk<R>(zm.x - zk.x, zm.y + zk.y);
        C2<R> o2 = mk<R>((R)0.5 * d2.y, (R)-0.5 * d2.x);
        C2<R> Xm = cadd<R>(e2, cmul<R>(wm, o2));
        buf[pad8(k)] = Xk;
        buf[pad8(H - k)] = Xm;
    }
    if (t == 0) {
        C2<R> z0 = buf[pad8(0)];
        buf[pad8(0)] = mk<R>(z0.x + z0.y, (R)0);
        C2<R> zh = buf[pad8(H / 2)];
        buf[pad8(H / 2)] = mk<R>(zh.x, -zh.y);
    }
    __syncthreads();
}

// Before the inverse length-H FFT: X[k], k in [0,H) (X[H] = 0, Im X[0] ignored) -> Z'[k] so
// that z = IFFT_H(Z') gives x[2m] = Re z[m], x[2m+1] = Im z[m] (unnormalised c2r).
template <typename R, int H>
__device__ __forceinline__ void c2r_merge(C2<R>* buf, const C2<R>* __restrict__ twr, int t) {
    constexpr int G = H / 8;
    for (int k = 1 + t; k < H / 2; k += G) {
        const C2<R> xk = buf[pad8(k)], xm = buf[pad8(H - k)];
        const C2<R> wk = __ldg(&twr[k]), wm = __ldg(&twr[H - k]);
        // Z'[k] = (xk + conj xm) + i (xk - conj xm) conj(w^k)
        C2<R> e = mk<R>(xk.x + xm.x, xk.y - xm.y);
        C2<R> o = cmul<R>(mk<R>(xk.x - xm.x, xk.y + xm.y), mk<R>(wk.x, -wk.y));
        C2<R> Zk = mk<R>(e.x - o.y, e.y + o.x);
        C2<R> e2 = mk<R>(xm.x + xk.x, xm.y - xk.y);
        C2<R> o2 = cmul<R>(mk<R>(xm.x - xk.x, xm.y + xk.y), mk<R>(wm.x, -wm.y));
        C2<R> Zm = mk<R>(e2.x - o2.y, e2.y + o2.x);
        buf[pad8(k)] = Zk;
        buf[pad8(H - k)] = Zm;
    }
    if (t == 0) {
        C2<R> x0 = buf[pad8(0)];
        buf[pad8(0)] = mk<R>(x0.x, x0.x);
        C2<R> xh = buf[pad8(H / 2)];
        buf[pad8(H / 2)] = mk<R>((R)2 * xh.x, (R)-2 * xh.y);
    }
    __syncthreads();
}

// r2c_split and c2r_merge of NB rows at buf + b * bstride (each row's arithmetic unchanged;
// the twiddles are loaded once for all rows).
template <typename R, int H, int NB>
__device__ __forceinline__ void r2c_split_m(C2<R>* buf, int bstride, const C2<R>* __restrict__ twr, int t) {
    constexpr int G = H / 8;
    for (int k = 1 + t; k < H / 2; k += G) {
        const C2<R> wk = __ldg(&twr[k]), wm = __ldg(&twr[H - k]);
#pragma unroll
        for (int b = 0; b < NB; ++b) {
            C2<R>* bb = buf + b * bstride;
            const C2<R> zk = bb[pad8(k)], zm = bb[pad8(H - k)];
            C2<R> e = mk<R>((R)0.5 * (zk.x + zm.x), (R)0.5 * (zk.y - zm.y));
            C2<R> d = mk<R>(zk.x - zm.x, zk.y + zm.y);
            C2<R> o = mk<R>((R)0.5 * d.y, (R)-0.5 * d.x);
            C2<R> Xk = cadd<R>(e, cmul<R>(wk, o));
            C2<R> e2 = mk<R>((R)0.5 * (zm.x + zk.x), (R)0.5 * (zm.y - zk.y));
            C2<R> d2 = mk<R>(zm.x - zk.x, zm.y + zk.y);
            C2<R> o2 = mk<R>((R)0.5 * d2.y, (R)-0.5 * d2.x);
            C2<R> Xm = cadd<R>(e2, cmul<R>(wm, o2));
            bb[pad8(k)] = Xk;
            bb[pad8(H - k)] = Xm;
        }
    }
    if (t == 0) {
#pragma unroll
        for (int b = 0; b < NB; ++b) {
            C2<R>* bb = buf + b * bstride;
            C2<R> z0 = bb[pad8(0)];
            bb[pad8(0)] = mk<R>(z0.x + z0.y, (R)0);
            C2<R> zh = bb[pad8(H / 2)];
            bb[pad8(H / 2)] = mk<R>(zh.x, -zh.y);
        }
    }
    __syncthreads();
}

template <typename R, int H, int NB>
__device__ __forceinline__ void c2r_merge_m(C2<R>* buf, int bstride, const C2<R>* __restrict__ twr, int t) {
    constexpr int G = H / 8;
    for (int k = 1 + t; k < H / 2; k += G) {
        const C2<R> wk = __ldg(&twr[k]), wm = __ldg(&twr[H - k]);
#pragma unroll
        for (int b = 0; b < NB; ++b) {
            C2<R>* bb = buf + b * bstride;
            const C2<R> xk = bb[pad8(k)], xm = bb[pad8(H - k)];
            C2<R> e = mk<R>(xk.x + xm.x, xk.y - xm.y);
            C2<R> o = cmul<R>(mk<R>(xk.x - xm.x, xk.y + xm.y), mk<R>(wk.x, -wk.y));
            C2<R> Zk = mk<R>(e.x - o.y, e.y + o.x);
            C2<R> e2 = mk<R>(xm.x + xk.x, xm.y - xk.y);
            C2<R> o2 = cmul<R>(mk<R>(xm.x - xk.x, xm.y + xk.y), mk<R>(wm.x, -wm.y));
            C2<R> Zm = mk<R>(e2.x - o2.y, e2.y + o2.x);
            bb[pad8(k)] = Zk;
            bb[pad8(H - k)] = Zm;
        }
    }
    if (t == 0) {
#pragma unroll
        for (int b = 0; b < NB; ++b) {
            C2<R>* bb = buf + b * bstride;
            C2<R> x0 = bb[pad8(0)];
            bb[pad8(0)] = mk<R>(x0.x, x0.x);
            C2<R> xh = bb[pad8(H / 2)];
            bb[pad8(H / 2)] = mk<R>((R)2 * xh.x, (R)-2 * xh.y);
        }
    }
    __syncthreads();
}

// ---- the x direction's split steps on paired rows (FP32) -----------------------------------
// A row of H complex values in the paired layout: element e is half e & 1 of the float4 slot
// padp(e >> 1) (pair_slots(H) slots a row).  The arithmetic is that of r2c_split_m and
// c2r_merge_m; nthr threads a row share the pairs (k, H - k).
__device__ __forceinline__ float2& pel(float4* row, int e) {
    return reinterpret_cast<float2*>(row + padp(e >> 1))[e & 1];
}

template <int H, int NB>
__device__ __forceinline__ void r2c_split_p(float4* buf, int bstride, const float2* __restrict__ twr, int t, int nthr) {
    for (int k = 1 + t; k < H / 2; k += nthr) {
        const float2 wk = __ldg(&twr[k]), wm = __ldg(&twr[H - k]);
#pragma unroll
        for (int b = 0; b < NB; ++b) {
            float4* bb = buf + b * bstride;
            const float2 zk = pel(bb, k), zm = pel(bb, H - k);
            float2 e = mk<float>(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
            float2 d = mk<float>(zk.x - zm.x, zk.y + zm.y);
            float2 o = mk<float>(0.5f * d.y, -0.5f * d.x);
            float2 Xk = cadd<float>(e, cmul<float>(wk, o));
            float2 e2 = mk<float>(0.5f * (zm.x + zk.x), 0.5f * (zm.y - zk.y));
            float2 d2 = mk<float>(zm.x - zk.x, zm.y + zk.y);
            float2 o2 = mk<float>(0.5f * d2.y, -0.5f * d2.x);
            float2 Xm = cadd<float>(e2, cmul<float>(wm, o2));
            pel(bb, k) = Xk;
            pel(bb, H - k) = Xm;
        }
    }
    if (t == 0) {
#pragma unroll
        for (int b = 0; b < NB; ++b) {
            float4* bb = buf + b * bstride;
            const float2 z0 = pel(bb, 0);
            pel(bb, 0) = mk<float>(z0.x + z0.y, 0.f);
            const float2 zh = pel(bb, H / 2);
            pel(bb, H / 2) = mk<float>(zh.x, -zh.y);
        }
    }
    __syncthreads();
}

template <int H, int NB>
__device__ __forceinline__ void c2r_merge_p(float4* buf, int bstride, const float2* __restrict__ twr, int t, int nthr) {
    for (int k = 1 + t; k < H / 2; k += nthr) {
        const float2 wk = __ldg(&twr[k]), wm = __ldg(&twr[H - k]);
#pragma unroll
        for (int b = 0; b < NB; ++b) {
            float4* bb = buf + b * bstride;
            const float2 xk = pel(bb, k), xm = pel(bb, H - k);
            float2 e = mk<float>(xk.x + xm.x, xk.y - xm.y);
            float2 o = cmul<float>(mk<float>(xk.x - xm.x, xk.y + xm.y), mk<float>(wk.x, -wk.y));
            float2 Zk = mk<float>(e.x - o.y, e.y + o.x);
            float2 e2 = mk<float>(xm.x + xk.x, xm.y - xk.y);
            float2 o2 = cmul<float>(mk<float>(xm.x - xk.x, xm.y + xk.y), mk<float>(wm.x, -wm.y));
            float2 Zm = mk<float>(e2.x - o2.y, e2.y + o2.x);
            pel(bb, k) = Zk;
            pel(bb, H - k) = Zm;
        }
    }
    if (t == 0) {
#pragma unroll
        for (int b = 0; b < NB; ++b) {
            float4* bb = buf + b * bstride;
            const float2 x0 = pel(bb, 0);
            pel(bb, 0) = mk<float>(x0.x, x0.x);
            const float2 xh = pel(bb, H / 2);
            pel(bb, H / 2) = mk<float>(2.f * xh.x, -2.f * xh.y);
        }
    }
    __syncthreads();
}

// Paired row transforms with the values in registers: v[b][2m + h] = element 2u + h + m (H/8)
// of row b (u < H/16).  c2r: merge in the rows (loaded by the caller, synchronised), then the
// inverse transform to registers; the rows are free on return.  r2c: the forward transform of
// registers into the rows, then the split; the rows must be free when called.
template <int H, int NB, int NBA>
__device__ __forceinline__ void row_c2r_reg2(float4* rb, int bstride, const float2* __restrict__ twR,
                                             const float2* __restrict__ twX, int u, float2 (&v)[NBA][16]) {
    constexpr int HG = H / 16;
    c2r_merge_p<H, NB>(rb, bstride, twR, u, HG);
#pragma unroll
    for (int b = 0; b < NB; ++b)
#pragma unroll
        for (int m = 0; m < 8; ++m) {
            const float4 q = rb[b * bstride + padp(u + m * HG)];
            v[b][2 * m] = make_float2(q.x, q.y);
            v[b][2 * m + 1] = make_float2(q.z, q.w);
        }
    __syncthreads();
    block_fft2_m<H, true, NB>(v, rb, bstride, twX, u);
}
template <int H, int NB, int NBA>
__device__ __forceinline__ void row_r2c_reg2(float2 (&v)[NBA][16], float4* rb, int bstride,
                                             const float2* __restrict__ twR, const float2* __restrict__ twX, int u) {
    constexpr int HG = H / 16;
    block_fft2_m<H, false, NB>(v, rb, bstride, twX, u);
#pragma unroll
    for (int b = 0; b < NB; ++b)
#pragma unroll
        for (int m = 0; m < 8; ++m)
            rb[b * bstride + padp(u + m * HG)] = make_float4(v[b][2 * m].x, v[b][2 * m].y, v[b][2 * m + 1].x, v[b][2 * m + 1].y);
    __syncthreads();
    r2c_split_p<H, NB>(rb, bstride, twR, u, HG);
}

}  // namespace fsibe
