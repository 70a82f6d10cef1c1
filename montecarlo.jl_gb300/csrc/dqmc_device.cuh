// CTA-cooperative FP64 building blocks of the DQMC sweep.
//
// Every function here is executed by all threads of one CTA with uniform
// control flow; one CTA owns one chain.  Matrices are column-major n x n FP64
// blocks in global memory (L2-resident per chain), staged through shared
// memory tiles.  On GB300 the FP64 pipe (DFMA) is the bound of this path, so
// the functions aim at keeping DFMA issue busy and at issuing no FP64
// instruction the reference's algorithm does not need.
#pragma once
#include <stdint.h>

#include "dqmc_chain.h"
#include "philox.h"

#define DQMC_NT 256
#define DQMC_NW (DQMC_NT / 32)
#define DQMC_NMAX 512

namespace dqmc {
namespace {  // internal linkage: each translation unit gets its own copy

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ void ident(int n, double* A) {
    for (int e = threadIdx.x; e < n * n; e += DQMC_NT) {
        int i = e % n, j = e / n;
        A[e] = (i == j) ? 1.0 : 0.0;
    }
}
__device__ __forceinline__ void fill(int cnt, double* d, double v) {
    for (int e = threadIdx.x; e < cnt; e += DQMC_NT) d[e] = v;
}
__device__ __forceinline__ void copy(int cnt, double* __restrict__ dst, const double* __restrict__ src) {
    for (int e = threadIdx.x; e < cnt; e += DQMC_NT) dst[e] = src[e];
}
// C = Diagonal(d) * B  (real.jl:27-37)
__device__ __forceinline__ void dleft(int n, double* __restrict__ C, const double* __restrict__ d,
                                      const double* __restrict__ B) {
    for (int e = threadIdx.x; e < n * n; e += DQMC_NT) C[e] = d[e % n] * B[e];
}
// C = A * Diagonal(d)  (real.jl:16-26)
__device__ __forceinline__ void dright(int n, double* __restrict__ C, const double* __restrict__ A,
                                       const double* __restrict__ d) {
    for (int e = threadIdx.x; e < n * n; e += DQMC_NT) C[e] = A[e] * d[e / n];
}

// Complex diagonal scalings on the real 2m x 2m representation
// [[Re, -Im], [Im, Re]] of m x m complex matrices (n = 2m; complex.jl:190-223,
// 257-277): d holds Re d_i at d[i] and Im d_i at d[m + i]; conj scales by the
// conjugate diagonal (adjoint(eV), stack.jl:359-367).
// C = Diagonal(d) * B: rows i and m + i mix.
__device__ __forceinline__ void dleft_c(int n, double* __restrict__ C, const double* __restrict__ d,
                                        const double* __restrict__ B, bool conj) {
    const int m = n >> 1;
    for (int e = threadIdx.x; e < n * n; e += DQMC_NT) {
        const int r = e % n, base = e - r;
        const int i = r < m ? r : r - m;
        const double dr = d[i], di = conj ? -d[m + i] : d[m + i];
        const double b0 = B[base + i], b1 = B[base + m + i];
        C[e] = r < m ? dr * b0 - di * b1 : di * b0 + dr * b1;
    }
}
// C = A * Diagonal(d): columns i and m + i mix.
__device__ __forceinline__ void dright_c(int n, double* __restrict__ C, const double* __restrict__ A,
                                         const double* __restrict__ d, bool conj) {
    const int m = n >> 1;
    for (int e = threadIdx.x; e < n * n; e += DQMC_NT) {
        const int r = e % n, col = e / n;
        const int i = col < m ? col : col - m;
        const double dr = d[i], di = conj ? -d[m + i] : d[m + i];
        const double a0 = A[r + (size_t)i * n], a1 = A[r + (size_t)(m + i) * n];
        C[e] = col < m ? a0 * dr + a1 * di : a1 * dr - a0 * di;
    }
}

// C = op(A) * op(B), op = transpose when TA / TB, on the FP64 FMA pipe (on
// GB300 measured at 1.16 TFLOP/s for 64 x 64 blocks, above the DMMA tensor
// path at 1.04).  64 x 64 output tiles,
// 4 x 4 outputs per thread, k staged 16 at a time through shared memory
// (sm: 2 * 16 * 64 doubles).  C must not alias A or B.  Summation over k is
// in ascending order with fused multiply-adds.
template <bool TA, bool TB>
__device__ __noinline__ void mm(int n, double* __restrict__ C, const double* __restrict__ A,
                   const double* __restrict__ B, double* sm) {
    double* sA = sm;            // [16][64]: sA[kk*64 + m]
    double* sB = sm + 16 * 64;  // [16][64]: sB[kk*64 + j]
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    for (int n0 = 0; n0 < n; n0 += 64) {
        // 16-column / 16-row groups of this tile that hold any output (all four
        // for n a multiple of 64; one for n = 16): the others are not computed
        const int qn = min(4, (n - n0 + 15) >> 4);
        for (int m0 = 0; m0 < n; m0 += 64) {
            const int rn = min(4, (n - m0 + 15) >> 4);
            const bool full = (rn == 4) && (qn == 4);
            double acc[4][4];
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[r][q] = 0.0;
            for (int k0 = 0; k0 < n; k0 += 16) {
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    int e = tid + t * DQMC_NT;
                    int mm_, kk;
                    if (!TA) { mm_ = e & 63; kk = e >> 6; } else { kk = e & 15; mm_ = e >> 4; }
                    int gm = m0 + mm_, gk = k0 + kk;
                    double v = 0.0;
                    if (gm < n && gk < n) v = TA ? A[gk + (size_t)gm * n] : A[gm + (size_t)gk * n];
                    sA[kk * 64 + mm_] = v;
                }
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    int e = tid + t * DQMC_NT;
                    int kk, jj;
                    if (!TB) { kk = e & 15; jj = e >> 4; } else { jj = e & 63; kk = e >> 6; }
                    int gk = k0 + kk, gj = n0 + jj;
                    double v = 0.0;
                    if (gk < n && gj < n) v = TB ? B[gj + (size_t)gk * n] : B[gk + (size_t)gj * n];
                    sB[kk * 64 + jj] = v;
                }
                __syncthreads();
                if (full) {
#pragma unroll
                    for (int kk = 0; kk < 16; ++kk) {
                        double a[4], b[4];
#pragma unroll
                        for (int r = 0; r < 4; ++r) a[r] = sA[kk * 64 + tx + 16 * r];
#pragma unroll
                        for (int q = 0; q < 4; ++q) b[q] = sB[kk * 64 + ty + 16 * q];
#pragma unroll
                        for (int r = 0; r < 4; ++r)
#pragma unroll
                            for (int q = 0; q < 4; ++q) acc[r][q] = fma(a[r], b[q], acc[r][q]);
                    }
                } else {
                    for (int kk = 0; kk < 16; ++kk) {
                        double a[4], b[4];
#pragma unroll
                        for (int r = 0; r < 4; ++r) a[r] = r < rn ? sA[kk * 64 + tx + 16 * r] : 0.0;
#pragma unroll
                        for (int q = 0; q < 4; ++q) b[q] = q < qn ? sB[kk * 64 + ty + 16 * q] : 0.0;
#pragma unroll
                        for (int r = 0; r < 4; ++r) {
                            if (r < rn) {
#pragma unroll
                                for (int q = 0; q < 4; ++q)
                                    if (q < qn) acc[r][q] = fma(a[r], b[q], acc[r][q]);
                            }
                        }
                    }
                }
                __syncthreads();
            }
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    int gm = m0 + tx + 16 * r, gj = n0 + ty + 16 * q;
                    if (gm < n && gj < n) C[gm + (size_t)gj * n] = acc[r][q];
                }
        }
    }
}

// ---- double-float storage (the mixed path's shared-memory G) ----------------
// A value is a float pair (hi, lo) with |lo| <= ulp(hi) / 2: ~48 significant
// bits.
__device__ __forceinline__ float2 d_to_df(double v) {
    const float h = __double2float_rn(v);
    return make_float2(h, __double2float_rn(v - (double)h));
}
__device__ __forceinline__ double df_to_d(float2 v) { return (double)v.x + (double)v.y; }
// (hi, lo) from an unnormalised pair (Fast2Sum, |s| >= |t|)
__device__ __forceinline__ float2 df_norm(float s, float t) {
    const float h = __fadd_rn(s, t);
    return make_float2(h, __fsub_rn(t, __fsub_rn(h, s)));
}
// a * b for double-float a, b (TwoProd by fmaf; the lo * lo term is dropped)
__device__ __forceinline__ float2 df_mul(float2 a, float2 b) {
    const float p = __fmul_rn(a.x, b.x);
    const float e = __fmaf_rn(a.x, b.x, -p);
    return df_norm(p, __fmaf_rn(a.x, b.y, __fmaf_rn(a.y, b.x, e)));
}
// g + a * b (the rank-1 update's element step): TwoProd, TwoSum, renormalise
__device__ __forceinline__ float2 df_fma(float2 a, float2 b, float2 g) {
    const float p = __fmul_rn(a.x, b.x);
    const float pe = __fmaf_rn(a.x, b.x, -p);
    const float pl = __fmaf_rn(a.x, b.y, __fmaf_rn(a.y, b.x, pe));
    const float s = __fadd_rn(g.x, p);
    const float z = __fsub_rn(s, g.x);
    const float er = __fadd_rn(__fsub_rn(g.x, __fsub_rn(s, z)), __fsub_rn(p, z));
    return df_norm(s, __fadd_rn(__fadd_rn(g.y, pl), er));
}
// C = Diagonal(d) * B and C = A * Diagonal(d) on double-float matrices
__device__ __forceinline__ void dleft_df(int n, float2* __restrict__ C, const float2* __restrict__ d,
                                         const float2* __restrict__ B) {
    for (int e = threadIdx.x; e < n * n; e += DQMC_NT) C[e] = df_mul(d[e % n], B[e]);
}
__device__ __forceinline__ void dright_df(int n, float2* __restrict__ C, const float2* __restrict__ A,
                                          const float2* __restrict__ d) {
    for (int e = threadIdx.x; e < n * n; e += DQMC_NT) C[e] = df_mul(A[e], d[e / n]);
}

// Double-float product for the mixed path: C = A * B on the FP32 pipe, each
// operand either FP64 (split X = Xh + Xl, Xh = fp32(X), Xl = fp32(X - Xh),
// while staging) or already split (ADF / BDF: a float2 array), the result
// FP64 or double-float (CDF).  The main term sum_k Ah Bh is accumulated
// exactly-rounded in a pair of floats: the product is split exactly with one
// fmaf (TwoProd) and added with TwoSum (Knuth); the cross terms Ah Bl + Al Bh
// are accumulated in plain FP32 and Al Bl is dropped.  Relative error ~1e-14
// per product (FP32 alone: ~1e-7, which the wraps' error amplification over
// ten slices turns into O(1)).  About 12 FP32 instructions per multiply-add,
// against one FP64 instruction on a pipe ~60x narrower on GB300.  64 x 64
// tiles, 4 x 4 per thread, k staged 16 at a time (sm: 4 * 16 * 64 floats).
// C must not alias A or B.  The split hopping exponentials and the
// shared-memory G of the mixed path enter without any FP64 instruction.
// TA / TB: the FP64 operand is read transposed (not for split operands).
template <bool ADF, bool BDF, bool CDF, bool TA = false, bool TB = false>
__device__ __noinline__ void mm_dfx(int n, void* __restrict__ Cv, const void* __restrict__ Av,
                                    const void* __restrict__ Bv, double* smd) {
    static_assert(!(ADF && TA) && !(BDF && TB), "split operands are read untransposed");
    float* sAh = reinterpret_cast<float*>(smd);  // [16][64]: sAh[kk*64 + m]
    float* sAl = sAh + 16 * 64;
    float* sBh = sAl + 16 * 64;                   // [16][64]: sBh[kk*64 + j]
    float* sBl = sBh + 16 * 64;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    for (int n0 = 0; n0 < n; n0 += 64) {
        for (int m0 = 0; m0 < n; m0 += 64) {
            float sh[4][4], sl[4][4], xx[4][4];
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int q = 0; q < 4; ++q) sh[r][q] = sl[r][q] = xx[r][q] = 0.f;
            for (int k0 = 0; k0 < n; k0 += 16) {
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    const int e = tid + t * DQMC_NT;
                    const int mm_ = TA ? e >> 4 : e & 63, kk = TA ? e & 15 : e >> 6;
                    const int gm = m0 + mm_, gk = k0 + kk;
                    float2 v = make_float2(0.f, 0.f);
                    if (gm < n && gk < n) {
                        const size_t at = TA ? gk + (size_t)gm * n : gm + (size_t)gk * n;
                        v = ADF ? static_cast<const float2*>(Av)[at]
                                : d_to_df(static_cast<const double*>(Av)[at]);
                    }
                    sAh[kk * 64 + mm_] = v.x;
                    sAl[kk * 64 + mm_] = v.y;
                }
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    const int e = tid + t * DQMC_NT;
                    const int kk = TB ? e >> 6 : e & 15, jj = TB ? e & 63 : e >> 4;
                    const int gk = k0 + kk, gj = n0 + jj;
                    float2 v = make_float2(0.f, 0.f);
                    if (gk < n && gj < n) {
                        const size_t at = TB ? gj + (size_t)gk * n : gk + (size_t)gj * n;
                        v = BDF ? static_cast<const float2*>(Bv)[at]
                                : d_to_df(static_cast<const double*>(Bv)[at]);
                    }
                    sBh[kk * 64 + jj] = v.x;
                    sBl[kk * 64 + jj] = v.y;
                }
                __syncthreads();
#pragma unroll 4
                for (int kk = 0; kk < 16; ++kk) {
                    float ah[4], al[4], bh[4], bl[4];
#pragma unroll
                    for (int r = 0; r < 4; ++r) {
                        ah[r] = sAh[kk * 64 + tx + 16 * r];
                        al[r] = sAl[kk * 64 + tx + 16 * r];
                    }
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        bh[q] = sBh[kk * 64 + ty + 16 * q];
                        bl[q] = sBl[kk * 64 + ty + 16 * q];
                    }
#pragma unroll
                    for (int r = 0; r < 4; ++r)
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            const float p = __fmul_rn(ah[r], bh[q]);
                            const float pe = __fmaf_rn(ah[r], bh[q], -p);
                            const float t = __fadd_rn(sh[r][q], p);
                            const float z = __fsub_rn(t, sh[r][q]);
                            const float er = __fadd_rn(__fsub_rn(sh[r][q], __fsub_rn(t, z)),
                                                       __fsub_rn(p, z));
                            sh[r][q] = t;
                            sl[r][q] = __fadd_rn(sl[r][q], __fadd_rn(er, pe));
                            xx[r][q] = __fmaf_rn(ah[r], bl[q], __fmaf_rn(al[r], bh[q], xx[r][q]));
                        }
                }
                __syncthreads();
            }
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int gm = m0 + tx + 16 * r, gj = n0 + ty + 16 * q;
                    if (gm < n && gj < n) {
                        const size_t at = gm + (size_t)gj * n;
                        if (CDF)
                            static_cast<float2*>(Cv)[at] =
                                df_norm(sh[r][q], __fadd_rn(sl[r][q], xx[r][q]));
                        else
                            static_cast<double*>(Cv)[at] =
                                (double)sh[r][q] + ((double)sl[r][q] + (double)xx[r][q]);
                    }
                }
        }
    }
}

// udt_AVX_pivot! (UDT.jl:216-334) on one n x n block in global memory (the
// blocks of n > 64 that do not fit shared memory; L2-resident): Householder
// QR with column pivoting, explicit Q by backward accumulation, D = |diag R|
// (0 -> 1), T = D^-1 R pivoted (apply = true) or left unpivoted with the
// reflectors below the diagonal (apply = false, consumed by rdivp).
//
// Organised for GB300's narrow FP64 pipe (a warp's FP64 instruction costs the
// pipe the same however few of its lanes do useful work):
//  * per step, warp 0 alone finds the pivot (bit patterns of the squared
//    norms compared on the integer pipe), swaps it in and forms the reflector
//    (scaled by the reciprocal of xi1, a rounding-level difference from the
//    division), staged in shared memory `xs`; one barrier;
//  * every warp then applies it to eight trailing columns at a time with four
//    lanes per column (rows interleaved by four from a 4-aligned start, so a
//    warp's load of one row quartet of eight columns touches eight whole
//    32-byte sectors; two shuffles combine a column's dot product); second
//    barrier.  Per column and row one FMA for the dot product, one for the
//    update, and one for the next step's squared norm;
//  * DOWNDATE (mixed-precision chains): the norms are downdated instead,
//    ||a(j+1:n)||^2 = ||a(j:n)||^2 - a_j^2 (LAPACK xGEQP3 / xLAQPS, Quintana-
//    Orti, Sun and Bischof 1998), and recomputed in the update pass only for
//    columns where cancellation has reduced the downdated value below
//    sqrt(eps) of the last recomputed one (warp-uniform: a pass recomputes
//    when one of its eight columns needs it); the reflector's own norm is
//    recomputed from its column.  Without DOWNDATE the norms are recomputed
//    every step as the reference's indmaxcolumn does;
//  * Q accumulates in blocks of reflectors (q_blocked).
// scr: n*n scratch (apply only); sv: n doubles of shared memory (squared
// norms); sxd: shared scalars; xs: 2048 doubles of shared memory (the
// reflector at 0, DOWNDATE reference norms at 1024); ws: DQMC_QWS doubles of
// shared memory.
// Strided column kernels of udt_pivot_g: rows r, r + 4, r + 8, ... < n of a
// column in global memory (L2), eight loads in flight per lane (four
// accumulation chains), which the L2 latency of the two-die part needs to
// keep the FP64 pipe fed.
__device__ __forceinline__ double dot_s4(const double* __restrict__ x, const double* a, int r,
                                         int n) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    for (; r + 28 < n; r += 32) {
        const double a0 = a[r], a1 = a[r + 4], a2 = a[r + 8], a3 = a[r + 12];
        const double a4 = a[r + 16], a5 = a[r + 20], a6 = a[r + 24], a7 = a[r + 28];
        s0 = fma(x[r], a0, s0);
        s1 = fma(x[r + 4], a1, s1);
        s2 = fma(x[r + 8], a2, s2);
        s3 = fma(x[r + 12], a3, s3);
        s0 = fma(x[r + 16], a4, s0);
        s1 = fma(x[r + 20], a5, s1);
        s2 = fma(x[r + 24], a6, s2);
        s3 = fma(x[r + 28], a7, s3);
    }
    for (; r < n; r += 4) s0 = fma(x[r], a[r], s0);
    return (s0 + s1) + (s2 + s3);
}
// a[r'] -= x[r'] v for the strided rows; with SQ, returns the sum of the new
// values' squares
template <bool SQ>
__device__ __forceinline__ double axpy_s4(double* a, const double* __restrict__ x, double v, int r,
                                          int n) {
    double q0 = 0.0, q1 = 0.0, q2 = 0.0, q3 = 0.0;
    for (; r + 28 < n; r += 32) {
        double b[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) b[u] = a[r + 4 * u];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            b[u] = fma(-x[r + 4 * u], v, b[u]);
            a[r + 4 * u] = b[u];
        }
        if (SQ) {
            q0 = fma(b[0], b[0], q0);
            q1 = fma(b[1], b[1], q1);
            q2 = fma(b[2], b[2], q2);
            q3 = fma(b[3], b[3], q3);
            q0 = fma(b[4], b[4], q0);
            q1 = fma(b[5], b[5], q1);
            q2 = fma(b[6], b[6], q2);
            q3 = fma(b[7], b[7], q3);
        }
    }
    for (; r < n; r += 4) {
        const double b = fma(-x[r], v, a[r]);
        a[r] = b;
        if (SQ) q0 = fma(b, b, q0);
    }
    return (q0 + q1) + (q2 + q3);
}

// Explicit Q of a Householder QR, Q = H_0 H_1 ... H_{n-1} I (UDT.jl:272-289),
// accumulated in blocks of DQMC_QB reflectors from the last block to the
// first: H_k0 ... H_k1-1 = I - V T V^T (compact WY form; Schreiber and Van
// Loan 1989, T as LAPACK's xLARFT builds it, forward and columnwise), so that
// each block updates the trailing rows and columns of Q with two products
// (W = V^T Q, Q -= V (T W)) staged through shared memory, in column passes of
// DQMC_QC, instead of one rank-1 pass over Q per reflector.  Same Q up to
// rounding.  In: the reflectors below the diagonal (unit diagonal implied),
// tau: their factors; ws: DQMC_QWS doubles of shared memory.
#define DQMC_QB 16
#define DQMC_QC 64
#define DQMC_QWS (2 * DQMC_QB * DQMC_QB + 32 * DQMC_QB + 32 * DQMC_QC + 2 * DQMC_QB * DQMC_QC)
// entry r of reflector k0 + i of a block of nb
__device__ __forceinline__ double qv(const double* In, int n, int k0, int i, int nb, int r) {
    const int k = k0 + i;
    if (i >= nb || r < k) return 0.0;
    return r == k ? 1.0 : In[(size_t)k * n + r];
}
__device__ __noinline__ void q_blocked(int n, double* __restrict__ U, const double* __restrict__ In,
                                       const double* __restrict__ tau, double* ws) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    double* Y = ws;                          // [QB][QB]: v_p . v_l for p < l
    double* T = Y + DQMC_QB * DQMC_QB;       // [QB][QB], upper triangular
    double* Vs = T + DQMC_QB * DQMC_QB;      // [32][QB]: a row slice of V
    double* Qs = Vs + 32 * DQMC_QB;          // [32][QC]: the same rows of Q's pass
    double* W = Qs + 32 * DQMC_QC;           // [QB][QC]: V^T Q
    double* W2 = W + DQMC_QB * DQMC_QC;      // [QB][QC]: T V^T Q
    ident(n, U);
    __syncthreads();
    if (tid == 0) U[(size_t)(n - 1) * n + (n - 1)] -= tau[n - 1];  // the 1 x 1 reflector
    __syncthreads();
    for (int k1 = n - 1; k1 > 0;) {
        const int k0 = ((k1 - 1) / DQMC_QB) * DQMC_QB, nb = k1 - k0;
        // Y[p][l] = v_p . v_l over the rows >= k0 + l (p < l < nb)
        for (int pl = warp; pl < DQMC_QB * DQMC_QB; pl += DQMC_NW) {
            const int p = pl / DQMC_QB, l = pl % DQMC_QB;
            if (p >= l || l >= nb) continue;
            double y = 0.0;
            for (int r = k0 + l + lane; r < n; r += 32)
                y = fma(qv(In, n, k0, p, nb, r), qv(In, n, k0, l, nb, r), y);
            y = warp_sum(y);
            if (lane == 0) Y[p * DQMC_QB + l] = y;
        }
        __syncthreads();
        // T[l][l] = tau_l, T[0:l][l] = -tau_l T[0:l][0:l] Y[0:l][l]; zero elsewhere
        if (warp == 0) {
            for (int e = lane; e < DQMC_QB * DQMC_QB; e += 32) T[e] = 0.0;
            __syncwarp();
            for (int l = 0; l < nb; ++l) {
                const double tl = tau[k0 + l];
                double v = 0.0;
                if (lane < l) {
                    for (int p = lane; p < l; ++p) v = fma(T[lane * DQMC_QB + p], Y[p * DQMC_QB + l], v);
                    v = -tl * v;
                }
                __syncwarp();
                if (lane < l) T[lane * DQMC_QB + l] = v;
                if (lane == l) T[l * DQMC_QB + l] = tl;
                __syncwarp();
            }
        }
        __syncthreads();
        const int wi = tid & (DQMC_QB - 1), wc = (tid >> 4) * 4;  // W outputs (wi, wc..wc+3)
        for (int c0 = k0; c0 < n; c0 += DQMC_QC) {
            // W = V^T Q[k0:n, c0:c0+QC]
            double acc[4] = {0.0, 0.0, 0.0, 0.0};
            for (int r0 = k0; r0 < n; r0 += 32) {
                for (int e = tid; e < 32 * DQMC_QB; e += DQMC_NT) {
                    const int rr = e & 31, i = e >> 5, r = r0 + rr;
                    Vs[rr * DQMC_QB + i] = r < n ? qv(In, n, k0, i, nb, r) : 0.0;
                }
                for (int e = tid; e < 32 * DQMC_QC; e += DQMC_NT) {
                    const int rr = e & 31, cc = e >> 5, r = r0 + rr, c = c0 + cc;
                    Qs[rr * DQMC_QC + cc] = (r < n && c < n) ? U[(size_t)c * n + r] : 0.0;
                }
                __syncthreads();
#pragma unroll 8
                for (int rr = 0; rr < 32; ++rr) {
                    const double v = Vs[rr * DQMC_QB + wi];
#pragma unroll
                    for (int q = 0; q < 4; ++q) acc[q] = fma(v, Qs[rr * DQMC_QC + wc + q], acc[q]);
                }
                __syncthreads();
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) W[wi * DQMC_QC + wc + q] = acc[q];
            __syncthreads();
            // W2 = T W
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                double sum = 0.0;
                for (int p = wi; p < DQMC_QB; ++p)
                    sum = fma(T[wi * DQMC_QB + p], W[p * DQMC_QC + wc + q], sum);
                W2[wi * DQMC_QC + wc + q] = sum;
            }
            __syncthreads();
            // Q[k0:n, pass] -= V W2: lanes along the rows, eight columns a thread
            {
                const int rr = lane, cg = warp * 8;
                for (int r = k0 + rr; r < n; r += 32) {
                    double v[DQMC_QB];
#pragma unroll
                    for (int i = 0; i < DQMC_QB; ++i) v[i] = qv(In, n, k0, i, nb, r);
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const int cc = cg + q, c = c0 + cc;
                        if (c < n) {
                            double sum = U[(size_t)c * n + r];
#pragma unroll
                            for (int i = 0; i < DQMC_QB; ++i) sum = fma(-v[i], W2[i * DQMC_QC + cc], sum);
                            U[(size_t)c * n + r] = sum;
                        }
                    }
                }
            }
            __syncthreads();
        }
        k1 = k0;
    }
}

template <bool DOWNDATE>
__device__ __noinline__ void udt_pivot_g(int n, double* __restrict__ U, double* __restrict__ D,
                                         double* __restrict__ In, int* __restrict__ piv,
                                         double* __restrict__ tau, bool apply,
                                         double* __restrict__ scr, double* sv, double* sxd,
                                         double* xs, double* ws) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int h = lane >> 3, cl = lane & 7;  // row quarter, column within the group of eight
    const double tol3z = 1.4901161193847656e-08;  // sqrt(2^-52)
    double* sv2 = xs + 1024;
    for (int i = tid; i < n; i += DQMC_NT) piv[i] = i + 1;
    // initial squared column norms
    for (int g = warp * 8; g < n; g += 8 * DQMC_NW) {
        const int c = g + cl;
        const bool act = c < n;
        const double* a = In + (size_t)(act ? c : g) * n;
        double q = act ? dot_s4(a, a, h, n) : 0.0;
        q += __shfl_xor_sync(0xffffffffu, q, 8);
        q += __shfl_xor_sync(0xffffffffu, q, 16);
        if (act && h == 0) {
            sv[c] = q;
            if (DOWNDATE) sv2[c] = q;
        }
    }
    __syncthreads();
    for (int j = 0; j < n; ++j) {
        const int rb = (j + 1) & ~3;  // first row of the aligned quartets below row j
        if (warp == 0) {
            // indmaxcolumn: first column of maximal norm among j..n-1
            long long best = -1;
            int bi = j;  // never out of range, also when every norm is NaN
            for (int col = j + lane; col < n; col += 32) {
                const long long v = __double_as_longlong(sv[col]);
                if (v > best) { best = v; bi = col; }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const long long ob = __shfl_xor_sync(0xffffffffu, best, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
            }
            const int jm = bi;
            double* x = In + (size_t)j * n;
            if (jm != j) {
                double* a = In + (size_t)jm * n;
                for (int r = lane; r < n; r += 32) {
                    const double t = a[r];
                    a[r] = x[r];
                    x[r] = t;
                }
                if (lane == 0) {
                    const int tp = piv[jm];
                    piv[jm] = piv[j];
                    piv[j] = tp;
                    sv[jm] = sv[j];
                    if (DOWNDATE) sv2[jm] = sv2[j];
                }
            }
            __syncwarp();
            // reflector! (UDT.jl:157-172)
            double normu = __longlong_as_double(best);
            if (DOWNDATE) {
                double s0 = 0.0, s1 = 0.0;
                int r = j + lane;
                for (; r + 32 < n; r += 64) {
                    s0 = fma(x[r], x[r], s0);
                    s1 = fma(x[r + 32], x[r + 32], s1);
                }
                if (r < n) s0 = fma(x[r], x[r], s0);
                normu = warp_sum(s0 + s1);
            }
            const double xi1 = x[j];
            double t = 0.0;
            if (normu != 0.0) {
                const double nu = copysign(sqrt(normu), xi1);
                const double xi = xi1 + nu;
                const double inv = 1.0 / xi;
                for (int r = j + 1 + lane; r < n; r += 32) {
                    const double v = x[r] * inv;
                    x[r] = v;
                    xs[r] = v;
                }
                if (lane == 0) x[j] = -nu;
                t = xi / nu;
            } else {
                for (int r = j + 1 + lane; r < n; r += 32) xs[r] = x[r];
            }
            // rows of the first quartet at or above row j take no part
            if (lane < 4 && rb + lane <= j) xs[rb + lane] = 0.0;
            if (lane == 0) { tau[j] = t; sxd[0] = t; }
        }
        __syncthreads();
        // reflectorApply! (UDT.jl:53-70) to columns j+1..n-1 and their norms
        const double t = sxd[0];
        for (int g = j + 1 + warp * 8; g < n; g += 8 * DQMC_NW) {
            const int c = g + cl;
            const bool act = c < n;
            double* a = In + (size_t)(act ? c : g) * n;
            double sdot = act ? dot_s4(xs, a, rb + h, n) : 0.0;
            sdot += __shfl_xor_sync(0xffffffffu, sdot, 8);
            sdot += __shfl_xor_sync(0xffffffffu, sdot, 16);
            const double aj = act ? a[j] : 0.0;
            const double vA = t * (aj + sdot);
            const double ajn = aj - vA;
            bool need = true;
            double down = 0.0;
            if (DOWNDATE) {
                const double s1v = act ? sv[c] : 0.0;
                down = fma(-ajn, ajn, s1v);
                need = act && s1v != 0.0 && down <= tol3z * sv2[c];
                if (s1v == 0.0) down = 0.0;
            }
            const bool norms = DOWNDATE ? __any_sync(0xffffffffu, need) : true;
            double q = 0.0;
            if (act) {
                // first quartet: rows at or above j stay
                const int r = rb + h;
                if (r > j && r < n) {
                    const double an = fma(-xs[r], vA, a[r]);
                    a[r] = an;
                    q = an * an;
                }
                if (norms) q += axpy_s4<true>(a, xs, vA, r + 4, n);
                else axpy_s4<false>(a, xs, vA, r + 4, n);
            }
            if (norms) {
                q += __shfl_xor_sync(0xffffffffu, q, 8);
                q += __shfl_xor_sync(0xffffffffu, q, 16);
            }
            __syncwarp();  // every lane has read a[j] and sv[c]
            if (act && h == 0) {
                a[j] = ajn;
                if (!DOWNDATE) {
                    sv[c] = q;
                } else if (need) {
                    sv[c] = q;
                    sv2[c] = q;
                } else {
                    sv[c] = down;
                }
            }
        }
        __syncthreads();
    }
    // Calculate Q (UDT.jl:272-289)
    q_blocked(n, U, In, tau, ws);
    // D (UDT.jl:293-301)
    for (int i = tid; i < n; i += DQMC_NT) {
        double xx = fabs(In[(size_t)i * n + i]);
        D[i] = (xx == 0.0) ? 1.0 : xx;
    }
    __syncthreads();
    // _apply_pivot! (UDT.jl:311-334)
    if (apply) {
        for (int e = tid; e < n * n; e += DQMC_NT) {
            int i = e % n, j = e / n;
            double d = 1.0 / D[i];
            double val = (j >= i) ? d * In[e] : 0.0;
            scr[i + (size_t)(piv[j] - 1) * n] = val;
        }
        __syncthreads();
        copy(n * n, In, scr);
    } else {
        for (int e = tid; e < n * n; e += DQMC_NT) {
            int i = e % n, j = e / n;
            if (j >= i) {
                double d = 1.0 / D[i];
                In[e] = d * In[e];
            }
        }
    }
    __syncthreads();
}

// udt_AVX_pivot! for n <= 64 with the factorisation held in shared memory
// (sIn, sU: n*(n+1) doubles each, leading dimension n+1).  Same algorithm and
// outputs as udt_pivot, organised for GB300's narrow FP64 pipe, where every
// FP64 warp instruction costs the same pipe time however few lanes do useful
// work and a dependent FP64 instruction waits about one warp-instruction pass
// of the pipe: four threads per column, each with two independent
// accumulation chains, run the dot products and updates down the column (two
// shuffles to combine), instead of a warp per column with a five-level
// reduction.  The column norms that the reference recomputes each
// step (indmaxcolumn) come out of the reflector-application pass, which
// already holds the updated columns; the pivot search compares the norms'
// bit patterns on the integer pipe (non-negative doubles order like their
// bits); the reflector scales by the reciprocal of xi1 (rounding-level
// difference from the division).  Two barriers per column.
__device__ __noinline__ void udt_pivot_sm(int n, double* __restrict__ U, double* __restrict__ D,
                                          double* __restrict__ In, int* __restrict__ piv,
                                          double* __restrict__ tau, bool apply, double* sIn,
                                          double* sU, double* sv, double* sxd) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int ld = n + 1;
    for (int e = tid; e < n * n; e += DQMC_NT) sIn[(e % n) + (e / n) * ld] = In[e];
    for (int i = tid; i < n; i += DQMC_NT) piv[i] = i + 1;
    __syncthreads();
    // initial squared column norms: four threads per column, two accumulation
    // chains each (the guard is warp-uniform so every lane of a participating
    // warp reaches the shuffles)
    if (warp * 32 < 4 * n) {
        const bool act = tid < 4 * n;
        const int col = act ? (tid >> 2) : 0, h = tid & 3;
        const double* a = sIn + col * ld;
        double q0 = 0.0, q1 = 0.0;
        if (act) {
            int r = h;
            for (; r + 4 < n; r += 8) {
                q0 = fma(a[r], a[r], q0);
                q1 = fma(a[r + 4], a[r + 4], q1);
            }
            if (r < n) q0 = fma(a[r], a[r], q0);
        }
        double q = q0 + q1;
        q += __shfl_xor_sync(0xffffffffu, q, 1);
        q += __shfl_xor_sync(0xffffffffu, q, 2);
        if (act && h == 0) sv[col] = q;
    }
    __syncthreads();
    for (int j = 0; j < n; ++j) {
        if (warp == 0) {
            // indmaxcolumn: first column of maximal norm among j..n-1
            long long best = -1;
            int bi = j;  // never out of range, also when every norm is NaN
            for (int col = j + lane; col < n; col += 32) {
                long long v = __double_as_longlong(sv[col]);
                if (v > best) { best = v; bi = col; }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                long long ob = __shfl_xor_sync(0xffffffffu, best, o);
                int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
            }
            const int jm = bi;
            const double normu = __longlong_as_double(best);
            if (jm != j) {
                double* a = sIn + jm * ld;
                double* b = sIn + j * ld;
                for (int r = lane; r < n; r += 32) {
                    double t = a[r];
                    a[r] = b[r];
                    b[r] = t;
                }
                if (lane == 0) {
                    int tp = piv[jm];
                    piv[jm] = piv[j];
                    piv[j] = tp;
                    sv[jm] = sv[j];
                }
            }
            __syncwarp();
            // reflector! (UDT.jl:157-172)
            double* x = sIn + j * ld;
            double xi1 = x[j];
            double t = 0.0;
            if (normu != 0.0) {
                double nu = copysign(sqrt(normu), xi1);
                xi1 += nu;
                const double inv = 1.0 / xi1;
                __syncwarp();
                for (int r = j + 1 + lane; r < n; r += 32) x[r] = x[r] * inv;
                if (lane == 0) x[j] = -nu;
                t = xi1 / nu;
            }
            if (lane == 0) { tau[j] = t; sxd[0] = t; }
        }
        __syncthreads();
        // reflectorApply! (UDT.jl:53-70) fused with the next step's column
        // norms: four threads per column, two accumulation chains each
        const int ncols = n - j - 1;
        if (warp * 32 < 4 * ncols) {
            const double t = sxd[0];
            const double* x = sIn + j * ld;
            const bool act = tid < 4 * ncols;
            const int col = j + 1 + (tid >> 2), h = tid & 3;
            double* a = sIn + (act ? col : j) * ld;
            const double aj = act ? a[j] : 0.0;
            double s0 = 0.0, s1 = 0.0;
            if (act) {
                int r = j + 1 + h;
                for (; r + 4 < n; r += 8) {
                    s0 = fma(x[r], a[r], s0);
                    s1 = fma(x[r + 4], a[r + 4], s1);
                }
                if (r < n) s0 = fma(x[r], a[r], s0);
            }
            double s = s0 + s1;
            s += __shfl_xor_sync(0xffffffffu, s, 1);
            s += __shfl_xor_sync(0xffffffffu, s, 2);
            const double vAj = t * (aj + s);
            double q0 = 0.0, q1 = 0.0;
            if (act) {
                if (h == 0) a[j] = aj - vAj;
                int r = j + 1 + h;
                for (; r + 4 < n; r += 8) {
                    const double v0 = fma(-x[r], vAj, a[r]);
                    const double v1 = fma(-x[r + 4], vAj, a[r + 4]);
                    a[r] = v0;
                    a[r + 4] = v1;
                    q0 = fma(v0, v0, q0);
                    q1 = fma(v1, v1, q1);
                }
                if (r < n) {
                    const double v0 = fma(-x[r], vAj, a[r]);
                    a[r] = v0;
                    q0 = fma(v0, v0, q0);
                }
            }
            double q = q0 + q1;
            q += __shfl_xor_sync(0xffffffffu, q, 1);
            q += __shfl_xor_sync(0xffffffffu, q, 2);
            if (act && h == 0) sv[col] = q;
        }
        __syncthreads();
    }
    // Calculate Q (UDT.jl:272-289)
    for (int e = tid; e < n * n; e += DQMC_NT) {
        int i = e % n, c = e / n;
        sU[i + c * ld] = (i == c) ? 1.0 : 0.0;
    }
    __syncthreads();
    if (tid == 0) sU[(n - 1) * ld + (n - 1)] -= tau[n - 1];
    __syncthreads();
    for (int k = n - 2; k >= 0; --k) {
        const int ncols = n - k;
        if (warp * 32 < 4 * ncols) {
            const double* v = sIn + k * ld;
            const double t = tau[k];
            const bool act = tid < 4 * ncols;
            const int col = k + (tid >> 2), h = tid & 3;
            double* u = sU + (act ? col : k) * ld;
            const double uk = act ? u[k] : 0.0;
            double s0 = 0.0, s1 = 0.0;
            if (act) {
                int r = k + 1 + h;
                for (; r + 4 < n; r += 8) {
                    s0 = fma(v[r], u[r], s0);
                    s1 = fma(v[r + 4], u[r + 4], s1);
                }
                if (r < n) s0 = fma(v[r], u[r], s0);
            }
            double s = s0 + s1;
            s += __shfl_xor_sync(0xffffffffu, s, 1);
            s += __shfl_xor_sync(0xffffffffu, s, 2);
            const double vB = t * (uk + s);
            if (act) {
                if (h == 0) u[k] = uk - vB;
                for (int r = k + 1 + h; r < n; r += 4) u[r] = fma(-v[r], vB, u[r]);
            }
        }
        __syncthreads();
    }
    // D (UDT.jl:293-301); 1/D per row as the reference's _apply_pivot!
    for (int i = tid; i < n; i += DQMC_NT) {
        double xx = fabs(sIn[i * ld + i]);
        double d = (xx == 0.0) ? 1.0 : xx;
        D[i] = d;
        sv[i] = 1.0 / d;
    }
    for (int e = tid; e < n * n; e += DQMC_NT) U[e] = sU[(e % n) + (e / n) * ld];
    __syncthreads();
    // _apply_pivot! (UDT.jl:311-334), straight from shared memory
    for (int e = tid; e < n * n; e += DQMC_NT) {
        int i = e % n, j = e / n;
        const double v = sIn[i + j * ld];
        if (apply) {
            In[i + (size_t)(piv[j] - 1) * n] = (j >= i) ? sv[i] * v : 0.0;
        } else {
            In[e] = (j >= i) ? sv[i] * v : v;
        }
    }
    __syncthreads();
}

// One flavour block's operands of udt_pivot_sm2.
struct UdtJob {
    double* U;
    double* D;
    double* In;
    int* piv;
    double* tau;
};

// udt_pivot_sm for the two flavour blocks of a BlockDiagonal matrix at once
// (UDT.jl:352-370 runs them one after the other; they are independent):
// threads 0-127 factor block 0, threads 128-255 block 1, each in its own half
// of `arena` (n <= 64, leading dimension n + 1, block g at g n (n + 1)) with
// two threads per column;
// the serial reflector step of the two blocks runs on warps 0 and 7 (different
// SM sub-partitions), so the two latency chains overlap, and Q is accumulated
// directly in U (global memory) instead of a second shared-memory block.
// sv: 2 * 64 doubles (block g at g * 64); sxd: 2 doubles.  Same algorithm and
// pivot rule as udt_pivot_sm.
__device__ __noinline__ void udt_pivot_sm2(int n, UdtJob j0, UdtJob j1, bool apply,
                                           double* arena, double* sv, double* sxd,
                                           bool one = false) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // block 1 numbers its warps backwards (warp 7 first): when a late step
    // keeps only the first warps of each block busy, the two blocks' warps
    // sit on different SM sub-partitions
    const int g = tid >> 7, gwarp = g ? 7 - warp : warp;
    // one: block j0 alone (threads 128-255 only keep the barriers), with the
    // same arithmetic per block as the pair
    const int gtid = (one && g) ? (1 << 20) : gwarp * 32 + lane;
    const UdtJob J = g ? j1 : j0;
    const int ld = n + 1;
    double* sIn = arena + (size_t)g * n * ld;
    double* svg = sv + g * 64;
    for (int e = gtid; e < n * n; e += 128) sIn[(e % n) + (e / n) * ld] = J.In[e];
    for (int i = gtid; i < n; i += 128) J.piv[i] = i + 1;
    __syncthreads();
    // initial squared column norms: two threads per column, two chains each
    if (gwarp * 32 < 2 * n) {
        const bool act = gtid < 2 * n;
        const int col = act ? (gtid >> 1) : 0, h = gtid & 1;
        const double* a = sIn + col * ld;
        double q0 = 0.0, q1 = 0.0;
        if (act) {
            int r = h;
            for (; r + 2 < n; r += 4) {
                q0 = fma(a[r], a[r], q0);
                q1 = fma(a[r + 2], a[r + 2], q1);
            }
            if (r < n) q0 = fma(a[r], a[r], q0);
        }
        double q = q0 + q1;
        q += __shfl_xor_sync(0xffffffffu, q, 1);
        if (act && h == 0) svg[col] = q;
    }
    __syncthreads();
    for (int j = 0; j < n; ++j) {
        if (gwarp == 0 && !(one && g)) {  // warp 0 for block 0, warp 7 for block 1
            long long best = -1;
            int bi = j;  // never out of range, also when every norm is NaN
            for (int col = j + lane; col < n; col += 32) {
                long long v = __double_as_longlong(svg[col]);
                if (v > best) { best = v; bi = col; }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                long long ob = __shfl_xor_sync(0xffffffffu, best, o);
                int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
            }
            const int jm = bi;
            const double normu = __longlong_as_double(best);
            if (jm != j) {
                double* a = sIn + jm * ld;
                double* b = sIn + j * ld;
                for (int r = lane; r < n; r += 32) {
                    double t = a[r];
                    a[r] = b[r];
                    b[r] = t;
                }
                if (lane == 0) {
                    int tp = J.piv[jm];
                    J.piv[jm] = J.piv[j];
                    J.piv[j] = tp;
                    svg[jm] = svg[j];
                }
            }
            __syncwarp();
            double* x = sIn + j * ld;
            double xi1 = x[j];
            double t = 0.0;
            if (normu != 0.0) {
                double nu = copysign(sqrt(normu), xi1);
                xi1 += nu;
                const double inv = 1.0 / xi1;
                __syncwarp();
                for (int r = j + 1 + lane; r < n; r += 32) x[r] = x[r] * inv;
                if (lane == 0) x[j] = -nu;
                t = xi1 / nu;
            }
            if (lane == 0) { J.tau[j] = t; sxd[g] = t; }
        }
        __syncthreads();
        const int ncols = n - j - 1;
        if (gwarp * 32 < 2 * ncols) {
            const double t = sxd[g];
            const double* x = sIn + j * ld;
            const bool act = gtid < 2 * ncols;
            const int col = j + 1 + (gtid >> 1), h = gtid & 1;
            double* a = sIn + (act ? col : j) * ld;
            const double aj = act ? a[j] : 0.0;
            double s0 = 0.0, s1 = 0.0;
            if (act) {
                int r = j + 1 + h;
                for (; r + 2 < n; r += 4) {
                    s0 = fma(x[r], a[r], s0);
                    s1 = fma(x[r + 2], a[r + 2], s1);
                }
                if (r < n) s0 = fma(x[r], a[r], s0);
            }
            double s = s0 + s1;
            s += __shfl_xor_sync(0xffffffffu, s, 1);
            const double vAj = t * (aj + s);
            double q0 = 0.0, q1 = 0.0;
            if (act) {
                if (h == 0) a[j] = aj - vAj;
                int r = j + 1 + h;
                for (; r + 2 < n; r += 4) {
                    const double v0 = fma(-x[r], vAj, a[r]);
                    const double v1 = fma(-x[r + 2], vAj, a[r + 2]);
                    a[r] = v0;
                    a[r + 2] = v1;
                    q0 = fma(v0, v0, q0);
                    q1 = fma(v1, v1, q1);
                }
                if (r < n) {
                    const double v0 = fma(-x[r], vAj, a[r]);
                    a[r] = v0;
                    q0 = fma(v0, v0, q0);
                }
            }
            double q = q0 + q1;
            q += __shfl_xor_sync(0xffffffffu, q, 1);
            if (act && h == 0) svg[col] = q;
        }
        __syncthreads();
    }
    // Calculate Q (UDT.jl:272-289), accumulated in U
    for (int e = gtid; e < n * n; e += 128) {
        int i = e % n, c = e / n;
        J.U[e] = (i == c) ? 1.0 : 0.0;
    }
    __syncthreads();
    if (gtid == 0) J.U[(size_t)(n - 1) * n + (n - 1)] -= J.tau[n - 1];
    __syncthreads();
    for (int k = n - 2; k >= 0; --k) {
        const int ncols = n - k;
        if (gwarp * 32 < 2 * ncols) {
            const double* v = sIn + k * ld;
            const double t = J.tau[k];
            const bool act = gtid < 2 * ncols;
            const int col = k + (gtid >> 1), h = gtid & 1;
            double* u = J.U + (size_t)(act ? col : k) * n;
            const double uk = act ? u[k] : 0.0;
            double s0 = 0.0, s1 = 0.0;
            if (act) {
                int r = k + 1 + h;
                for (; r + 2 < n; r += 4) {
                    s0 = fma(v[r], u[r], s0);
                    s1 = fma(v[r + 2], u[r + 2], s1);
                }
                if (r < n) s0 = fma(v[r], u[r], s0);
            }
            double s = s0 + s1;
            s += __shfl_xor_sync(0xffffffffu, s, 1);
            const double vB = t * (uk + s);
            if (act) {
                if (h == 0) u[k] = uk - vB;
                for (int r = k + 1 + h; r < n; r += 2) u[r] = fma(-v[r], vB, u[r]);
            }
        }
        __syncthreads();
    }
    // D (UDT.jl:293-301); 1/D per row as the reference's _apply_pivot!
    for (int i = gtid; i < n; i += 128) {
        double xx = fabs(sIn[i * ld + i]);
        double d = (xx == 0.0) ? 1.0 : xx;
        J.D[i] = d;
        svg[i] = 1.0 / d;
    }
    __syncthreads();
    // _apply_pivot! (UDT.jl:311-334), straight from shared memory
    for (int e = gtid; e < n * n; e += 128) {
        int i = e % n, jj = e / n;
        const double v = sIn[i + jj * ld];
        if (apply) {
            J.In[i + (size_t)(J.piv[jj] - 1) * n] = (jj >= i) ? svg[i] * v : 0.0;
        } else {
            J.In[e] = (jj >= i) ? svg[i] * v : v;
        }
    }
    __syncthreads();
}

// rdivp for the two flavour blocks at once (n <= 64): threads 0-63 run the
// rows of block 0 and threads 64-127 those of block 1 (four warps, one per SM
// sub-partition, where one block alone keeps two of them busy).  rcp: 2 * 64
// doubles.  Same arithmetic per row as rdivp.
__device__ __noinline__ void rdivp2(int n, double* A0, const double* T0, double* O0, const int* p0,
                                    double* A1, const double* T1, double* O1, const int* p1,
                                    double* rcp, int nb = 2) {
    // nb = 1: block 0 alone, the same arithmetic per row
    const int tid = threadIdx.x;
    for (int e = tid; e < nb * n; e += DQMC_NT) {
        const int b = e / n, j = e % n;
        const double* T = b ? T1 : T0;
        rcp[b * 64 + j] = 1.0 / T[(size_t)j * n + j];
    }
    for (int e = tid; e < nb * n * n; e += DQMC_NT) {
        const int b = e / (n * n), f = e % (n * n);
        const int i = f % n, j = f / n;
        const double* A = b ? A1 : A0;
        const int* piv = b ? p1 : p0;
        (b ? O1 : O0)[f] = A[i + (size_t)(piv[j] - 1) * n];
    }
    __syncthreads();
    if (tid < 64 * nb) {
        const int b = tid >> 6, i = tid & 63;
        if (i < n) {
            double* A = b ? A1 : A0;
            const double* T = b ? T1 : T0;
            const double* O = b ? O1 : O0;
            const double* rc = rcp + b * 64;
            for (int j = 0; j < n; ++j) {
                const double* tj = T + (size_t)j * n;
                double x0 = O[i + (size_t)j * n], x1 = 0.0;
                int k = 0;
                for (; k + 1 < j; k += 2) {
                    x0 = fma(-A[i + (size_t)k * n], tj[k], x0);
                    x1 = fma(-A[i + (size_t)(k + 1) * n], tj[k + 1], x1);
                }
                if (k < j) x0 = fma(-A[i + (size_t)k * n], tj[k], x0);
                A[i + (size_t)j * n] = (x0 + x1) * rc[j];
            }
        }
    }
    __syncthreads();
}

// rdivp!: A <- A * P * T^-1 with T upper triangular (real.jl:198-226 for the
// dense form, blockdiagonal.jl:286-324 for the block form, which multiplies
// by 1/T[j,j] instead of dividing).  Rows of A are independent: one thread per
// row runs the forward substitution.
__device__ __noinline__ void rdivp(int n, double* __restrict__ A, const double* __restrict__ T,
                      double* __restrict__ O, const int* __restrict__ piv, bool block_form,
                      double* __restrict__ rcp) {
    // 1/T[j,j] once per column (the block form's invtjj); the dense form's
    // division x / T[j,j] becomes the same multiply (rounding-level change),
    // which keeps DP divisions off the narrow FP64 pipe's critical path
    (void)block_form;
    for (int j = threadIdx.x; j < n; j += DQMC_NT) rcp[j] = 1.0 / T[(size_t)j * n + j];
    for (int e = threadIdx.x; e < n * n; e += DQMC_NT) {
        int i = e % n, j = e / n;
        O[e] = A[i + (size_t)(piv[j] - 1) * n];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += DQMC_NT) {
        for (int j = 0; j < n; ++j) {
            const double* tj = T + (size_t)j * n;
            // two independent accumulation chains halve the dependent-FMA latency
            // (eight loads of the row in flight, four accumulation chains)
            double x0 = O[i + (size_t)j * n], x1 = 0.0, x2 = 0.0, x3 = 0.0;
            const double* ai = A + i;
            int k = 0;
            for (; k + 7 < j; k += 8) {
                double b[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) b[u] = ai[(size_t)(k + u) * n];
                x0 = fma(-b[0], tj[k], x0);
                x1 = fma(-b[1], tj[k + 1], x1);
                x2 = fma(-b[2], tj[k + 2], x2);
                x3 = fma(-b[3], tj[k + 3], x3);
                x0 = fma(-b[4], tj[k + 4], x0);
                x1 = fma(-b[5], tj[k + 5], x1);
                x2 = fma(-b[6], tj[k + 6], x2);
                x3 = fma(-b[7], tj[k + 7], x3);
            }
            for (; k < j; ++k) x0 = fma(-ai[(size_t)k * n], tj[k], x0);
            A[i + (size_t)j * n] = ((x0 + x1) + (x2 + x3)) * rcp[j];
        }
    }
    __syncthreads();
}

}  // namespace
}  // namespace dqmc
