// Tensor-core (tcgen05) products with FP64-class accuracy for the mixed path.
//
// C = op(A) * op(B) for n x n matrices (n <= 256), computed on the 5th-gen
// tensor cores by splitting both operands into BF16 digit slices (the
// error-free splitting of Ozaki et al., "Error-free transformations of
// matrix multiplication by using fast routines of matrix multiplication and
// its applications", Numer. Algorithms 59 (2012)):
//
//   row r of op(A) is scaled by 2^-e_r (max_k |A[r,k]| < 2^e_r) and written as
//   A[r,k] = 2^(e_r - 7) * sum_i s_i 2^(-8i),  s_i integers, |s_i| <= 129,
//
// i = 0..6 (55 bits of the row's scale; the digits are signed, round to
// nearest); columns of op(B) likewise with 2^f_c.  A BF16 holds every
// s_i 2^(-8i) exactly (8 significant bits).  Every slice product A_i B_j is a
// sum of at most K <= 256 integer terms of magnitude <= 2^14 in units of
// 2^(-8(i+j)), so the FP32 accumulators of tcgen05.mma (kind::f16, BF16
// inputs) hold the digit levels l = i + j = 0, 1, 2, 3 (1 to 4 products)
// exactly -- each in its own TMEM accumulator -- and the fifth accumulator
// takes levels 4 to 6 (18 products), whose rounding (the tensor core
// truncates when it aligns addends) is 2^-32 below level 0.  Pairs with
// i + j > 6 are dropped (below 2^-55 of max_k |A_rk| sum_k |B_kc|).  The
// epilogue adds the five accumulators in double-float arithmetic and scales by
// 2^(e_r + f_c - 14).  The digits are relative to each row's (column's)
// largest entry, so an entry far below it keeps fewer bits than in the
// double-float products on the FP32 pipe (mm_dfx), which are relative to
// each entry: the seventh digit keeps that loss below 2^-55 of the row's
// scale.
//
// Mapping: one CTA (256 threads).  (1) The CTA splits op(A) and op(B) once
// into their digit slices in a global scratch buffer (L2-resident), laid out
// as the shared-memory blocks the MMAs read: per (tile, 16-wide K step) the
// seven slices of a 128 x 16 block of A (rows of the 128-row tile) and of a
// 48 x 16 block of B, each in the no-swizzle K-major canonical layout (8 x 8
// core matrices, 16-byte rows).  (2) Per output tile of 128 rows x 48 columns
// one thread drives a two-stage pipeline: bulk copies (cp.async.bulk,
// completing on an mbarrier) bring the next K step's slices into shared
// memory while the tensor core runs the current step's 28 slice-pair MMAs
// (M = 128, N = 48, K = 16) into the five accumulators (5 x 48 TMEM
// columns); each stage's MMAs are committed to a second mbarrier that frees
// the stage.  (3) All eight warps read the accumulators back with
// tcgen05.ld (warp w reads TMEM lanes 32 (w % 4) .. + 31) and combine them.
// No FP64 arithmetic is issued before the epilogue: FP64 operands are split
// from their bit patterns.
//
// Every wait on an mbarrier is bounded (DQMC_TC_SPIN_NS); on timeout the
// state's status is set, the remaining waits are still bounded, and the
// product returns false.
#pragma once
#include <stdint.h>

#include "dqmc_device.cuh"

#define DQMC_TC_NMAX 256   // largest n (K <= 256 keeps the level sums exact)
#define DQMC_TC_TM 128     // rows per tile (MMA M)
#define DQMC_TC_TN 48      // columns per tile (MMA N)
#define DQMC_TC_KB 16      // K per step (one MMA K step for 16-bit inputs)
#define DQMC_TC_S 7        // digit slices per operand
#define DQMC_TC_NACC 5     // accumulators: levels 0, 1, 2, 3 and 4..6
#define DQMC_TC_COLS 256   // TMEM columns a CTA allocates (5 x 48 used)
#define DQMC_TC_SPIN_NS 2000000000ull  // give up on an mbarrier after 2 s
// bytes of one slice block (rows x 16 BF16) and of all slices of one K step
#define DQMC_TC_ABLK (DQMC_TC_TM * DQMC_TC_KB * 2)
#define DQMC_TC_BBLK (DQMC_TC_TN * DQMC_TC_KB * 2)
#define DQMC_TC_ASTEP (DQMC_TC_S * DQMC_TC_ABLK)
#define DQMC_TC_BSTEP (DQMC_TC_S * DQMC_TC_BBLK)
#define DQMC_TC_STAGE (DQMC_TC_ASTEP + DQMC_TC_BSTEP)
// shared memory of mm_tc: 2 stages + 2 n exponents (ints)
#define DQMC_TC_SMEM (2 * DQMC_TC_STAGE + 2 * DQMC_TC_NMAX * 4)

// global scratch bytes of mm_tc for n x n operands (A slices, then B slices)
__host__ __device__ inline size_t dqmc_tc_scratch_a(int n) {
    const size_t nk = (size_t)(n + DQMC_TC_KB - 1) / DQMC_TC_KB;
    return (size_t)((n + DQMC_TC_TM - 1) / DQMC_TC_TM) * nk * DQMC_TC_ASTEP;
}
__host__ __device__ inline size_t dqmc_tc_scratch_bytes(int n) {
    const size_t nk = (size_t)(n + DQMC_TC_KB - 1) / DQMC_TC_KB;
    return dqmc_tc_scratch_a(n) + (size_t)((n + DQMC_TC_TN - 1) / DQMC_TC_TN) * nk * DQMC_TC_BSTEP;
}
// a chain's scratch holds one such area per flavour block (256-byte aligned),
// so that the two CTAs of a flavour-split chain split their products apart
__host__ __device__ inline size_t dqmc_tc_scratch_stride(int n) {
    return (dqmc_tc_scratch_bytes(n) + 255) & ~(size_t)255;
}

namespace dqmc {

// Shared state of mm_tc in one CTA: the accumulators' TMEM base, a status
// word (nonzero: a wait timed out), and per staging buffer one mbarrier for
// its bulk copies (full) and one for the MMAs reading it (mma), with their
// completed-phase counts (at most one phase of each is outstanding, so the
// parity waits are unambiguous).
struct __align__(16) TcState {
    unsigned long long full[2];
    unsigned long long mma[2];
    uint32_t tmem;
    uint32_t status;
    uint32_t ph_full[2];
    uint32_t ph_mma[2];
    uint32_t pad[2];
};

namespace {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// ---- TMEM allocation (one warp) --------------------------------------------
__device__ __forceinline__ void tc_alloc(uint32_t* dst_smem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(dst_smem)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tc_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// generic-proxy global writes visible to the async proxy (the bulk copies)
__device__ __forceinline__ void fence_proxy_async_global() {
    asm volatile("fence.proxy.async.global;" ::: "memory");
}

// ---- mbarrier ------------------------------------------------------------------
__device__ __forceinline__ void mbar_init(unsigned long long* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
// wait for the phase with parity `parity` to complete; false after the time limit
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, uint32_t parity) {
    const uint32_t a = smem_u32(bar);
    uint64_t t0 = 0;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    while (true) {
        uint32_t ok = 0;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(a), "r"(parity)
            : "memory");
        if (ok) return true;
        uint64_t t1 = 0;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
        if (t1 - t0 > DQMC_TC_SPIN_NS) return false;
    }
}

// one bulk copy global -> shared completing on `bar` (16-byte aligned, size
// a multiple of 16)
__device__ __forceinline__ void bulk_g2s(void* dst_smem, const void* src, uint32_t bytes,
                                         unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst_smem)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// ---- descriptors -------------------------------------------------------------
// Shared-memory matrix descriptor (no swizzle, K-major): start address, byte
// offset between core matrices adjacent in K (leading) and in M / N (stride),
// fixed 0b001 at bits 46-48, base offset 0, swizzle mode 0.
__device__ __forceinline__ uint64_t tc_sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}
#define DQMC_TC_LBO 128u  // K-adjacent core matrices
#define DQMC_TC_SBO 256u  // row-group-adjacent core matrices
// Instruction descriptor of kind::f16: D FP32, A and B BF16, both K-major,
// no negation, N >> 3 at bits 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t tc_idesc_bf16(int M, int N) {
    return (1u << 4)            // D format: F32
           | (1u << 7)          // A format: BF16
           | (1u << 10)         // B format: BF16
           | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t dtmem, uint64_t adesc, uint64_t bdesc,
                                       uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void tc_commit(unsigned long long* bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(bar))
        : "memory");
}
// 8 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tc_ld8(uint32_t taddr, float* v) {
    uint32_t r[8];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = __uint_as_float(r[q]);
}

// ---- splitting -----------------------------------------------------------------
// 2^e as a float (e clamped to [-126, 127])
__device__ __forceinline__ float pow2f(int e) {
    e = e < -126 ? -126 : (e > 127 ? 127 : e);
    return __int_as_float((e + 127) << 23);
}
// exponent e with v < 2^e (v > 0 a float); 0 for v = 0
__device__ __forceinline__ int exp_above_f(float v) {
    if (!(v > 0.0f)) return 0;
    const int E = (int)((__float_as_uint(v) >> 23) & 0xff);
    return E - 126;
}

// The scaled value t = x * 2^(7 - e) (|t| < 2^7) of an FP64 x (|x| < 2^e),
// from its bits with no FP64 instruction: th = its top 24 significand bits
// (an exact float), and the remaining 29 bits in units of 2^-48 of t (the
// seventh digit's unit), rounded to nearest: t = th + low * 2^-48.
__device__ __forceinline__ void scaled_split_d(double x, int e, float& th, long long& low) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
    const int E = (int)((hi >> 20) & 0x7ff);
    const int q = E - 1023 + 7 - e;  // t = 1.m 2^q, q <= 6
    th = 0.0f;
    low = 0;
    if (E == 0 || q < -56) return;   // |t| < 2^-55: below the last digit
    const uint32_t sign = hi & 0x80000000u;
    const uint32_t top23 = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    if (q >= -126) th = __uint_as_float(sign | ((uint32_t)(q + 127) << 23) | top23);
    // the low 29 bits are worth 2^(q - 52) each: 2^(q - 4) digit-6 units
    const long long r29 = (long long)(lo & 0x1FFFFFFFu);
    const int sh = 4 - q;  // >= -2
    long long v;
    if (sh <= 0) v = r29 << (-sh);
    else if (sh >= 31) v = 0;
    else v = (r29 + (1ll << (sh - 1))) >> sh;
    low = sign ? -v : v;
}

// The seven signed digits s_i 2^(-8i) of t = th + low 2^-48 (|t| < 2^7),
// round to nearest: s_0, s_1, s_2 from th by exact float steps (rint, then the
// remainder times 2^8), then the remainder of th and `low` as one integer in
// units of 2^-48 split into four signed bytes (|s_i| <= 128), whose carry
// (-1, 0 or 1) goes back to s_2.
__device__ __forceinline__ void digits7(float th, long long low, float* d) {
    float s0 = rintf(th);
    float r = __fsub_rn(th, s0);
    r = __fmul_rn(r, 256.0f);
    const float s1 = rintf(r);
    r = __fsub_rn(r, s1);
    r = __fmul_rn(r, 256.0f);
    float s2 = rintf(r);
    r = __fsub_rn(r, s2);
    // |r| <= 1/2 in digit-2 units: 2^32 digit-6 units (exact scaling)
    long long R = __float2ll_rn(__fmul_rn(r, 4294967296.0f)) + low;
    int dd[4];
#pragma unroll
    for (int i = 3; i >= 0; --i) {
        const long long t = ((R + 128) & 255) - 128;
        dd[i] = (int)t;
        R = (R - t) >> 8;
    }
    s2 = __fadd_rn(s2, (float)R);
    d[0] = s0;
    d[1] = s1 * 0x1p-8f;
    d[2] = s2 * 0x1p-16f;
    d[3] = (float)dd[0] * 0x1p-24f;
    d[4] = (float)dd[1] * 0x1p-32f;
    d[5] = (float)dd[2] * 0x1p-40f;
    d[6] = (float)dd[3] * 0x1p-48f;
}

// BF16 bits of a float that has at most 8 significant bits (exact)
__device__ __forceinline__ uint32_t bf16_bits(float v) { return __float_as_uint(v) >> 16; }

// byte offset of element (row, k) (k in 0..15) inside a slice block in the
// no-swizzle K-major canonical layout: core matrix (row / 8, k / 8) of 8 rows
// x 16 bytes; K-adjacent core matrices 128 bytes apart, row groups 256 apart
__device__ __forceinline__ uint32_t tc_off(int row, int k) {
    return (uint32_t)((row >> 3) * 256 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// Element (r, k) of op(X), X column-major n x n, T = read transposed; FP64
// (split from its bits) or double-float (float2).
template <bool T>
__device__ __forceinline__ size_t op_at(int n, int r, int k) {
    return T ? (size_t)k + (size_t)r * n : (size_t)r + (size_t)k * n;
}
template <bool DF, bool T>
__device__ __forceinline__ void load_split(const void* X, int n, int r, int k, int e, float& th,
                                           long long& low) {
    const size_t at = op_at<T>(n, r, k);
    if (DF) {
        // a pair (hi, lo): hi scaled is exact; lo (|lo| <= ulp(hi) / 2, so
        // |lo * 2^48| < 2^31 after the scaling) rounded to digit-6 units
        const float2 v = static_cast<const float2*>(X)[at];
        const float p = pow2f(7 - e);
        th = __fmul_rn(v.x, p);
        low = __float2ll_rn(__fmul_rn(__fmul_rn(v.y, p), 281474976710656.0f));
    } else {
        scaled_split_d(static_cast<const double*>(X)[at], e, th, low);
    }
}
// a float with the exponent bound of |op(X)[r][k]| (a power of two <= it, or
// |hi| of a pair): only its exponent is used
template <bool DF, bool T>
__device__ __forceinline__ float mag_elem(const void* X, int n, int r, int k) {
    const size_t at = op_at<T>(n, r, k);
    if (DF) return fabsf(static_cast<const float2*>(X)[at].x);
    const unsigned long long b =
        (unsigned long long)__double_as_longlong(static_cast<const double*>(X)[at]);
    const int e = (int)((b >> 52) & 0x7ff) - 1022;  // |x| < 2^e
    if (e <= -125) return 0.0f;
    return e > 127 ? __int_as_float(0x7f000000) : pow2f(e - 1);
}
// ex[r] = e with max_k |op(X)[r][k]| < 2^e, for every row r < n of op(X)
template <bool DF, bool T>
__device__ __forceinline__ void row_exponents(const void* X, int n, int* ex) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (!T) {  // a row runs across columns: one thread per row, coalesced over r
        for (int r = tid; r < n; r += DQMC_NT) {
            float m = 0.0f;
#pragma unroll 8
            for (int k = 0; k < n; ++k) m = fmaxf(m, mag_elem<DF, T>(X, n, r, k));
            ex[r] = exp_above_f(m);
        }
    } else {  // a row is contiguous: one warp per row
        for (int r = warp; r < n; r += DQMC_NW) {
            float m = 0.0f;
            for (int k = lane; k < n; k += 32) m = fmaxf(m, mag_elem<DF, T>(X, n, r, k));
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
            if (lane == 0) ex[r] = exp_above_f(m);
        }
    }
}

// Split op(X) (n x n, rows in `rows`-row tiles) into its slice blocks in
// global scratch: block (tile, step, slice) at ((tile * nk + step) * S + slice)
// * (rows * 32) bytes; rows and K beyond n are zero.
template <bool DF, bool T>
__device__ __forceinline__ void split_all(const void* X, int n, int rows, const int* ex,
                                          unsigned char* dst) {
    const int nk = (n + DQMC_TC_KB - 1) / DQMC_TC_KB;
    const int rpad = ((n + rows - 1) / rows) * rows;
    const int wpr = nk * (DQMC_TC_KB / 2);  // 32-bit words (two K) per padded row
    const uint32_t blk = (uint32_t)rows * DQMC_TC_KB * 2;
    const int words = rpad * wpr;
    for (int w = threadIdx.x; w < words; w += DQMC_NT) {
        // coalesced global reads: consecutive threads take consecutive r when
        // a column is contiguous, consecutive k when a row is
        const int r = T ? w / wpr : w % rpad;
        const int kp = T ? w % wpr : w / rpad;
        const int k = 2 * kp;
        float d0[DQMC_TC_S], d1[DQMC_TC_S];
#pragma unroll
        for (int i = 0; i < DQMC_TC_S; ++i) d0[i] = d1[i] = 0.0f;
        if (r < n) {
            const int e = ex[r];
            float th;
            long long low;
            if (k < n) {
                load_split<DF, T>(X, n, r, k, e, th, low);
                digits7(th, low, d0);
            }
            if (k + 1 < n) {
                load_split<DF, T>(X, n, r, k + 1, e, th, low);
                digits7(th, low, d1);
            }
        }
        const int tile = r / rows, step = k / DQMC_TC_KB;
        unsigned char* base = dst + ((size_t)tile * nk + step) * DQMC_TC_S * blk +
                              tc_off(r - tile * rows, k - step * DQMC_TC_KB);
#pragma unroll
        for (int i = 0; i < DQMC_TC_S; ++i)
            *reinterpret_cast<uint32_t*>(base + (size_t)i * blk) =
                bf16_bits(d0[i]) | (bf16_bits(d1[i]) << 16);
    }
}

// double-float (h, l) += v (TwoSum of the leading parts)
__device__ __forceinline__ void df_acc(float& h, float& l, float v) {
    const float s = __fadd_rn(h, v);
    const float z = __fsub_rn(s, h);
    const float e = __fadd_rn(__fsub_rn(h, __fsub_rn(s, z)), __fsub_rn(v, z));
    h = s;
    l = __fadd_rn(l, e);
}

// wait for the oldest outstanding phase of a barrier (bounded)
__device__ __forceinline__ bool tc_wait(unsigned long long* bar, uint32_t* ph) {
    const bool ok = mbar_wait(bar, *ph & 1);
    *ph += 1;
    return ok;
}

// issue the bulk copies of K step kb of tile (mt, nt) into stage kb & 1
__device__ __forceinline__ void tc_issue(TcState* ts, unsigned char* stage, const unsigned char* scA,
                                         const unsigned char* scB, int mt, int nt, int nk, int kb,
                                         int* issued) {
    issued[kb & 1] += 1;
    unsigned char* st = stage + (kb & 1) * DQMC_TC_STAGE;
    mbar_expect_tx(&ts->full[kb & 1], DQMC_TC_STAGE);
    bulk_g2s(st, scA + ((size_t)mt * nk + kb) * DQMC_TC_ASTEP, DQMC_TC_ASTEP, &ts->full[kb & 1]);
    bulk_g2s(st + DQMC_TC_ASTEP, scB + ((size_t)nt * nk + kb) * DQMC_TC_BSTEP, DQMC_TC_BSTEP,
             &ts->full[kb & 1]);
}

// C = op(A) * op(B) on the tensor cores (see the top of this file).
// ADF / BDF: operand is double-float (float2), else FP64; TA / TB: read
// transposed; CDF: write C as double-float, else FP64.  stage:
// DQMC_TC_SMEM bytes of shared memory (16-byte aligned); ts: the CTA's
// TcState (TMEM allocated, DQMC_TC_COLS columns; barriers initialised);
// scratch: dqmc_tc_scratch_bytes(n) bytes of global memory (16-byte
// aligned).  All threads of the CTA call it.  Returns false when a wait timed
// out (C is then incomplete).
template <bool ADF, bool BDF, bool CDF, bool TA = false, bool TB = false>
__device__ __noinline__ bool mm_tc(int n, void* __restrict__ Cv, const void* __restrict__ Av,
                                   const void* __restrict__ Bv, unsigned char* stage,
                                   TcState* ts, unsigned char* scratch) {
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (ts->status) return false;
    int* exA = reinterpret_cast<int*>(stage + 2 * DQMC_TC_STAGE);
    int* exB = exA + DQMC_TC_NMAX;
    unsigned char* scA = scratch;
    unsigned char* scB = scratch + dqmc_tc_scratch_a(n);
    // (1) exponents, then the slices of op(A) (its rows) and of op(B) (its
    // columns: the rows of op(B)^T, read with the transpose flipped)
    row_exponents<ADF, TA>(Av, n, exA);
    row_exponents<BDF, !TB>(Bv, n, exB);
    __syncthreads();
    split_all<ADF, TA>(Av, n, DQMC_TC_TM, exA, scA);
    split_all<BDF, !TB>(Bv, n, DQMC_TC_TN, exB, scB);
    fence_proxy_async_global();
    __syncthreads();
    const uint32_t idesc = tc_idesc_bf16(DQMC_TC_TM, DQMC_TC_TN);
    const uint32_t tmem = ts->tmem;
    const int nk = (n + DQMC_TC_KB - 1) / DQMC_TC_KB;
    const int nmt = (n + DQMC_TC_TM - 1) / DQMC_TC_TM, nnt = (n + DQMC_TC_TN - 1) / DQMC_TC_TN;
    for (int mt = 0; mt < nmt; ++mt) {
        for (int nt = 0; nt < nnt; ++nt) {
            // (2) one thread: bulk copies two steps ahead of the MMAs
            if (tid == 0) {
                bool ok = true;
                int issued[2] = {0, 0}, landed[2] = {0, 0};  // bulk copies per stage
                tc_issue(ts, stage, scA, scB, mt, nt, nk, 0, issued);
                if (nk > 1) tc_issue(ts, stage, scA, scB, mt, nt, nk, 1, issued);
                int waited = 0;  // MMA commits waited for
                for (int kb = 0; kb < nk && ok; ++kb) {
                    const int sb = kb & 1;
                    ok = tc_wait(&ts->full[sb], &ts->ph_full[sb]);
                    landed[sb] += 1;
                    if (!ok) break;
                    tc_fence_after();
                    const uint32_t sa = smem_u32(stage + sb * DQMC_TC_STAGE);
                    const uint32_t sbb = sa + DQMC_TC_ASTEP;
#pragma unroll
                    for (int i = 0; i < DQMC_TC_S; ++i) {
#pragma unroll
                        for (int j = 0; j < DQMC_TC_S; ++j) {
                            if (i + j >= DQMC_TC_S) continue;
                            const int acc = i + j < 4 ? i + j : 4;
                            // the first product into an accumulator overwrites it
                            const bool first = kb == 0 && i == 0 && (acc < 4 || j == 4);
                            tc_mma(tmem + (uint32_t)(acc * DQMC_TC_TN),
                                   tc_sdesc(sa + i * DQMC_TC_ABLK, DQMC_TC_LBO, DQMC_TC_SBO),
                                   tc_sdesc(sbb + j * DQMC_TC_BBLK, DQMC_TC_LBO, DQMC_TC_SBO),
                                   idesc, first ? 0u : 1u);
                        }
                    }
                    tc_commit(&ts->mma[sb]);
                    if (kb + 2 < nk) {  // this stage is free once its MMAs are done
                        ok = tc_wait(&ts->mma[sb], &ts->ph_mma[sb]);
                        waited = kb + 1;
                        if (ok) tc_issue(ts, stage, scA, scB, mt, nt, nk, kb + 2, issued);
                    }
                }
                // the MMA commits not waited for yet, oldest first (all of
                // them complete before the accumulators are read)
                for (int kb = waited; kb < nk && ok; ++kb)
                    ok = tc_wait(&ts->mma[kb & 1], &ts->ph_mma[kb & 1]);
                if (!ok) {
                    // give the copies still in flight their (bounded) time to
                    // land before the staging memory is used for anything else
                    for (int sb = 0; sb < 2; ++sb)
                        while (landed[sb] < issued[sb]) {
                            tc_wait(&ts->full[sb], &ts->ph_full[sb]);
                            landed[sb] += 1;
                        }
                    ts->status = 1;
                }
            }
            __syncthreads();
            if (ts->status) return false;
            tc_fence_after();
            // (3) epilogue: warp w reads lanes 32 (w % 4) .. + 31 (tile rows),
            // columns 24 (w / 4) .. + 23, eight at a time
            {
                const int row = mt * DQMC_TC_TM + 32 * (warp & 3) + lane;
                const uint32_t lane_addr = (uint32_t)(32 * (warp & 3)) << 16;
                const int er = row < n ? exA[row] : 0;
#pragma unroll 1
                for (int g8 = 0; g8 < 3; ++g8) {
                    const int c0 = 24 * (warp >> 2) + 8 * g8;
                    float h[8], l[8], v[8];
                    tc_ld8(tmem + lane_addr + (uint32_t)(4 * DQMC_TC_TN + c0), v);
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        h[q] = v[q];
                        l[q] = 0.0f;
                    }
#pragma unroll 1
                    for (int a = 3; a >= 0; --a) {
                        tc_ld8(tmem + lane_addr + (uint32_t)(a * DQMC_TC_TN + c0), v);
#pragma unroll
                        for (int q = 0; q < 8; ++q) df_acc(h[q], l[q], v[q]);
                    }
                    if (row < n) {
#pragma unroll
                        for (int q = 0; q < 8; ++q) {
                            const int col = nt * DQMC_TC_TN + c0 + q;
                            if (col < n) {
                                const float sc = pow2f(er + exB[col] - 14);
                                // renormalise and scale (powers of two: exact)
                                const float hh = __fadd_rn(h[q], l[q]);
                                const float ll = __fadd_rn(__fsub_rn(h[q], hh), l[q]);
                                const size_t at = (size_t)row + (size_t)col * n;
                                if (CDF)
                                    static_cast<float2*>(Cv)[at] =
                                        make_float2(__fmul_rn(hh, sc), __fmul_rn(ll, sc));
                                else
                                    static_cast<double*>(Cv)[at] =
                                        (double)__fmul_rn(hh, sc) + (double)__fmul_rn(ll, sc);
                            }
                        }
                    }
                }
            }
            tc_fence_before();
            __syncthreads();
        }
    }
    return true;
}

}  // namespace
}  // namespace dqmc
