// Tensor-core (tcgen05) products with FP64-class accuracy for the mixed path.
//
// C = op(A) * op(B) for n x n matrices (n <= 256), computed on the 5th-gen
// tensor cores by splitting both operands into BF16 digit slices (the
// error-free splitting of Ozaki et al., "Error-free transformations of
// matrix multiplication by using fast routines of matrix multiplication and
// its applications", Numer. Algorithms 59 (2012)):
//
//   row r of A is scaled by 2^-e_r (max_k |A[r,k]| < 2^e_r) and written as
//   A[r,k] = 2^(e_r - 7) * sum_i s_i 2^(-8i),  s_i integers, |s_i| <= 128,
//
// i = 0..5 (47 bits of the row's scale); columns of B likewise with 2^f_c.
// A BF16 holds every s_i 2^(-8i) exactly (8 significant bits).  Every slice
// product A_i B_j is an integer sum of at most K terms of magnitude <= 2^14 in
// units of 2^(-8(i+j)); for K <= 256 the FP32 accumulator of tcgen05.mma
// (kind::f16, BF16 inputs) holds sums of up to four such products exactly
// (4 * 2^22 = 2^24).  Levels l = i + j = 0, 1, 2 (1, 2, 3 products) are
// therefore accumulated exactly in three TMEM accumulators, and levels 3..5
// (4 + 5 + 6 products, each 2^8 below the previous) in a fourth, whose
// rounding is below 2^-45 of sum_k |A_rk||B_kc|.  Pairs with i + j > 5 are
// dropped (their sum is below 2^-47 of the same bound).  The epilogue adds
// the four accumulators in double-float arithmetic and scales by
// 2^(e_r + f_c - 14): about 46 correct bits, the accuracy class of the
// double-float products on the FP32 pipe (mm_dfx) that this replaces, at a
// fraction of their issue cost.
//
// Mapping: one CTA (256 threads) computes C tile by tile, 128 rows x 64
// columns per tile (M = 128, N = 64 MMAs, one thread issues), K staged 16 at
// a time: for each K step the CTA splits the 128 x 16 block of A and the
// 64 x 16 block of B into their six slices in shared memory (the no-swizzle
// K-major canonical layout: 8 x 8 core matrices, 16-byte rows), one elected
// thread issues the 21 slice-pair MMAs into the four accumulators (4 x 64
// TMEM columns) and commits them to an mbarrier; two stages alternate, so the
// split of step k + 1 overlaps the MMAs of step k.  The accumulators are read
// back with tcgen05.ld (warp w reads TMEM lanes 32 (w % 4) .. + 31).  No FP64
// instruction is issued: FP64 operands are split from their bit patterns.
//
// Every wait on an mbarrier is bounded (DQMC_TC_SPIN_NS); on timeout the
// caller's status flag is set and the product is abandoned.
#pragma once
#include <stdint.h>

#include "dqmc_device.cuh"

#define DQMC_TC_NMAX 256          // largest n (K <= 256 keeps the level sums exact)
#define DQMC_TC_TM 128            // rows per tile (MMA M)
#define DQMC_TC_TN 64             // columns per tile (MMA N)
#define DQMC_TC_KB 16             // K per stage (one MMA K step for 16-bit inputs)
#define DQMC_TC_S 6               // digit slices per operand
#define DQMC_TC_COLS 256          // TMEM columns a CTA allocates (4 accumulators x 64)
#define DQMC_TC_SPIN_NS 2000000000ull  // give up on an mbarrier after 2 s
// bytes of one slice block: rows x 16 BF16 = rows * 32 bytes
#define DQMC_TC_ABYTES (DQMC_TC_TM * DQMC_TC_KB * 2)
#define DQMC_TC_BBYTES (DQMC_TC_TN * DQMC_TC_KB * 2)
#define DQMC_TC_STAGE (DQMC_TC_S * (DQMC_TC_ABYTES + DQMC_TC_BBYTES))
// shared memory of mm_tc: 2 stages + 2 n exponents (ints)
#define DQMC_TC_SMEM (2 * DQMC_TC_STAGE + 2 * DQMC_TC_NMAX * 4)

namespace dqmc {
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
// generic-proxy writes to shared memory visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ---- mbarrier ------------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}
// wait for the phase with parity `parity` to complete; false after the time limit
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
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
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(bar))
        : "memory");
}
// 16 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
        "%11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = __uint_as_float(r[q]);
}

// ---- splitting -----------------------------------------------------------------
// 2^e as a float (e in [-126, 127])
__device__ __forceinline__ float pow2f(int e) {
    e = e < -126 ? -126 : (e > 127 ? 127 : e);
    return __int_as_float((e + 127) << 23);
}
// exponent e with |v| < 2^e for the largest |v| (v >= 0 given as its bits'
// magnitude); 0 for v = 0
__device__ __forceinline__ int exp_above(double v) {
    if (!(v > 0.0)) return 0;
    const int E = (int)((__double_as_longlong(v) >> 52) & 0x7ff);
    return E - 1022;  // v = 1.m 2^(E-1023) < 2^(E-1022)
}
__device__ __forceinline__ int exp_above_f(float v) {
    if (!(v > 0.0f)) return 0;
    const int E = (int)((__float_as_uint(v) >> 23) & 0xff);
    return E - 126;
}

// (th, tl) = x * 2^(7 - e) as an unevaluated float pair, from the bits of
// the FP64 x (|x| < 2^e): th carries the top 24 significand bits, tl the
// next ~24 (rounded).  No FP64 instruction.
__device__ __forceinline__ void scaled_pair_d(double x, int e, float& th, float& tl) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
    const int E = (int)((hi >> 20) & 0x7ff);
    const int q = E - 1023 + 7 - e;  // t = 1.m 2^q, q <= 6
    if (E == 0 || q < -48) {  // |t| < 2^-47: below the last digit
        th = 0.0f;
        tl = 0.0f;
        return;
    }
    const uint32_t sign = hi & 0x80000000u;
    const uint32_t top23 = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    th = __uint_as_float(sign | ((uint32_t)(q + 127) << 23) | top23);
    const uint32_t r29 = lo & 0x1FFFFFFFu;
    float t = __uint2float_rn(r29) * pow2f(q - 52);
    tl = sign ? -t : t;
}

// The six digits s_i 2^(-8i) of t = th + tl (|t| < 2^7), round to nearest:
// s_0 = rint(th), then each digit from the exact remainder times 2^8; tl
// enters at digit 3, where the remainder of th has few bits left.
__device__ __forceinline__ void digits6(float th, float tl, float* d) {
    float s = rintf(th);
    float r = __fsub_rn(th, s);
    d[0] = s;
    r = __fmul_rn(r, 256.0f);
    s = rintf(r);
    r = __fsub_rn(r, s);
    d[1] = s * 0x1p-8f;
    r = __fmul_rn(r, 256.0f);
    s = rintf(r);
    r = __fsub_rn(r, s);
    d[2] = s * 0x1p-16f;
    r = __fmaf_rn(r, 256.0f, __fmul_rn(tl, 16777216.0f));
    s = rintf(r);
    r = __fsub_rn(r, s);
    d[3] = s * 0x1p-24f;
    r = __fmul_rn(r, 256.0f);
    s = rintf(r);
    r = __fsub_rn(r, s);
    d[4] = s * 0x1p-32f;
    r = __fmul_rn(r, 256.0f);
    s = rintf(r);
    d[5] = s * 0x1p-40f;
}

// BF16 bits of a float that has at most 8 significant bits (exact)
__device__ __forceinline__ uint32_t bf16_bits(float v) { return __float_as_uint(v) >> 16; }

// byte offset of element (row, k) (k in 0..15) inside a slice block in the
// no-swizzle K-major canonical layout: core matrix (row / 8, k / 8) of 8 rows
// x 16 bytes; K-adjacent core matrices 128 bytes apart, row groups 256 apart
__device__ __forceinline__ uint32_t tc_off(int row, int k) {
    return (uint32_t)((row >> 3) * 256 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}
#ifndef DQMC_TC_LBO
#define DQMC_TC_LBO 128u
#endif
#ifndef DQMC_TC_SBO
#define DQMC_TC_SBO 256u
#endif

// Operand access: element (r, k) of op(X) with X column-major n x n, FP64
// (split from its bits) or double-float (float2, already a pair).
template <bool DF, bool T>
__device__ __forceinline__ void load_pair(const void* X, int n, int r, int k, int e, float& th,
                                          float& tl) {
    const size_t at = T ? (size_t)k + (size_t)r * n : (size_t)r + (size_t)k * n;
    if (DF) {
        const float2 v = static_cast<const float2*>(X)[at];
        const float p = pow2f(7 - e);
        th = __fmul_rn(v.x, p);
        tl = __fmul_rn(v.y, p);
    } else {
        scaled_pair_d(static_cast<const double*>(X)[at], e, th, tl);
    }
}
template <bool DF, bool T>
__device__ __forceinline__ float absmax_elem(const void* X, int n, int r, int k) {
    const size_t at = T ? (size_t)k + (size_t)r * n : (size_t)r + (size_t)k * n;
    if (DF) return fabsf(static_cast<const float2*>(X)[at].x);
    // a float power of two that has the exponent bound of the FP64 value
    const unsigned long long b =
        (unsigned long long)__double_as_longlong(static_cast<const double*>(X)[at]);
    const int E = (int)((b >> 52) & 0x7ff);
    if (E == 0) return 0.0f;
    // 2^(E-1023) * 1.999.. < 2^(E-1022): report the upper power directly
    const int e = E - 1022;
    return e > 127 ? __int_as_float(0x7f000000) : (e < -125 ? 0.0f : pow2f(e - 1));
}

// Split rows [r0, r0 + rows) x k-block [k0, k0 + 16) of op(X) into the six
// slice blocks at `dst` (slice i at dst + i * blockbytes); rows / ks beyond n
// are zero.  `ex[r]`: the row's exponent.
template <bool DF, bool T>
__device__ __forceinline__ void split_block(const void* X, int n, int r0, int rows, int k0,
                                            const int* ex, unsigned char* dst,
                                            uint32_t blockbytes) {
    // each thread handles pairs of adjacent k (one 32-bit word of two BF16)
    const int words = rows * (DQMC_TC_KB / 2);
    for (int w = threadIdx.x; w < words; w += DQMC_NT) {
        const int row = T ? w / (DQMC_TC_KB / 2) : w % rows;
        const int kk = 2 * (T ? w % (DQMC_TC_KB / 2) : w / rows);
        const int r = r0 + row;
        float d0[DQMC_TC_S], d1[DQMC_TC_S];
        if (r < n) {
            const int e = ex[r];
            float th, tl;
            if (k0 + kk < n) {
                load_pair<DF, T>(X, n, r, k0 + kk, e, th, tl);
                digits6(th, tl, d0);
            } else {
#pragma unroll
                for (int i = 0; i < DQMC_TC_S; ++i) d0[i] = 0.0f;
            }
            if (k0 + kk + 1 < n) {
                load_pair<DF, T>(X, n, r, k0 + kk + 1, e, th, tl);
                digits6(th, tl, d1);
            } else {
#pragma unroll
                for (int i = 0; i < DQMC_TC_S; ++i) d1[i] = 0.0f;
            }
        } else {
#pragma unroll
            for (int i = 0; i < DQMC_TC_S; ++i) d0[i] = d1[i] = 0.0f;
        }
        const uint32_t off = tc_off(row, kk);
#pragma unroll
        for (int i = 0; i < DQMC_TC_S; ++i)
            *reinterpret_cast<uint32_t*>(dst + (size_t)i * blockbytes + off) =
                bf16_bits(d0[i]) | (bf16_bits(d1[i]) << 16);
    }
}

// double-float a + b for floats (TwoSum) added into (h, l)
__device__ __forceinline__ void df_acc(float& h, float& l, float v) {
    const float s = __fadd_rn(h, v);
    const float z = __fsub_rn(s, h);
    const float e = __fadd_rn(__fsub_rn(h, __fsub_rn(s, z)), __fsub_rn(v, z));
    h = s;
    l = __fadd_rn(l, e);
}

}  // namespace

// Shared state of mm_tc in one CTA: TMEM base, one mbarrier per staging
// buffer (each tracks the MMAs that read it; at most one commit outstanding,
// so parity waits are unambiguous) with its completed-phase count, and a
// status word (nonzero: a wait timed out).
struct __align__(16) TcState {
    uint32_t tmem;
    uint32_t status;
    uint32_t phase[2];
    uint64_t bar[2];
};

namespace {

// wait for the oldest outstanding commit on buffer b's barrier
__device__ __forceinline__ bool tc_wait(TcState* ts, int b) {
    const bool ok = mbar_wait(&ts->bar[b], ts->phase[b] & 1);
    ts->phase[b] += 1;
    return ok;
}

// C = op(A) * op(B) on the tensor cores (see the top of this file).
// ADF / BDF: operand is double-float (float2), else FP64; TA / TB: read
// transposed (FP64 operands only); CDF: write C as double-float, else FP64.
// stage: DQMC_TC_SMEM bytes of shared memory (16-byte aligned); ts: the CTA's
// TcState (TMEM allocated, DQMC_TC_COLS columns; barrier initialised).
// All threads of the CTA call it.  Returns false when a wait timed out.
template <bool ADF, bool BDF, bool CDF, bool TA = false, bool TB = false>
__device__ __noinline__ bool mm_tc(int n, void* __restrict__ Cv, const void* __restrict__ Av,
                                   const void* __restrict__ Bv, unsigned char* stage,
                                   TcState* ts) {
    static_assert(!(ADF && TA) && !(BDF && TB), "split operands are read untransposed");
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    int* exA = reinterpret_cast<int*>(stage + 2 * DQMC_TC_STAGE);
    int* exB = exA + DQMC_TC_NMAX;
    // row exponents of op(A), column exponents of op(B)
    for (int r = tid; r < n; r += DQMC_NT) {
        float m = 0.0f;
        for (int k = 0; k < n; ++k) m = fmaxf(m, absmax_elem<ADF, TA>(Av, n, r, k));
        exA[r] = exp_above_f(m);
        float mb = 0.0f;
        for (int k = 0; k < n; ++k) mb = fmaxf(mb, absmax_elem<BDF, !TB>(Bv, n, r, k));
        exB[r] = exp_above_f(mb);
    }
    __syncthreads();
    const uint32_t idesc = tc_idesc_bf16(DQMC_TC_TM, DQMC_TC_TN);
    const uint32_t tmem = ts->tmem;
    const int nk = (n + DQMC_TC_KB - 1) / DQMC_TC_KB;
    for (int m0 = 0; m0 < n; m0 += DQMC_TC_TM) {
        for (int n0 = 0; n0 < n; n0 += DQMC_TC_TN) {
            for (int kb = 0; kb < nk; ++kb) {
                const int sidx = kb & 1;
                unsigned char* st = stage + sidx * DQMC_TC_STAGE;
                // the MMAs of two steps back read this buffer: wait for them
                if (kb >= 2) {
                    if (tid == 0 && !tc_wait(ts, sidx)) ts->status = 1;
                    __syncthreads();
                    if (ts->status) return false;
                }
                split_block<ADF, TA>(Av, n, m0, DQMC_TC_TM, kb * DQMC_TC_KB, exA, st,
                                     DQMC_TC_ABYTES);
                // op(B) is K x N; its slice block is N rows x K: row = column c
                split_block<BDF, !TB>(Bv, n, n0, DQMC_TC_TN, kb * DQMC_TC_KB, exB,
                                      st + DQMC_TC_S * DQMC_TC_ABYTES, DQMC_TC_BBYTES);
                fence_proxy_async_smem();
                __syncthreads();
                if (tid == 0) {
                    tc_fence_after();
                    const uint32_t sa = smem_u32(st);
                    const uint32_t sb = sa + DQMC_TC_S * DQMC_TC_ABYTES;
#pragma unroll
                    for (int i = 0; i < DQMC_TC_S; ++i) {
#pragma unroll
                        for (int j = 0; j < DQMC_TC_S; ++j) {
                            if (i + j >= DQMC_TC_S) continue;
                            const int lvl = i + j < 3 ? i + j : 3;
                            // the first product into an accumulator in this tile
                            // overwrites it
                            const bool first = kb == 0 && (lvl < 3 ? i == 0 : (i == 0 && j == 3));
                            tc_mma(tmem + (uint32_t)(lvl * DQMC_TC_TN),
                                   tc_sdesc(sa + i * DQMC_TC_ABYTES, DQMC_TC_LBO, DQMC_TC_SBO),
                                   tc_sdesc(sb + j * DQMC_TC_BBYTES, DQMC_TC_LBO, DQMC_TC_SBO),
                                   idesc, first ? 0u : 1u);
                        }
                    }
                    tc_commit(&ts->bar[sidx]);
                }
            }
            // the tile's outstanding commits (the last two steps), in order
            if (tid == 0) {
                bool w = true;
                if (nk >= 2) w = tc_wait(ts, (nk - 2) & 1);
                if (w) w = tc_wait(ts, (nk - 1) & 1);
                if (!w) ts->status = 1;
            }
            __syncthreads();
            if (ts->status) return false;
            tc_fence_after();
            // epilogue: warp w reads lanes 32 (w % 4) .. + 31 (tile rows),
            // columns 32 (w / 4) .. + 31
            {
                const int row = m0 + 32 * (warp & 3) + lane;
                const int cb = 32 * (warp >> 2);
                const uint32_t lane_addr = (uint32_t)(32 * (warp & 3)) << 16;
#pragma unroll 1
                for (int half = 0; half < 2; ++half) {
                    const int c0 = cb + 16 * half;
                    float h[16], l[16], v[16];
                    tc_ld16(tmem + lane_addr + (uint32_t)(3 * DQMC_TC_TN + c0), v);
#pragma unroll
                    for (int q = 0; q < 16; ++q) {
                        h[q] = v[q];
                        l[q] = 0.0f;
                    }
#pragma unroll 1
                    for (int a = 2; a >= 0; --a) {
                        tc_ld16(tmem + lane_addr + (uint32_t)(a * DQMC_TC_TN + c0), v);
#pragma unroll
                        for (int q = 0; q < 16; ++q) df_acc(h[q], l[q], v[q]);
                    }
                    if (row < n) {
                        const int er = exA[row];
#pragma unroll
                        for (int q = 0; q < 16; ++q) {
                            const int col = n0 + c0 + q;
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
