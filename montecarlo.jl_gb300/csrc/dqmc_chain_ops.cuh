// Chain-level device operations of the DQMC sweep (one CTA = one chain):
// slice matrices, wraps, stack building, UDT stabilisation, Green's function
// reconstruction, propagate and the local sweep.  Included by the kernel
// translation units; every function is executed by all threads of a CTA.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "dqmc_device.cuh"

namespace dqmc {
namespace {  // internal linkage: each translation unit gets its own copy

struct Smem {
    union {                      // never live at the same time
        double tiles[2 * 16 * 64];  // mm() / mm_df() staging
        struct {
            double col[2][DQMC_NMAX];  // rank-1: (I - G)[:, i] per block
            double row[2][DQMC_NMAX];  // rank-1: (Delta/R) G[i, :] per block
        } r1;
    };
    double sv[DQMC_NMAX];        // column norms / small vectors
    double ev[2 * DQMC_NMAX];    // interaction exponential of the current slice
    double sxd[4];
    double red[DQMC_NW];
    int sxi[4];
    DqmcChain c;                 // this CTA's chain (state mutated here, written back at exit)
    double arena[2 * 64 * 65];   // shared-memory QR of one block when n <= 64; between
                                 // stabilisations of a sweep it holds G (G-resident mode)
    double* Gglob;               // the chain's G in global memory
    int gres;                    // G currently lives in `arena`
};

struct Ctx {
    Smem* s;
    DqmcChain* c;  // == &s->c
    int n, nf;
    size_t nn;
};

__device__ __forceinline__ double* blk(double* p, const Ctx& x, int b) { return p + (size_t)b * x.nn; }

// G-resident mode (n <= 64): during sweeps G stays in shared memory for the
// rank-1 updates and wraps, and moves to global memory while a stabilisation
// needs the arena for its QR factorisations.
__device__ __forceinline__ bool g_resident_possible(const Ctx& x) {
    return x.n <= 64 && (size_t)x.nf * x.nn <= sizeof(x.s->arena) / sizeof(double);
}
__device__ void g_to_arena(const Ctx& x) {
    __syncthreads();
    for (int e = threadIdx.x; e < x.nf * (int)x.nn; e += DQMC_NT) x.s->arena[e] = x.s->Gglob[e];
    __syncthreads();
    if (threadIdx.x == 0) { x.c->G = x.s->arena; x.s->gres = 1; }
    __syncthreads();
}
__device__ void g_to_global(const Ctx& x) {
    __syncthreads();
    for (int e = threadIdx.x; e < x.nf * (int)x.nn; e += DQMC_NT) x.s->Gglob[e] = x.s->arena[e];
    __syncthreads();
    if (threadIdx.x == 0) { x.c->G = x.s->Gglob; x.s->gres = 0; }
    __syncthreads();
}

// UDT of one flavour block: in shared memory for n <= 64, else from global memory
__device__ __forceinline__ void udt_one(const Ctx& x, double* U, double* D, double* In, int b,
                                        bool apply) {
    if (x.n <= 64)
        udt_pivot_sm(x.n, U, D, In, x.c->pivot + b * x.n, x.c->tempv + b * x.n, apply,
                     x.s->arena, x.s->arena + x.n * (x.n + 1), x.s->sv, x.s->sxd);
    else
        udt_pivot(x.n, U, D, In, x.c->pivot + b * x.n, x.c->tempv + b * x.n, apply,
                  blk(x.c->out, x, b), x.s->sv, x.s->sxd, x.s->sxi);
}


// nanoseconds of the GPU-wide timer (comparable across SMs)
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// phase timers: thread 0 accumulates SM cycles per DQMC_PHASE_*
__device__ __forceinline__ long long phase_start() { return threadIdx.x == 0 ? clock64() : 0; }
__device__ __forceinline__ void phase_stop(const Ctx& x, int phase, long long t0) {
    if (threadIdx.x == 0) x.c->timers[phase] += (unsigned long long)(clock64() - t0);
}

// Slice-matrix products (wraps and slice chains): FP64, or on a
// mixed-precision chain the double-float product on the FP32 pipe.  The UDT,
// the Green's reconstruction, the T updates, the determinant ratios and the
// rank-1 updates stay FP64 on every chain.
template <bool TA, bool TB>
__device__ __forceinline__ void smm(const Ctx& x, bool wrap, double* C, const double* A,
                                    const double* B) {
    (void)wrap;
    if (x.c->prec == DQMC_PREC_MIXED_ID)
        mm_df<TA, TB>(x.n, C, A, B, x.s->tiles);
    else
        mm<TA, TB>(x.n, C, A, B, x.s->tiles);
}

// interaction_matrix_exp! (fields.jl:380-386, 429-438, 548-560, 618-624)
// into shared memory: ev[b*n + i]
__device__ __noinline__ void interaction_exp(const Ctx& x, int slice, bool inverse) {
    const DqmcChain& c = *x.c;
    const int8_t* s = c.conf + (size_t)(slice - 1) * x.n;
    const bool ghq = (c.kind >= 2);
    for (int e = threadIdx.x; e < x.nf * x.n; e += DQMC_NT) {
        int b = e / x.n, i = e % x.n;
        int v = ghq ? (int)s[i] - 1 : (s[i] > 0 ? 1 : 0);
        x.s->ev[e] = inverse ? c.evinv[b][v] : c.ev[b][v];
    }
    __syncthreads();
}

// multiply_slice_matrix_left!: M <- eT2 * eV * M  (stack.jl:319-327)
__device__ __noinline__ void slice_left(const Ctx& x, int slice, double* M, bool wrap = false) {
    interaction_exp(x, slice, false);
    for (int b = 0; b < x.nf; ++b) {
        dleft(x.n, blk(x.c->tmp1, x, b), x.s->ev + b * x.n, blk(M, x, b));
        __syncthreads();
        smm<true, false>(x, wrap, blk(M, x, b), x.c->eT2, blk(x.c->tmp1, x, b));
        __syncthreads();
    }
}
// multiply_slice_matrix_right!: M <- M * eT2 * eV  (stack.jl:329-337)
__device__ __noinline__ void slice_right(const Ctx& x, int slice, double* M, bool wrap = false) {
    interaction_exp(x, slice, false);
    for (int b = 0; b < x.nf; ++b) {
        smm<false, true>(x, wrap, blk(x.c->tmp1, x, b), blk(M, x, b), x.c->eT2);
        __syncthreads();
        dright(x.n, blk(M, x, b), blk(x.c->tmp1, x, b), x.s->ev + b * x.n);
        __syncthreads();
    }
}
// multiply_slice_matrix_inv_right!: M <- M * eV^-1 * eT2^-1  (stack.jl:339-347)
__device__ __noinline__ void slice_inv_right(const Ctx& x, int slice, double* M, bool wrap = false) {
    interaction_exp(x, slice, true);
    for (int b = 0; b < x.nf; ++b) {
        dright(x.n, blk(x.c->tmp1, x, b), blk(M, x, b), x.s->ev + b * x.n);
        __syncthreads();
        smm<false, true>(x, wrap, blk(M, x, b), blk(x.c->tmp1, x, b), x.c->eT2inv);
        __syncthreads();
    }
}
// multiply_slice_matrix_inv_left!: M <- eV^-1 * eT2^-1 * M  (stack.jl:349-357)
__device__ __noinline__ void slice_inv_left(const Ctx& x, int slice, double* M, bool wrap = false) {
    interaction_exp(x, slice, true);
    for (int b = 0; b < x.nf; ++b) {
        smm<true, false>(x, wrap, blk(x.c->tmp1, x, b), x.c->eT2inv, blk(M, x, b));
        __syncthreads();
        dleft(x.n, blk(M, x, b), x.s->ev + b * x.n, blk(x.c->tmp1, x, b));
        __syncthreads();
    }
}
// multiply_daggered_slice_matrix_left!: M <- eV * eT2 * M (stack.jl:359-367)
__device__ __noinline__ void slice_dagger_left(const Ctx& x, int slice, double* M) {
    interaction_exp(x, slice, false);
    for (int b = 0; b < x.nf; ++b) {
        smm<true, false>(x, false, blk(x.c->tmp1, x, b), x.c->eT2, blk(M, x, b));
        __syncthreads();
        dleft(x.n, blk(M, x, b), x.s->ev + b * x.n, blk(x.c->tmp1, x, b));
        __syncthreads();
    }
}

// wrap_greens! (stack.jl:594-603)
__device__ void wrap_greens(const Ctx& x, double* gf, int curr_slice, int direction) {
    if (direction == -1) {
        slice_inv_left(x, curr_slice - 1, gf, true);
        slice_right(x, curr_slice - 1, gf, true);
    } else {
        slice_left(x, curr_slice, gf, true);
        slice_inv_right(x, curr_slice, gf, true);
    }
}

__device__ __forceinline__ double* ustk(const Ctx& x, int idx) {
    return x.c->ustack + (size_t)(idx - 1) * x.nf * x.nn;
}
__device__ __forceinline__ double* tstk(const Ctx& x, int idx) {
    return x.c->tstack + (size_t)(idx - 1) * x.nf * x.nn;
}
__device__ __forceinline__ double* dstk(const Ctx& x, int idx) {
    return x.c->dstack + (size_t)(idx - 1) * x.nf * x.n;
}

__device__ void mat_ident(const Ctx& x, double* A) {
    for (int b = 0; b < x.nf; ++b) ident(x.n, blk(A, x, b));
}

__device__ __noinline__ void udt_blocks(const Ctx& x, double* U, double* D, double* In, bool apply) {
    for (int b = 0; b < x.nf; ++b) udt_one(x, blk(U, x, b), D + b * x.n, blk(In, x, b), b, apply);
}
__device__ __noinline__ void mm_blocks(const Ctx& x, double* C, double* A, double* B) {
    for (int b = 0; b < x.nf; ++b) {
        mm<false, false>(x.n, blk(C, x, b), blk(A, x, b), blk(B, x, b), x.s->tiles);
    }
    __syncthreads();
}
__device__ void dright_blocks(const Ctx& x, double* C, double* A, const double* d) {
    for (int b = 0; b < x.nf; ++b) dright(x.n, blk(C, x, b), blk(A, x, b), d + b * x.n);
    __syncthreads();
}

// add_slice_sequence_left (stack.jl:377-393)
__device__ __noinline__ void add_slice_sequence_left(const Ctx& x, int idx) {
    DqmcChain& c = *x.c;
    copy(x.nf * (int)x.nn, c.currU, ustk(x, idx));
    __syncthreads();
    long long t0 = phase_start();
    for (int s = c.rfirst[idx - 1]; s <= c.rlast[idx - 1]; ++s) slice_left(x, s, c.currU);
    dright_blocks(x, c.tmp1, c.currU, dstk(x, idx));
    phase_stop(x, DQMC_PHASE_SLICE_CHAIN, t0);
    t0 = phase_start();
    udt_blocks(x, ustk(x, idx + 1), dstk(x, idx + 1), c.tmp1, true);
    phase_stop(x, DQMC_PHASE_UDT, t0);
    t0 = phase_start();
    mm_blocks(x, tstk(x, idx + 1), c.tmp1, tstk(x, idx));
    phase_stop(x, DQMC_PHASE_T_UPDATE, t0);
}
// add_slice_sequence_right (stack.jl:402-416)
__device__ __noinline__ void add_slice_sequence_right(const Ctx& x, int idx) {
    DqmcChain& c = *x.c;
    copy(x.nf * (int)x.nn, c.currU, ustk(x, idx + 1));
    __syncthreads();
    long long t0 = phase_start();
    for (int s = c.rlast[idx - 1]; s >= c.rfirst[idx - 1]; --s) slice_dagger_left(x, s, c.currU);
    dright_blocks(x, c.tmp1, c.currU, dstk(x, idx + 1));
    phase_stop(x, DQMC_PHASE_SLICE_CHAIN, t0);
    t0 = phase_start();
    udt_blocks(x, ustk(x, idx), dstk(x, idx), c.tmp1, true);
    phase_stop(x, DQMC_PHASE_UDT, t0);
    t0 = phase_start();
    mm_blocks(x, tstk(x, idx), c.tmp1, tstk(x, idx + 1));
    phase_stop(x, DQMC_PHASE_T_UPDATE, t0);
}

// calculate_greens_AVX! (stack.jl:442-496), per flavour block
__device__ __noinline__ void calculate_greens(const Ctx& x, double* Gout) {
    DqmcChain& c = *x.c;
    const int n = x.n;
    const bool bf = x.nf > 1;
    for (int b = 0; b < x.nf; ++b) {
        double *ul = blk(c.Ul, x, b), *tl = blk(c.Tl, x, b), *ur = blk(c.Ur, x, b),
               *tr = blk(c.Tr, x, b), *g = blk(Gout, x, b);
        double *dl = c.Dl + b * n, *dr = c.Dr + b * n;
        int* pv = c.pivot + b * n;
        double* tv = c.tempv + b * n;
        mm<false, true>(n, g, tl, tr, x.s->tiles);
        __syncthreads();
        dright(n, tr, g, dr);
        __syncthreads();
        dleft(n, g, dl, tr);
        __syncthreads();
        udt_one(x, tr, dr, g, b, false);
        mm<false, false>(n, tl, ul, tr, x.s->tiles);
        __syncthreads();
        rdivp(n, ur, g, ul, pv, bf, x.s->sv);
        mm<true, false>(n, tr, tl, ur, x.s->tiles);
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += DQMC_NT) tr[(size_t)i * n + i] += dr[i];
        __syncthreads();
        udt_one(x, ul, dr, tr, b, false);
        rdivp(n, ur, tr, g, pv, bf, x.s->sv);
        mm<false, false>(n, tr, tl, ul, x.s->tiles);
        for (int i = threadIdx.x; i < n; i += DQMC_NT) dl[i] = 1.0 / dr[i];
        __syncthreads();
        dright(n, ul, ur, dl);
        __syncthreads();
        mm<false, true>(n, g, ul, tr, x.s->tiles);
        __syncthreads();
    }
}

__device__ void set_ones(const Ctx& x, double* d) {
    fill(x.nf * x.n, d, 1.0);
}

// reverse_build_stack (stack.jl:284-308)
__device__ __noinline__ void reverse_build_stack(const Ctx& x) {
    DqmcChain& c = *x.c;
    const int nr = c.nr;
    mat_ident(x, ustk(x, nr + 1));
    set_ones(x, dstk(x, nr + 1));
    mat_ident(x, tstk(x, nr + 1));
    __syncthreads();
    for (int i = nr; i >= 1; --i) add_slice_sequence_right(x, i);
    mat_ident(x, c.Ul);
    set_ones(x, c.Dl);
    mat_ident(x, c.Tl);
    copy(x.nf * (int)x.nn, c.Ur, ustk(x, 1));
    copy(x.nf * x.n, c.Dr, dstk(x, 1));
    copy(x.nf * (int)x.nn, c.Tr, tstk(x, 1));
    __syncthreads();
    calculate_greens(x, c.G);
    if (threadIdx.x == 0) {
        c.current_slice = 0;
        c.current_range = 1;
        c.direction = 1;
    }
    __syncthreads();
}

// build_stack (stack.jl:257-281)
__device__ __noinline__ void build_stack(const Ctx& x) {
    DqmcChain& c = *x.c;
    const int nr = c.nr;
    mat_ident(x, ustk(x, 1));
    set_ones(x, dstk(x, 1));
    mat_ident(x, tstk(x, 1));
    __syncthreads();
    for (int i = 1; i <= nr; ++i) add_slice_sequence_left(x, i);
    copy(x.nf * (int)x.nn, c.Ul, ustk(x, nr + 1));
    copy(x.nf * x.n, c.Dl, dstk(x, nr + 1));
    copy(x.nf * (int)x.nn, c.Tl, tstk(x, nr + 1));
    mat_ident(x, c.Ur);
    set_ones(x, c.Dr);
    mat_ident(x, c.Tr);
    __syncthreads();
    calculate_greens(x, c.G);
    if (threadIdx.x == 0) {
        c.current_slice = c.M + 1;
        c.current_range = nr;
        c.direction = -1;
    }
    __syncthreads();
}

// max |Gtmp - G| (stack.jl:646, 701); NaN propagates
__device__ __noinline__ void record_prop_error(const Ctx& x) {
    DqmcChain& c = *x.c;
    const int cnt = x.nf * (int)x.nn;
    double m = 0.0;
    for (int e = threadIdx.x; e < cnt; e += DQMC_NT) {
        double d = fabs(c.Gtmp[e] - c.G[e]);
        if (d > m || d != d) m = d;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        double om = __shfl_xor_sync(0xffffffffu, m, o);
        if (om > m || om != om) m = om;
    }
    if ((threadIdx.x & 31) == 0) x.s->red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double mx = 0.0;
        for (int w = 0; w < DQMC_NW; ++w) {
            double v = x.s->red[w];
            if (v > mx || v != v) mx = v;
        }
        if (mx > c.prop_err_max || mx != mx) c.prop_err_max = mx;
        // a non-finite Green's function is reported to the host as a
        // numerical error (status 2) instead of propagating silently
        if (mx != mx || mx > 1e300) c.status = 2;
        if (mx > 1e-7) {
            c.n_prop_err += 1;
            if (mx > c.prop_err_reported) c.prop_err_reported = mx;
        }
    }
    __syncthreads();
}

// propagate (stack.jl:605-730); the direction flips at 0 and M+1 recurse once
__device__ __noinline__ void propagate(const Ctx& x) {
    DqmcChain& c = *x.c;
    for (int depth = 0; depth < 2; ++depth) {
        __syncthreads();
        const int dir = c.direction;
        const int cs = c.current_slice + dir;
        const int cr = c.current_range;
        __syncthreads();
        if (threadIdx.x == 0) c.current_slice = cs;
        __syncthreads();
        bool recurse = false;
        if (dir == 1) {
            if (cs == 1) {
                mat_ident(x, ustk(x, 1));
                set_ones(x, dstk(x, 1));
                mat_ident(x, tstk(x, 1));
                __syncthreads();
            } else if (cs - 1 == c.rlast[cr - 1]) {
                const int idx = cr;
                const bool was_res = x.s->gres;
                if (was_res) g_to_global(x);
                copy(x.nf * (int)x.nn, c.Ur, ustk(x, idx + 1));
                copy(x.nf * x.n, c.Dr, dstk(x, idx + 1));
                copy(x.nf * (int)x.nn, c.Tr, tstk(x, idx + 1));
                __syncthreads();
                add_slice_sequence_left(x, idx);
                copy(x.nf * (int)x.nn, c.Ul, ustk(x, idx + 1));
                copy(x.nf * x.n, c.Dl, dstk(x, idx + 1));
                copy(x.nf * (int)x.nn, c.Tl, tstk(x, idx + 1));
                long long t0 = phase_start();
                if (c.check_prop) copy(x.nf * (int)x.nn, c.Gtmp, c.G);
                __syncthreads();
                wrap_greens(x, c.Gtmp, cs - 1, 1);
                phase_stop(x, DQMC_PHASE_PROP_CHECK, t0);
                t0 = phase_start();
                calculate_greens(x, c.G);
                phase_stop(x, DQMC_PHASE_GREENS, t0);
                t0 = phase_start();
                if (c.check_prop) record_prop_error(x);
                phase_stop(x, DQMC_PHASE_PROP_CHECK, t0);
                if (cr == c.nr) {
                    if (threadIdx.x == 0) c.direction = -1;
                    recurse = true;
                } else {
                    if (threadIdx.x == 0) c.current_range = cr + 1;
                }
                if (was_res) g_to_arena(x);
            } else {
                {
                    long long tw = phase_start();
                    wrap_greens(x, c.G, cs - 1, 1);
                    phase_stop(x, DQMC_PHASE_WRAP, tw);
                }
            }
        } else {
            if (cs == c.M) {
                mat_ident(x, ustk(x, c.nr + 1));
                set_ones(x, dstk(x, c.nr + 1));
                mat_ident(x, tstk(x, c.nr + 1));
                __syncthreads();
                {
                    long long tw = phase_start();
                    wrap_greens(x, c.G, cs + 1, -1);
                    phase_stop(x, DQMC_PHASE_WRAP, tw);
                }
            } else if (cs + 1 == c.rfirst[cr - 1]) {
                const int idx = cr;
                const bool was_res = x.s->gres;
                if (was_res) g_to_global(x);
                copy(x.nf * (int)x.nn, c.Ul, ustk(x, idx));
                copy(x.nf * x.n, c.Dl, dstk(x, idx));
                copy(x.nf * (int)x.nn, c.Tl, tstk(x, idx));
                __syncthreads();
                add_slice_sequence_right(x, idx);
                copy(x.nf * (int)x.nn, c.Ur, ustk(x, idx));
                copy(x.nf * x.n, c.Dr, dstk(x, idx));
                copy(x.nf * (int)x.nn, c.Tr, tstk(x, idx));
                long long t0 = phase_start();
                if (c.check_prop) copy(x.nf * (int)x.nn, c.Gtmp, c.G);
                __syncthreads();
                phase_stop(x, DQMC_PHASE_PROP_CHECK, t0);
                t0 = phase_start();
                calculate_greens(x, c.G);
                phase_stop(x, DQMC_PHASE_GREENS, t0);
                t0 = phase_start();
                if (c.check_prop) record_prop_error(x);
                phase_stop(x, DQMC_PHASE_PROP_CHECK, t0);
                if (cr == 1) {
                    if (threadIdx.x == 0) c.direction = 1;
                    recurse = true;
                } else {
                    {
                        long long tw = phase_start();
                        wrap_greens(x, c.G, cs + 1, -1);
                        phase_stop(x, DQMC_PHASE_WRAP, tw);
                    }
                    if (threadIdx.x == 0) c.current_range = cr - 1;
                }
                if (was_res) g_to_arena(x);
            } else {
                {
                    long long tw = phase_start();
                    wrap_greens(x, c.G, cs + 1, -1);
                    phase_stop(x, DQMC_PHASE_WRAP, tw);
                }
            }
        }
        __syncthreads();
        if (!recurse) break;
    }
}

#define DQMC_DELAY 16  // pending rank-1 updates per flush when G is in global memory

// G -= U W for the pending updates (U: n x p columns u_m = (I - G)[:, i_m],
// W: p x n rows w_m = (Delta/R) G[i_m, :], stored column / row contiguous
// with stride n), one flavour block.  Each thread keeps its row's p entries
// of U in registers.
__device__ void flush_delayed(const Ctx& x, int p) {
    const int n = x.n;
    for (int b = 0; b < x.nf; ++b) {
        double* g = x.c->G + (size_t)b * x.nn;
        const double* U = x.c->tmp2 + (size_t)b * x.nn;
        const double* W = x.c->currU + (size_t)b * x.nn;
        for (int k = threadIdx.x & 63; k < n; k += 64) {
            double uk[DQMC_DELAY];
#pragma unroll
            for (int m = 0; m < DQMC_DELAY; ++m) uk[m] = m < p ? U[(size_t)m * n + k] : 0.0;
            for (int l = threadIdx.x >> 6; l < n; l += DQMC_NT / 64) {
                double v = g[k + (size_t)l * n];
#pragma unroll
                for (int m = 0; m < DQMC_DELAY; ++m)
                    if (m < p) v = fma(-uk[m], W[(size_t)m * n + l], v);
                g[k + (size_t)l * n] = v;
            }
        }
    }
    __syncthreads();
}

// sweep_spatial (local_updates.jl:23-60) with propose_local / accept_local!
// (fields.jl:58-84, 176-209, 271-286, 340-344, 388-393, 440-449, 497-503,
// 563-573, 627-637).  Thread 0 makes the sequential decisions with the
// reference's operation order (no contraction), scanning on through rejected
// proposals without a barrier; at an accepted one, warps 1.. apply the rank-1
// update G -= (I - G)[:, i] (Delta/R) G[i, :] per flavour block while warp 0
// applies the same fused multiply-add to a shared-memory copy of G's diagonal
// and thread 0 goes on deciding from it: the next decisions overlap the update
// and read bit-identical diagonal values.
__device__ __noinline__ long long sweep_spatial(const Ctx& x) {
    DqmcChain& c = *x.c;
    const int n = x.n, nf = x.nf;
    const int slice = c.current_slice;
    int8_t* s = c.conf + (size_t)(slice - 1) * n;
    const bool ghq = (c.kind >= 2);
    const bool twoflv = (nf == 2);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    double* diag = x.s->ev;  // [nf * n] mirror of the diagonals (ev is free here)
    for (int e = tid; e < nf * n; e += DQMC_NT) {
        const int b = e / n, k = e % n;
        diag[e] = c.G[(size_t)b * x.nn + (size_t)k * n + k];
    }
    __syncthreads();
    long long acc_count = 0;
    int i = 0, round = 0;
    // G in global memory: delay the rank-1 updates and apply them DQMC_DELAY
    // at a time (one pass over G instead of one per accepted move)
    const bool delayed = !x.s->gres;
    const int kcap = n < DQMC_DELAY ? n : DQMC_DELAY;  // U, W columns fit the n*n scratch
    int pending = 0;
    while (true) {
        if (tid == 0) {
            int j = i;
            for (; j < n; ++j) {
                const double g0 = diag[j];
                const double g1 = twoflv ? diag[n + j] : 0.0;
                int t;
                int xnew = 0;
                double gr = 1.0, gq = 1.0;
                if (ghq) {
                    const int xold = s[j];
                    const uint64_t w = dqmc_philox_word(c.key, c.ctr);
                    c.ctr += 1;
                    const int r = dqmc_word_to_choice3(w);
                    xnew = r + (r + 1 >= xold ? 2 : 1);  // choices[x_old, r+1] (fields.jl:534)
                    t = (xold - 1) * 4 + (xnew - 1);
                    gr = c.gam[xnew - 1];
                    gq = c.gam[xold - 1];
                } else {
                    t = s[j] > 0 ? 1 : 0;
                }
                const double d0 = c.delta0[t], d1 = c.delta1[t];
                const double R0 = __dadd_rn(1.0, __dmul_rn(d0, __dsub_rn(1.0, g0)));
                double detratio;
                double R1 = 0.0;
                if (twoflv) {
                    R1 = __dadd_rn(1.0, __dmul_rn(d1, __dsub_rn(1.0, g1)));
                    detratio = __dmul_rn(R0, R1);
                } else {
                    detratio = __dmul_rn(R0, R0);
                }
                if (ghq) detratio = __ddiv_rn(__dmul_rn(detratio, gr), gq);
                const double p = __dmul_rn(c.wboson[t], detratio);
                if (p < 0.0) c.n_neg_p += 1;
                int accept;
                if (p > 1.0) {
                    accept = 1;
                } else {
                    const uint64_t w = dqmc_philox_word(c.key, c.ctr);
                    c.ctr += 1;
                    accept = dqmc_word_to_uniform(w) < p;
                }
                c.proposals += 1;
                if (accept) {
                    x.s->sxd[0] = __ddiv_rn(d0, R0);
                    x.s->sxd[1] = twoflv ? __ddiv_rn(d1, R1) : 0.0;
                    s[j] = ghq ? (int8_t)xnew : (int8_t)(-s[j]);
                    c.accepted += 1;
                    break;
                }
            }
            // double-buffered slot: thread 0 writes the next round's slot
            // while slow threads may still read this one
            x.s->sxi[2 + (round & 1)] = j;
        }
        __syncthreads();  // also: the previous round's update is complete
        const int j = x.s->sxi[2 + (round & 1)];
        ++round;
        if (j >= n) {
            if (pending > 0) flush_delayed(x, pending);
            break;
        }
        acc_count += 1;
        for (int e = tid; e < nf * n; e += DQMC_NT) {
            const int b = e / n, k = e % n;
            const double* g = c.G + (size_t)b * x.nn;
            double gkj = g[(size_t)j * n + k], gjk = g[(size_t)k * n + j];
            if (delayed) {
                // current G[k, j] and G[j, k] with the pending updates applied
                const double* U = c.tmp2 + (size_t)b * x.nn;
                const double* W = c.currU + (size_t)b * x.nn;
                for (int m = 0; m < pending; ++m) {
                    gkj = fma(-U[(size_t)m * n + k], W[(size_t)m * n + j], gkj);
                    gjk = fma(-U[(size_t)m * n + j], W[(size_t)m * n + k], gjk);
                }
            }
            double ig = -gkj;
            if (k == j) ig += 1.0;
            const double rw = x.s->sxd[b] * gjk;
            x.s->r1.col[b][k] = ig;
            x.s->r1.row[b][k] = rw;
            if (delayed) {
                c.tmp2[(size_t)b * x.nn + (size_t)pending * n + k] = ig;
                c.currU[(size_t)b * x.nn + (size_t)pending * n + k] = rw;
            }
        }
        __syncthreads();
        if (delayed) {
            if (warp == 0) {
                for (int e = lane; e < nf * n; e += 32) {
                    const int b = e / n, k = e % n;
                    diag[e] = fma(-x.s->r1.col[b][k], x.s->r1.row[b][k], diag[e]);
                }
                __syncwarp();
            }
            ++pending;
            if (pending == kcap) {
                __syncthreads();
                flush_delayed(x, pending);
                pending = 0;
            }
            i = j + 1;
            continue;
        }
        if (warp == 0) {
            for (int e = lane; e < nf * n; e += 32) {
                const int b = e / n, k = e % n;
                diag[e] = fma(-x.s->r1.col[b][k], x.s->r1.row[b][k], diag[e]);
            }
            __syncwarp();
        } else {
            const int w = tid - 32, nw = DQMC_NT / 32 - 1;
            for (int b = 0; b < nf; ++b) {
                double* g = c.G + (size_t)b * x.nn;
                const double* cl = x.s->r1.col[b];
                const double* rw = x.s->r1.row[b];
                for (int k = w & 31; k < n; k += 32) {
                    const double ck = -cl[k];
                    for (int l = w >> 5; l < n; l += nw)
                        g[k + (size_t)l * n] = fma(ck, rw[l], g[k + (size_t)l * n]);
                }
            }
        }
        i = j + 1;
    }
    return acc_count;
}

// calculate_greens(mc, slice, output, field, safe_mult) (stack.jl:525-583)
__device__ __noinline__ void calculate_greens_at(const Ctx& x, int slice, int safe_mult, double* out) {
    DqmcChain& c = *x.c;
    if (safe_mult <= 0) safe_mult = c.k;
    const int sz = x.nf * (int)x.nn;
    mat_ident(x, c.currU);
    mat_ident(x, c.Ur);
    set_ones(x, c.Dr);
    mat_ident(x, c.Tr);
    __syncthreads();
    if (slice + 1 <= c.M) {
        for (int k = c.M; k >= slice + 1; --k) {
            slice_dagger_left(x, k, c.currU);
            if (k % safe_mult == 0) {
                dright_blocks(x, c.tmp1, c.currU, c.Dr);
                udt_blocks(x, c.currU, c.Dr, c.tmp1, true);
                copy(sz, c.tmp2, c.Tr);
                __syncthreads();
                mm_blocks(x, c.Tr, c.tmp1, c.tmp2);
            }
        }
        dright_blocks(x, c.tmp1, c.currU, c.Dr);
        udt_blocks(x, c.Ur, c.Dr, c.tmp1, true);
        copy(sz, c.tmp2, c.Tr);
        __syncthreads();
        mm_blocks(x, c.Tr, c.tmp1, c.tmp2);
    }
    mat_ident(x, c.currU);
    mat_ident(x, c.Ul);
    set_ones(x, c.Dl);
    mat_ident(x, c.Tl);
    __syncthreads();
    if (slice >= 1) {
        for (int k = 1; k <= slice; ++k) {
            slice_left(x, k, c.currU);
            if (k % safe_mult == 0) {
                dright_blocks(x, c.tmp1, c.currU, c.Dl);
                udt_blocks(x, c.currU, c.Dl, c.tmp1, true);
                copy(sz, c.tmp2, c.Tl);
                __syncthreads();
                mm_blocks(x, c.Tl, c.tmp1, c.tmp2);
            }
        }
        dright_blocks(x, c.tmp1, c.currU, c.Dl);
        udt_blocks(x, c.Ul, c.Dl, c.tmp1, true);
        copy(sz, c.tmp2, c.Tl);
        __syncthreads();
        mm_blocks(x, c.Tl, c.tmp1, c.tmp2);
    }
    calculate_greens(x, out);
}

// _greens! (greens.jl:114-125): out = eThalfplus * (G * eThalfminus)
__device__ __noinline__ void greens_physical(const Ctx& x, const double* src, double* out) {
    DqmcChain& c = *x.c;
    for (int b = 0; b < x.nf; ++b) {
        mm<false, true>(x.n, blk(c.tmp1, x, b), src + (size_t)b * x.nn, c.eTh, x.s->tiles);
        __syncthreads();
        mm<true, false>(x.n, blk(out, x, b), c.eThinv, blk(c.tmp1, x, b), x.s->tiles);
        __syncthreads();
    }
}

}  // namespace
}  // namespace dqmc
