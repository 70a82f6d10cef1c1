// Chain-level device operations of the DQMC sweep (one CTA = one chain):
// slice matrices, wraps, stack building, UDT stabilisation, Green's function
// reconstruction, propagate and the local sweep.  Included by the kernel
// translation units; every function is executed by all threads of a CTA.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/dqmc_gb300.h"
#include "dqmc_device.cuh"
#include "dqmc_tc.cuh"

namespace dqmc {
namespace {  // internal linkage: each translation unit gets its own copy

struct Smem {
    double sv[DQMC_NMAX];        // column norms / small vectors
    double ev[2 * DQMC_NMAX];    // interaction exponential of the current slice
    double sxd[4];
    double red[DQMC_NW];
    int sxi[4];
    DqmcChain c;                 // this CTA's chain (state mutated here, written back at exit)
    double* Gglob;               // the chain's G in global memory
    int gres;                    // G currently lives in `arena`
    int arena_cap;               // doubles of `arena` this launch allocated
    int tc_on;                   // this chain's products run on the tensor cores (mm_tc)
    int gdfg;                    // G stays in global memory but holds float pairs (n > 64)
    // flavour-split chains (one flavour block per CTA of a two-CTA cluster):
    // this CTA's exchange counter as its partner reads it, the epochs it has
    // published, a partner that stopped answering, values for the partner,
    // and a configuration flip published after the partner has read the site
    unsigned int xflag;
    unsigned int xepoch;
    int xdead;
    int xflip_val;
    double xval[2];
    TcState tc;                  // TMEM base and mbarriers of mm_tc (16-byte aligned)
    // `tiles` and `arena` are adjacent and 16-byte aligned: mm_tc stages its
    // operand slices in both (chains with n > 64 use neither otherwise)
    union {                      // never live at the same time
        double tiles[2 * 16 * 64];  // mm() / mm_dfx() staging
        struct {
            double col[2][DQMC_NMAX];  // rank-1: (I - G)[:, i] per block
            double row[2][DQMC_NMAX];  // rank-1: (Delta/R) G[i, :] per block
        } r1;
    };
    // last member: a launch allocates only the 2 n (n + 1) doubles its chains
    // use (max over chains with n <= 64).  Shared-memory QR of one or two
    // blocks when n <= 64; between stabilisations of a sweep it holds G
    // (G-resident mode).
    double arena[2 * 64 * 65];
};
static_assert(sizeof(double) * 2 * 16 * 64 + sizeof(double) * 2 * 64 * 65 >= DQMC_TC_SMEM,
              "mm_tc staging must fit tiles + arena");
static_assert(2 * 64 * 65 >= DQMC_QWS, "the blocked Q accumulation's workspace must fit the arena");

// Products of a chain run on the tensor cores (mm_tc) when it is a real,
// mixed-precision chain with dense hopping and DQMC_TC_NMIN <= n <= 256, its
// tensor products are enabled, and the launch has the whole arena (then
// `tiles` + `arena` hold mm_tc's staging).
#define DQMC_TC_NMIN 96
// the tensor-core products are compiled only into the tensor-core build of
// the chain kernel (dqmc_kernels_tc.cu)
#ifndef DQMC_TC_BUILD
#define DQMC_TC_BUILD 0
#endif
#define DQMC_TC_COMPILED DQMC_TC_BUILD
__device__ __forceinline__ bool tc_eligible(const DqmcChain& c, int arena_cap) {
    return c.prec == DQMC_PREC_MIXED_ID && !c.cplx && !c.cb && c.tc_enable && c.tcs &&
           c.n >= DQMC_TC_NMIN && c.n <= DQMC_TC_NMAX && arena_cap >= 2 * 64 * 65;
}
__device__ __forceinline__ unsigned char* tc_stage(Smem* s) {
    return reinterpret_cast<unsigned char*>(s->tiles);
}

struct Ctx {
    Smem* s;
    DqmcChain* c;  // == &s->c
    int n, nf;
    size_t nn;
    // flavour blocks this CTA owns: [0, nf), or block `b0` alone on a
    // flavour-split chain, whose other block the cluster partner (`peer`,
    // its rank; -1: none) owns
    int b0, b1, peer;
};

__device__ __forceinline__ double* blk(double* p, const Ctx& x, int b) { return p + (size_t)b * x.nn; }
__device__ __forceinline__ bool split(const Ctx& x) { return x.peer >= 0; }
// the tensor products' operand scratch of this CTA (one area per flavour
// block; a CTA that owns both blocks uses the first)
__device__ __forceinline__ unsigned char* tc_scratch(const Ctx& x) {
    return x.c->tcs + (size_t)x.b0 * dqmc_tc_scratch_stride(x.n);
}
// A chain whose two flavour blocks can run on two CTAs: real field, dense
// hopping, and nothing coupling the blocks besides the local updates'
// determinant ratio and the propagation error (no device measurements,
// global updates or replica exchange); and large enough (n >= 48) that
// halving its matrix work clearly outweighs the two rendezvous per accepted
// move (measured on the served stream: 64- to 128-site two-flavour chains
// 1.1-1.7x faster per 10-sweep block).
#define DQMC_SPLIT_NMIN 48
__device__ __forceinline__ bool flavour_split_ok(const DqmcChain& c) {
    return c.nf == 2 && c.n >= DQMC_SPLIT_NMIN && !c.cplx && !c.cb && !c.meas_enable &&
           !c.td_enable && c.global_kind < 0 && c.partner < 0;
}
// the owned blocks' part of an nf x (n x n) matrix / an nf x n vector
__device__ __forceinline__ void copy_mats(const Ctx& x, double* dst, const double* src) {
    const size_t o = (size_t)x.b0 * x.nn;
    copy((x.b1 - x.b0) * (int)x.nn, dst + o, src + o);
}
__device__ __forceinline__ void copy_vecs(const Ctx& x, double* dst, const double* src) {
    const int o = x.b0 * x.n;
    copy((x.b1 - x.b0) * x.n, dst + o, src + o);
}

// The field of site j of a slice row; `fresh`: read past L1 (on a
// flavour-split chain the partner CTA's SM writes the configuration).
__device__ __forceinline__ int conf_at(const int8_t* s, int j, bool fresh) {
    return fresh ? *reinterpret_cast<const volatile int8_t*>(s + j) : s[j];
}

// ---- exchanges between the two CTAs of a flavour-split chain ---------------
__device__ __forceinline__ unsigned int cluster_ncta() {
    unsigned int r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned int cluster_rank() {
    unsigned int r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
// all threads of the cluster (every CTA has started; its prior writes visible)
__device__ __forceinline__ void cluster_barrier() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;"
                 ::: "memory");
}
// the address of `p` (this CTA's shared memory) in CTA `rank` of the cluster
__device__ __forceinline__ uint32_t peer_addr(const void* p, int rank) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
    return r;
}
__device__ __forceinline__ double peer_ld(uint32_t a) {
    double v;
    asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(a) : "memory");
    return v;
}
__device__ __forceinline__ int peer_ld_s32(uint32_t a) {
    int v;
    asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(a) : "memory");
    return v;
}
__device__ __forceinline__ unsigned int peer_ld_acquire(uint32_t a) {
    unsigned int v;
    asm volatile("ld.acquire.cluster.shared::cluster.u32 %0, [%1];" : "=r"(v) : "r"(a) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_cluster(uint32_t a, unsigned int v) {
    asm volatile("st.release.cluster.shared::cluster.u32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}
#define DQMC_STATUS_PEER 9  // the partner CTA of a flavour-split chain stopped answering
// Rendezvous of the two CTAs of a flavour-split chain: every write either CTA
// made before it is visible to the other after it.  Thread 0 publishes its
// epoch with a cluster-scope release and waits (bounded: 2 s of the global
// timer or 2^28 polls) until the partner has published the same epoch; after
// a time-out the chain's status is set, further rendezvous return at once
// and false, and the callers skip the partner's data.  Executed by all
// threads of both CTAs the same number of times (both run the same control
// flow: the decisions are identical) unless one of them timed out.  Neither
// CTA leaves the kernel before the other has passed its last rendezvous
// (a cluster barrier ends the chain's launch; every wait before it is
// bounded), so a partner's shared memory is never read after it has left.
__device__ bool xsync(const Ctx& x) {
    __syncthreads();
    if (threadIdx.x == 0 && !x.s->xdead) {
        const unsigned int e = ++x.s->xepoch;
        const int quiet = x.c->x_silent_from;
        if (!(quiet > 0 && x.b0 == 1 && e >= (unsigned int)quiet))
            st_release_cluster(peer_addr(&x.s->xflag, (int)cluster_rank()), e);
        const uint32_t pa = peer_addr(&x.s->xflag, x.peer);
        unsigned long long t0;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
        for (unsigned int spin = 0;; ++spin) {
            if ((int)(peer_ld_acquire(pa) - e) >= 0) break;
            if ((spin & 1023) == 1023) {
                unsigned long long t;
                asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
                if (t - t0 > 2000000000ull || spin > (1u << 28)) {
                    x.s->xdead = 1;
                    x.c->status = DQMC_STATUS_PEER;
                    break;
                }
            }
        }
    }
    __syncthreads();
    return !x.s->xdead;
}

// G-resident mode (n <= 64): during sweeps G stays in shared memory for the
// rank-1 updates and wraps, and moves to global memory while a stabilisation
// needs the arena for its QR factorisations.
// On a mixed-precision chain with n >= 32 the resident G is double-float
// (float2 per entry, same bytes): the rank-1 updates and the wraps then run
// entirely on the FP32 pipe; it is rounded back to FP64 whenever it leaves
// shared memory.  (At n = 16 the split arithmetic costs more than it saves.)
// A mixed chain with n > 64 keeps G in its global buffer but, between
// stabilisations, as float pairs in place (gdfg): the delayed rank-k updates
// and the wraps then issue no FP64 instruction either.
__device__ __forceinline__ bool df_mode(const Ctx& x) {
    return x.c->prec == DQMC_PREC_MIXED_ID && x.n >= 32 && !x.c->cb && !x.c->cplx;
}
__device__ __forceinline__ bool df_global_possible(const Ctx& x) { return df_mode(x) && x.n > 64; }
__device__ __forceinline__ bool g_resident_possible(const Ctx& x) {
    return (x.n <= 64 && (size_t)x.nf * x.nn <= (size_t)x.s->arena_cap) || df_global_possible(x);
}
__device__ __forceinline__ bool df_resident(const Ctx& x) {
    return df_mode(x) && (x.s->gres || x.s->gdfg);
}
__device__ __forceinline__ float2* arena_df(const Ctx& x) {
    return reinterpret_cast<float2*>(x.s->arena);
}
// the double-float G wherever it lives (shared arena or its global buffer)
__device__ __forceinline__ float2* gdf_ptr(const Ctx& x) {
    return reinterpret_cast<float2*>(x.c->G);
}
// the resident G (either form) as FP64 into dst (dst may be G's own global
// buffer: element e is read before it is written, by the same thread)
__device__ void g_resident_to(const Ctx& x, double* dst) {
    if (!x.s->gres && !x.s->gdfg) return;  // G is in global memory as FP64 already
    const int e0 = x.b0 * (int)x.nn, e1 = x.b1 * (int)x.nn;
    if (df_mode(x)) {
        const float2* a = gdf_ptr(x);
        for (int e = e0 + threadIdx.x; e < e1; e += DQMC_NT) dst[e] = df_to_d(a[e]);
    } else {
        for (int e = e0 + threadIdx.x; e < e1; e += DQMC_NT) dst[e] = x.s->arena[e];
    }
}
__device__ void g_to_arena(const Ctx& x) {
    __syncthreads();
    const int e0 = x.b0 * (int)x.nn, e1 = x.b1 * (int)x.nn;
    if (x.n > 64) {  // in place, float pairs in the global buffer
        float2* a = reinterpret_cast<float2*>(x.s->Gglob);
        for (int e = e0 + threadIdx.x; e < e1; e += DQMC_NT) a[e] = d_to_df(x.s->Gglob[e]);
        __syncthreads();
        if (threadIdx.x == 0) x.s->gdfg = 1;
        __syncthreads();
        return;
    }
    if (df_mode(x)) {
        float2* a = arena_df(x);
        for (int e = e0 + threadIdx.x; e < e1; e += DQMC_NT) a[e] = d_to_df(x.s->Gglob[e]);
    } else {
        for (int e = e0 + threadIdx.x; e < e1; e += DQMC_NT) x.s->arena[e] = x.s->Gglob[e];
    }
    __syncthreads();
    if (threadIdx.x == 0) { x.c->G = x.s->arena; x.s->gres = 1; }
    __syncthreads();
}
__device__ void g_to_global(const Ctx& x) {
    __syncthreads();
    g_resident_to(x, x.s->Gglob);
    __syncthreads();
    if (threadIdx.x == 0) { x.c->G = x.s->Gglob; x.s->gres = 0; x.s->gdfg = 0; }
    __syncthreads();
}

// UDT of one flavour block: in shared memory for n <= 64, else from global memory
__device__ __forceinline__ void udt_one(const Ctx& x, double* U, double* D, double* In, int b,
                                        bool apply) {
    if (x.n <= 64)
        udt_pivot_sm(x.n, U, D, In, x.c->pivot + b * x.n, x.c->tempv + b * x.n, apply,
                     x.s->arena, x.s->arena + x.n * (x.n + 1), x.s->sv, x.s->sxd);
    else if (x.c->prec == DQMC_PREC_MIXED_ID)  // norms downdated (see udt_pivot_g)
        udt_pivot_g<true>(x.n, U, D, In, x.c->pivot + b * x.n, x.c->tempv + b * x.n, apply,
                          blk(x.c->out, x, b), x.s->sv, x.s->sxd, x.s->tiles, x.s->arena);
    else
        udt_pivot_g<false>(x.n, U, D, In, x.c->pivot + b * x.n, x.c->tempv + b * x.n, apply,
                           blk(x.c->out, x, b), x.s->sv, x.s->sxd, x.s->tiles, x.s->arena);
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
// mixed-precision chain the double-float product on the FP32 pipe (so are
// the products of the Green's reconstruction, rmm below).  The UDT
// factorisations, the triangular solves, the T updates, the determinant ratios
// and the rank-1 updates stay FP64 on every chain.
// Every transposed left operand (TA) of these products is a hopping
// exponential, which is symmetric, so the double-float product reads it
// untransposed (identical sums; the untransposed staging needs fewer
// registers).  Below n = 48 the mixed path keeps the FP64 product: the
// matrices are too small for the split arithmetic to pay.
// A failed tensor-core product (an mbarrier wait that timed out) sets the
// chain's status to DQMC_STATUS_TC_TIMEOUT and turns the tensor path off for
// the rest of the launch.
#define DQMC_STATUS_TC_TIMEOUT 7
__device__ __forceinline__ void tc_failed(const Ctx& x) {
    if (threadIdx.x == 0) {
        x.c->status = DQMC_STATUS_TC_TIMEOUT;
        x.s->tc_on = 0;
    }
    __syncthreads();
}

template <bool TA, bool TB>
__device__ __forceinline__ void smm(const Ctx& x, bool wrap, double* C, const double* A,
                                    const double* B) {
    const DqmcChain& c = *x.c;
    if (c.prec == DQMC_PREC_MIXED_ID && x.n >= 48) {
        // the transposed operand is eT2 or eT2inv: take its float-pair split
        if (DQMC_TC_COMPILED && x.s->tc_on && (c.tc_enable & (wrap ? DQMC_TC_WRAPS : DQMC_TC_SLICES))) {
            const bool ok = TA ? mm_tc<true, false, false>(x.n, C, A == c.eT2 ? c.eT2df : c.eT2invdf,
                                                          B, tc_stage(x.s), &x.s->tc, tc_scratch(x))
                               : mm_tc<false, true, false>(x.n, C, A,
                                                           B == c.eT2 ? c.eT2df : c.eT2invdf,
                                                           tc_stage(x.s), &x.s->tc, tc_scratch(x));
            if (ok) return;
            tc_failed(x);
        }
        if (TA)
            mm_dfx<true, false, false>(x.n, C, A == c.eT2 ? c.eT2df : c.eT2invdf, B, x.s->tiles);
        else
            mm_dfx<false, true, false>(x.n, C, A, B == c.eT2 ? c.eT2df : c.eT2invdf, x.s->tiles);
    } else {
        mm<TA, TB>(x.n, C, A, B, x.s->tiles);
    }
}

// Checkerboard products (linalg/checkerboard.jl:272-473) on one flavour
// block.  Factor m (0 exp(-dtau T), 1 exp(+dtau T), 2 exp(-dtau T/2),
// 3 exp(+dtau T/2)) is X = P_1 ... P_N D; mode 0: out = X in, 1: out = in X,
// 2: out = X^T in = D P_N ... P_1 in.  One pass per part: row (mode 1: column)
// i becomes c_i times itself plus s_i times its partner's, D fused into the
// first (mode 0) or last (modes 1, 2) pass.  Passes alternate between out and
// scr so that the last lands in out; in must differ from out and scr.
// O(n^2) per part instead of the dense product's O(n^3), FP64 on every chain.
__device__ __noinline__ void cb_apply(const Ctx& x, int m, int mode, double* out,
                                      const double* in, double* scr) {
    const DqmcChain& c = *x.c;
    const int n = x.n, np = c.cb_np;
    const double* D = c.cb + (size_t)m * n * (1 + 2 * (size_t)np);
    const double* P = D + n;
    const int* PT = c.cbp + (size_t)m * np * n;
    if (np == 0) {
        for (int e = threadIdx.x; e < n * n; e += DQMC_NT) {
            const int i = e % n, k = e / n;
            out[e] = (mode == 1) ? in[e] * D[k] : D[i] * in[e];
        }
        __syncthreads();
        return;
    }
    const double* src = in;
    for (int step = 0; step < np; ++step) {
        const int part = (mode == 0) ? np - 1 - step : step;
        const double* cc = P + (size_t)part * 2 * n;
        const double* ss = cc + n;
        const int* pt = PT + (size_t)part * n;
        const bool first = (step == 0), last = (step == np - 1);
        double* dst = ((np - 1 - step) & 1) ? scr : out;
        for (int e = threadIdx.x; e < n * n; e += DQMC_NT) {
            const int i = e % n, k = e / n;
            double y;
            if (mode == 1) {
                const int q = pt[k];
                const double v = src[e];
                y = (q >= 0) ? fma(src[i + (size_t)q * n], ss[k], v * cc[k]) : v;
                if (last) y = y * D[k];
            } else {
                const int q = pt[i];
                double v = src[e];
                double w = (q >= 0) ? src[q + (size_t)k * n] : 0.0;
                if (mode == 0 && first) {
                    v = D[i] * v;
                    if (q >= 0) w = D[q] * w;
                }
                y = (q >= 0) ? fma(ss[i], w, cc[i] * v) : v;
                if (mode == 2 && last) y = D[i] * y;
            }
            dst[e] = y;
        }
        __syncthreads();
        src = dst;
    }
}

// interaction_matrix_exp! (fields.jl:380-386, 429-438, 548-560, 618-624)
// into shared memory: ev[b*n + i]; on a complex chain Re at ev[b*n + i] and
// Im at ev[b*n + ns + i] (i < ns)
__device__ __noinline__ void interaction_exp(const Ctx& x, int slice, bool inverse) {
    const DqmcChain& c = *x.c;
    const int ns = c.ns;
    const int8_t* s = c.conf + (size_t)(slice - 1) * ns;
    const bool ghq = (c.kind >= 2);
    for (int e = threadIdx.x; e < x.nf * ns; e += DQMC_NT) {
        int b = e / ns, i = e % ns;
        const int f = conf_at(s, i, x.peer >= 0);
        int v = ghq ? f - 1 : (f > 0 ? 1 : 0);
        x.s->ev[b * x.n + i] = inverse ? c.evinv[b][v] : c.ev[b][v];
        if (c.cplx) x.s->ev[b * x.n + ns + i] = inverse ? c.evinvi[b][v] : c.evi[b][v];
    }
    __syncthreads();
}
// Diagonal(eV) * B and A * Diagonal(eV) with the current slice's exponentials
// (complex on a complex chain; conj: adjoint(eV))
__device__ __forceinline__ void ev_left(const Ctx& x, double* C, const double* d, const double* B,
                                        bool conj = false) {
    if (x.c->cplx) dleft_c(x.n, C, d, B, conj);
    else dleft(x.n, C, d, B);
}
__device__ __forceinline__ void ev_right(const Ctx& x, double* C, const double* A, const double* d) {
    if (x.c->cplx) dright_c(x.n, C, A, d, false);
    else dright(x.n, C, A, d);
}

// multiply_slice_matrix_left!: M <- eT2 * eV * M  (stack.jl:319-327)
__device__ __noinline__ void slice_left(const Ctx& x, int slice, double* M, bool wrap = false) {
    interaction_exp(x, slice, false);
    for (int b = x.b0; b < x.b1; ++b) {
        ev_left(x, blk(x.c->tmp1, x, b), x.s->ev + b * x.n, blk(M, x, b));
        __syncthreads();
        if (x.c->cb)
            cb_apply(x, 0, 0, blk(M, x, b), blk(x.c->tmp1, x, b), blk(x.c->tmp2, x, b));
        else
            smm<true, false>(x, wrap, blk(M, x, b), x.c->eT2, blk(x.c->tmp1, x, b));
        __syncthreads();
    }
}
// multiply_slice_matrix_right!: M <- M * eT2 * eV  (stack.jl:329-337)
__device__ __noinline__ void slice_right(const Ctx& x, int slice, double* M, bool wrap = false) {
    interaction_exp(x, slice, false);
    for (int b = x.b0; b < x.b1; ++b) {
        if (x.c->cb)
            cb_apply(x, 0, 1, blk(x.c->tmp1, x, b), blk(M, x, b), blk(x.c->tmp2, x, b));
        else
            smm<false, true>(x, wrap, blk(x.c->tmp1, x, b), blk(M, x, b), x.c->eT2);
        __syncthreads();
        ev_right(x, blk(M, x, b), blk(x.c->tmp1, x, b), x.s->ev + b * x.n);
        __syncthreads();
    }
}
// multiply_slice_matrix_inv_right!: M <- M * eV^-1 * eT2^-1  (stack.jl:339-347)
__device__ __noinline__ void slice_inv_right(const Ctx& x, int slice, double* M, bool wrap = false) {
    interaction_exp(x, slice, true);
    for (int b = x.b0; b < x.b1; ++b) {
        ev_right(x, blk(x.c->tmp1, x, b), blk(M, x, b), x.s->ev + b * x.n);
        __syncthreads();
        if (x.c->cb)
            cb_apply(x, 1, 1, blk(M, x, b), blk(x.c->tmp1, x, b), blk(x.c->tmp2, x, b));
        else
            smm<false, true>(x, wrap, blk(M, x, b), blk(x.c->tmp1, x, b), x.c->eT2inv);
        __syncthreads();
    }
}
// multiply_slice_matrix_inv_left!: M <- eV^-1 * eT2^-1 * M  (stack.jl:349-357)
__device__ __noinline__ void slice_inv_left(const Ctx& x, int slice, double* M, bool wrap = false) {
    interaction_exp(x, slice, true);
    for (int b = x.b0; b < x.b1; ++b) {
        if (x.c->cb)
            cb_apply(x, 1, 0, blk(x.c->tmp1, x, b), blk(M, x, b), blk(x.c->tmp2, x, b));
        else
            smm<true, false>(x, wrap, blk(x.c->tmp1, x, b), x.c->eT2inv, blk(M, x, b));
        __syncthreads();
        ev_left(x, blk(M, x, b), x.s->ev + b * x.n, blk(x.c->tmp1, x, b));
        __syncthreads();
    }
}
// multiply_daggered_slice_matrix_left!: M <- eV * eT2 * M (stack.jl:359-367)
__device__ __noinline__ void slice_dagger_left(const Ctx& x, int slice, double* M) {
    interaction_exp(x, slice, false);
    for (int b = x.b0; b < x.b1; ++b) {
        if (x.c->cb)
            cb_apply(x, 0, 2, blk(x.c->tmp1, x, b), blk(M, x, b), blk(x.c->tmp2, x, b));
        else
            smm<true, false>(x, false, blk(x.c->tmp1, x, b), x.c->eT2, blk(M, x, b));
        __syncthreads();
        ev_left(x, blk(M, x, b), x.s->ev + b * x.n, blk(x.c->tmp1, x, b), true);
        __syncthreads();
    }
}

// C = A B for double-float operands and result: tensor cores when the chain
// has them, else the FP32-pipe product
__device__ __forceinline__ void mm_df3(const Ctx& x, float2* C, const float2* A, const float2* B) {
    if (DQMC_TC_COMPILED && x.s->tc_on && (x.c->tc_enable & DQMC_TC_WRAPS)) {
        if (mm_tc<true, true, true>(x.n, C, A, B, tc_stage(x.s), &x.s->tc, tc_scratch(x))) return;
        tc_failed(x);
    }
    mm_dfx<true, true, true>(x.n, C, A, B, x.s->tiles);
}

// wrap_greens! of the resident double-float G of a mixed chain: the same
// four slice-matrix steps with double-float diagonals (exact float pairs of
// the interaction exponentials) and double-float products; tmp1 holds the
// float-pair intermediate.  The pairs of one flavour block's diagonal go into
// `sv` (n <= DQMC_NMAX pairs; `sv` is used only by the stabilisations).
__device__ __noinline__ void wrap_greens_df(const Ctx& x, int curr_slice, int direction) {
    const DqmcChain& c = *x.c;
    const int n = x.n;
    float2* G = gdf_ptr(x);
    float2* T = reinterpret_cast<float2*>(c.tmp1);
    float2* d = reinterpret_cast<float2*>(x.s->sv);
    const int slice = direction == -1 ? curr_slice - 1 : curr_slice;
    for (int half = 0; half < 2; ++half) {
        // direction +1: B(l) G B(l)^-1 = eT2 (eV (G eV^-1)) eT2inv, as
        //   slice_left then slice_inv_right; direction -1: B(l)^-1 G B(l) as
        //   slice_inv_left then slice_right (stack.jl:319-357)
        const bool inverse = (direction == 1) ? (half == 1) : (half == 0);
        interaction_exp(x, slice, inverse);
        const float2* hop = inverse ? c.eT2invdf : c.eT2df;
        for (int b = x.b0; b < x.b1; ++b) {
            float2* g = G + (size_t)b * x.nn;
            float2* t = T + (size_t)b * x.nn;
            __syncthreads();  // the previous block's last reads of d are done
            for (int i = threadIdx.x; i < n; i += DQMC_NT) d[i] = d_to_df(x.s->ev[b * n + i]);
            __syncthreads();
            if (half == 0) {
                if (direction == 1) {  // G <- eT2 * (eV * G)
                    dleft_df(n, t, d, g);
                    __syncthreads();
                    mm_df3(x, g, hop, t);
                } else {                 // G <- eV^-1 * (eT2inv * G)
                    mm_df3(x, t, hop, g);
                    __syncthreads();
                    dleft_df(n, g, d, t);
                }
            } else {
                if (direction == 1) {  // G <- (G * eV^-1) * eT2inv
                    dright_df(n, t, g, d);
                    __syncthreads();
                    mm_df3(x, g, t, hop);
                } else {                 // G <- (G * eT2) * eV
                    mm_df3(x, t, g, hop);
                    __syncthreads();
                    dright_df(n, g, t, d);
                }
            }
            __syncthreads();
        }
    }
}

// wrap_greens! (stack.jl:594-603)
// A complex chain's G projected back onto the representation subspace
// [[X, -Y], [Y, X]] (each pair of copies replaced by its mean).  Rounding in
// the wraps and rank-2 updates leaves a component outside the subspace,
// which the next wraps carry along; the projection removes it.
__device__ void rep_project(const Ctx& x, double* gf) {
    const int n = x.n, m = n >> 1;
    for (int e = threadIdx.x; e < x.nf * m * m; e += DQMC_NT) {
        const int b = e / (m * m), r = e % m, col = (e / m) % m;
        double* g = gf + (size_t)b * x.nn;
        const size_t tl = (size_t)col * n + r, br = (size_t)(m + col) * n + m + r;
        const size_t bl = (size_t)col * n + m + r, tr = (size_t)(m + col) * n + r;
        const double xa = 0.5 * (g[tl] + g[br]), ya = 0.5 * (g[bl] - g[tr]);
        g[tl] = xa;
        g[br] = xa;
        g[bl] = ya;
        g[tr] = -ya;
    }
    __syncthreads();
}

__device__ void wrap_greens(const Ctx& x, double* gf, int curr_slice, int direction) {
    if (df_resident(x) && gf == x.c->G) {
        wrap_greens_df(x, curr_slice, direction);
        return;
    }
    if (direction == -1) {
        slice_inv_left(x, curr_slice - 1, gf, true);
        slice_right(x, curr_slice - 1, gf, true);
    } else {
        slice_left(x, curr_slice, gf, true);
        slice_inv_right(x, curr_slice, gf, true);
    }
    if (x.c->cplx) rep_project(x, gf);
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
    for (int b = x.b0; b < x.b1; ++b) ident(x.n, blk(A, x, b));
}

// two flavour blocks that fit the shared-memory QR: factor them together
__device__ __forceinline__ bool paired(const Ctx& x) { return x.nf == 2 && x.n <= 64; }
__device__ __forceinline__ UdtJob udt_job(const Ctx& x, double* U, double* D, double* In, int b) {
    return UdtJob{blk(U, x, b), D + b * x.n, blk(In, x, b), x.c->pivot + b * x.n,
                  x.c->tempv + b * x.n};
}
// (a flavour-split chain factors its own block with the pair's arithmetic)
__device__ __forceinline__ void udt_pair(const Ctx& x, double* U, double* D, double* In, bool apply) {
    if (split(x)) {
        const UdtJob j = udt_job(x, U, D, In, x.b0);
        udt_pivot_sm2(x.n, j, j, apply, x.s->arena, x.s->sv, x.s->sxd, true);
        return;
    }
    udt_pivot_sm2(x.n, udt_job(x, U, D, In, 0), udt_job(x, U, D, In, 1), apply, x.s->arena,
                  x.s->sv, x.s->sxd);
}
__device__ __forceinline__ void rdivp_pair(const Ctx& x, double* A, double* T, double* O) {
    const int n = x.n;
    if (split(x)) {
        const int b = x.b0;
        rdivp2(n, blk(A, x, b), blk(T, x, b), blk(O, x, b), x.c->pivot + b * n, nullptr, nullptr,
               nullptr, nullptr, x.s->sv, 1);
        return;
    }
    rdivp2(n, A, T, O, x.c->pivot, blk(A, x, 1), blk(T, x, 1), blk(O, x, 1), x.c->pivot + n,
           x.s->sv);
}

__device__ __noinline__ void udt_blocks(const Ctx& x, double* U, double* D, double* In, bool apply) {
    if (paired(x)) {
        udt_pair(x, U, D, In, apply);
        return;
    }
    for (int b = x.b0; b < x.b1; ++b) udt_one(x, blk(U, x, b), D + b * x.n, blk(In, x, b), b, apply);
}
__device__ __noinline__ void mm_blocks(const Ctx& x, double* C, double* A, double* B) {
    for (int b = x.b0; b < x.b1; ++b) {
        mm<false, false>(x.n, blk(C, x, b), blk(A, x, b), blk(B, x, b), x.s->tiles);
    }
    __syncthreads();
}
__device__ void dright_blocks(const Ctx& x, double* C, double* A, const double* d) {
    for (int b = x.b0; b < x.b1; ++b) dright(x.n, blk(C, x, b), blk(A, x, b), d + b * x.n);
    __syncthreads();
}

// add_slice_sequence_left (stack.jl:377-393)
__device__ __noinline__ void add_slice_sequence_left(const Ctx& x, int idx) {
    DqmcChain& c = *x.c;
    copy_mats(x, c.currU, ustk(x, idx));
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
    copy_mats(x, c.currU, ustk(x, idx + 1));
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

// calculate_greens_AVX! for two flavour blocks in lock step (the blocks are
// independent; each sees exactly the per-block sequence below), so that the
// two QR factorisations and the two triangular solves of each step run
// together.
// Products of the Green's reconstruction: FP64, or on a mixed-precision
// chain with n >= 48 the double-float product on the FP32 pipe (FP64
// operands split while staged; ~1e-14 relative per product).  The UDT
// factorisations and triangular solves between them stay FP64, and so does
// everything of a checkerboard chain.
template <bool TA, bool TB>
__device__ __forceinline__ void rmm(const Ctx& x, double* C, const double* A, const double* B) {
    if (x.c->prec == DQMC_PREC_MIXED_ID && x.n >= 48 && !x.c->cplx && !x.c->cb) {
        if (DQMC_TC_COMPILED && x.s->tc_on && (x.c->tc_enable & DQMC_TC_GREENS)) {
            if (mm_tc<false, false, false, TA, TB>(x.n, C, A, B, tc_stage(x.s), &x.s->tc, tc_scratch(x)))
                return;
            tc_failed(x);
        }
        mm_dfx<false, false, false, TA, TB>(x.n, C, A, B, x.s->tiles);
    } else {
        mm<TA, TB>(x.n, C, A, B, x.s->tiles);
    }
}

__device__ __noinline__ void calculate_greens_pair(const Ctx& x, double* Gout, bool finish) {
    DqmcChain& c = *x.c;
    const int n = x.n;
    for (int b = x.b0; b < x.b1; ++b) rmm<false, true>(x, blk(Gout, x, b), blk(c.Tl, x, b), blk(c.Tr, x, b));
    __syncthreads();
    for (int b = x.b0; b < x.b1; ++b) dright(n, blk(c.Tr, x, b), blk(Gout, x, b), c.Dr + b * n);
    __syncthreads();
    for (int b = x.b0; b < x.b1; ++b) dleft(n, blk(Gout, x, b), c.Dl + b * n, blk(c.Tr, x, b));
    __syncthreads();
    udt_pair(x, c.Tr, c.Dr, Gout, false);
    for (int b = x.b0; b < x.b1; ++b) rmm<false, false>(x, blk(c.Tl, x, b), blk(c.Ul, x, b), blk(c.Tr, x, b));
    __syncthreads();
    rdivp_pair(x, c.Ur, Gout, c.Ul);
    for (int b = x.b0; b < x.b1; ++b) rmm<true, false>(x, blk(c.Tr, x, b), blk(c.Tl, x, b), blk(c.Ur, x, b));
    __syncthreads();
    for (int e = x.b0 * n + threadIdx.x; e < x.b1 * n; e += DQMC_NT) {
        const int b = e / n, i = e % n;
        blk(c.Tr, x, b)[(size_t)i * n + i] += c.Dr[b * n + i];
    }
    __syncthreads();
    udt_pair(x, c.Ul, c.Dr, c.Tr, false);
    if (!finish) return;
    rdivp_pair(x, c.Ur, c.Tr, Gout);
    for (int b = x.b0; b < x.b1; ++b) rmm<false, false>(x, blk(c.Tr, x, b), blk(c.Tl, x, b), blk(c.Ul, x, b));
    for (int e = x.b0 * n + threadIdx.x; e < x.b1 * n; e += DQMC_NT) c.Dl[e] = 1.0 / c.Dr[e];
    __syncthreads();
    for (int b = x.b0; b < x.b1; ++b) dright(n, blk(c.Ul, x, b), blk(c.Ur, x, b), c.Dl + b * n);
    __syncthreads();
    for (int b = x.b0; b < x.b1; ++b) rmm<false, true>(x, blk(Gout, x, b), blk(c.Ul, x, b), blk(c.Tr, x, b));
    __syncthreads();
}

// calculate_greens_AVX! (stack.jl:442-496), per flavour block.  finish =
// false stops after the second UDT: calculate_inv_greens_udt
// (global_updates.jl:26-49), leaving det(G) = 1 / prod(Dr) up to phases.
// A complex chain's result is projected onto the representation subspace.
__device__ __noinline__ void calculate_greens(const Ctx& x, double* Gout, bool finish = true) {
    if (paired(x)) {
        calculate_greens_pair(x, Gout, finish);
        if (finish && x.c->cplx) rep_project(x, Gout);
        return;
    }
    DqmcChain& c = *x.c;
    const int n = x.n;
    const bool bf = x.nf > 1;
    for (int b = x.b0; b < x.b1; ++b) {
        double *ul = blk(c.Ul, x, b), *tl = blk(c.Tl, x, b), *ur = blk(c.Ur, x, b),
               *tr = blk(c.Tr, x, b), *g = blk(Gout, x, b);
        double *dl = c.Dl + b * n, *dr = c.Dr + b * n;
        int* pv = c.pivot + b * n;
        rmm<false, true>(x, g, tl, tr);
        __syncthreads();
        dright(n, tr, g, dr);
        __syncthreads();
        dleft(n, g, dl, tr);
        __syncthreads();
        udt_one(x, tr, dr, g, b, false);
        rmm<false, false>(x, tl, ul, tr);
        __syncthreads();
        rdivp(n, ur, g, ul, pv, bf, x.s->sv);
        rmm<true, false>(x, tr, tl, ur);
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += DQMC_NT) tr[(size_t)i * n + i] += dr[i];
        __syncthreads();
        udt_one(x, ul, dr, tr, b, false);
        if (!finish) continue;
        rdivp(n, ur, tr, g, pv, bf, x.s->sv);
        rmm<false, false>(x, tr, tl, ul);
        for (int i = threadIdx.x; i < n; i += DQMC_NT) dl[i] = 1.0 / dr[i];
        __syncthreads();
        dright(n, ul, ur, dl);
        __syncthreads();
        rmm<false, true>(x, g, ul, tr);
        __syncthreads();
    }
    if (finish && x.c->cplx) rep_project(x, Gout);
}

__device__ void set_ones(const Ctx& x, double* d) {
    fill((x.b1 - x.b0) * x.n, d + x.b0 * x.n, 1.0);
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
    copy_mats(x, c.Ur, ustk(x, 1));
    copy_vecs(x, c.Dr, dstk(x, 1));
    copy_mats(x, c.Tr, tstk(x, 1));
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
    copy_mats(x, c.Ul, ustk(x, nr + 1));
    copy_vecs(x, c.Dl, dstk(x, nr + 1));
    copy_mats(x, c.Tl, tstk(x, nr + 1));
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

// max |Gtmp - G| (stack.jl:646, 701); NaN propagates.  On a complex chain
// the modulus of the complex difference, read from the representation's
// left half (Re rows 0..ns-1, Im rows ns..2ns-1).
__device__ __noinline__ void record_prop_error(const Ctx& x) {
    DqmcChain& c = *x.c;
    double m = 0.0;
    if (c.cplx) {
        const int ns = c.ns, cnt = x.nf * ns * ns;
        for (int e = threadIdx.x; e < cnt; e += DQMC_NT) {
            const int b = e / (ns * ns), r = e % ns, col = (e / ns) % ns;
            const size_t at = (size_t)b * x.nn + (size_t)col * x.n + r;
            double d = hypot(c.Gtmp[at] - c.G[at], c.Gtmp[at + ns] - c.G[at + ns]);
            if (d > m || d != d) m = d;
        }
    } else {
        for (int e = x.b0 * (int)x.nn + threadIdx.x; e < x.b1 * (int)x.nn; e += DQMC_NT) {
            double d = fabs(c.Gtmp[e] - c.G[e]);
            if (d > m || d != d) m = d;
        }
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
        x.s->xval[0] = mx;
    }
    if (split(x) && xsync(x)) {
        // the chain's error is the larger of the two blocks' (both CTAs
        // record the same value); the partner reads xval[0] before the
        // next rendezvous, which precedes the next write of it
        if (threadIdx.x == 0) {
            const double v = peer_ld(peer_addr(&x.s->xval[0], x.peer));
            if (v > x.s->xval[0] || v != v) x.s->xval[0] = v;
        }
        xsync(x);
    }
    if (threadIdx.x == 0) {
        const double mx = x.s->xval[0];
        if (mx > c.prop_err_max || mx != mx) c.prop_err_max = mx;
        // a non-finite Green's function is reported to the host as a
        // numerical error (status 2) instead of propagating silently
        if (mx != mx || mx > 1e300) c.status = 2;
        if (mx > 1e-7) {
            c.n_prop_err += 1;
            if (mx > c.prop_err_reported) c.prop_err_reported = mx;
            DQMC_MS_PUSH(c.ms_prop, mx);
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
                const bool was_res = x.s->gres || x.s->gdfg;
                if (was_res) g_to_global(x);
                copy_mats(x, c.Ur, ustk(x, idx + 1));
                copy_vecs(x, c.Dr, dstk(x, idx + 1));
                copy_mats(x, c.Tr, tstk(x, idx + 1));
                __syncthreads();
                add_slice_sequence_left(x, idx);
                copy_mats(x, c.Ul, ustk(x, idx + 1));
                copy_vecs(x, c.Dl, dstk(x, idx + 1));
                copy_mats(x, c.Tl, tstk(x, idx + 1));
                long long t0 = phase_start();
                if (c.check_prop) copy_mats(x, c.Gtmp, c.G);
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
                const bool was_res = x.s->gres || x.s->gdfg;
                if (was_res) g_to_global(x);
                copy_mats(x, c.Ul, ustk(x, idx));
                copy_vecs(x, c.Dl, dstk(x, idx));
                copy_mats(x, c.Tl, tstk(x, idx));
                __syncthreads();
                add_slice_sequence_right(x, idx);
                copy_mats(x, c.Ur, ustk(x, idx));
                copy_vecs(x, c.Dr, dstk(x, idx));
                copy_mats(x, c.Tr, tstk(x, idx));
                long long t0 = phase_start();
                if (c.check_prop) copy_mats(x, c.Gtmp, c.G);
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
    for (int b = x.b0; b < x.b1; ++b) {
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

// flush_delayed for a mixed chain whose global G holds float pairs (n > 64):
// G -= U W in double-float arithmetic on the FP32 pipe.  W's p rows are split
// into float pairs once (in the arena, free on such chains), each thread keeps
// the pairs of -U for its row in registers; per element the p products are
// summed exactly-rounded in a float pair (TwoProd by fmaf, TwoSum) with the
// cross terms in FP32, then added to G with one TwoSum: no FP64 instruction
// beyond the O(p n) splits.
// one term u w of flush_delayed_df's sum: the leading products summed
// exactly rounded in (sh, sl) (TwoProd by fmaf, TwoSum), the cross terms in xx
__device__ __forceinline__ void df_delay_term(float2 u, float2 w, float& sh, float& sl, float& xx) {
    const float pr = __fmul_rn(u.x, w.x);
    const float pe = __fmaf_rn(u.x, w.x, -pr);
    const float t = __fadd_rn(sh, pr);
    const float z = __fsub_rn(t, sh);
    const float er = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, z)), __fsub_rn(pr, z));
    sh = t;
    sl = __fadd_rn(sl, __fadd_rn(er, pe));
    xx = __fmaf_rn(u.x, w.y, __fmaf_rn(u.y, w.x, xx));
}
// (gv.x + gv.y) + (sh + (sl + xx)): TwoSum of the leading parts
__device__ __forceinline__ float2 df_delay_add(float2 gv, float sh, float sl, float xx) {
    const float s = __fadd_rn(gv.x, sh);
    const float z = __fsub_rn(s, gv.x);
    const float er = __fadd_rn(__fsub_rn(gv.x, __fsub_rn(s, z)), __fsub_rn(sh, z));
    return df_norm(s, __fadd_rn(__fadd_rn(gv.y, __fadd_rn(sl, xx)), er));
}
__device__ void flush_delayed_df(const Ctx& x, int p) {
    const int n = x.n;
    float2* wdf = arena_df(x);  // p * n pairs <= 16 * 256 (32 KB of the arena)
    for (int b = x.b0; b < x.b1; ++b) {
        float2* g = gdf_ptr(x) + (size_t)b * x.nn;
        const double* U = x.c->tmp2 + (size_t)b * x.nn;
        const double* W = x.c->currU + (size_t)b * x.nn;
        for (int e = threadIdx.x; e < p * n; e += DQMC_NT) wdf[e] = d_to_df(W[e]);
        __syncthreads();
        for (int k = threadIdx.x & 63; k < n; k += 64) {
            float2 uk[DQMC_DELAY];
#pragma unroll
            for (int m = 0; m < DQMC_DELAY; ++m)
                uk[m] = m < p ? d_to_df(-U[(size_t)m * n + k]) : make_float2(0.f, 0.f);
            // four columns of the thread's stride at a time: four independent
            // dependency chains, and their G entries loaded before the sums
            // (a column past n repeats the first one and is not stored)
            constexpr int LS = DQMC_NT / 64, NC = 4;
            for (int l = threadIdx.x >> 6; l < n; l += NC * LS) {
                int lc[NC];
                float2 gv[NC];
                float sh[NC], sl[NC], xx[NC];
#pragma unroll
                for (int q = 0; q < NC; ++q) {
                    lc[q] = l + q * LS < n ? l + q * LS : l;
                    gv[q] = g[(size_t)k + (size_t)lc[q] * n];
                    sh[q] = sl[q] = xx[q] = 0.f;
                }
#pragma unroll
                for (int m = 0; m < DQMC_DELAY; ++m) {
                    if (m < p) {
#pragma unroll
                        for (int q = 0; q < NC; ++q)
                            df_delay_term(uk[m], wdf[(size_t)m * n + lc[q]], sh[q], sl[q], xx[q]);
                    }
                }
#pragma unroll
                for (int q = 0; q < NC; ++q)
                    if (q == 0 || lc[q] != l)
                        g[(size_t)k + (size_t)lc[q] * n] = df_delay_add(gv[q], sh[q], sl[q], xx[q]);
            }
        }
        __syncthreads();
    }
}

__device__ __forceinline__ void flush_pending(const Ctx& x, int p, bool df) {
    if (df) flush_delayed_df(x, p);
    else flush_delayed(x, p);
}

// Flavour-split chain: bring the partner's block of the diagonal mirror into
// this CTA's after a rendezvous (accepted site j >= 0: rank 0 first writes
// the site's new field, `xflip_val`, now that both have read the old one);
// a second rendezvous keeps the partner from changing its mirror before this
// CTA has read it.
__device__ void pull_peer_diag(const Ctx& x, double* diag, int j) {
    if (!xsync(x)) return;
    if (j >= 0 && x.b0 == 0 && threadIdx.x == 0)
        x.c->conf[(size_t)(x.c->current_slice - 1) * x.n + j] = (int8_t)x.s->xflip_val;
    const int pb = 1 - x.b0, n = x.n;
    const uint32_t base = peer_addr(diag + pb * n, x.peer);
    for (int k = threadIdx.x; k < n; k += DQMC_NT) diag[pb * n + k] = peer_ld(base + 8u * k);
    xsync(x);
}

// sweep_spatial on a complex chain (local_updates.jl:23-60 with the complex
// calculate_detratio! methods, fields.jl:63-66 and 128-140, vldiv22!,
// fields.jl:215-227, and update_greens!, fields.jl:271-286) on the real
// representation E of G (n = 2 ns).  An accepted move at site j updates
// G -= u v^T with u = (I - G)[:, j], v = (Delta/R) G[j, :]; on E that is the
// rank-2 update E -= a1 b1^T + a2 b2^T with a1 = [Re u; Im u],
// a2 = [-Im u; Re u], b1 = [Re v, -Im v], b2 = [Im v, Re v], all formed from
// the left half [X; Y] of E.
// Thread 0 decides in the reference's complex operation order from a
// shared-memory mirror of G_jj = (E[j, j], E[ns+j, j]); the update vectors are
// formed from E (plus the pending updates when E is in global memory) and
// applied as in sweep_spatial.
__device__ __noinline__ long long sweep_spatial_cplx(const Ctx& x) {
    DqmcChain& c = *x.c;
    const int n = x.n, nf = x.nf, m = c.ns;
    const int slice = c.current_slice;
    int8_t* s = c.conf + (size_t)(slice - 1) * m;
    const bool ghq = (c.kind >= 2);
    const bool twoflv = (nf == 2);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    double* diag = x.s->ev;  // [b*n + k]: Re G_b[k, k]; [b*n + m + k]: Im G_b[k, k]
    for (int e = tid; e < nf * m; e += DQMC_NT) {
        const int b = e / m, k = e % m;
        const size_t at = (size_t)b * x.nn + (size_t)k * n + k;
        diag[b * n + k] = c.G[at];
        diag[b * n + m + k] = c.G[at + m];
    }
    __syncthreads();
    // per block b: a1, a2, b1, b2 at vec + (4 b + q) n (4 nf n <= 2048 doubles)
    double* vec = &x.s->r1.col[0][0];
    long long acc_count = 0;
    int i = 0, round = 0;
    const bool delayed = !x.s->gres;
    const int kcap = n < DQMC_DELAY ? n : DQMC_DELAY;  // even: two columns per accepted move
    int pending = 0;
    while (true) {
        if (tid == 0) {
            int j = i;
            for (; j < m; ++j) {
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
                const double dre[2] = {c.delta0[t], c.delta1[t]};
                const double dim[2] = {c.delta0i[t], c.delta1i[t]};
                double Rr[2] = {0.0, 0.0}, Ri[2] = {0.0, 0.0};
                double detr, deti;
                if (!twoflv) {
                    // R = 1.0 + Delta * (1.0 - G[i, i]); detratio = R * R
                    const double o_r = __dsub_rn(1.0, diag[j]), o_i = -diag[m + j];
                    const double pr = __dsub_rn(__dmul_rn(dre[0], o_r), __dmul_rn(dim[0], o_i));
                    const double pi = __dadd_rn(__dmul_rn(dre[0], o_i), __dmul_rn(dim[0], o_r));
                    Rr[0] = __dadd_rn(1.0, pr);
                    Ri[0] = pi;
                    detr = __dsub_rn(__dmul_rn(Rr[0], Rr[0]), __dmul_rn(Ri[0], Ri[0]));
                    deti = __dadd_rn(__dmul_rn(Rr[0], Ri[0]), __dmul_rn(Ri[0], Rr[0]));
                } else {
                    // R.re = 1 + Dr (1 - G.re) + Di G.im; R.im = Di (1 - G.re) - Dr G.im;
                    // detratio = prod(R)
                    for (int b = 0; b < 2; ++b) {
                        const double omg = __dsub_rn(1.0, diag[b * n + j]);
                        const double gim = diag[b * n + m + j];
                        Rr[b] = __dadd_rn(__dadd_rn(1.0, __dmul_rn(dre[b], omg)),
                                          __dmul_rn(dim[b], gim));
                        Ri[b] = __dsub_rn(__dmul_rn(dim[b], omg), __dmul_rn(dre[b], gim));
                    }
                    detr = __dsub_rn(__dmul_rn(Rr[0], Rr[1]), __dmul_rn(Ri[0], Ri[1]));
                    deti = __dadd_rn(__dmul_rn(Rr[0], Ri[1]), __dmul_rn(Ri[0], Rr[1]));
                }
                if (ghq) {  // detratio * gamma[x_new] / gamma[x_old]
                    detr = __ddiv_rn(__dmul_rn(detr, gr), gq);
                    deti = __ddiv_rn(__dmul_rn(deti, gr), gq);
                }
                // p = exp(-dE_boson) * detratio
                const double wr = c.wboson[t], wi = c.wbosoni[t];
                const double p = __dsub_rn(__dmul_rn(wr, detr), __dmul_rn(wi, deti));
                const double pim = __dadd_rn(__dmul_rn(wr, deti), __dmul_rn(wi, detr));
                if (fabs(pim) > 1e-6) {
                    c.n_imag_p += 1;
                    if (fabs(pim) > c.max_imag_p) c.max_imag_p = fabs(pim);
                    DQMC_MS_PUSH(c.ms_imag, pim);
                }
                if (p < 0.0) {
                    c.n_neg_p += 1;
                    DQMC_MS_PUSH(c.ms_neg, p);
                }
                int accept;
                if (p > 1.0) {
                    accept = 1;
                } else {
                    const uint64_t w = dqmc_philox_word(c.key, c.ctr);
                    c.ctr += 1;
                    const double u = dqmc_word_to_uniform(w);
                    accept = u < p;
                    note_tie(c, u, p);
                }
                c.proposals += 1;
                if (accept) {
                    // invRDelta_b = Delta_b / R_b = f (Delta conj(R)), f = 1 / |R|^2
                    for (int b = 0; b < nf; ++b) {
                        const double f =
                            1.0 / (Rr[b] * Rr[b] + Ri[b] * Ri[b]);
                        x.s->sxd[2 * b] = f * (dre[b] * Rr[b] + dim[b] * Ri[b]);
                        x.s->sxd[2 * b + 1] = f * (dim[b] * Rr[b] - dre[b] * Ri[b]);
                    }
                    s[j] = ghq ? (int8_t)xnew : (int8_t)(-s[j]);
                    c.accepted += 1;
                    break;
                }
            }
            x.s->sxi[2 + (round & 1)] = j;
        }
        __syncthreads();  // also: the previous round's update is complete
        const int j = x.s->sxi[2 + (round & 1)];
        ++round;
        if (j >= m) {
            if (pending > 0) flush_delayed(x, pending);
            break;
        }
        acc_count += 1;
        // every vector from the left half [X; Y] of E only (column j and
        // rows j, m + j of its first m columns): the increment is then the
        // representation of the complex update even where rounding has left
        // E slightly off the subspace, so no such component is amplified
        for (int e = tid; e < nf * m; e += DQMC_NT) {
            const int b = e / m, k = e % m;
            const double* g = c.G + (size_t)b * x.nn;
            double xc = g[(size_t)j * n + k];      // X[k, j] = E[k, j]
            double yc = g[(size_t)j * n + m + k];  // Y[k, j] = E[m + k, j]
            double xr = g[(size_t)k * n + j];      // X[j, k] = E[j, k]
            double yr = g[(size_t)k * n + m + j];  // Y[j, k] = E[m + j, k]
            if (delayed) {
                const double* U = c.tmp2 + (size_t)b * x.nn;
                const double* W = c.currU + (size_t)b * x.nn;
                for (int q = 0; q < pending; ++q) {
                    const double* u = U + (size_t)q * n;
                    const double* w = W + (size_t)q * n;
                    xc = fma(-u[k], w[j], xc);
                    yc = fma(-u[m + k], w[j], yc);
                    xr = fma(-u[j], w[k], xr);
                    yr = fma(-u[m + j], w[k], yr);
                }
            }
            // u = e_j - G[:, j]; v = w G[j, :]
            const double ur = (k == j ? 1.0 : 0.0) - xc, ui = -yc;
            const double wr = x.s->sxd[2 * b], wi = x.s->sxd[2 * b + 1];
            const double vr = wr * xr - wi * yr, vi = wr * yr + wi * xr;
            double* v = vec + (size_t)4 * b * n;
            v[k] = ur;           // a1 = [ur; ui]
            v[m + k] = ui;
            v[n + k] = -ui;      // a2 = [-ui; ur]
            v[n + m + k] = ur;
            v[2 * n + k] = vr;   // b1 = [vr, -vi]
            v[2 * n + m + k] = -vi;
            v[3 * n + k] = vi;   // b2 = [vi, vr]
            v[3 * n + m + k] = vr;
            if (delayed) {
                double* U = c.tmp2 + (size_t)b * x.nn + (size_t)pending * n;
                double* W = c.currU + (size_t)b * x.nn + (size_t)pending * n;
                U[k] = ur;
                U[m + k] = ui;
                U[n + k] = -ui;
                U[n + m + k] = ur;
                W[k] = vr;
                W[m + k] = -vi;
                W[n + k] = vi;
                W[n + m + k] = vr;
            }
        }
        __syncthreads();
        if (warp == 0) {  // the mirrored diagonal, with the same fused operations as E
            for (int e = lane; e < nf * m; e += 32) {
                const int b = e / m, k = e % m;
                const double* v = vec + (size_t)4 * b * n;
                double re = diag[b * n + k], im = diag[b * n + m + k];
                re = fma(-v[k], v[2 * n + k], re);
                re = fma(-v[n + k], v[3 * n + k], re);
                im = fma(-v[m + k], v[2 * n + k], im);
                im = fma(-v[n + m + k], v[3 * n + k], im);
                diag[b * n + k] = re;
                diag[b * n + m + k] = im;
            }
            __syncwarp();
        }
        if (delayed) {
            pending += 2;
            if (pending == kcap) {
                __syncthreads();
                flush_delayed(x, pending);
                pending = 0;
            }
            i = j + 1;
            continue;
        }
        if (warp != 0) {
            const int w = tid - 32, nw = DQMC_NT / 32 - 1;
            for (int b = 0; b < nf; ++b) {
                double* g = c.G + (size_t)b * x.nn;
                const double* v = vec + (size_t)4 * b * n;
                for (int k = w & 31; k < n; k += 32) {
                    const double na1 = -v[k], na2 = -v[n + k];
                    for (int l = w >> 5; l < n; l += nw) {
                        double y = g[k + (size_t)l * n];
                        y = fma(na1, v[2 * n + l], y);
                        y = fma(na2, v[3 * n + l], y);
                        g[k + (size_t)l * n] = y;
                    }
                }
            }
        }
        i = j + 1;
    }
    return acc_count;
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
    if (x.c->cplx) return sweep_spatial_cplx(x);
    DqmcChain& c = *x.c;
    const int n = x.n, nf = x.nf;
    const int slice = c.current_slice;
    int8_t* s = c.conf + (size_t)(slice - 1) * n;
    const bool ghq = (c.kind >= 2);
    const bool twoflv = (nf == 2);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    double* diag = x.s->ev;  // [nf * n] mirror of the diagonals (ev is free here)
    // mixed chain with G resident: G is double-float; decisions still use FP64
    // values (the diagonal and the update vectors are formed in FP64), the
    // n x n rank-1 update runs in double-float on the FP32 pipe
    const bool dfg = df_resident(x);
    const float2* gdf = gdf_ptr(x);
    const int e0 = x.b0 * n, e1 = x.b1 * n;  // the owned blocks' entries
    for (int e = e0 + tid; e < e1; e += DQMC_NT) {
        const int b = e / n, k = e % n;
        const size_t at = (size_t)b * x.nn + (size_t)k * n + k;
        diag[e] = dfg ? df_to_d(gdf[at]) : c.G[at];
    }
    // the slice's fields as the decisions read them (a shared-memory copy:
    // the decision loop's serial chain then waits on no global load; `sv` is
    // free during the local sweep); a site is not read again after it flips
    int8_t* sc = reinterpret_cast<int8_t*>(x.s->sv);
    for (int k = tid; k < n; k += DQMC_NT) sc[k] = (int8_t)conf_at(s, k, split(x));
    __syncthreads();
    if (split(x)) pull_peer_diag(x, diag, -1);
    long long acc_count = 0;
    int i = 0, round = 0;
    // G in global memory: delay the rank-1 updates and apply them DQMC_DELAY
    // at a time (one pass over G instead of one per accepted move)
    const bool delayed = !x.s->gres;
    const int kcap = n < DQMC_DELAY ? n : DQMC_DELAY;  // U, W columns fit the n*n scratch
    int pending = 0;
    while (true) {
        if (!ghq && warp == 0) {
            // Hirsch fields: warp 0 evaluates up to 32 proposals at once.  From
            // site i on, lane k computes the ratio of site i + k on the current
            // diagonal (valid for every site up to the first acceptance, which
            // alone changes it), takes its uniform at the counter the
            // sequential loop would reach (a ballot and prefix count of the
            // proposals with p <= 1 before it), and the first accepting lane
            // wins: the sequential loop's decisions and draws exactly.
            uint64_t ctr = c.ctr;
            long long props = c.proposals, ties = c.n_near_tie;
            double tie_gap = c.min_tie_gap;
            int j = i, win = n;
            const unsigned FULL = 0xffffffffu, below = (1u << lane) - 1u;
            while (j < n) {
                const int jj = j + lane;
                const bool valid = jj < n;
                double p = 0.0, R0 = 1.0, R1 = 1.0, d0 = 0.0, d1 = 0.0;
                if (valid) {
                    const int t = sc[jj] > 0 ? 1 : 0;
                    d0 = c.delta0[t];
                    d1 = c.delta1[t];
                    R0 = __dadd_rn(1.0, __dmul_rn(d0, __dsub_rn(1.0, diag[jj])));
                    double detratio;
                    if (twoflv) {
                        R1 = __dadd_rn(1.0, __dmul_rn(d1, __dsub_rn(1.0, diag[n + jj])));
                        detratio = __dmul_rn(R0, R1);
                    } else {
                        detratio = __dmul_rn(R0, R0);
                    }
                    p = __dmul_rn(c.wboson[t], detratio);
                }
                const unsigned need = __ballot_sync(FULL, valid && !above_one(p));
                bool acc = false;
                double gap = INFINITY;  // |u - p| of this lane's drawn uniform
                if (valid) {
                    if (above_one(p)) {
                        acc = true;
                    } else {
                        const uint64_t w = dqmc_philox_word(c.key, ctr + (uint64_t)__popc(need & below));
                        const long long ub = uniform_bits(w);
                        acc = uniform_below(ub, p);
                        gap = fabs(__longlong_as_double(ub) - p);
                    }
                }
                const unsigned am = __ballot_sync(FULL, acc);
                const unsigned vm = __ballot_sync(FULL, valid);
                const int last = am ? __ffs(am) - 1 : 31 - __clz(vm);  // last proposal made
                const unsigned done = last == 31 ? FULL : ((2u << last) - 1u);
                // near ties and the smallest gap of the proposals made (the
                // gaps' bit patterns compared on the integer pipe)
                ties += __popc(__ballot_sync(FULL, gap < DQMC_NEAR_TIE) & done);
                long long gb = ((done >> lane) & 1u) ? __double_as_longlong(gap)
                                                     : __double_as_longlong(INFINITY);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    const long long og = __shfl_xor_sync(FULL, gb, o);
                    gb = og < gb ? og : gb;
                }
                const double gmin = __longlong_as_double(gb);
                if (gmin < tie_gap) tie_gap = gmin;
                // negative probabilities of the proposals made, in order
                unsigned neg = __ballot_sync(FULL, valid && below_zero(p)) & done;
                while (neg) {
                    const int k = __ffs(neg) - 1;
                    const double pk = __shfl_sync(FULL, p, k);
                    if (lane == 0) {
                        c.n_neg_p += 1;
                        DQMC_MS_PUSH(c.ms_neg, pk);
                    }
                    neg &= neg - 1u;
                }
                ctr += (uint64_t)__popc(need & done);
                props += __popc(vm & done);
                if (am) {
                    win = j + last;
                    if (lane == last) {  // accept_local! of site `win`
                        x.s->sxd[0] = __ddiv_rn(d0, R0);
                        x.s->sxd[1] = twoflv ? __ddiv_rn(d1, R1) : 0.0;
                        const int8_t flipped = (int8_t)(-sc[win]);
                        if (split(x)) x.s->xflip_val = (int)flipped;
                        else s[win] = flipped;
                        c.accepted += 1;
                    }
                    break;
                }
                j += 32;
            }
            if (lane == 0) {
                c.ctr = ctr;
                c.proposals = props;
                c.n_near_tie = ties;
                c.min_tie_gap = tie_gap;
                x.s->sxi[2 + (round & 1)] = win;
            }
        } else if (tid == 0) {
            // the chain's counters in registers for the loop
            uint64_t ctr = c.ctr;
            long long props = c.proposals, ties = c.n_near_tie;
            double tie_gap = c.min_tie_gap;
            int j = i;
            for (; j < n; ++j) {
                const double g0 = diag[j];
                const double g1 = twoflv ? diag[n + j] : 0.0;
                int t;
                int xnew = 0;
                double gr = 1.0, gq = 1.0;
                if (ghq) {
                    const int xold = sc[j];
                    const uint64_t w = dqmc_philox_word(c.key, ctr);
                    ctr += 1;
                    const int r = dqmc_word_to_choice3(w);
                    xnew = r + (r + 1 >= xold ? 2 : 1);  // choices[x_old, r+1] (fields.jl:534)
                    t = (xold - 1) * 4 + (xnew - 1);
                    gr = c.gam[xnew - 1];
                    gq = c.gam[xold - 1];
                } else {
                    t = sc[j] > 0 ? 1 : 0;
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
                // the uniform's word, drawn only when p <= 1 but computed
                // ahead (it does not depend on p)
                const uint64_t wu = dqmc_philox_word(c.key, ctr);
                const double p = __dmul_rn(c.wboson[t], detratio);
                if (below_zero(p)) {
                    c.n_neg_p += 1;
                    DQMC_MS_PUSH(c.ms_neg, p);
                }
                int accept;
                if (above_one(p)) {
                    accept = 1;
                } else {
                    ctr += 1;
                    const long long ub = uniform_bits(wu);
                    accept = uniform_below(ub, p);
                    const double gap = fabs(__longlong_as_double(ub) - p);  // note_tie
                    if (gap < DQMC_NEAR_TIE) ties += 1;
                    if (gap < tie_gap) tie_gap = gap;
                }
                props += 1;
                if (accept) {
                    x.s->sxd[0] = __ddiv_rn(d0, R0);
                    x.s->sxd[1] = twoflv ? __ddiv_rn(d1, R1) : 0.0;
                    const int8_t flipped = ghq ? (int8_t)xnew : (int8_t)(-sc[j]);
                    // a flavour-split chain flips after the partner has read
                    // the site (rank 0 alone writes the configuration)
                    if (split(x)) x.s->xflip_val = (int)flipped;
                    else s[j] = flipped;
                    c.accepted += 1;
                    break;
                }
            }
            c.ctr = ctr;
            c.proposals = props;
            c.n_near_tie = ties;
            c.min_tie_gap = tie_gap;
            // double-buffered slot: thread 0 writes the next round's slot
            // while slow threads may still read this one
            x.s->sxi[2 + (round & 1)] = j;
        }
        __syncthreads();  // also: the previous round's update is complete
        const int j = x.s->sxi[2 + (round & 1)];
        ++round;
        if (j >= n) {
            if (pending > 0) flush_pending(x, pending, dfg);
            break;
        }
        acc_count += 1;
        for (int e = e0 + tid; e < e1; e += DQMC_NT) {
            const int b = e / n, k = e % n;
            const double* g = c.G + (size_t)b * x.nn;
            double gkj, gjk;
            if (dfg) {
                const float2* gb = gdf + (size_t)b * x.nn;
                gkj = df_to_d(gb[(size_t)j * n + k]);
                gjk = df_to_d(gb[(size_t)k * n + j]);
            } else {
                gkj = g[(size_t)j * n + k];
                gjk = g[(size_t)k * n + j];
            }
            if (delayed) {
                // current G[k, j] and G[j, k] with the pending updates applied
                // (in the order m = 0, 1, ...); the loads of a batch of eight
                // terms are issued together (one L2 round trip per batch, not
                // per term)
                const double* U = c.tmp2 + (size_t)b * x.nn;
                const double* W = c.currU + (size_t)b * x.nn;
#pragma unroll
                for (int m0 = 0; m0 < DQMC_DELAY; m0 += 8) {
                    if (m0 >= pending) break;
                    double uk[8], wk[8], uj[8], wj[8];
#pragma unroll
                    for (int m = 0; m < 8; ++m) {
                        const bool on = m0 + m < pending;
                        const size_t r = (size_t)(m0 + m) * n;
                        uk[m] = on ? U[r + k] : 0.0;
                        wk[m] = on ? W[r + k] : 0.0;
                        uj[m] = on ? U[r + j] : 0.0;
                        wj[m] = on ? W[r + j] : 0.0;
                    }
#pragma unroll
                    for (int m = 0; m < 8; ++m) {
                        if (m0 + m < pending) {
                            gkj = fma(-uk[m], wj[m], gkj);
                            gjk = fma(-uj[m], wk[m], gjk);
                        }
                    }
                }
            }
            double ig = -gkj;
            if (k == j) ig += 1.0;
            const double rw = x.s->sxd[b] * gjk;
            x.s->r1.col[b][k] = ig;
            x.s->r1.row[b][k] = rw;
            if (dfg && !delayed) {  // float pairs of -col and row behind the FP64 vectors
                reinterpret_cast<float2*>(x.s->r1.col[b] + 256)[k] = d_to_df(-ig);
                reinterpret_cast<float2*>(x.s->r1.row[b] + 256)[k] = d_to_df(rw);
            }
            if (delayed) {
                c.tmp2[(size_t)b * x.nn + (size_t)pending * n + k] = ig;
                c.currU[(size_t)b * x.nn + (size_t)pending * n + k] = rw;
            }
        }
        __syncthreads();
        if (delayed) {
            if (warp == 0) {
                for (int e = e0 + lane; e < e1; e += 32) {
                    const int b = e / n, k = e % n;
                    diag[e] = fma(-x.s->r1.col[b][k], x.s->r1.row[b][k], diag[e]);
                }
                __syncwarp();
            }
            ++pending;
            if (pending == kcap) {
                __syncthreads();
                flush_pending(x, pending, dfg);
                pending = 0;
            }
            if (split(x)) pull_peer_diag(x, diag, j);
            i = j + 1;
            continue;
        }
        if (warp == 0) {
            for (int e = e0 + lane; e < e1; e += 32) {
                const int b = e / n, k = e % n;
                diag[e] = fma(-x.s->r1.col[b][k], x.s->r1.row[b][k], diag[e]);
            }
            __syncwarp();
        } else if (dfg) {
            const int w = tid - 32, nw = DQMC_NT / 32 - 1;
            for (int b = x.b0; b < x.b1; ++b) {
                float2* g = arena_df(x) + (size_t)b * x.nn;
                const float2* cl = reinterpret_cast<const float2*>(x.s->r1.col[b] + 256);
                const float2* rw = reinterpret_cast<const float2*>(x.s->r1.row[b] + 256);
                for (int k = w & 31; k < n; k += 32) {
                    const float2 ck = cl[k];
                    for (int l = w >> 5; l < n; l += nw)
                        g[k + (size_t)l * n] = df_fma(ck, rw[l], g[k + (size_t)l * n]);
                }
            }
        } else {
            const int w = tid - 32, nw = DQMC_NT / 32 - 1;
            for (int b = x.b0; b < x.b1; ++b) {
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
        if (split(x)) pull_peer_diag(x, diag, j);
        i = j + 1;
    }
    return acc_count;
}

// the UDT chains of calculate_greens(mc, slice, ...) (stack.jl:525-583) and
// of inv_det (global_updates.jl:65-133): Ur,Dr,Tr = B(slice+1)'...B(M)' and
// Ul,Dl,Tl = B(slice)...B(1), stabilised every safe_mult slices
__device__ __noinline__ void udt_chains_from_scratch(const Ctx& x, int slice, int safe_mult) {
    DqmcChain& c = *x.c;
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
}

// calculate_greens(mc, slice, output, field, safe_mult) (stack.jl:525-583)
__device__ __noinline__ void calculate_greens_at(const Ctx& x, int slice, int safe_mult, double* out) {
    if (safe_mult <= 0) safe_mult = x.c->k;
    udt_chains_from_scratch(x, slice, safe_mult);
    calculate_greens(x, out);
}

// ---- global updates ---------------------------------------------------------

// sum of a configuration's entries (exact), all threads get it
__device__ long long conf_sum(const Ctx& x, const int8_t* conf) {
    const int cnt = x.n * x.c->M;
    long long v = 0;
    for (int e = threadIdx.x; e < cnt; e += DQMC_NT) v += conf[e];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    long long* red = reinterpret_cast<long long*>(x.s->red);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    long long t = 0;
    for (int w = 0; w < DQMC_NW; ++w) t += red[w];
    __syncthreads();
    return t;
}

// propose_global_from_conf (global_updates.jl:137-166) for the proposal
// `prop` replacing `old`, at current_slice 1: tempvf = Dl of the current G,
// inv_det(current_slice - 1) with the proposal (G_tmp as scratch, so G is
// untouched), detratio = prod tempvf_i Dr_i (squared for one flavour block),
// Delta E_boson = E(prop) - E(old) (fields.jl:395, 451, 544, 614).  Returns
// p = exp(-Delta E) detratio to thread 0 (sxd[1]).
__device__ __noinline__ void global_weight(const Ctx& x, const int8_t* prop, const int8_t* old) {
    DqmcChain& c = *x.c;
    const int cnt = x.nf * x.n;
    copy(cnt, c.tempvf, c.Dl);
    __syncthreads();
    int8_t* own = c.conf;
    if (threadIdx.x == 0) c.conf = const_cast<int8_t*>(prop);  // the slice matrices read c.conf
    __syncthreads();
    udt_chains_from_scratch(x, c.current_slice - 1, c.k);
    calculate_greens(x, c.Gtmp, false);
    __syncthreads();
    if (threadIdx.x == 0) c.conf = own;
    const bool dens = (c.kind == 0 || c.kind == 2);
    const long long s_new = dens ? conf_sum(x, prop) : 0;
    const long long s_old = dens ? conf_sum(x, old) : 0;
    if (threadIdx.x == 0) {
        double detratio = 1.0;
        for (int i = 0; i < cnt; ++i) detratio = __dmul_rn(detratio, __dmul_rn(c.tempvf[i], c.Dr[i]));
        const double dE = dens ? __dsub_rn(__dmul_rn(c.alpha_field, (double)s_new),
                                           __dmul_rn(c.alpha_field, (double)s_old))
                               : 0.0;
        if (x.nf == 1) detratio = __dmul_rn(detratio, detratio);
        x.s->sxd[1] = __dmul_rn(exp(-dE), detratio);
    }
    __syncthreads();
}

// global_update (global_updates.jl:188-203) after propose_conf! of
// GlobalFlip (kind 0, :244-256: s -> -s, GHQ x -> 5 - x) or GlobalShuffle
// (kind 1, :270-278: Fisher-Yates over the whole configuration with
// j = floor(w (i+1) / 2^64) from the chain's stream, i = nM-1 ... 1);
// accepted: accept_global! (:169-185: full rebuild), rejected: the old
// configuration back.  G must be in global memory.
__device__ __noinline__ void global_update(const Ctx& x, int kind) {
    DqmcChain& c = *x.c;
    const int cnt = x.n * c.M;
    const bool ghq = c.kind >= 2;
    for (int e = threadIdx.x; e < cnt; e += DQMC_NT) c.temp_conf[e] = c.conf[e];
    __syncthreads();
    if (kind == 0) {
        for (int e = threadIdx.x; e < cnt; e += DQMC_NT)
            c.conf[e] = ghq ? (int8_t)(5 - c.temp_conf[e]) : (int8_t)(-c.temp_conf[e]);
    } else if (threadIdx.x == 0) {
        for (int i = cnt - 1; i >= 1; --i) {
            const uint64_t w = dqmc_philox_word(c.key, c.ctr);
            c.ctr += 1;
            const int j = (int)__umul64hi(w, (unsigned long long)(i + 1));
            const int8_t t = c.conf[i];
            c.conf[i] = c.conf[j];
            c.conf[j] = t;
        }
    }
    __syncthreads();
    global_weight(x, c.conf, c.temp_conf);
    if (threadIdx.x == 0) {
        const double p = fabs(x.s->sxd[1]);
        int acc = 1;
        if (!(p > 1.0)) {
            const uint64_t w = dqmc_philox_word(c.key, c.ctr);
            c.ctr += 1;
            acc = dqmc_word_to_uniform(w) < p;
        }
        c.g_proposals += 1;
        c.g_accepted += acc;
        x.s->sxi[0] = acc;
    }
    __syncthreads();
    if (x.s->sxi[0]) {
        reverse_build_stack(x);
        propagate(x);
    } else {
        for (int e = threadIdx.x; e < cnt; e += DQMC_NT) c.conf[e] = c.temp_conf[e];
        __syncthreads();
    }
}

// ReplicaExchange (parallel_updates.jl:116-150) between chains of one launch,
// step 1: the weight exp(-Delta E) detratio of adopting the partner's
// configuration (copied into temp_conf: the partner's own buffer is only read)
// and one uniform draw.  Nothing of the chain's configuration or G changes.
__device__ __noinline__ void replica_weight(const Ctx& x, const DqmcChain* all) {
    DqmcChain& c = *x.c;
    const int cnt = x.n * c.M;
    const int8_t* pc = all[c.partner].conf;
    for (int e = threadIdx.x; e < cnt; e += DQMC_NT) c.temp_conf[e] = pc[e];
    __syncthreads();
    global_weight(x, c.temp_conf, c.conf);
    if (threadIdx.x == 0) {
        c.r_weight = x.s->sxd[1];
        const uint64_t w = dqmc_philox_word(c.key, c.ctr);
        c.ctr += 1;
        c.r_prob = dqmc_word_to_uniform(w);
    }
    __syncthreads();
}

// step 2 (a later launch, so both weights are final): w = w_self w_partner,
// the lower chain index's uniform decides for both; accepted chains take the
// partner's configuration (from temp_conf) and rebuild.
__device__ __noinline__ void replica_accept(const Ctx& x, const DqmcChain* all, int self) {
    DqmcChain& c = *x.c;
    const DqmcChain& q = all[c.partner];
    if (threadIdx.x == 0) {
        const double w = __dmul_rn(c.r_weight, q.r_weight);
        const double u = self < c.partner ? c.r_prob : q.r_prob;
        const int acc = u < w;
        c.g_proposals += 1;
        c.g_accepted += acc;
        x.s->sxi[0] = acc;
    }
    __syncthreads();
    if (x.s->sxi[0]) {
        const int cnt = x.n * c.M;
        for (int e = threadIdx.x; e < cnt; e += DQMC_NT) c.conf[e] = c.temp_conf[e];
        __syncthreads();
        reverse_build_stack(x);
        propagate(x);
    }
}

// _greens! (greens.jl:114-125): out = eThalfplus * (G * eThalfminus)
__device__ __noinline__ void greens_physical(const Ctx& x, const double* src, double* out) {
    DqmcChain& c = *x.c;
    for (int b = x.b0; b < x.b1; ++b) {
        if (c.cb) {
            cb_apply(x, 2, 1, blk(c.tmp1, x, b), src + (size_t)b * x.nn, blk(c.tmp2, x, b));
            cb_apply(x, 3, 0, blk(out, x, b), blk(c.tmp1, x, b), blk(c.tmp2, x, b));
            continue;
        }
        mm<false, true>(x.n, blk(c.tmp1, x, b), src + (size_t)b * x.nn, c.eTh, x.s->tiles);
        __syncthreads();
        mm<true, false>(x.n, blk(out, x, b), c.eThinv, blk(c.tmp1, x, b), x.s->tiles);
        __syncthreads();
    }
}

// One value into the log binner of scalar k: level l keeps the Welford mean
// and M2 of the completed bins of 2^l consecutive values (the binning levels
// of BinningAnalysis' LogBinner); a completed pair moves up as its mean.
// Thread 0 only.
__device__ void binner_push(double* m, int k, double v) {
    for (int l = 0; l < DQMC_MEAS_LEVELS; ++l) {
        double* b = m + DQMC_MEAS_HEADER + (k * DQMC_MEAS_LEVELS + l) * DQMC_MEAS_BIN_WORDS;
        const double cnt = b[0] + 1.0;
        const double d = v - b[1];
        b[0] = cnt;
        b[1] += d / cnt;
        b[2] += d * (v - b[1]);
        if (b[4] == 0.0) {
            b[3] = v;
            b[4] = 1.0;
            return;
        }
        v = 0.5 * (b[3] + v);
        b[4] = 0.0;
    }
}

// Equal-time measurements of the current G (the reference measures after a
// sweep, DQMC.jl:205-222), all on the device: the physical G (greens!,
// greens.jl:94-125), then per site i with d_b = G^b_ii (one block: d_2 = d_1)
//   density            (1/n) sum_i (1 - d_1) + (1 - d_2)          (occupation.jl:44-55)
//   double occupancy   (1/n) sum_i (1 - d_1)(1 - d_2)
//   interaction energy -U sum_i (d_1 - 1/2)(d_2 - 1/2)            (HubbardModel.jl:160-183)
//   S^z(q)             (1/n) sum_ij cos(q.(r_i - r_j)) <m_z(i) m_z(j)> with the
//                      equal-time Wick form of full_sdc_z_kernel (spin_density.jl:182-227):
//                      m_i m_j + (2/nf) sum_b (delta_ij - G^b_ji) G^b_ij, m_i = d_2 - d_1
// pushed into the chain's log binners, plus running sums of the occupations
// 1 - d_b and (optionally) of the physical G.
__device__ __noinline__ void measure(const Ctx& x) {
    DqmcChain& c = *x.c;
    const int n = x.n, nf = x.nf;
    const size_t nn = x.nn;
    const double* src = c.G;
    if (df_resident(x)) {  // FP64 snapshot of the double-float resident G
        double* snap = x.s->gdfg ? c.Gtmp : x.s->Gglob;
        g_resident_to(x, snap);
        __syncthreads();
        src = snap;
    }
    greens_physical(x, src, c.out);
    const double* g1 = c.out;
    const double* g2 = c.out + (size_t)(nf - 1) * nn;
    double* occ = c.meas + DQMC_MEAS_OCC_OFF;
    const double* qc = c.qcs;
    const double* qs = c.qcs ? c.qcs + n : nullptr;
    double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int i = threadIdx.x; i < n; i += DQMC_NT) {
        const double d1 = g1[(size_t)i * n + i], d2 = g2[(size_t)i * n + i];
        acc[0] += (1.0 - d1) + (1.0 - d2);
        acc[1] += (1.0 - d1) * (1.0 - d2);
        acc[2] += (d1 - 0.5) * (d2 - 0.5);
        if (qc) {
            const double m = d2 - d1;
            acc[3] += qc[i] * m;
            acc[4] += qs[i] * m;
        }
        occ[i] += 1.0 - d1;
        if (nf > 1) occ[n + i] += 1.0 - d2;
    }
    if (qc) {
        for (int b = 0; b < nf; ++b) {
            const double* g = c.out + (size_t)b * nn;
            for (int e = threadIdx.x; e < n * n; e += DQMC_NT) {
                const int i = e % n, j = e / n;
                const double w = qc[i] * qc[j] + qs[i] * qs[j];
                acc[5] += w * ((i == j ? 1.0 : 0.0) - g[(size_t)i * n + j]) * g[e];
            }
        }
    }
    if (c.meas_greens) {
        double* gs = occ + (size_t)nf * n;
        for (int e = threadIdx.x; e < nf * (int)nn; e += DQMC_NT) gs[e] += c.out[e];
    }
    // block reduction of the six partial sums through the staging tiles
    double* red = x.s->tiles;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        const double v = warp_sum(acc[q]);
        if (lane == 0) red[q * DQMC_NW + warp] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t[6];
        for (int q = 0; q < 6; ++q) {
            t[q] = 0.0;
            for (int w = 0; w < DQMC_NW; ++w) t[q] += red[q * DQMC_NW + w];
        }
        const double inv_n = 1.0 / n;
        binner_push(c.meas, 0, t[0] * inv_n);
        binner_push(c.meas, 1, t[1] * inv_n);
        binner_push(c.meas, 2, -c.meas_U * t[2]);
        binner_push(c.meas, 3, qc ? (t[3] * t[3] + t[4] * t[4] + (2.0 / nf) * t[5]) * inv_n : 0.0);
        c.meas[0] += 1.0;
    }
    __syncthreads();
}

// end of a sweep: count it and measure at the measurement points
__device__ void td_measure(const Ctx& x);

__device__ void after_sweep(const Ctx& x) {
    if (threadIdx.x == 0) x.c->sweep += 1;
    __syncthreads();
    if (x.c->meas_enable && x.c->meas && x.c->meas_rate > 0 && x.c->sweep % x.c->meas_rate == 0)
        measure(x);
    if (x.c->td_enable && x.c->td && x.c->ut && x.c->td_rate > 0 &&
        x.c->sweep % x.c->td_rate == 0) {
        // the unequal-time stack factors in the arena (n <= 64): G leaves it
        const bool was_res = x.s->gres || x.s->gdfg;
        if (was_res) g_to_global(x);
        td_measure(x);
        if (was_res) g_to_arena(x);
    }
}

}  // namespace
}  // namespace dqmc

namespace dqmc {
namespace {

// ---- unequal-time Green's function (unequal_time_stack.jl) -----------------
// calculate_greens(mc, k, l) through the UnequalTimeStack: forward, backward
// and inverse UDT stacks of the current configuration (build_stack,
// :124-178), then per (k, l) the inverse block, the forward and backward
// blocks and the stabilised combination (calculate_greens_full1! / full2!,
// :536-697).  Overwrites Ul..Tr, tmp1, tmp2, curr_U, pivot and tempv, which
// are scratch between stabilisations (as the reference documents for
// greens(mc, k, l)).

struct UtView {
    double *fu, *ft, *bu, *bt, *iu, *it, *U, *T, *G;
    double *fd, *bd, *id, *D;
};
__device__ UtView ut_view(const Ctx& x) {
    const size_t ms = (size_t)x.nf * x.nn, vs = (size_t)x.nf * x.n;
    const int nr = x.c->nr;
    double* p = x.c->ut;
    UtView v;
    v.fu = p; p += ms * (nr + 1);
    v.ft = p; p += ms * (nr + 1);
    v.bu = p; p += ms * (nr + 1);
    v.bt = p; p += ms * (nr + 1);
    v.iu = p; p += ms * nr;
    v.it = p; p += ms * nr;
    v.U = p; p += ms;
    v.T = p; p += ms;
    v.G = p; p += ms;
    v.fd = p; p += vs * (nr + 1);
    v.bd = p; p += vs * (nr + 1);
    v.id = p; p += vs * nr;
    v.D = p;
    return v;
}
__device__ __forceinline__ double* utm(const Ctx& x, double* p, int idx) {
    return p + (size_t)(idx - 1) * x.nf * x.nn;
}
__device__ __forceinline__ double* utv(const Ctx& x, double* p, int idx) {
    return p + (size_t)(idx - 1) * x.nf * x.n;
}

__device__ void mm_nt_blocks(const Ctx& x, double* C, double* A, double* B) {
    for (int b = x.b0; b < x.b1; ++b) mm<false, true>(x.n, blk(C, x, b), blk(A, x, b), blk(B, x, b), x.s->tiles);
    __syncthreads();
}
__device__ void mm_tn_blocks(const Ctx& x, double* C, double* A, double* B) {
    for (int b = x.b0; b < x.b1; ++b) mm<true, false>(x.n, blk(C, x, b), blk(A, x, b), blk(B, x, b), x.s->tiles);
    __syncthreads();
}
__device__ void dleft_blocks(const Ctx& x, double* C, const double* d, double* B) {
    for (int b = x.b0; b < x.b1; ++b) dleft(x.n, blk(C, x, b), d + b * x.n, blk(B, x, b));
    __syncthreads();
}
__device__ void rdivp_blocks(const Ctx& x, double* A, double* T, double* O) {
    if (paired(x)) {
        rdivp_pair(x, A, T, O);
        return;
    }
    for (int b = x.b0; b < x.b1; ++b)
        rdivp(x.n, blk(A, x, b), blk(T, x, b), blk(O, x, b), x.c->pivot + b * x.n, x.nf > 1, x.s->sv);
}
// vmaxinv! / vmin! (real.jl:143-170), rvadd! (:123-127), copyto!(A, Diagonal(d))
__device__ void vmaxinv_v(const Ctx& x, double* v, const double* w) {
    __syncthreads();
    for (int i = threadIdx.x; i < x.nf * x.n; i += DQMC_NT) v[i] = 1.0 / fmax(1.0, w[i]);
    __syncthreads();
}
__device__ void vmin_v(const Ctx& x, double* v, const double* w) {
    __syncthreads();
    for (int i = threadIdx.x; i < x.nf * x.n; i += DQMC_NT) v[i] = fmin(1.0, w[i]);
    __syncthreads();
}
__device__ void vinv_v(const Ctx& x, double* v) {
    __syncthreads();
    for (int i = threadIdx.x; i < x.nf * x.n; i += DQMC_NT) v[i] = 1.0 / v[i];
    __syncthreads();
}
__device__ void mat_add(const Ctx& x, double* A, const double* B) {
    for (int e = threadIdx.x; e < x.nf * (int)x.nn; e += DQMC_NT) A[e] += B[e];
    __syncthreads();
}
__device__ void mat_diag(const Ctx& x, double* A, const double* d) {
    for (int e = threadIdx.x; e < x.nf * (int)x.nn; e += DQMC_NT) {
        const int b = e / (int)x.nn, f = e % (int)x.nn, i = f % x.n, j = f / x.n;
        A[e] = (i == j) ? d[b * x.n + i] : 0.0;
    }
    __syncthreads();
}

// build_stack(mc, ::UnequalTimeStack) (:124-178)
__device__ __noinline__ void ut_build(const Ctx& x, const UtView& s) {
    DqmcChain& c = *x.c;
    const int nr = c.nr, ms = x.nf * (int)x.nn;
    mat_ident(x, utm(x, s.fu, 1));
    set_ones(x, utv(x, s.fd, 1));
    mat_ident(x, utm(x, s.ft, 1));
    mat_ident(x, utm(x, s.bu, nr + 1));
    set_ones(x, utv(x, s.bd, nr + 1));
    mat_ident(x, utm(x, s.bt, nr + 1));
    __syncthreads();
    for (int idx = 1; idx <= nr; ++idx) {
        copy(ms, c.currU, utm(x, s.fu, idx));
        __syncthreads();
        for (int sl = c.rfirst[idx - 1]; sl <= c.rlast[idx - 1]; ++sl) slice_left(x, sl, c.currU);
        dright_blocks(x, c.tmp1, c.currU, utv(x, s.fd, idx));
        udt_blocks(x, utm(x, s.fu, idx + 1), utv(x, s.fd, idx + 1), c.tmp1, true);
        mm_blocks(x, utm(x, s.ft, idx + 1), c.tmp1, utm(x, s.ft, idx));
    }
    for (int idx = nr; idx >= 1; --idx) {
        copy(ms, c.currU, utm(x, s.bu, idx + 1));
        __syncthreads();
        for (int sl = c.rlast[idx - 1]; sl >= c.rfirst[idx - 1]; --sl) slice_dagger_left(x, sl, c.currU);
        dright_blocks(x, c.tmp1, c.currU, utv(x, s.bd, idx + 1));
        udt_blocks(x, utm(x, s.bu, idx), utv(x, s.bd, idx), c.tmp1, true);
        mm_blocks(x, utm(x, s.bt, idx), c.tmp1, utm(x, s.bt, idx + 1));
    }
    for (int idx = 1; idx <= nr; ++idx) {
        double* it = utm(x, s.it, idx);
        mat_ident(x, it);
        __syncthreads();
        for (int sl = c.rlast[idx - 1]; sl >= c.rfirst[idx - 1]; --sl) slice_inv_left(x, sl, it);
        udt_blocks(x, utm(x, s.iu, idx), utv(x, s.id, idx), it, true);
    }
}

// _find_range_with_value (:354-390): chunk (1-based) holding slice val
__device__ int find_range(const Ctx& x, int val) {
    const DqmcChain& c = *x.c;
    if (val < 1) return 0;
    if (val > c.rlast[c.nr - 1]) return c.nr + 1;
    for (int i = 0; i < c.nr; ++i)
        if (c.rfirst[i] <= val && val <= c.rlast[i]) return i + 1;
    return c.nr + 1;
}

// compute_inverse_udt_block! (:400-463): U D T = B_{low+1}^-1 ... B_high^-1
__device__ __noinline__ void ut_inverse_block(const Ctx& x, const UtView& s, int low, int high) {
    DqmcChain& c = *x.c;
    const int ms = x.nf * (int)x.nn;
    const int lower = find_range(x, low) + 1, upper = find_range(x, high + 1) - 1;
    mat_ident(x, s.U);
    set_ones(x, s.D);
    mat_ident(x, s.T);
    __syncthreads();
    for (int idx = lower; idx <= upper; ++idx) {
        mm_blocks(x, c.tmp1, s.T, utm(x, s.iu, idx));
        dleft_blocks(x, c.tmp2, s.D, c.tmp1);
        dright_blocks(x, c.tmp1, c.tmp2, utv(x, s.id, idx));
        udt_blocks(x, c.tmp2, s.D, c.tmp1, true);
        mm_blocks(x, s.T, c.tmp1, utm(x, s.it, idx));
        mm_blocks(x, c.tmp1, s.U, c.tmp2);
        copy(ms, s.U, c.tmp1);
        __syncthreads();
    }
    const int lower_slice = lower <= c.nr ? c.rfirst[lower - 1] : c.rlast[c.nr - 1] + 1;
    const int upper_slice = upper > 0 ? c.rlast[upper - 1] : 0;
    const int top = min(lower_slice - 1, high);
    for (int sl = top; sl >= low + 1; --sl) slice_inv_left(x, sl, s.U);
    if (top >= low + 1) {
        dright_blocks(x, c.tmp1, s.U, s.D);
        udt_blocks(x, s.U, s.D, c.tmp1, true);
        mm_blocks(x, c.tmp2, c.tmp1, s.T);
        copy(ms, s.T, c.tmp2);
        __syncthreads();
    }
    for (int sl = max(upper_slice + 1, top + 1); sl <= high; ++sl) slice_inv_right(x, sl, s.T);
}

// compute_forward_udt_block! (:474-497): Ul Dl Tl = B_slice ... B_1
__device__ __noinline__ void ut_forward_block(const Ctx& x, const UtView& s, int slice) {
    DqmcChain& c = *x.c;
    const int idx = max(0, find_range(x, slice) - 1);
    copy_mats(x, c.Tl, utm(x, s.fu, idx + 1));
    __syncthreads();
    const int target = idx > 0 ? c.rlast[idx - 1] + 1 : 1;
    for (int l = target; l <= slice; ++l) slice_left(x, l, c.Tl);
    dright_blocks(x, c.tmp1, c.Tl, utv(x, s.fd, idx + 1));
    udt_blocks(x, c.Ul, c.Dl, c.tmp1, true);
    mm_blocks(x, c.Tl, c.tmp1, utm(x, s.ft, idx + 1));
}

// compute_backward_udt_block! (:509-533): (Ur Dr Tr)^T = B_M ... B_{slice+1}
__device__ __noinline__ void ut_backward_block(const Ctx& x, const UtView& s, int slice) {
    DqmcChain& c = *x.c;
    const int idx = find_range(x, slice) + 1;
    copy_mats(x, c.Ur, utm(x, s.bu, idx));
    __syncthreads();
    const int target = idx <= c.nr ? c.rfirst[idx - 1] - 1 : c.rlast[c.nr - 1];
    for (int l = target; l >= slice + 1; --l) slice_dagger_left(x, l, c.Ur);
    dright_blocks(x, c.tmp1, c.Ur, utv(x, s.bd, idx));
    udt_blocks(x, c.Ur, c.Dr, c.tmp1, true);
    mm_blocks(x, c.Tr, c.tmp1, utm(x, s.bt, idx));
}

// calculate_greens_full1! (:536-619), slice1 >= slice2
__device__ __noinline__ void ut_full1(const Ctx& x, const UtView& s, int slice1, int slice2) {
    DqmcChain& c = *x.c;
    ut_inverse_block(x, s, slice2, slice1);
    ut_forward_block(x, s, slice2);
    ut_backward_block(x, s, slice1);
    mm_nt_blocks(x, s.G, c.Tl, c.Tr);
    dright_blocks(x, c.tmp1, s.G, c.Dr);
    dleft_blocks(x, s.G, c.Dl, c.tmp1);
    udt_blocks(x, c.Tr, c.Dr, s.G, false);
    mm_blocks(x, c.Tl, c.Ul, c.Tr);
    rdivp_blocks(x, c.Ur, s.G, c.Ul);
    mm_tn_blocks(x, c.Tr, s.U, c.Tl);
    vmaxinv_v(x, c.Dl, s.D);
    dleft_blocks(x, c.tmp1, c.Dl, c.Tr);
    vmin_v(x, c.Dl, c.Dr);
    dright_blocks(x, c.Tr, c.tmp1, c.Dl);
    mm_blocks(x, c.Tl, s.T, c.Ur);
    vmin_v(x, c.Dl, s.D);
    dleft_blocks(x, c.tmp1, c.Dl, c.Tl);
    vmaxinv_v(x, c.Dl, c.Dr);
    dright_blocks(x, c.Tl, c.tmp1, c.Dl);
    mat_add(x, c.Tl, c.Tr);
    udt_blocks(x, c.Tr, c.Dl, c.Tl, false);
    vmaxinv_v(x, c.Dr, c.Dr);
    mat_diag(x, c.Ul, c.Dr);
    rdivp_blocks(x, c.Ul, c.Tl, c.tmp1);
    vinv_v(x, c.Dl);
    dright_blocks(x, c.tmp1, c.Ul, c.Dl);
    mm_nt_blocks(x, c.Ul, c.tmp1, c.Tr);
    vmaxinv_v(x, c.Dl, s.D);
    dright_blocks(x, s.G, c.Ul, c.Dl);
    mm_nt_blocks(x, c.Tr, s.G, s.U);
    mm_blocks(x, s.G, c.Ur, c.Tr);
}

// calculate_greens_full2! (:621-697), slice1 < slice2
__device__ __noinline__ void ut_full2(const Ctx& x, const UtView& s, int slice1, int slice2) {
    DqmcChain& c = *x.c;
    ut_inverse_block(x, s, slice1, slice2);
    ut_forward_block(x, s, slice1);
    ut_backward_block(x, s, slice2);
    mm_nt_blocks(x, s.G, c.Tl, c.Tr);
    dleft_blocks(x, c.tmp1, c.Dl, s.G);
    dright_blocks(x, s.G, c.tmp1, c.Dr);
    udt_blocks(x, c.Tr, c.Dr, s.G, false);
    mm_blocks(x, c.Tl, c.Ul, c.Tr);
    mm_tn_blocks(x, c.Ul, s.U, c.Tl);
    vmaxinv_v(x, c.Dl, s.D);
    dleft_blocks(x, s.U, c.Dl, c.Ul);
    vmin_v(x, c.Dl, c.Dr);
    dright_blocks(x, c.Ul, s.U, c.Dl);
    mm_blocks(x, s.U, s.T, c.Ur);
    rdivp_blocks(x, s.U, s.G, c.Ur);
    vmin_v(x, c.Dl, s.D);
    dleft_blocks(x, c.Ur, c.Dl, s.U);
    vmaxinv_v(x, c.Dl, c.Dr);
    dright_blocks(x, c.Tr, c.Ur, c.Dl);
    mat_add(x, c.Tr, c.Ul);
    udt_blocks(x, c.Ul, c.Dl, c.Tr, false);
    vmin_v(x, c.Dr, c.Dr);
    mat_diag(x, s.U, c.Dr);
    rdivp_blocks(x, s.U, c.Tr, c.Ur);
    vinv_v(x, c.Dl);
    dright_blocks(x, c.Ur, s.U, c.Dl);
    mm_nt_blocks(x, s.U, c.Ur, c.Ul);
    vmin_v(x, s.D, s.D);
    dright_blocks(x, c.Ur, s.U, s.D);
    mm_blocks(x, c.Tr, c.Ur, s.T);
    mm_blocks(x, s.G, c.Tl, c.Tr);
    for (int e = threadIdx.x; e < x.nf * (int)x.nn; e += DQMC_NT) s.G[e] = -s.G[e];
    __syncthreads();
}

// OP_GREENS_KL: one stack build, then G(k, l) for each requested pair
// (physical: the _greens! transform of the result, greens.jl:114-125)
// ---- time-displaced measurements (TimeIntegral, generic.jl:337-366) ----------
// For l = 0..M with the trapezoid weights w_l = (1/2 at l = 0, M; else 1) dtau,
// from the physical G(0,0), G(0,l), G(l,0), G(l,l) of the UnequalTimeStack
// (the reference's CombinedGreensIterator order), the Wick kernels per site
// pair (i, j), X_b = delta_ij [l = 0] - G0l_b[j, i], Y_b = Gl0_b[i, j],
// occupations o^l_b(i) = 1 - Gll_b[i, i], o^0_b(j) = 1 - G00_b[j, j]:
//   charge   full_cdc_kernel   (charge_density.jl:65-112)
//            sum_ab o^l_a(i) o^0_b(j) + sum_b X_b Y_b
//   spin x,y full_sdc_x/y_kernel (spin_density.jl:100-169): X_0 Y_1 + X_1 Y_0
//   spin z   full_sdc_z_kernel (spin_density.jl:182-227):
//            (o^l_0 - o^l_1)(i) (o^0_0 - o^0_1)(j) + sum_b X_b Y_b
//   pairing  pc_combined_kernel on site (pairing.jl:95-161): Y_0 Y_1 + X_1 X_0
// (one flavour block stands for both spins: 4 o^l o^0 + 2 X Y, 2 X Y, Y^2 + X^2),
// reduced by distance as EachSitePairByDistance does (slot of the pair, sum,
// divided by the number of sites: lattice_iterators.jl:160-260,
// generic.jl:434-461, 582-584) and as q-resolved susceptibilities
// (1/n) sum_l w_l sum_ij (cos q r_i cos q r_j + sin sin) C(i, j); the pairing
// susceptibility is the q = 0 sum.  Form-factor pairing (extended s, d):
// (1/n) sum_l w_l [sum F_ab F_cd (Gl0_up[c,a] Gl0_dn[d,b] + X_up[c,a] X_dn[d,b])]
// over the bonds (a, b), (c, d) of the form factor; current: (1/n) sum_l w_l
// Re[T_l T_0 + E] with T_l = rep sum_b tr(A (I - Gll_b)), T_0 likewise with
// G00, E = rep sum_b tr(A Gl0_b A X_b) for the sparse current operator A (rep
// = 2 for one flavour block).  Each measurement's 8 susceptibilities and 5 P
// by-distance values go into log binners (the layout of the equal-time ones).
__device__ __noinline__ void td_contract(const Ctx& x, const TdLayout& L, bool at_zero, double w,
                                         double* bd, double* sacc) {
    const DqmcChain& c = *x.c;
    const int n = x.n, nf = x.nf, P = c.td_P;
    const size_t nn = x.nn;
    const int* slot = reinterpret_cast<const int*>(c.td + L.slot);
    const double* qc = c.td + L.q;
    const double* qs = qc + n;
    const double* G00 = c.td + L.g;
    const double* G0l = G00 + nf * nn;
    const double* Gl0 = G0l + nf * nn;
    const double* Gll = Gl0 + nf * nn;
    const int b1 = nf - 1;
    for (int e = threadIdx.x; e < n * n; e += DQMC_NT) {
        const int i = e % n, j = e / n;
        const double id = (at_zero && i == j) ? 1.0 : 0.0;
        const double X0 = id - G0l[(size_t)i * n + j], X1 = id - G0l[b1 * nn + (size_t)i * n + j];
        const double Y0 = Gl0[e], Y1 = Gl0[b1 * nn + e];
        const double ol0 = 1.0 - Gll[(size_t)i * n + i], ol1 = 1.0 - Gll[b1 * nn + (size_t)i * n + i];
        const double o00 = 1.0 - G00[(size_t)j * n + j], o01 = 1.0 - G00[b1 * nn + (size_t)j * n + j];
        double ch, sx, sz, pr;
        if (nf == 2) {
            const double ex = X0 * Y0 + X1 * Y1;
            ch = (ol0 + ol1) * (o00 + o01) + ex;
            sx = X0 * Y1 + X1 * Y0;
            sz = (ol0 - ol1) * (o00 - o01) + ex;
            pr = Y0 * Y1 + X1 * X0;
        } else {
            const double ex = X0 * Y0;
            ch = 4.0 * ol0 * o00 + 2.0 * ex;
            sx = 2.0 * ex;
            sz = 2.0 * ex;
            pr = Y0 * Y0 + X0 * X0;
        }
        const double ph = qc[i] * qc[j] + qs[i] * qs[j];
        sacc[0] += w * ch * ph;
        sacc[1] += w * sx * ph;
        sacc[2] += w * sx * ph;
        sacc[3] += w * sz * ph;
        sacc[4] += w * pr;
        const int sl = slot[e];
        atomicAdd(&bd[sl], w * ch);
        atomicAdd(&bd[P + sl], w * sx);
        atomicAdd(&bd[2 * P + sl], w * sx);
        atomicAdd(&bd[3 * P + sl], w * sz);
        atomicAdd(&bd[4 * P + sl], w * pr);
    }
    // form-factor pairing: bonds of form f are entries [f0, f0 + nb) of the
    // (a, b, F) list
    const double* fl = c.td + L.form;
    const int dn = nf - 1;
    for (int f = 0; f < 2; ++f) {
        const int f0 = f == 0 ? 0 : c.td_nform0, nb = f == 0 ? c.td_nform0 : c.td_nform1;
        double t = 0.0;
        for (int p = threadIdx.x; p < nb; p += DQMC_NT) {
            const int a = (int)fl[3 * (f0 + p)], b = (int)fl[3 * (f0 + p) + 1];
            const double Fab = fl[3 * (f0 + p) + 2];
            double u = 0.0;
            for (int q = 0; q < nb; ++q) {
                const int cc = (int)fl[3 * (f0 + q)], d = (int)fl[3 * (f0 + q) + 1];
                const double Fcd = fl[3 * (f0 + q) + 2];
                const double xu = ((at_zero && cc == a) ? 1.0 : 0.0) - G0l[(size_t)a * n + cc];
                const double xd = ((at_zero && d == b) ? 1.0 : 0.0) - G0l[dn * nn + (size_t)b * n + d];
                u += Fcd * (Gl0[(size_t)a * n + cc] * Gl0[dn * nn + (size_t)b * n + d] + xu * xd);
            }
            t += Fab * u;
        }
        sacc[5 + f] += w * t;
    }
    // current: the trace terms need the whole sum before their product
    const double* cl = c.td + L.cur;
    const int nc = c.td_ncur;
    const double rep = nf == 1 ? 2.0 : 1.0;
    double tlr = 0.0, tli = 0.0, t0r = 0.0, t0i = 0.0, er = 0.0;
    for (int p = threadIdx.x; p < nc; p += DQMC_NT) {
        const int r = (int)cl[4 * p], s = (int)cl[4 * p + 1];
        const double ar = cl[4 * p + 2], ai = cl[4 * p + 3];
        for (int b = 0; b < nf; ++b) {
            const double il = (r == s ? 1.0 : 0.0) - Gll[b * nn + (size_t)r * n + s];
            const double i0 = (r == s ? 1.0 : 0.0) - G00[b * nn + (size_t)r * n + s];
            tlr += ar * il;
            tli += ai * il;
            t0r += ar * i0;
            t0i += ai * i0;
            // sum_q A_p Gl0[s_p, r_q] A_q X[s_q, r_p]
            for (int q = 0; q < nc; ++q) {
                const int r2 = (int)cl[4 * q], s2 = (int)cl[4 * q + 1];
                const double br = cl[4 * q + 2], bi = cl[4 * q + 3];
                const double g = Gl0[b * nn + (size_t)r2 * n + s];
                const double xx = ((at_zero && s2 == r) ? 1.0 : 0.0) - G0l[b * nn + (size_t)r * n + s2];
                // Re[(ar + i ai)(br + i bi)] * g * xx
                er += (ar * br - ai * bi) * g * xx;
            }
        }
    }
    // block sums of the trace terms (tiles are free here)
    double* red = x.s->tiles;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double v4[4] = {tlr, tli, t0r, t0i};
    for (int q = 0; q < 4; ++q) {
        const double v = warp_sum(v4[q]);
        if (lane == 0) red[q * DQMC_NW + warp] = v;
    }
    __syncthreads();
    double T[4] = {0.0, 0.0, 0.0, 0.0};
    for (int q = 0; q < 4; ++q)
        for (int ww = 0; ww < DQMC_NW; ++ww) T[q] += red[q * DQMC_NW + ww];
    __syncthreads();
    // Re[T_l T_0] once (thread 0), the exchange term from every thread
    double cur = rep * er;
    if (threadIdx.x == 0) cur += rep * rep * (T[0] * T[2] - T[1] * T[3]);
    sacc[7] += w * cur;
}

__device__ __noinline__ void td_measure(const Ctx& x) {
    DqmcChain& c = *x.c;
    const int n = x.n, nf = x.nf, M = c.M, P = c.td_P;
    const TdLayout L = td_layout(n, nf, P, c.td_nform0 + c.td_nform1, c.td_ncur);
    const size_t ms = (size_t)nf * x.nn;
    double* G00 = c.td + L.g;
    double* G0l = G00 + ms;
    double* Gl0 = G0l + ms;
    double* Gll = Gl0 + ms;
    const UtView s = ut_view(x);
    ut_build(x, s);
    ut_full1(x, s, 0, 0);
    greens_physical(x, s.G, G00);
    // by-distance sums of this measurement (global: the arena holds the
    // unequal-time QR factorisations of small chains)
    double* bd = c.td + L.stage;
    fill(DQMC_TD_KINDS * P, bd, 0.0);
    double sacc[DQMC_TD_SCALARS];
    for (int q = 0; q < DQMC_TD_SCALARS; ++q) sacc[q] = 0.0;
    __syncthreads();
    for (int l = 0; l <= M; ++l) {
        const double w = ((l == 0 || l == M) ? 0.5 : 1.0) * c.td_dtau;
        if (l == 0) ut_full1(x, s, 0, 0);
        else ut_full2(x, s, 0, l);
        greens_physical(x, s.G, G0l);
        ut_full1(x, s, l, 0);
        greens_physical(x, s.G, Gl0);
        ut_full1(x, s, l, l);
        greens_physical(x, s.G, Gll);
        __syncthreads();
        td_contract(x, L, l == 0, w, bd, sacc);
        __syncthreads();
    }
    // block sums of the susceptibilities
    double* red = x.s->tiles;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int q = 0; q < DQMC_TD_SCALARS; ++q) {
        const double v = warp_sum(sacc[q]);
        if (lane == 0) red[q * DQMC_NW + warp] = v;
    }
    __syncthreads();
    double* acc = c.td + L.acc;
    const double inv_n = 1.0 / n;
    // one binner per thread: the scalars first, then the by-distance values
    for (int k = threadIdx.x; k < DQMC_TD_SCALARS + DQMC_TD_KINDS * P; k += DQMC_NT) {
        double v;
        if (k < DQMC_TD_SCALARS) {
            v = 0.0;
            for (int ww = 0; ww < DQMC_NW; ++ww) v += red[k * DQMC_NW + ww];
        } else {
            v = bd[k - DQMC_TD_SCALARS];
        }
        binner_push(acc, k, v * inv_n);
    }
    __syncthreads();
    if (threadIdx.x == 0) acc[0] += 1.0;
    __syncthreads();
}

__device__ __noinline__ void greens_kl(const Ctx& x, int npairs, bool physical) {
    const DqmcChain& c = *x.c;
    const UtView s = ut_view(x);
    ut_build(x, s);
    const int ms = x.nf * (int)x.nn;
    for (int p = 0; p < npairs; ++p) {
        const int k = c.ut_pairs[2 * p], l = c.ut_pairs[2 * p + 1];
        if (k >= l) ut_full1(x, s, k, l);
        else ut_full2(x, s, k, l);
        if (physical) {
            greens_physical(x, s.G, c.ut_out + (size_t)p * ms);
        } else {
            copy(ms, c.ut_out + (size_t)p * ms, s.G);
            __syncthreads();
        }
    }
}

}  // namespace
}  // namespace dqmc
