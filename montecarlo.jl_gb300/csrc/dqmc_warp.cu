// The DQMC sweep for small lattices (n <= 32 sites): one warp runs one chain,
// eight chains share a CTA.
//
// For n = 16 the CTA-per-chain kernel is latency-bound: its 256 threads wait
// on block barriers around 16 x 16 products, 16-step QR factorisations and one
// Metropolis decision at a time, and four such CTAs per SM (the register file's
// limit) leave the FP64 pipe mostly idle.  Here every operation is
// warp-synchronous (no block barrier anywhere): products give each lane one
// column (two lanes per column when n <= 16), the Householder QR gives each
// lane one trailing column, triangular solves give each lane one row, and the
// rank-1 update is lane-strided over G, which stays in shared memory for the
// whole launch.  Sixteen chains run per SM instead of four.
//
// Same algorithm, state and workspace as the CTA kernel (dqmc_chain_ops.cuh),
// for the sweep operation only: the decision arithmetic is the same sequence
// of correctly rounded FP64 operations (so accept/reject decisions agree with
// the oracle's bit for bit); products, factorisations and solves sum in a
// different order (agreement to rounding).  The host runs it for handles whose
// chains are all real, FP64, dense-hopping, without device measurements or
// scheduled global updates, with n <= 32; everything else goes to the CTA
// kernel.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "dqmc_chain.h"
#include "dqmc_kernels.h"
#include "philox.h"

namespace dqmc_warp {
namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int WPC = 8;  // warps (chains) per CTA

// per-warp shared memory: descriptor, G (nf blocks of n x n), the current
// slice's interaction exponentials, rank-1 vectors, small scratch
struct Layout {
    int off_G, off_ev, off_u, off_w, off_sv, bytes;
};
__host__ __device__ inline int align16(int x) { return (x + 15) & ~15; }
__host__ __device__ inline Layout layout(int nmax) {
    Layout L;
    L.off_G = align16((int)sizeof(DqmcChain));
    L.off_ev = L.off_G + 2 * nmax * nmax * 8;
    L.off_u = L.off_ev + 2 * nmax * 8;
    L.off_w = L.off_u + 2 * nmax * 8;
    L.off_sv = L.off_w + 2 * nmax * 8;
    L.bytes = align16(L.off_sv + 2 * nmax * 8);
    return L;
}

struct W {
    DqmcChain* c;
    double *G, *ev, *u, *w, *sv;  // shared memory
    int n, nf, lane;
    int nn;
};

__device__ __forceinline__ double* blk(double* p, const W& x, int b) { return p + (size_t)b * x.nn; }

__device__ __forceinline__ void wcopy(const W& x, int cnt, double* dst, const double* src) {
    for (int e = x.lane; e < cnt; e += 32) dst[e] = src[e];
    __syncwarp();
}
__device__ __forceinline__ void wident(const W& x, double* A) {
    for (int e = x.lane; e < x.nf * x.nn; e += 32) {
        const int r = e % x.nn;
        A[e] = (r % x.n == r / x.n) ? 1.0 : 0.0;
    }
    __syncwarp();
}
__device__ __forceinline__ void wfill(const W& x, int cnt, double* d, double v) {
    for (int e = x.lane; e < cnt; e += 32) d[e] = v;
    __syncwarp();
}
// C = Diagonal(d) * B and C = A * Diagonal(d), one block
__device__ __forceinline__ void wdleft(const W& x, double* C, const double* d, const double* B) {
    for (int e = x.lane; e < x.nn; e += 32) C[e] = d[e % x.n] * B[e];
    __syncwarp();
}
__device__ __forceinline__ void wdright(const W& x, double* C, const double* A, const double* d) {
    for (int e = x.lane; e < x.nn; e += 32) C[e] = A[e] * d[e / x.n];
    __syncwarp();
}

// C = op(A) op(B) for one n x n block (n <= NB): n <= 16: lane l owns
// column l % 16 and rows [8 (l / 16), ... + 8); n <= 32: lane l owns column l
// in two passes of 16 rows (16 accumulators either way).  Fused
// multiply-adds in ascending k.  C must not alias A or B.
template <int NB, bool TA, bool TB>
__device__ __noinline__ void wmm(const W& x, double* __restrict__ C, const double* __restrict__ A,
                                 const double* __restrict__ B) {
    constexpr int LPC = NB == 16 ? 2 : 1, RPL = NB == 16 ? 8 : 16, PASSES = NB == 16 ? 1 : 2;
    const int n = x.n, col = x.lane % (32 / LPC);
    if (col < n) {
        for (int pass = 0; pass < PASSES; ++pass) {
            const int r0 = NB == 16 ? (x.lane / 16) * RPL : pass * RPL;
            if (r0 >= n) break;
            double acc[RPL];
#pragma unroll
            for (int r = 0; r < RPL; ++r) acc[r] = 0.0;
            for (int k = 0; k < n; ++k) {
                const double b = TB ? B[col + (size_t)k * n] : B[k + (size_t)col * n];
#pragma unroll
                for (int r = 0; r < RPL; ++r) {
                    const int i = r0 + r;
                    if (i < n)
                        acc[r] = fma(TA ? A[k + (size_t)i * n] : A[i + (size_t)k * n], b, acc[r]);
                }
            }
#pragma unroll
            for (int r = 0; r < RPL; ++r)
                if (r0 + r < n) C[r0 + r + (size_t)col * n] = acc[r];
        }
    }
    __syncwarp();
}
template <bool TA, bool TB>
__device__ __forceinline__ void mm(const W& x, double* C, const double* A, const double* B) {
    if (x.n <= 16) wmm<16, TA, TB>(x, C, A, B);
    else wmm<32, TA, TB>(x, C, A, B);
}

// udt_AVX_pivot! (UDT.jl:216-334) of one block, warp-synchronous: the same
// outputs as the CTA kernel's udt_pivot (pivot 1-based, reflectors below the
// diagonal, tau, D = |diag R| (0 -> 1), T pivoted or not).  Each trailing
// column of a step is owned by LPC lanes: two for n <= 16 (lane l: column
// j + l % 16, rows of parity l / 16, sums combined by a shuffle), one above.
// scr: n x n (apply only).
template <int LPC>
__device__ __noinline__ void wudt_t(const W& x, double* __restrict__ U, double* __restrict__ D,
                                    double* __restrict__ In, int* __restrict__ piv,
                                    double* __restrict__ tau, bool apply, double* __restrict__ scr) {
    const int n = x.n, lane = x.lane;
    const int co = LPC == 2 ? (lane & 15) : lane;  // column offset this lane works on
    const int h = LPC == 2 ? (lane >> 4) : 0;       // its row parity
    for (int i = lane; i < n; i += 32) piv[i] = i + 1;
    __syncwarp();
    for (int j = 0; j < n; ++j) {
        // indmaxcolumn: squared norms of the trailing columns, first maximum
        const int col = j + co;
        double s = 0.0;
        if (col < n) {
            const double* xc = In + (size_t)col * n;
            for (int r = j + h; r < n; r += LPC) s = fma(xc[r], xc[r], s);
        }
        if (LPC == 2) s += __shfl_xor_sync(FULL, s, 16);
        double best = -1.0;
        int bi = j;
        if (col < n) {
            best = s;
            bi = col;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double ob = __shfl_down_sync(FULL, best, o);
            const int oi = __shfl_down_sync(FULL, bi, o);
            if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        const int jm = __shfl_sync(FULL, bi, 0);
        const double normu = __shfl_sync(FULL, best, 0);
        if (jm != j) {
            double* a = In + (size_t)jm * n;
            double* b = In + (size_t)j * n;
            for (int r = lane; r < n; r += 32) {
                const double t = a[r];
                a[r] = b[r];
                b[r] = t;
            }
            if (lane == 0) {
                const int tp = piv[jm];
                piv[jm] = piv[j];
                piv[j] = tp;
            }
        }
        __syncwarp();
        // reflector! (UDT.jl:157-172)
        double* xj = In + (size_t)j * n;
        double xi1 = xj[j];
        double t = 0.0;
        __syncwarp();
        if (normu != 0.0) {
            const double nu = copysign(sqrt(normu), xi1);
            xi1 += nu;
            for (int r = j + 1 + lane; r < n; r += 32) xj[r] = xj[r] / xi1;
            if (lane == 0) xj[j] = -nu;
            t = xi1 / nu;
        }
        if (lane == 0) tau[j] = t;
        __syncwarp();
        // reflectorApply! (UDT.jl:53-70)
        const int ac = j + 1 + co;
        double* a = In + (size_t)ac * n;
        double aj = 0.0, s2 = 0.0;
        if (ac < n) {
            if (h == 0) aj = a[j];
            for (int r = j + 1 + h; r < n; r += LPC) s2 = fma(xj[r], a[r], s2);
        }
        if (LPC == 2) s2 += __shfl_xor_sync(FULL, s2, 16);
        double vAj = t * (aj + s2);
        if (LPC == 2) vAj = __shfl_sync(FULL, vAj, co);  // the parity-0 lane's value
        if (ac < n) {
            if (h == 0) a[j] = aj - vAj;
            for (int r = j + 1 + h; r < n; r += LPC) a[r] = fma(-xj[r], vAj, a[r]);
        }
        __syncwarp();
    }
    // explicit Q by backward accumulation (UDT.jl:272-289)
    for (int e = lane; e < x.nn; e += 32) U[e] = (e % n == e / n) ? 1.0 : 0.0;
    __syncwarp();
    if (lane == 0) U[(size_t)(n - 1) * n + (n - 1)] -= tau[n - 1];
    __syncwarp();
    for (int k = n - 2; k >= 0; --k) {
        const double* v = In + (size_t)k * n;
        const double tk = tau[k];
        const int col = k + co;
        double* u = U + (size_t)col * n;
        double uk = 0.0, s = 0.0;
        if (col < n) {
            if (h == 0) uk = u[k];
            for (int r = k + 1 + h; r < n; r += LPC) s = fma(v[r], u[r], s);
        }
        if (LPC == 2) s += __shfl_xor_sync(FULL, s, 16);
        double vB = tk * (uk + s);
        if (LPC == 2) vB = __shfl_sync(FULL, vB, co);
        if (col < n) {
            if (h == 0) u[k] = uk - vB;
            for (int r = k + 1 + h; r < n; r += LPC) u[r] = fma(-v[r], vB, u[r]);
        }
        __syncwarp();
    }
    // D (UDT.jl:293-301)
    for (int i = lane; i < n; i += 32) {
        const double av = fabs(In[(size_t)i * n + i]);
        D[i] = (av == 0.0) ? 1.0 : av;
    }
    __syncwarp();
    // _apply_pivot! (UDT.jl:311-334)
    if (apply) {
        for (int e = lane; e < x.nn; e += 32) {
            const int i = e % n, jj = e / n;
            const double d = 1.0 / D[i];
            scr[i + (size_t)(piv[jj] - 1) * n] = (jj >= i) ? d * In[e] : 0.0;
        }
        __syncwarp();
        for (int e = lane; e < x.nn; e += 32) In[e] = scr[e];
    } else {
        for (int e = lane; e < x.nn; e += 32) {
            const int i = e % n, jj = e / n;
            if (jj >= i) In[e] = (1.0 / D[i]) * In[e];
        }
    }
    __syncwarp();
}
__device__ __forceinline__ void wudt(const W& x, double* U, double* D, double* In, int* piv,
                                     double* tau, bool apply, double* scr) {
    if (x.n <= 16) wudt_t<2>(x, U, D, In, piv, tau, apply, scr);
    else wudt_t<1>(x, U, D, In, piv, tau, apply, scr);
}

// rdivp! (real.jl:198-226): A <- A[:, piv] triu(T)^-1.  Row i is owned by
// LPC lanes (two for n <= 16: the k-sum split by parity, combined by a
// shuffle), one above (two accumulation chains).  O: n x n scratch.
template <int LPC>
__device__ __noinline__ void wrdivp_t(const W& x, double* __restrict__ A,
                                      const double* __restrict__ T, double* __restrict__ O,
                                      const int* __restrict__ piv) {
    const int n = x.n, lane = x.lane;
    for (int j = lane; j < n; j += 32) x.sv[j] = 1.0 / T[(size_t)j * n + j];
    for (int e = lane; e < x.nn; e += 32) {
        const int i = e % n, j = e / n;
        O[e] = A[i + (size_t)(piv[j] - 1) * n];
    }
    __syncwarp();
    const int i = LPC == 2 ? (lane & 15) : lane, h = LPC == 2 ? (lane >> 4) : 0;
    for (int j = 0; j < n; ++j) {
        const double* tj = T + (size_t)j * n;
        double x0 = 0.0, x1 = 0.0;
        if (i < n) {
            if (h == 0) x0 = O[i + (size_t)j * n];
            if (LPC == 2) {
                for (int k = h; k < j; k += 2) x0 = fma(-A[i + (size_t)k * n], tj[k], x0);
            } else {
                int k = 0;
                for (; k + 1 < j; k += 2) {
                    x0 = fma(-A[i + (size_t)k * n], tj[k], x0);
                    x1 = fma(-A[i + (size_t)(k + 1) * n], tj[k + 1], x1);
                }
                if (k < j) x0 = fma(-A[i + (size_t)k * n], tj[k], x0);
            }
        }
        if (LPC == 2) x0 += __shfl_xor_sync(FULL, x0, 16);
        if (i < n && h == 0) A[i + (size_t)j * n] = (x0 + x1) * x.sv[j];
        if (LPC == 2) __syncwarp();  // the parity-1 lane reads A[i, j] in later columns
    }
    __syncwarp();
}
__device__ __forceinline__ void wrdivp(const W& x, double* A, const double* T, double* O,
                                       const int* piv) {
    if (x.n <= 16) wrdivp_t<2>(x, A, T, O, piv);
    else wrdivp_t<1>(x, A, T, O, piv);
}

// ---- chain-level operations (the CTA kernel's, warp-synchronous) -----------

__device__ __forceinline__ long long tstart(const W& x) { return x.lane == 0 ? clock64() : 0; }
__device__ __forceinline__ void tstop(const W& x, int phase, long long t0) {
    if (x.lane == 0) x.c->timers[phase] += (unsigned long long)(clock64() - t0);
}

// interaction_matrix_exp! of a slice into ev[b*n + i]
__device__ void interaction_exp(const W& x, int slice, bool inverse) {
    const DqmcChain& c = *x.c;
    const int8_t* s = c.conf + (size_t)(slice - 1) * x.n;
    const bool ghq = (c.kind >= 2);
    for (int e = x.lane; e < x.nf * x.n; e += 32) {
        const int b = e / x.n, i = e % x.n;
        const int v = ghq ? (int)s[i] - 1 : (s[i] > 0 ? 1 : 0);
        x.ev[e] = inverse ? c.evinv[b][v] : c.ev[b][v];
    }
    __syncwarp();
}
// multiply_slice_matrix_left!/right!/inv_right!/inv_left!, the daggered left
// product (stack.jl:319-367); tmp1 is the scratch block
__device__ void slice_left(const W& x, int slice, double* M) {
    interaction_exp(x, slice, false);
    for (int b = 0; b < x.nf; ++b) {
        wdleft(x, blk(x.c->tmp1, x, b), x.ev + b * x.n, blk(M, x, b));
        mm<true, false>(x, blk(M, x, b), x.c->eT2, blk(x.c->tmp1, x, b));
    }
}
__device__ void slice_right(const W& x, int slice, double* M) {
    interaction_exp(x, slice, false);
    for (int b = 0; b < x.nf; ++b) {
        mm<false, true>(x, blk(x.c->tmp1, x, b), blk(M, x, b), x.c->eT2);
        wdright(x, blk(M, x, b), blk(x.c->tmp1, x, b), x.ev + b * x.n);
    }
}
__device__ void slice_inv_right(const W& x, int slice, double* M) {
    interaction_exp(x, slice, true);
    for (int b = 0; b < x.nf; ++b) {
        wdright(x, blk(x.c->tmp1, x, b), blk(M, x, b), x.ev + b * x.n);
        mm<false, true>(x, blk(M, x, b), blk(x.c->tmp1, x, b), x.c->eT2inv);
    }
}
__device__ void slice_inv_left(const W& x, int slice, double* M) {
    interaction_exp(x, slice, true);
    for (int b = 0; b < x.nf; ++b) {
        mm<true, false>(x, blk(x.c->tmp1, x, b), x.c->eT2inv, blk(M, x, b));
        wdleft(x, blk(M, x, b), x.ev + b * x.n, blk(x.c->tmp1, x, b));
    }
}
__device__ void slice_dagger_left(const W& x, int slice, double* M) {
    interaction_exp(x, slice, false);
    for (int b = 0; b < x.nf; ++b) {
        mm<true, false>(x, blk(x.c->tmp1, x, b), x.c->eT2, blk(M, x, b));
        wdleft(x, blk(M, x, b), x.ev + b * x.n, blk(x.c->tmp1, x, b));
    }
}
// wrap_greens! (stack.jl:594-603)
__device__ void wrap_greens(const W& x, double* gf, int curr_slice, int direction) {
    if (direction == -1) {
        slice_inv_left(x, curr_slice - 1, gf);
        slice_right(x, curr_slice - 1, gf);
    } else {
        slice_left(x, curr_slice, gf);
        slice_inv_right(x, curr_slice, gf);
    }
}

__device__ __forceinline__ double* ustk(const W& x, int idx) {
    return x.c->ustack + (size_t)(idx - 1) * x.nf * x.nn;
}
__device__ __forceinline__ double* tstk(const W& x, int idx) {
    return x.c->tstack + (size_t)(idx - 1) * x.nf * x.nn;
}
__device__ __forceinline__ double* dstk(const W& x, int idx) {
    return x.c->dstack + (size_t)(idx - 1) * x.nf * x.n;
}
__device__ void udt_blocks(const W& x, double* U, double* D, double* In, bool apply) {
    for (int b = 0; b < x.nf; ++b)
        wudt(x, blk(U, x, b), D + b * x.n, blk(In, x, b), x.c->pivot + b * x.n,
             x.c->tempv + b * x.n, apply, blk(x.c->out, x, b));
}

// add_slice_sequence_left / _right (stack.jl:377-416)
__device__ __noinline__ void add_slice_sequence_left(const W& x, int idx) {
    DqmcChain& c = *x.c;
    wcopy(x, x.nf * x.nn, c.currU, ustk(x, idx));
    long long t0 = tstart(x);
    for (int s = c.rfirst[idx - 1]; s <= c.rlast[idx - 1]; ++s) slice_left(x, s, c.currU);
    for (int b = 0; b < x.nf; ++b)
        wdright(x, blk(c.tmp1, x, b), blk(c.currU, x, b), dstk(x, idx) + b * x.n);
    tstop(x, DQMC_PHASE_SLICE_CHAIN, t0);
    t0 = tstart(x);
    udt_blocks(x, ustk(x, idx + 1), dstk(x, idx + 1), c.tmp1, true);
    tstop(x, DQMC_PHASE_UDT, t0);
    t0 = tstart(x);
    for (int b = 0; b < x.nf; ++b)
        mm<false, false>(x, blk(tstk(x, idx + 1), x, b), blk(c.tmp1, x, b), blk(tstk(x, idx), x, b));
    tstop(x, DQMC_PHASE_T_UPDATE, t0);
}
__device__ __noinline__ void add_slice_sequence_right(const W& x, int idx) {
    DqmcChain& c = *x.c;
    wcopy(x, x.nf * x.nn, c.currU, ustk(x, idx + 1));
    long long t0 = tstart(x);
    for (int s = c.rlast[idx - 1]; s >= c.rfirst[idx - 1]; --s) slice_dagger_left(x, s, c.currU);
    for (int b = 0; b < x.nf; ++b)
        wdright(x, blk(c.tmp1, x, b), blk(c.currU, x, b), dstk(x, idx + 1) + b * x.n);
    tstop(x, DQMC_PHASE_SLICE_CHAIN, t0);
    t0 = tstart(x);
    udt_blocks(x, ustk(x, idx), dstk(x, idx), c.tmp1, true);
    tstop(x, DQMC_PHASE_UDT, t0);
    t0 = tstart(x);
    for (int b = 0; b < x.nf; ++b)
        mm<false, false>(x, blk(tstk(x, idx), x, b), blk(c.tmp1, x, b), blk(tstk(x, idx + 1), x, b));
    tstop(x, DQMC_PHASE_T_UPDATE, t0);
}

// calculate_greens_AVX! (stack.jl:442-496), per flavour block, into Gout
__device__ __noinline__ void calculate_greens(const W& x, double* Gout) {
    DqmcChain& c = *x.c;
    const int n = x.n;
    for (int b = 0; b < x.nf; ++b) {
        double *ul = blk(c.Ul, x, b), *tl = blk(c.Tl, x, b), *ur = blk(c.Ur, x, b),
               *tr = blk(c.Tr, x, b), *g = blk(Gout, x, b);
        double *dl = c.Dl + b * n, *dr = c.Dr + b * n;
        int* pv = c.pivot + b * n;
        double* tv = c.tempv + b * n;
        mm<false, true>(x, g, tl, tr);
        wdright(x, tr, g, dr);
        wdleft(x, g, dl, tr);
        wudt(x, tr, dr, g, pv, tv, false, blk(c.out, x, b));
        mm<false, false>(x, tl, ul, tr);
        wrdivp(x, ur, g, ul, pv);
        mm<true, false>(x, tr, tl, ur);
        for (int i = x.lane; i < n; i += 32) tr[(size_t)i * n + i] += dr[i];
        __syncwarp();
        wudt(x, ul, dr, tr, pv, tv, false, blk(c.out, x, b));
        wrdivp(x, ur, tr, g, pv);
        mm<false, false>(x, tr, tl, ul);
        for (int i = x.lane; i < n; i += 32) dl[i] = 1.0 / dr[i];
        __syncwarp();
        wdright(x, ul, ur, dl);
        mm<false, true>(x, g, ul, tr);
    }
}

// max |Gtmp - G| (stack.jl:646, 701); NaN propagates; a non-finite G sets status 2
__device__ void record_prop_error(const W& x) {
    DqmcChain& c = *x.c;
    double m = 0.0;
    for (int e = x.lane; e < x.nf * x.nn; e += 32) {
        const double d = fabs(c.Gtmp[e] - x.G[e]);
        if (d > m || d != d) m = d;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double om = __shfl_xor_sync(FULL, m, o);
        if (om > m || om != om) m = om;
    }
    if (x.lane == 0) {
        if (m > c.prop_err_max || m != m) c.prop_err_max = m;
        if (m != m || m > 1e300) c.status = 2;
        if (m > 1e-7) {
            c.n_prop_err += 1;
            if (m > c.prop_err_reported) c.prop_err_reported = m;
            DQMC_MS_PUSH(c.ms_prop, m);
        }
    }
    __syncwarp();
}

// propagate (stack.jl:605-730); the direction flips at 0 and M+1 recurse once
__device__ __noinline__ void propagate(const W& x) {
    DqmcChain& c = *x.c;
    for (int depth = 0; depth < 2; ++depth) {
        const int dir = c.direction;
        const int cs = c.current_slice + dir;
        const int cr = c.current_range;
        __syncwarp();
        if (x.lane == 0) c.current_slice = cs;
        __syncwarp();
        bool recurse = false;
        if (dir == 1) {
            if (cs == 1) {
                wident(x, ustk(x, 1));
                wfill(x, x.nf * x.n, dstk(x, 1), 1.0);
                wident(x, tstk(x, 1));
            } else if (cs - 1 == c.rlast[cr - 1]) {
                const int idx = cr;
                wcopy(x, x.nf * x.nn, c.Ur, ustk(x, idx + 1));
                wcopy(x, x.nf * x.n, c.Dr, dstk(x, idx + 1));
                wcopy(x, x.nf * x.nn, c.Tr, tstk(x, idx + 1));
                add_slice_sequence_left(x, idx);
                wcopy(x, x.nf * x.nn, c.Ul, ustk(x, idx + 1));
                wcopy(x, x.nf * x.n, c.Dl, dstk(x, idx + 1));
                wcopy(x, x.nf * x.nn, c.Tl, tstk(x, idx + 1));
                long long t0 = tstart(x);
                if (c.check_prop) {
                    wcopy(x, x.nf * x.nn, c.Gtmp, x.G);
                    wrap_greens(x, c.Gtmp, cs - 1, 1);
                }
                tstop(x, DQMC_PHASE_PROP_CHECK, t0);
                t0 = tstart(x);
                calculate_greens(x, x.G);
                tstop(x, DQMC_PHASE_GREENS, t0);
                if (c.check_prop) record_prop_error(x);
                if (cr == c.nr) {
                    if (x.lane == 0) c.direction = -1;
                    recurse = true;
                } else if (x.lane == 0) {
                    c.current_range = cr + 1;
                }
            } else {
                const long long tw = tstart(x);
                wrap_greens(x, x.G, cs - 1, 1);
                tstop(x, DQMC_PHASE_WRAP, tw);
            }
        } else {
            if (cs == c.M) {
                wident(x, ustk(x, c.nr + 1));
                wfill(x, x.nf * x.n, dstk(x, c.nr + 1), 1.0);
                wident(x, tstk(x, c.nr + 1));
                const long long tw = tstart(x);
                wrap_greens(x, x.G, cs + 1, -1);
                tstop(x, DQMC_PHASE_WRAP, tw);
            } else if (cs + 1 == c.rfirst[cr - 1]) {
                const int idx = cr;
                wcopy(x, x.nf * x.nn, c.Ul, ustk(x, idx));
                wcopy(x, x.nf * x.n, c.Dl, dstk(x, idx));
                wcopy(x, x.nf * x.nn, c.Tl, tstk(x, idx));
                add_slice_sequence_right(x, idx);
                wcopy(x, x.nf * x.nn, c.Ur, ustk(x, idx));
                wcopy(x, x.nf * x.n, c.Dr, dstk(x, idx));
                wcopy(x, x.nf * x.nn, c.Tr, tstk(x, idx));
                if (c.check_prop) wcopy(x, x.nf * x.nn, c.Gtmp, x.G);
                long long t0 = tstart(x);
                calculate_greens(x, x.G);
                tstop(x, DQMC_PHASE_GREENS, t0);
                if (c.check_prop) record_prop_error(x);
                if (cr == 1) {
                    if (x.lane == 0) c.direction = 1;
                    recurse = true;
                } else {
                    const long long tw = tstart(x);
                    wrap_greens(x, x.G, cs + 1, -1);
                    tstop(x, DQMC_PHASE_WRAP, tw);
                    if (x.lane == 0) c.current_range = cr - 1;
                }
            } else {
                const long long tw = tstart(x);
                wrap_greens(x, x.G, cs + 1, -1);
                tstop(x, DQMC_PHASE_WRAP, tw);
            }
        }
        __syncwarp();
        if (!recurse) break;
    }
}

// sweep_spatial (local_updates.jl:23-60) with propose_local / accept_local!:
// lane 0 decides with the CTA kernel's (and the oracle's) sequence of
// correctly rounded operations; an accepted move updates G (shared memory)
// with every lane: G -= (I - G)[:, j] (Delta/R) G[j, :] per flavour block.
__device__ __noinline__ void sweep_spatial(const W& x) {
    DqmcChain& c = *x.c;
    const int n = x.n, nf = x.nf;
    int8_t* s = c.conf + (size_t)(c.current_slice - 1) * n;
    const bool ghq = (c.kind >= 2);
    const bool twoflv = (nf == 2);
    for (int j = 0; j < n; ++j) {
        int accept = 0;
        double sx0 = 0.0, sx1 = 0.0;
        if (x.lane == 0) {
            const double g0 = x.G[(size_t)j * n + j];
            const double g1 = twoflv ? x.G[(size_t)x.nn + (size_t)j * n + j] : 0.0;
            int t, xnew = 0;
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
            // the uniform's word ahead of p (drawn only when p <= 1); the
            // uniform and the comparisons on the integer pipe (uniform_bits)
            const uint64_t wu = dqmc_philox_word(c.key, c.ctr);
            const double p = __dmul_rn(c.wboson[t], detratio);
            if (below_zero(p)) {
                c.n_neg_p += 1;
                DQMC_MS_PUSH(c.ms_neg, p);
            }
            if (above_one(p)) {
                accept = 1;
            } else {
                c.ctr += 1;
                const long long ub = uniform_bits(wu);
                accept = uniform_below(ub, p);
                note_tie(c, __longlong_as_double(ub), p);
            }
            c.proposals += 1;
            if (accept) {
                sx0 = __ddiv_rn(d0, R0);
                sx1 = twoflv ? __ddiv_rn(d1, R1) : 0.0;
                s[j] = ghq ? (int8_t)xnew : (int8_t)(-s[j]);
                c.accepted += 1;
            }
        }
        accept = __shfl_sync(FULL, accept, 0);
        if (!accept) continue;
        sx0 = __shfl_sync(FULL, sx0, 0);
        sx1 = __shfl_sync(FULL, sx1, 0);
        // u = (I - G)[:, j], w = (Delta/R) G[j, :] per block
        for (int e = x.lane; e < nf * n; e += 32) {
            const int b = e / n, k = e % n;
            const double* g = x.G + (size_t)b * x.nn;
            double ig = -g[(size_t)j * n + k];
            if (k == j) ig += 1.0;
            x.u[e] = ig;
            x.w[e] = (b ? sx1 : sx0) * g[(size_t)k * n + j];
        }
        __syncwarp();
        for (int e = x.lane; e < nf * x.nn; e += 32) {
            const int b = e / x.nn, r = e % x.nn;
            const int k = r % n, l = r / n;
            x.G[e] = fma(-x.u[b * n + k], x.w[b * n + l], x.G[e]);
        }
        __syncwarp();
    }
}

// The same sweep for Hirsch fields with the proposals evaluated in parallel:
// from site j on, lane k computes the ratio of site j + k on the current G
// (valid for every site up to the first acceptance, since G changes only
// there), each lane takes its uniform at the counter the sequential loop
// would reach (a ballot and prefix count of the proposals with p <= 1 before
// it), and the first accepting lane wins; the proposals after it are
// evaluated again on the updated G.  Every decision is the sequential loop's
// (same operations, same uniforms); on GB300 a scalar FP64 operation of lane 0
// costs as much FP64-pipe time as a full warp's, so up to 32 proposals cost
// one.
__device__ __noinline__ void sweep_spatial_hirsch(const W& x) {
    DqmcChain& c = *x.c;
    const int n = x.n, nf = x.nf, lane = x.lane;
    int8_t* s = c.conf + (size_t)(c.current_slice - 1) * n;
    const bool twoflv = (nf == 2);
    int j = 0;
    while (j < n) {
        const int jj = j + lane;
        const bool valid = jj < n;
        double p = 0.0, R0 = 1.0, R1 = 1.0, d0 = 0.0, d1 = 0.0;
        if (valid) {
            const double g0 = x.G[(size_t)jj * n + jj];
            const double g1 = twoflv ? x.G[(size_t)x.nn + (size_t)jj * n + jj] : 0.0;
            const int t = s[jj] > 0 ? 1 : 0;
            d0 = c.delta0[t];
            d1 = c.delta1[t];
            R0 = __dadd_rn(1.0, __dmul_rn(d0, __dsub_rn(1.0, g0)));
            double detratio;
            if (twoflv) {
                R1 = __dadd_rn(1.0, __dmul_rn(d1, __dsub_rn(1.0, g1)));
                detratio = __dmul_rn(R0, R1);
            } else {
                detratio = __dmul_rn(R0, R0);
            }
            p = __dmul_rn(c.wboson[t], detratio);
        }
        const unsigned need = __ballot_sync(FULL, valid && !above_one(p));
        const unsigned below = (1u << lane) - 1u;  // lanes before this one
        bool acc = false;
        double gap = INFINITY;  // |u - p| of this lane's drawn uniform
        if (valid) {
            if (above_one(p)) {
                acc = true;
            } else {
                const uint64_t w = dqmc_philox_word(c.key, c.ctr + (uint64_t)__popc(need & below));
                const long long ub = uniform_bits(w);
                acc = uniform_below(ub, p);
                gap = fabs(__longlong_as_double(ub) - p);
            }
        }
        const unsigned am = __ballot_sync(FULL, acc);
        const unsigned vm = __ballot_sync(FULL, valid);
        const int last = am ? __ffs(am) - 1 : 31 - __clz(vm);  // last proposal of this pass
        const unsigned done = last == 31 ? FULL : ((2u << last) - 1u);
        {
            // near ties among the proposals made; the smallest gap by the bit
            // patterns of the non-negative gaps (integer pipe)
            const unsigned ties = __ballot_sync(FULL, gap < DQMC_NEAR_TIE) & done;
            long long gb = ((done >> lane) & 1u) ? __double_as_longlong(gap)
                                                 : __double_as_longlong(INFINITY);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const long long og = __shfl_xor_sync(FULL, gb, o);
                gb = og < gb ? og : gb;
            }
            if (lane == 0) {
                c.n_near_tie += __popc(ties);
                const double gmin = __longlong_as_double(gb);
                if (gmin < c.min_tie_gap) c.min_tie_gap = gmin;
            }
        }
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
        if (lane == 0) {
            c.ctr += (uint64_t)__popc(need & done);
            c.proposals += __popc(vm & done);
        }
        if (!am) break;
        // accept_local! of site j + last
        const int ja = j + last;
        double sx0 = 0.0, sx1 = 0.0;
        if (lane == last) {
            sx0 = __ddiv_rn(d0, R0);
            sx1 = twoflv ? __ddiv_rn(d1, R1) : 0.0;
            s[ja] = (int8_t)(-s[ja]);
            c.accepted += 1;
        }
        sx0 = __shfl_sync(FULL, sx0, last);
        sx1 = __shfl_sync(FULL, sx1, last);
        __syncwarp();
        for (int e = lane; e < nf * n; e += 32) {
            const int b = e / n, k = e % n;
            const double* g = x.G + (size_t)b * x.nn;
            double ig = -g[(size_t)ja * n + k];
            if (k == ja) ig += 1.0;
            x.u[e] = ig;
            x.w[e] = (b ? sx1 : sx0) * g[(size_t)k * n + ja];
        }
        __syncwarp();
        for (int e = lane; e < nf * x.nn; e += 32) {
            const int b = e / x.nn, r = e % x.nn;
            const int k = r % n, l = r / n;
            x.G[e] = fma(-x.u[b * n + k], x.w[b * n + l], x.G[e]);
        }
        __syncwarp();
        j = ja + 1;
    }
}

// One warp per chain: `nsweeps` sweeps (local_sweep, local_updates.jl:7-14)
// of every chain, the sweep counter advanced after each (the scheduler's
// mc.last_sweep).  MINB CTAs per SM: two for n <= 16 (16 chains per SM, 71 KB
// of shared memory each; a third CTA measured no faster: the FP64 pipe and
// issue are busy), one for n <= 32 (8 chains per SM, 178 KB).
template <int MINB>
__global__ void __launch_bounds__(32 * WPC, MINB)
    warp_sweep_kernel(DqmcChain* chains, int nchains, int nsweeps, int nmax) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Layout L = layout(nmax);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int chain = blockIdx.x * WPC + warp;
    if (chain >= nchains) return;  // whole warps only: no block barrier below
    unsigned char* base = smem_raw + (size_t)warp * L.bytes;
    DqmcChain* c = reinterpret_cast<DqmcChain*>(base);
    {
        const int words = (int)(sizeof(DqmcChain) / 4);
        const uint32_t* src = reinterpret_cast<const uint32_t*>(chains + chain);
        uint32_t* dst = reinterpret_cast<uint32_t*>(c);
        for (int e = lane; e < words; e += 32) dst[e] = src[e];
    }
    __syncwarp();
    if (!c->active) return;
    W x;
    x.c = c;
    x.n = c->n;
    x.nf = c->nf;
    x.nn = x.n * x.n;
    x.lane = lane;
    x.G = reinterpret_cast<double*>(base + L.off_G);
    x.ev = reinterpret_cast<double*>(base + L.off_ev);
    x.u = reinterpret_cast<double*>(base + L.off_u);
    x.w = reinterpret_cast<double*>(base + L.off_w);
    x.sv = reinterpret_cast<double*>(base + L.off_sv);
    if (x.n < 1 || x.n > nmax || x.nf < 1 || x.nf > 2 || c->cplx || c->cb) {
        if (lane == 0) chains[chain].status = 1;
        return;
    }
    wcopy(x, x.nf * x.nn, x.G, c->G);
    for (int sw = 0; sw < nsweeps; ++sw) {
        for (int t = 0; t < 2 * c->M; ++t) {
            const long long t0 = tstart(x);
            if (c->kind >= 2) sweep_spatial(x);
            else sweep_spatial_hirsch(x);
            tstop(x, DQMC_PHASE_SWEEP_SPATIAL, t0);
            propagate(x);
        }
        if (lane == 0) c->sweep += 1;
        __syncwarp();
    }
    wcopy(x, x.nf * x.nn, c->G, x.G);
    if (lane == 0) {
        DqmcChain& g = chains[chain];
        g.ctr = c->ctr;
        g.current_slice = c->current_slice;
        g.current_range = c->current_range;
        g.direction = c->direction;
        g.prop_err_max = c->prop_err_max;
        g.prop_err_reported = c->prop_err_reported;
        g.n_prop_err = c->n_prop_err;
        g.n_neg_p = c->n_neg_p;
        g.n_near_tie = c->n_near_tie;
        g.min_tie_gap = c->min_tie_gap;
        g.accepted = c->accepted;
        g.proposals = c->proposals;
        for (int p = 0; p < 8; ++p) g.timers[p] = c->timers[p];
        for (int q = 0; q < 3; ++q) {
            g.ms_prop[q] = c->ms_prop[q];
            g.ms_neg[q] = c->ms_neg[q];
        }
        g.sweep = c->sweep;
        if (c->status) g.status = c->status;
    }
}

}  // namespace
}  // namespace dqmc_warp

bool dqmc_warp_kernel_eligible(const DqmcChain& d) {
    return !d.active || (d.n <= 32 && d.prec == DQMC_PREC_FP64_ID && !d.cplx && !d.cb &&
                         d.global_kind < 0 && !d.meas_enable && !d.td_enable);
}

cudaError_t dqmc_launch_warp_kernel(DqmcChain* d_chains, int nchains, int nsweeps,
                                    cudaStream_t stream, int n_max) {
    if (n_max < 1 || n_max > 32) return cudaErrorInvalidValue;
    const int nmax = n_max <= 16 ? 16 : 32;
    const size_t smem = (size_t)dqmc_warp::WPC * dqmc_warp::layout(nmax).bytes;
    static bool attr_set[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev >= 0 && dev < 64 && !attr_set[dev]) {
        e = cudaFuncSetAttribute(dqmc_warp::warp_sweep_kernel<2>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(dqmc_warp::WPC * dqmc_warp::layout(16).bytes));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(dqmc_warp::warp_sweep_kernel<1>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)(dqmc_warp::WPC * dqmc_warp::layout(32).bytes));
        if (e != cudaSuccess) return e;
        attr_set[dev] = true;
    }
    const int grid = (nchains + dqmc_warp::WPC - 1) / dqmc_warp::WPC;
    if (nmax == 16)
        dqmc_warp::warp_sweep_kernel<2><<<grid, 32 * dqmc_warp::WPC, smem, stream>>>(
            d_chains, nchains, nsweeps, nmax);
    else
        dqmc_warp::warp_sweep_kernel<1><<<grid, 32 * dqmc_warp::WPC, smem, stream>>>(
            d_chains, nchains, nsweeps, nmax);
    return cudaGetLastError();
}
