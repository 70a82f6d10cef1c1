// The DQMC chain kernel: one CTA runs one chain of the reference's DQMC
// (src/flavors/DQMC) entirely on the device -- local sweeps with rank-1
// Green's function updates, wraps, slice-matrix chains, UDT stabilisation and
// Green's function reconstruction -- for as many sweeps as requested, so a
// whole batch of chains advances in one launch.
//
// The file is compiled twice: as is (DQMC_TC_BUILD 0, no tensor-core code:
// the occupancy calculation of a kernel that contains tcgen05 instructions
// allows one CTA per SM, while these kernels are built for two), and by
// dqmc_kernels_tc.cu with DQMC_TC_BUILD 1, whose kernels run the products of
// tensor-core-capable mixed chains on the tensor cores.  Each build's kernels
// have internal linkage; the host entry points carry a _tc suffix in the
// second.
#include <cuda_runtime.h>
#include <stdint.h>

#ifndef DQMC_TC_BUILD
#define DQMC_TC_BUILD 0
#endif
#include "dqmc_chain_ops.cuh"
#include "dqmc_kernels.h"

#if DQMC_TC_BUILD
#define DQMC_KERNEL_ENTRY(name) name##_tc
#else
#define DQMC_KERNEL_ENTRY(name) name
#endif

namespace dqmc {
namespace {

// MINB CTAs per SM: 2 in general (128 registers a thread); 4 for ensembles of
// small lattices (n <= 32), whose chains are latency-bound and leave the
// pipes idle, so that twice as many chains share an SM.
template <int MINB>
__global__ void __launch_bounds__(DQMC_NT, MINB) chain_kernel(DqmcChain* chains, int nchains,
                                                           int op, int arg0, int arg1,
                                                           int arena_cap) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem* s = reinterpret_cast<Smem*>(smem_raw);
    // launched in two-CTA clusters (a pool with flavour-split chains): both
    // CTAs of a cluster take the same slot; a two-flavour chain that can be
    // split runs one flavour block on each, any other chain on rank 0 alone
    const bool pair = cluster_ncta() == 2;
    const int slot = pair ? (int)(blockIdx.x >> 1) : (int)blockIdx.x;
    const int rank = pair ? (int)cluster_rank() : 0;
    if (pair) {
        if (threadIdx.x == 0) {
            s->xflag = 0;
            s->xepoch = 0;
            s->xdead = 0;
        }
        cluster_barrier();  // both CTAs have started and cleared their exchange counters
    }
    if (slot >= nchains) return;
    // stage this chain's descriptor in shared memory
    {
        const int words = (int)(sizeof(DqmcChain) / 4);
        const uint32_t* src = reinterpret_cast<const uint32_t*>(chains + slot);
        uint32_t* dst = reinterpret_cast<uint32_t*>(&s->c);
        for (int e = threadIdx.x; e < words; e += DQMC_NT) dst[e] = src[e];
    }
    __syncthreads();
    Ctx x;
    x.s = s;
    x.c = &s->c;
    x.n = s->c.n;
    x.nf = s->c.nf;
    x.nn = (size_t)x.n * x.n;
    x.b0 = 0;
    x.b1 = x.nf;
    x.peer = -1;
    if (threadIdx.x == 0) {
        s->Gglob = s->c.G;
        s->gres = 0;
        s->gdfg = 0;
        s->tc_on = 0;
        s->arena_cap = arena_cap;
    }
    __syncthreads();
    if (!s->c.active) return;  // free pool slot
    if (x.n > DQMC_NMAX || x.nf < 1 || x.nf > 2) {
        if (threadIdx.x == 0 && rank == 0) chains[slot].status = 1;
        return;
    }
    const bool fsplit = pair && op == DQMC_OP_RUN && flavour_split_ok(s->c);
    if (pair && rank == 1 && !fsplit) return;
    if (fsplit) {
        x.b0 = rank;
        x.b1 = rank + 1;
        x.peer = rank ^ 1;
    }
    // tensor-core products: one warp allocates the accumulators' TMEM columns
    // (two CTAs per SM at most, 2 x 256 of the SM's 512 columns) and thread 0
    // sets up the mbarriers; released after the operation
    const bool use_tc = DQMC_TC_BUILD && tc_eligible(s->c, arena_cap);
#if DQMC_TC_BUILD
    // a CTA of the tensor-core variant that will not allocate TMEM gives up
    // its allocation permit at once: an SM admits the next CTA of a kernel that
    // may allocate TMEM only after the resident one has allocated or
    // relinquished
    if (!use_tc && (threadIdx.x >> 5) == 0)
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
#endif
    if (use_tc) {
#if DQMC_TC_BUILD
        if ((threadIdx.x >> 5) == 0) tc_alloc(&s->tc.tmem, DQMC_TC_COLS);
#endif
        if (threadIdx.x == 0) {
            for (int b = 0; b < 2; ++b) {
                mbar_init(&s->tc.full[b], 1);
                mbar_init(&s->tc.mma[b], 1);
                s->tc.ph_full[b] = s->tc.ph_mma[b] = 0;
            }
            s->tc.status = 0;
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        tc_fence_before();
    }
    if (threadIdx.x == 0) s->tc_on = use_tc ? 1 : 0;
    __syncthreads();
    if (use_tc) tc_fence_after();
    switch (op) {
    case DQMC_OP_RUN: {
        // time slice of a pool: build the stack of a newly admitted chain,
        // then run slice visits (sweep_spatial + propagate) until the chain's
        // quota is used up or the time slice is over; the chain's state
        // carries over to the next slice.  The slice is work-conserving: a
        // chain past its budget (arg0 microseconds) keeps visiting until every
        // chain of the launch is past its own (the pool's visit counters), so
        // no SM idles while the launch waits for a chain with long visits.
        // No chain waits for another: each only reads the counters.
        const unsigned long long t_start = global_ns();
        const unsigned long long budget = 1000ull * (unsigned long long)arg0;
        // (a flavour-split chain counts once, on rank 0, which also decides
        // when the chain stops and tells its partner)
        unsigned int* sync = rank == 0 ? s->c.run_sync : nullptr;
        bool counted = false;  // thread 0: this chain is counted as past its budget
        const bool works = s->c.needs_build || s->c.visits_quota > 0;
        if (threadIdx.x == 0 && sync && works) atomicAdd(&sync[0], 1u);
        if (s->c.needs_build) {
            reverse_build_stack(x);
            propagate(x);
            if (threadIdx.x == 0) s->c.needs_build = 0;
            __syncthreads();
        }
        const bool res = g_resident_possible(x);
        if (res && s->c.visits_quota > 0) g_to_arena(x);
        bool in_arena = res && s->c.visits_quota > 0;
        while (s->c.visits_quota > 0) {
            long long t0 = phase_start();
            sweep_spatial(x);
            phase_stop(x, DQMC_PHASE_SWEEP_SPATIAL, t0);
            propagate(x);
            if (threadIdx.x == 0) {
                s->c.visits_quota -= 1;
                s->c.visits_done += 1;
                const bool over = (global_ns() - t_start) >= budget;
                bool stop = over;
                if (sync) {
                    if (over && !counted) {
                        atomicAdd(&sync[1], 1u);
                        counted = true;
                    }
                    const volatile unsigned int* vs = sync;
                    stop = counted && vs[1] >= vs[0];
                }
                s->sxi[1] = stop;
                s->xval[1] = stop ? 1.0 : 0.0;
            }
            if (fsplit) {  // rank 1 follows rank 0 (a partner gone: stop)
                const bool ok = xsync(x);
                if (threadIdx.x == 0 && rank == 1)
                    s->sxi[1] = !ok || peer_ld(peer_addr(&s->xval[1], x.peer)) != 0.0;
            }
            __syncthreads();
            if (s->c.visits_done % (2 * s->c.M) == 0) after_sweep(x);
            if (s->sxi[1]) break;
        }
        // a chain that stops early (quota used up) no longer holds the others
        if (threadIdx.x == 0 && sync && works && !counted) atomicAdd(&sync[1], 1u);
        if (in_arena) g_to_global(x);
        break;
    }
    case DQMC_OP_SWEEP: {
        const bool res = g_resident_possible(x);
        if (res) g_to_arena(x);
        for (int sw = 0; sw < arg0; ++sw) {
            // SimpleScheduler(LocalSweep(), <global update>) (scheduler.jl:281-289):
            // every call after the first starts with the global update
            if (s->c.global_kind >= 0) {
                // every thread reads the call count before thread 0 bumps it
                const bool global_first = s->c.sched_calls > 0;
                __syncthreads();
                if (global_first) {
                    if (res) g_to_global(x);
                    global_update(x, s->c.global_kind);
                    if (res) g_to_arena(x);
                }
                if (threadIdx.x == 0) s->c.sched_calls += 1;
                __syncthreads();
            }
            for (int t = 0; t < 2 * s->c.M; ++t) {
                long long t0 = phase_start();
                sweep_spatial(x);
                phase_stop(x, DQMC_PHASE_SWEEP_SPATIAL, t0);
                propagate(x);
            }
            after_sweep(x);
        }
        if (res) g_to_global(x);
        break;
    }
    case DQMC_OP_BUILD:
        reverse_build_stack(x);
        propagate(x);
        break;
    case DQMC_OP_BUILD_FWD:
        build_stack(x);
        break;
    case DQMC_OP_GREENS_AT:
        calculate_greens_at(x, arg0, arg1, s->c.out);
        break;
    case DQMC_OP_PHYSICAL:
        greens_physical(x, s->c.G, s->c.out);
        break;
    case DQMC_OP_PROPAGATE:
        propagate(x);
        break;
    case DQMC_OP_SWEEP_SPATIAL:
        sweep_spatial(x);
        break;
    case DQMC_OP_GLOBAL:
        global_update(x, arg0);
        break;
    case DQMC_OP_REPLICA_WEIGHT:
        if (s->c.partner >= 0) replica_weight(x, chains);
        break;
    case DQMC_OP_REPLICA_ACCEPT:
        if (s->c.partner >= 0) replica_accept(x, chains, (int)blockIdx.x);
        break;
    case DQMC_OP_TD_MEASURE:  // chains without time-displaced measurements skip
        if (s->c.td && s->c.ut) td_measure(x);
        break;
    case DQMC_OP_GREENS_KL:
        if (s->c.ut && s->c.ut_pairs && s->c.ut_out) greens_kl(x, arg0, arg1 != 0);
        else if (threadIdx.x == 0) s->c.status = 1;
        break;
    default:
        break;
    }
    __syncthreads();
    if (use_tc) {
        // every product waited for its MMAs; release the columns
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
#if DQMC_TC_BUILD
        if ((threadIdx.x >> 5) == 0) tc_dealloc(s->tc.tmem, DQMC_TC_COLS);
#endif
    }
    if (fsplit) {
        // rank 0 takes over its partner's status; then both leave together
        // (also after a rendezvous time-out: no CTA leaves while its partner
        // may still read its shared memory)
        if (xsync(x)) {
            if (threadIdx.x == 0 && rank == 0) {
                const int st = peer_ld_s32(peer_addr(&s->c.status, x.peer));
                if (st != 0 && s->c.status == 0) s->c.status = st;
            }
            xsync(x);
        }
        cluster_barrier();
        if (rank == 1) return;
    }
    // write back the mutable state
    if (threadIdx.x == 0) {
        DqmcChain& g = chains[slot];
        g.ctr = s->c.ctr;
        g.current_slice = s->c.current_slice;
        g.current_range = s->c.current_range;
        g.direction = s->c.direction;
        g.prop_err_max = s->c.prop_err_max;
        g.prop_err_reported = s->c.prop_err_reported;
        g.n_prop_err = s->c.n_prop_err;
        g.n_neg_p = s->c.n_neg_p;
        g.n_near_tie = s->c.n_near_tie;
        g.min_tie_gap = s->c.min_tie_gap;
        g.n_imag_p = s->c.n_imag_p;
        g.max_imag_p = s->c.max_imag_p;
        for (int q = 0; q < 3; ++q) {
            g.ms_prop[q] = s->c.ms_prop[q];
            g.ms_neg[q] = s->c.ms_neg[q];
            g.ms_imag[q] = s->c.ms_imag[q];
        }
        g.accepted = s->c.accepted;
        g.proposals = s->c.proposals;
        for (int p = 0; p < 8; ++p) g.timers[p] = s->c.timers[p];
        g.needs_build = s->c.needs_build;
        g.visits_quota = s->c.visits_quota;
        g.visits_done = s->c.visits_done;
        g.sweep = s->c.sweep;
        g.g_accepted = s->c.g_accepted;
        g.g_proposals = s->c.g_proposals;
        g.sched_calls = s->c.sched_calls;
        if (op == DQMC_OP_REPLICA_WEIGHT) {  // read by the partner in the next launch only
            g.r_weight = s->c.r_weight;
            g.r_prob = s->c.r_prob;
        }
        if (s->c.status) g.status = s->c.status;
    }
}

}  // namespace
}  // namespace dqmc

#if !DQMC_TC_BUILD
size_t dqmc_chain_kernel_smem() { return sizeof(dqmc::Smem); }
#endif

static bool g_attr_set[64] = {};

cudaError_t DQMC_KERNEL_ENTRY(dqmc_prepare_chain_kernel)() {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    if (!g_attr_set[dev]) {
        e = cudaFuncSetAttribute(dqmc::chain_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sizeof(dqmc::Smem));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(dqmc::chain_kernel<4>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)sizeof(dqmc::Smem));
        // the whole unified L1 / shared array as shared memory: two CTAs of
        // ~97 KB per SM need more than the smaller carve-outs leave
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(dqmc::chain_kernel<2>,
                                     cudaFuncAttributePreferredSharedMemoryCarveout,
                                     cudaSharedmemCarveoutMaxShared);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(dqmc::chain_kernel<4>,
                                     cudaFuncAttributePreferredSharedMemoryCarveout,
                                     cudaSharedmemCarveoutMaxShared);
        if (e != cudaSuccess) return e;
        g_attr_set[dev] = true;
    }
    return cudaSuccess;
}

cudaError_t DQMC_KERNEL_ENTRY(dqmc_launch_chain_kernel)(DqmcChain* d_chains, int nchains, int op,
                                                        int arg0, int arg1, cudaStream_t stream,
                                                        int n_max, bool pairs) {
    cudaError_t e = DQMC_KERNEL_ENTRY(dqmc_prepare_chain_kernel)();
    if (e != cudaSuccess) return e;
    // arena the chains need: 2 n (n + 1) doubles for the largest n <= 64
    // (n_max <= 0: unknown, e.g. a pool whose chains change between replays:
    // the whole arena)
    const int na = (n_max <= 0 || n_max > 64) ? 64 : n_max;
    const int cap = 2 * na * (na + 1);
    const size_t smem = offsetof(dqmc::Smem, arena) + (size_t)cap * sizeof(double);
    if (pairs) {
        // two CTAs per chain in two-CTA clusters (flavour-split chains)
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(2u * (unsigned)nchains);
        cfg.blockDim = dim3(DQMC_NT);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = stream;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = 2;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        return cudaLaunchKernelEx(&cfg, dqmc::chain_kernel<2>, d_chains, nchains, op, arg0, arg1,
                                  cap);
    }
    if (n_max > 0 && n_max <= 32)
        dqmc::chain_kernel<4><<<nchains, DQMC_NT, smem, stream>>>(d_chains, nchains, op, arg0,
                                                                  arg1, cap);
    else
        dqmc::chain_kernel<2><<<nchains, DQMC_NT, smem, stream>>>(d_chains, nchains, op, arg0,
                                                                  arg1, cap);
    return cudaGetLastError();
}

#if !DQMC_TC_BUILD
cudaError_t dqmc_prepare_chain_kernels() {
    cudaError_t e = dqmc_prepare_chain_kernel();
    return e == cudaSuccess ? dqmc_prepare_chain_kernel_tc() : e;
}
cudaError_t dqmc_launch_chain_kernel(DqmcChain* d_chains, int nchains, int op, int arg0, int arg1,
                                     cudaStream_t stream, int n_max, bool tc, bool pairs) {
    return tc ? dqmc_launch_chain_kernel_tc(d_chains, nchains, op, arg0, arg1, stream, n_max, pairs)
              : dqmc_launch_chain_kernel(d_chains, nchains, op, arg0, arg1, stream, n_max, pairs);
}
#endif
