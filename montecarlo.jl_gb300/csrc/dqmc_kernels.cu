// The DQMC chain kernel: one CTA runs one chain of the reference's DQMC
// (src/flavors/DQMC) entirely on the device -- local sweeps with rank-1
// Green's function updates, wraps, slice-matrix chains, UDT stabilisation and
// Green's function reconstruction -- for as many sweeps as requested, so a
// whole batch of chains advances in one launch.
#include <cuda_runtime.h>
#include <stdint.h>

#include "dqmc_chain_ops.cuh"
#include "dqmc_kernels.h"

namespace dqmc {

__global__ void __launch_bounds__(DQMC_NT, 2) chain_kernel(DqmcChain* chains, int nchains, int op,
                                                        int arg0, int arg1) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem* s = reinterpret_cast<Smem*>(smem_raw);
    if ((int)blockIdx.x >= nchains) return;
    // stage this chain's descriptor in shared memory
    {
        const int words = (int)(sizeof(DqmcChain) / 4);
        const uint32_t* src = reinterpret_cast<const uint32_t*>(chains + blockIdx.x);
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
    if (threadIdx.x == 0) {
        s->Gglob = s->c.G;
        s->gres = 0;
    }
    __syncthreads();
    if (x.n > DQMC_NMAX || x.nf < 1 || x.nf > 2) {
        if (threadIdx.x == 0) chains[blockIdx.x].status = 1;
        return;
    }
    switch (op) {
    case DQMC_OP_SWEEP: {
        const bool res = g_resident_possible(x);
        if (res) g_to_arena(x);
        for (int sw = 0; sw < arg0; ++sw) {
            for (int t = 0; t < 2 * s->c.M; ++t) {
                long long t0 = phase_start();
                sweep_spatial(x);
                phase_stop(x, DQMC_PHASE_SWEEP_SPATIAL, t0);
                propagate(x);
            }
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
    default:
        break;
    }
    __syncthreads();
    // write back the mutable state
    if (threadIdx.x == 0) {
        DqmcChain& g = chains[blockIdx.x];
        g.ctr = s->c.ctr;
        g.current_slice = s->c.current_slice;
        g.current_range = s->c.current_range;
        g.direction = s->c.direction;
        g.prop_err_max = s->c.prop_err_max;
        g.prop_err_reported = s->c.prop_err_reported;
        g.n_prop_err = s->c.n_prop_err;
        g.n_neg_p = s->c.n_neg_p;
        g.accepted = s->c.accepted;
        g.proposals = s->c.proposals;
        for (int p = 0; p < 8; ++p) g.timers[p] = s->c.timers[p];
    }
}

}  // namespace dqmc

size_t dqmc_chain_kernel_smem() { return sizeof(dqmc::Smem); }

cudaError_t dqmc_launch_chain_kernel(DqmcChain* d_chains, int nchains, int op, int arg0, int arg1,
                                     cudaStream_t stream) {
    static bool attr_set = false;
    const size_t smem = sizeof(dqmc::Smem);
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(dqmc::chain_kernel,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    dqmc::chain_kernel<<<nchains, DQMC_NT, smem, stream>>>(d_chains, nchains, op, arg0, arg1);
    return cudaGetLastError();
}
