#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#include "dqmc_chain.h"

size_t dqmc_chain_kernel_smem();
// Sets the kernels' shared-memory attributes once per device (call before any
// stream capture of a launch).
cudaError_t dqmc_prepare_chain_kernel();
cudaError_t dqmc_prepare_chain_kernel_tc();
cudaError_t dqmc_prepare_chain_kernels();  // both builds
// One CTA per chain; op is one of DQMC_OP_*.  n_max: the largest n_sites of
// the launch's chains (sizes the shared-memory arena and picks the kernel
// variant); <= 0 when the chains may change between replays of a captured
// launch (pools): the full arena.  The first two take one build; the third
// picks the tensor-core build when tc (the launch holds chains whose
// products may run on the tensor cores).  pairs: two CTAs per chain in
// two-CTA clusters (DQMC_OP_RUN of a pool with flavour-split chains).
cudaError_t dqmc_launch_chain_kernel(DqmcChain* d_chains, int nchains, int op, int arg0, int arg1,
                                     cudaStream_t stream, int n_max, bool pairs);
cudaError_t dqmc_launch_chain_kernel_tc(DqmcChain* d_chains, int nchains, int op, int arg0,
                                        int arg1, cudaStream_t stream, int n_max, bool pairs);
cudaError_t dqmc_launch_chain_kernel(DqmcChain* d_chains, int nchains, int op, int arg0, int arg1,
                                     cudaStream_t stream, int n_max, bool tc, bool pairs);

// The sweep of chains with n <= 32 sites, one warp per chain (dqmc_warp.cu):
// nsweeps sweeps of every chain.  n_max: the largest n of the launch (<= 32).
// Eligible chains: real, FP64, dense hopping, no device measurements, no
// scheduled global update (free pool slots are skipped).
bool dqmc_warp_kernel_eligible(const DqmcChain& d);
cudaError_t dqmc_launch_warp_kernel(DqmcChain* d_chains, int nchains, int nsweeps,
                                    cudaStream_t stream, int n_max);

#include <string>
// Records `msg` as the calling thread's dqmc_last_error() text; returns `code`.
int dqmc_report_error(int code, const std::string& msg);
