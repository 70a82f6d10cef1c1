#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#include "dqmc_chain.h"

size_t dqmc_chain_kernel_smem();
// Sets the kernel's shared-memory attribute once per device (call before any
// stream capture of a launch).
cudaError_t dqmc_prepare_chain_kernel();
// One CTA per chain; op is one of DQMC_OP_*.  n_max: the largest n_sites of
// the launch's chains (sizes the shared-memory arena and picks the kernel
// variant); <= 0 when the chains may change between replays of a captured
// launch (pools): the full arena.
cudaError_t dqmc_launch_chain_kernel(DqmcChain* d_chains, int nchains, int op, int arg0, int arg1,
                                     cudaStream_t stream, int n_max);

#include <string>
// Records `msg` as the calling thread's dqmc_last_error() text; returns `code`.
int dqmc_report_error(int code, const std::string& msg);
