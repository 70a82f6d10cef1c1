// The chain kernel with the tensor-core products (mm_tc, dqmc_tc.cuh)
// compiled in: launched for handles and pools whose chains may run their
// products on the tensor cores (real mixed-precision chains with
// 96 <= n <= 256); everything else uses the build of dqmc_kernels.cu.
#define DQMC_TC_BUILD 1
#include "dqmc_kernels.cu"
