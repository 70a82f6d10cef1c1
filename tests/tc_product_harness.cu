// Harness of the tensor-core product mm_tc (dqmc_tc.cuh): one CTA computes
// C = op(A) op(B) for random n x n FP64 operands whose rows and columns span
// scales of 2^-12 .. 2^12, on the tensor cores (mode 0), as the double-float
// FP32-pipe product (mode 1) and as the FP64 product (mode 2); prints per
// product the largest error relative to sum_k |a_ik b_kj| (against a
// double-double host reference), the largest error relative to |c_ij|, the
// time per product (CUDA events) and the status of the mbarrier waits.
// Usage: tc_product_harness [n]  (n: only that size, tensor-core product
// only; default: every size, all three products at n = 144 and 256).
// Exit status 2 when a tensor-core product misses 1e-13 of sum |a b| or a
// wait timed out.
#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <math.h>
#include <vector>
#include <random>
#include "../montecarlo.jl_gb300/csrc/dqmc_tc.cuh"

using namespace dqmc;

template <int MODE, bool TA, bool TB>
__global__ void __launch_bounds__(256, 1) probe(int n, const double* A, const double* B, double* C,
                                                int reps, unsigned* status, long long* cyc,
                                                unsigned char* scratch) {
    extern __shared__ __align__(128) unsigned char sm[];
    __shared__ TcState ts;
    __shared__ uint32_t tbase;
    const int tid = threadIdx.x, warp = tid >> 5;
    if (MODE == 0) {
        if (warp == 0) tc_alloc(&tbase, DQMC_TC_COLS);
        if (tid == 0) {
            for (int b = 0; b < 2; ++b) {
                mbar_init(&ts.full[b], 1);
                mbar_init(&ts.mma[b], 1);
                ts.ph_full[b] = ts.ph_mma[b] = 0;
            }
            ts.status = 0;
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) ts.tmem = tbase;
        __syncthreads();
    }
    long long t0 = clock64();
    for (int r = 0; r < reps; ++r) {
        if (MODE == 0) {
            if (!mm_tc<false, false, false, TA, TB>(n, C, A, B, sm, &ts, scratch)) break;
        } else if (MODE == 1) {
            mm_dfx<false, false, false, TA, TB>(n, C, A, B, (double*)sm);
        } else {
            mm<TA, TB>(n, C, A, B, (double*)sm);
        }
        __syncthreads();
    }
    long long t1 = clock64();
    if (MODE == 0) {
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (warp == 0) tc_dealloc(ts.tmem, DQMC_TC_COLS);
        if (tid == 0) *status = ts.status;
    }
    if (tid == 0) *cyc = t1 - t0;
}

// double-double dot product reference
static void two_prod(double a, double b, double& p, double& e) { p = a * b; e = fma(a, b, -p); }
static void two_sum(double a, double b, double& s, double& e) {
    s = a + b; double z = s - a; e = (a - (s - z)) + (b - z);
}

#define CK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { printf("CUDA %s at %d: %s\n", #x, __LINE__, cudaGetErrorString(e_)); exit(1);} } while (0)

static int g_bad = 0;
template <int MODE, bool TA, bool TB>
void run(int n, const std::vector<double>& A, const std::vector<double>& B, int reps, const char* name) {
    double *dA, *dB, *dC;
    unsigned* dst;
    long long* dcyc;
    size_t bytes = (size_t)n * n * 8;
    CK(cudaMalloc(&dA, bytes)); CK(cudaMalloc(&dB, bytes)); CK(cudaMalloc(&dC, bytes));
    CK(cudaMalloc(&dst, 4)); CK(cudaMalloc(&dcyc, 8));
    unsigned char* dscr;
    CK(cudaMalloc(&dscr, dqmc_tc_scratch_bytes(n)));
    CK(cudaMemcpy(dA, A.data(), bytes, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dB, B.data(), bytes, cudaMemcpyHostToDevice));
    CK(cudaMemset(dC, 0, bytes)); CK(cudaMemset(dst, 0, 4));
    int smem = MODE == 0 ? DQMC_TC_SMEM : 4 * 16 * 64 * 8;
    CK(cudaFuncSetAttribute(probe<MODE, TA, TB>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    probe<MODE, TA, TB><<<1, 256, smem>>>(n, dA, dB, dC, 1, dst, dcyc, dscr);
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0); cudaEventCreate(&e1);
    cudaEventRecord(e0);
    probe<MODE, TA, TB><<<1, 256, smem>>>(n, dA, dB, dC, reps, dst, dcyc, dscr);
    cudaEventRecord(e1);
    CK(cudaDeviceSynchronize());
    float ms = 0; cudaEventElapsedTime(&ms, e0, e1);
    std::vector<double> C((size_t)n * n);
    unsigned st = 0; long long cyc = 0;
    CK(cudaMemcpy(C.data(), dC, bytes, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&st, dst, 4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&cyc, dcyc, 8, cudaMemcpyDeviceToHost));
    // reference
    double maxbound = 0, maxrel = 0;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            double s = 0, c = 0, ab = 0;
            for (int k = 0; k < n; ++k) {
                double a = TA ? A[k + (size_t)i * n] : A[i + (size_t)k * n];
                double b = TB ? B[j + (size_t)k * n] : B[k + (size_t)j * n];
                double p, e, s2, e2;
                two_prod(a, b, p, e);
                two_sum(s, p, s2, e2);
                s = s2; c += e + e2;
                ab += fabs(a * b);
            }
            double ref = s + c;
            double got = C[i + (size_t)j * n];
            double err = fabs(got - ref);
            if (ab > 0) maxbound = fmax(maxbound, err / ab);
            if (ref != 0) maxrel = fmax(maxrel, err / fabs(ref));
            if (err != err) maxbound = INFINITY;
        }
    if (MODE == 0 && (st != 0 || !(maxbound < 1e-13))) g_bad = 1;
    printf("%-28s n=%3d status=%u  err/sum|ab| = %.3e  maxrel = %.3e  per-product %.1f us (%lld cyc)\n",
           name, n, st, maxbound, maxrel, 1e3 * ms / reps, cyc / reps);
    cudaFree(dA); cudaFree(dB); cudaFree(dC); cudaFree(dst); cudaFree(dcyc); cudaFree(dscr);
}

int main(int argc, char** argv) {
    std::mt19937_64 g(7);
    std::normal_distribution<double> N01(0, 1);
    std::uniform_int_distribution<int> ex(-12, 12);
    int ns[] = {16, 64, 100, 144, 256};
    const int only = argc > 1 ? atoi(argv[1]) : 0;
    for (int n : ns) {
        if (only && n != only) continue;
        std::vector<double> A((size_t)n * n), B((size_t)n * n);
        std::vector<int> rs(n), cs(n);
        for (int i = 0; i < n; ++i) { rs[i] = ex(g); cs[i] = ex(g); }
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) {
                A[i + (size_t)j * n] = ldexp(N01(g), rs[i]);
                B[i + (size_t)j * n] = ldexp(N01(g), cs[j]);
            }
        int reps = n <= 64 ? 20 : 5;
        run<0, false, false>(n, A, B, only ? 1 : reps, "tc");
        if (!only && (n == 144 || n == 256)) {
            run<0, true, false>(n, A, B, reps, "tc TA");
            run<0, false, true>(n, A, B, reps, "tc TB");
            run<1, false, false>(n, A, B, reps, "dfx");
            run<2, false, false>(n, A, B, reps, "fp64");
        }
    }
    printf(g_bad ? "TC_PROBE_BAD\n" : "TC_PROBE_OK\n");
    return g_bad ? 2 : 0;
}
