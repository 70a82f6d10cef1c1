// Allocation-free Green's function entry point.
//
// Some hosts cannot allocate device memory at the moment they need a Green's
// function: a host that has handed the whole device memory budget to its own
// pool allocator (so a cudaMalloc from a library would fail or break the
// budget), or a latency-critical loop in which cudaMalloc / cudaFree would add
// device-wide synchronisation.  For them, dqmc_calculate_greens_noalloc
// computes calculate_greens(mc, slice) -- the same device code as
// dqmc_calculate_greens -- with every work matrix in one file-scope device
// array of fixed size instead of a handle's workspace.  The caller passes its
// inputs and its output in device memory; the call allocates nothing.
//
// Limits and rules:
//   - n_flavors * n_sites^2 <= DQMC_NOALLOC_MAX_MAT (8192, e.g. an 8x8 lattice
//     with two flavour blocks or n_sites <= 90 with one); larger chains are
//     rejected with DQMC_ERR_INVALID.  The array is 8 * 8192 doubles plus
//     vectors, about 0.53 MB, held by every GPU that loads the library until
//     the process exits.
//   - The first call on a device (that device current) looks up the array's
//     device address with cudaGetSymbolAddress; make that first call before
//     any stream capture.
//   - All calls share the one array, which keeps the previous call's contents;
//     every element a call reads is written by that call first, so nothing
//     needs clearing.  Calls whose work overlaps on the GPU (different streams,
//     host threads, or devices sharing a context) race on the array and must be
//     serialised by the caller.
#include <cuda_runtime.h>
#include <string.h>

#include <mutex>
#include <string>

#include "../../include/dqmc_gb300.h"
#include "dqmc_chain_ops.cuh"
#include "dqmc_host_tables.h"
#include "dqmc_kernels.h"

#define DQMC_NOALLOC_MAX_MAT 8192
#define DQMC_NOALLOC_MAX_VEC 256
#define DQMC_NOALLOC_MAX_DEVICES 64

namespace {

struct NoallocScratch {
    double mats[8][DQMC_NOALLOC_MAX_MAT];  // currU, Ur, Ul, Tr, Tl, tmp1, tmp2, UDT scratch
    double vecs[3][DQMC_NOALLOC_MAX_VEC];  // Dl, Dr, Householder tau
    int pivot[DQMC_NOALLOC_MAX_VEC];
};

static __device__ __align__(256) NoallocScratch g_noalloc_scratch;

__global__ void __launch_bounds__(DQMC_NT, 2)
    greens_at_noalloc_kernel(const __grid_constant__ DqmcChain desc, int slice, int safe_mult,
                             double* out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    dqmc::Smem* s = reinterpret_cast<dqmc::Smem*>(smem_raw);
    {
        const int words = (int)(sizeof(DqmcChain) / 4);
        const uint32_t* src = reinterpret_cast<const uint32_t*>(&desc);
        uint32_t* dst = reinterpret_cast<uint32_t*>(&s->c);
        for (int e = threadIdx.x; e < words; e += DQMC_NT) dst[e] = src[e];
    }
    if (threadIdx.x == 0) {  // G stays in global memory; no tensor products here
        s->Gglob = s->c.G;
        s->gres = 0;
        s->gdfg = 0;
        s->tc_on = 0;
        s->arena_cap = (int)(sizeof(s->arena) / sizeof(double));
    }
    __syncthreads();
    dqmc::Ctx x;
    x.s = s;
    x.c = &s->c;
    x.n = s->c.n;
    x.nf = s->c.nf;
    x.nn = (size_t)x.n * x.n;
    x.b0 = 0;
    x.b1 = x.nf;
    x.peer = -1;
    dqmc::calculate_greens_at(x, slice, safe_mult, out);
}

std::mutex g_setup_mutex;
void* g_scratch_addr[DQMC_NOALLOC_MAX_DEVICES] = {};
bool g_attr_set[DQMC_NOALLOC_MAX_DEVICES] = {};

}  // namespace

extern "C" int dqmc_calculate_greens_noalloc(const dqmc_chain_config* cfg,
                                             const double* d_hopping, const int8_t* d_conf,
                                             int slice, int safe_mult, double* d_out,
                                             void* cuda_stream) {
    if (!cfg || !d_hopping || !d_conf || !d_out)
        return dqmc_report_error(DQMC_ERR_INVALID, "dqmc_calculate_greens_noalloc: null argument");
    const dqmc_chain_config& c = *cfg;
    int want_nf = (c.field == DQMC_FIELD_MAGNETIC_HIRSCH || c.field == DQMC_FIELD_MAGNETIC_GHQ) ? 2 : 1;
    if (c.n_sites < 1 || c.slices < 1 || c.field < 0 || c.field > 3 || c.n_flavors != want_nf)
        return dqmc_report_error(DQMC_ERR_INVALID,
                                 "dqmc_calculate_greens_noalloc: invalid chain configuration");
    const long long mat = (long long)c.n_flavors * c.n_sites * c.n_sites;
    if (mat > DQMC_NOALLOC_MAX_MAT || (long long)c.n_flavors * c.n_sites > DQMC_NOALLOC_MAX_VEC)
        return dqmc_report_error(
            DQMC_ERR_INVALID,
            "dqmc_calculate_greens_noalloc: n_flavors * n_sites^2 = " + std::to_string(mat) +
                " exceeds the fixed scratch of " + std::to_string(DQMC_NOALLOC_MAX_MAT) +
                " elements per matrix (use dqmc_calculate_greens with a handle instead)");
    if (slice < 0 || slice > c.slices)
        return dqmc_report_error(DQMC_ERR_INVALID,
                                 "dqmc_calculate_greens_noalloc: slice out of range 0..M");
    if (c.alpha_imag != 0.0)
        return dqmc_report_error(DQMC_ERR_INVALID,
                                 "dqmc_calculate_greens_noalloc: real chains only (alpha_imag != 0)");
    if (safe_mult <= 0) safe_mult = c.safe_mult;
    if (safe_mult <= 0)
        return dqmc_report_error(DQMC_ERR_INVALID, "dqmc_calculate_greens_noalloc: safe_mult <= 0");

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return dqmc_report_error(DQMC_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= DQMC_NOALLOC_MAX_DEVICES)
        return dqmc_report_error(DQMC_ERR_INVALID, "dqmc_calculate_greens_noalloc: device index too large");
    void* base = nullptr;
    {
        // set-up, once per device, with that device current
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_scratch_addr[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p)
                return dqmc_report_error(DQMC_ERR_CUDA, std::string("cudaGetSymbolAddress: ") +
                                                            cudaGetErrorString(e));
            g_scratch_addr[dev] = p;
        }
        if (!g_attr_set[dev]) {
            e = cudaFuncSetAttribute(greens_at_noalloc_kernel,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)sizeof(dqmc::Smem));
            if (e != cudaSuccess)
                return dqmc_report_error(DQMC_ERR_CUDA, std::string("cudaFuncSetAttribute: ") +
                                                            cudaGetErrorString(e));
            g_attr_set[dev] = true;
        }
        base = g_scratch_addr[dev];
    }
    NoallocScratch* sc = reinterpret_cast<NoallocScratch*>(base);

    DqmcChain d;
    memset(&d, 0, sizeof(d));
    d.n = c.n_sites; d.nf = c.n_flavors; d.M = c.slices; d.k = safe_mult; d.kind = c.field;
    d.ns = c.n_sites;
    d.check_prop = 0;
    d.prec = DQMC_PREC_FP64;
    d.nr = 0;
    dqmc_host::fill_tables(d, c.field, c.alpha);
    const size_t nn = (size_t)c.n_sites * c.n_sites;
    d.conf = const_cast<int8_t*>(d_conf);
    d.eT2 = d_hopping; d.eT2inv = d_hopping + nn; d.eTh = d_hopping + 2 * nn;
    d.eThinv = d_hopping + 3 * nn;
    d.currU = sc->mats[0]; d.Ur = sc->mats[1]; d.Ul = sc->mats[2]; d.Tr = sc->mats[3];
    d.Tl = sc->mats[4]; d.tmp1 = sc->mats[5]; d.tmp2 = sc->mats[6]; d.out = sc->mats[7];
    d.Dl = sc->vecs[0]; d.Dr = sc->vecs[1]; d.tempv = sc->vecs[2];
    d.pivot = sc->pivot;
    d.key = c.seed;

    cudaStream_t stream = (cudaStream_t)cuda_stream;
    greens_at_noalloc_kernel<<<1, DQMC_NT, sizeof(dqmc::Smem), stream>>>(d, slice, safe_mult, d_out);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return dqmc_report_error(DQMC_ERR_CUDA, std::string("noalloc kernel launch: ") +
                                                    cudaGetErrorString(e));
    return DQMC_OK;
}
