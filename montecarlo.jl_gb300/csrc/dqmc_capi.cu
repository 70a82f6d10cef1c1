// C ABI of libdqmc_gb300.so (declared in include/dqmc_gb300.h): handle and
// device-memory management, host-side tables, launches and error reporting.
#include <cuda_runtime.h>
#include <math.h>
#include <cmath>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <map>
#include <vector>

#include "../../include/dqmc_gb300.h"
#include "dqmc_chain.h"
#include "dqmc_host_tables.h"
#include "dqmc_kernels.h"
#include "dqmc_tc.cuh"
#include "philox.h"

using dqmc_host::fill_tables;
using dqmc_host::fill_tables_complex;
using dqmc_host::generate_chunks;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    return fail(e == cudaErrorMemoryAllocation ? DQMC_ERR_OOM : DQMC_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

#define CUDA_TRY(expr, what)                       \
    do {                                           \
        cudaError_t _e = (expr);                   \
        if (_e != cudaSuccess) return cuda_fail(_e, what); \
    } while (0)

bool is_cplx(const dqmc_chain_config& c) { return c.alpha_imag != 0.0; }
// matrix dimension on the device: a complex chain keeps the real 2n x 2n
// representation [[Re, -Im], [Im, Re]] of its n x n complex matrices
size_t mat_n(const dqmc_chain_config& c) {
    return is_cplx(c) ? 2 * (size_t)c.n_sites : (size_t)c.n_sites;
}
size_t mat_elems(const dqmc_chain_config& c) { return (size_t)c.n_flavors * mat_n(c) * mat_n(c); }
// doubles of one matrix as the caller passes it (complex: re, im per entry)
size_t user_elems(const dqmc_chain_config& c) {
    return (is_cplx(c) ? 2 : 1) * (size_t)c.n_flavors * c.n_sites * c.n_sites;
}
// representation -> interleaved complex (Julia's Matrix{ComplexF64} layout), nf blocks
void rep_to_complex(const dqmc_chain_config& c, const double* E, double* out) {
    const size_t n = c.n_sites, n2 = 2 * n;
    for (size_t b = 0; b < (size_t)c.n_flavors; ++b) {
        const double* Eb = E + b * n2 * n2;
        double* ob = out + 2 * b * n * n;
        for (size_t col = 0; col < n; ++col)
            for (size_t r = 0; r < n; ++r) {
                ob[2 * (col * n + r)] = Eb[col * n2 + r];
                ob[2 * (col * n + r) + 1] = Eb[col * n2 + n + r];
            }
    }
}
void complex_to_rep(const dqmc_chain_config& c, const double* in, double* E) {
    const size_t n = c.n_sites, n2 = 2 * n;
    for (size_t b = 0; b < (size_t)c.n_flavors; ++b) {
        double* Eb = E + b * n2 * n2;
        const double* ib = in + 2 * b * n * n;
        for (size_t col = 0; col < n; ++col)
            for (size_t r = 0; r < n; ++r) {
                const double re = ib[2 * (col * n + r)], im = ib[2 * (col * n + r) + 1];
                Eb[col * n2 + r] = re;
                Eb[col * n2 + n + r] = im;
                Eb[(n + col) * n2 + r] = -im;
                Eb[(n + col) * n2 + n + r] = re;
            }
    }
}
// a real n x n matrix as the representation of a complex one: diag(A, A)
void real_to_rep(size_t n, const double* A, double* E) {
    const size_t n2 = 2 * n;
    for (size_t e = 0; e < n2 * n2; ++e) E[e] = 0.0;
    for (size_t col = 0; col < n; ++col)
        for (size_t r = 0; r < n; ++r) {
            E[col * n2 + r] = A[col * n + r];
            E[(n + col) * n2 + n + r] = A[col * n + r];
        }
}

struct Layout {
    size_t bytes;
    size_t off_conf, off_hop, off_G, off_Gtmp, off_Ul, off_Ur, off_Tl, off_Tr, off_tmp1, off_tmp2,
        off_currU, off_out, off_ustack, off_tstack, off_dstack, off_Dl, off_Dr, off_tempv,
        off_pivot, off_meas, off_qcs, off_tconf, off_tempvf, off_hopdf, off_tcs;
};

// chains whose products may run on the tensor cores (mm_tc, dqmc_tc.cuh):
// real, mixed precision, 96 <= n <= 256; they carry its slice scratch
bool tc_capable(const dqmc_chain_config& c, int prec) {
    return prec == DQMC_PREC_MIXED && !is_cplx(c) && c.n_sites >= 96 && c.n_sites <= DQMC_TC_NMAX;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

Layout layout_of(const dqmc_chain_config& c, int prec) {
    Layout L;
    const size_t n = mat_n(c), nf = c.n_flavors, ms = mat_elems(c) * sizeof(double);
    const size_t nconf = (size_t)c.n_sites * c.slices;
    const int nr = (c.slices + c.safe_mult - 1) / c.safe_mult;
    size_t o = 0;
    L.off_conf = o; o = align256(o + nconf);
    L.off_hop = o; o = align256(o + 4 * n * n * sizeof(double));
    size_t* mats[] = {&L.off_G, &L.off_Gtmp, &L.off_Ul, &L.off_Ur, &L.off_Tl, &L.off_Tr,
                      &L.off_tmp1, &L.off_tmp2, &L.off_currU, &L.off_out};
    for (size_t* m : mats) { *m = o; o = align256(o + ms); }
    L.off_ustack = o; o = align256(o + ms * (nr + 1));
    L.off_tstack = o; o = align256(o + ms * (nr + 1));
    L.off_dstack = o; o = align256(o + nf * n * sizeof(double) * (nr + 1));
    L.off_Dl = o; o = align256(o + nf * n * sizeof(double));
    L.off_Dr = o; o = align256(o + nf * n * sizeof(double));
    L.off_tempv = o; o = align256(o + nf * n * sizeof(double));
    L.off_pivot = o; o = align256(o + nf * n * sizeof(int));
    L.off_meas = o; o = align256(o + DQMC_MEAS_DOUBLES(n, nf) * sizeof(double));
    L.off_qcs = o; o = align256(o + 2 * n * sizeof(double));
    L.off_tconf = o; o = align256(o + nconf);
    L.off_tempvf = o; o = align256(o + nf * n * sizeof(double));
    L.off_hopdf = o; o = align256(o + 2 * n * n * sizeof(float2));
    L.off_tcs = o;
    if (tc_capable(c, prec)) o = align256(o + nf * dqmc_tc_scratch_stride((int)n));
    L.bytes = o;
    return L;
}

}  // namespace

struct dqmc_handle {
    int device = 0;
    int precision = DQMC_PREC_FP64;
    cudaStream_t stream = nullptr;      // stream in use (own or caller's)
    cudaStream_t own_stream = nullptr;
    std::vector<dqmc_chain_config> cfg;
    std::vector<Layout> lay;
    std::vector<DqmcChain> host;  // descriptors (pointers into `arena`)
    char* arena = nullptr;
    DqmcChain* d_chains = nullptr;
    bool host_dirty = false;      // host descriptors changed (must upload before launch)
    bool busy = false;
    // pool: slots admitted and released while others run, sub-allocated from
    // one device arena of `budget` bytes (first fit, 256-byte granules)
    bool pool = false;
    size_t budget = 0;
    std::map<size_t, size_t> free_blocks;  // offset -> bytes
    std::vector<size_t> slot_off, slot_bytes;
    DqmcChain* pinned = nullptr;           // pinned mirror for graph replays
    unsigned int* d_sync = nullptr;        // pools: the launch's visit counters (DqmcChain::run_sync)
    bool flavour_split = false;            // pools: two-flavour chains on two CTAs (dqmc_pool_set_flavour_split)
    int n_max = 0;                         // largest n_sites of a fixed handle's chains
    bool tc = false;                       // launches use the tensor-core kernel build
    bool small_kernel = true;              // sweeps of small chains one warp per chain
    std::vector<double*> ut_mem;           // per-chain unequal-time workspaces (lazy)
    std::vector<double*> cb_mem;           // per-chain checkerboard factors
    std::vector<double*> td_mem;           // per-chain time-displaced measurement buffers
    cudaGraphExec_t graph = nullptr;
    int graph_budget_us = -1;
};

namespace {

int check_chain(dqmc_handle* h, int chain) {
    if (!h) return fail(DQMC_ERR_INVALID, "null handle");
    if (chain < 0 || chain >= (int)h->cfg.size())
        return fail(DQMC_ERR_INVALID, "chain index " + std::to_string(chain) + " out of range");
    if (!h->host[chain].active)
        return fail(DQMC_ERR_INVALID, "slot " + std::to_string(chain) + " holds no chain");
    return DQMC_OK;
}

// refresh the host mirror of the mutable device state
int pull_descriptors(dqmc_handle* h) {
    CUDA_TRY(cudaMemcpyAsync(h->host.data(), h->d_chains, sizeof(DqmcChain) * h->host.size(),
                             cudaMemcpyDeviceToHost, h->stream),
             "download chain descriptors");
    CUDA_TRY(cudaStreamSynchronize(h->stream), "synchronize");
    return DQMC_OK;
}
int push_descriptors(dqmc_handle* h) {
    CUDA_TRY(cudaMemcpyAsync(h->d_chains, h->host.data(), sizeof(DqmcChain) * h->host.size(),
                             cudaMemcpyHostToDevice, h->stream),
             "upload chain descriptors");
    CUDA_TRY(cudaStreamSynchronize(h->stream), "synchronize");
    h->host_dirty = false;
    return DQMC_OK;
}

int launch(dqmc_handle* h, int op, int arg0, int arg1, bool sync) {
    // launches are stream-ordered, so queued asynchronous sweeps need no host
    // synchronisation here; host-side descriptor edits synchronise first
    if (h->busy && (sync || h->host_dirty)) {
        int st = dqmc_synchronize(h);
        if (st != DQMC_OK) return st;
    }
    CUDA_TRY(cudaSetDevice(h->device), "cudaSetDevice");
    if (h->host_dirty) {
        int st = push_descriptors(h);
        if (st != DQMC_OK) return st;
    }
    bool warp = op == DQMC_OP_SWEEP && !h->pool && h->small_kernel && h->n_max <= 32;
    for (size_t i = 0; warp && i < h->host.size(); ++i)
        warp = dqmc_warp_kernel_eligible(h->host[i]);
    if (warp)
        CUDA_TRY(dqmc_launch_warp_kernel(h->d_chains, (int)h->host.size(), arg0, h->stream, h->n_max),
                 "warp sweep kernel launch");
    else
        CUDA_TRY(dqmc_launch_chain_kernel(h->d_chains, (int)h->host.size(), op, arg0, arg1,
                                          h->stream, h->pool ? 0 : h->n_max, h->tc,
                                          h->pool && h->flavour_split && op == DQMC_OP_RUN),
                 "chain kernel launch");
    if (!sync) {
        h->busy = true;
        return DQMC_OK;
    }
    CUDA_TRY(cudaStreamSynchronize(h->stream), "chain kernel");
    int st = pull_descriptors(h);
    if (st != DQMC_OK) return st;
    for (size_t i = 0; i < h->host.size(); ++i)
        if (h->host[i].status != 0)
            return fail(DQMC_ERR_NUMERICAL, "chain " + std::to_string(i) + " reported status " +
                                                 std::to_string(h->host[i].status));
    return DQMC_OK;
}

int validate_config(const dqmc_chain_config& c, int i) {
    if (c.n_sites < 1 || c.n_sites > 512 || c.slices < 1 || c.safe_mult < 1 ||
        (c.n_flavors != 1 && c.n_flavors != 2) || c.field < 0 || c.field > 3)
        return fail(DQMC_ERR_INVALID, "invalid config for chain " + std::to_string(i) +
                                          " (need 1 <= n_sites <= 512, slices >= 1, safe_mult >= 1, "
                                          "n_flavors in {1,2}, field in 0..3)");
    int want_nf = (c.field == DQMC_FIELD_MAGNETIC_HIRSCH || c.field == DQMC_FIELD_MAGNETIC_GHQ) ? 2 : 1;
    if (c.n_flavors != want_nf)
        return fail(DQMC_ERR_INVALID, "n_flavors does not match the field kind");
    if ((c.slices + c.safe_mult - 1) / c.safe_mult > DQMC_MAX_CHUNKS)
        return fail(DQMC_ERR_INVALID, "too many stabilisation chunks (max 256)");
    if (!std::isfinite(c.alpha) || !std::isfinite(c.alpha_imag))
        return fail(DQMC_ERR_INVALID, "alpha is not finite");
    if (is_cplx(c) && c.n_sites > 128)
        return fail(DQMC_ERR_INVALID, "complex chains (alpha_imag != 0) need n_sites <= 128");
    return DQMC_OK;
}

// Fill the descriptor of a chain whose workspace starts at `b` (layout L).
void fill_descriptor(DqmcChain& d, const dqmc_chain_config& c, char* b, const Layout& L,
                     int precision) {
    memset(&d, 0, sizeof(d));
    d.n = (int)mat_n(c); d.nf = c.n_flavors; d.M = c.slices; d.k = c.safe_mult; d.kind = c.field;
    d.ns = c.n_sites;
    d.cplx = is_cplx(c) ? 1 : 0;
    d.check_prop = c.check_propagation_error ? 1 : 0;
    d.prec = precision;
    d.nr = generate_chunks(c.slices, c.safe_mult, d.rfirst, d.rlast);
    if (d.cplx) fill_tables_complex(d, c.field, c.alpha, c.alpha_imag);
    else fill_tables(d, c.field, c.alpha);
    const size_t nn = mat_n(c) * mat_n(c);
    double* hop = (double*)(b + L.off_hop);
    d.conf = (int8_t*)(b + L.off_conf);
    d.eT2 = hop; d.eT2inv = hop + nn; d.eTh = hop + 2 * nn; d.eThinv = hop + 3 * nn;
    d.eT2df = (const float2*)(b + L.off_hopdf);
    d.eT2invdf = d.eT2df + nn;
    d.G = (double*)(b + L.off_G); d.Gtmp = (double*)(b + L.off_Gtmp);
    d.Ul = (double*)(b + L.off_Ul); d.Ur = (double*)(b + L.off_Ur);
    d.Tl = (double*)(b + L.off_Tl); d.Tr = (double*)(b + L.off_Tr);
    d.tmp1 = (double*)(b + L.off_tmp1); d.tmp2 = (double*)(b + L.off_tmp2);
    d.currU = (double*)(b + L.off_currU); d.out = (double*)(b + L.off_out);
    d.ustack = (double*)(b + L.off_ustack); d.tstack = (double*)(b + L.off_tstack);
    d.dstack = (double*)(b + L.off_dstack);
    d.Dl = (double*)(b + L.off_Dl); d.Dr = (double*)(b + L.off_Dr);
    d.tempv = (double*)(b + L.off_tempv);
    d.pivot = (int*)(b + L.off_pivot);
    d.meas = (double*)(b + L.off_meas);
    d.qcs = nullptr;  // set with the measurement's q
    d.meas_rate = 1;
    d.temp_conf = (int8_t*)(b + L.off_tconf);
    d.tempvf = (double*)(b + L.off_tempvf);
    d.tcs = tc_capable(c, precision) ? (unsigned char*)(b + L.off_tcs) : nullptr;
    d.alpha_field = c.alpha;
    d.partner = -1;
    d.global_kind = -1;
    for (double* ms : {d.ms_prop, d.ms_neg, d.ms_imag}) {  // MagnitudeStats() (statistics.jl:16)
        ms[0] = -INFINITY;
        ms[1] = INFINITY;
        ms[2] = 0.0;
    }
    d.min_tie_gap = INFINITY;
    d.tc_enable = DQMC_TC_DEFAULT;
    d.key = c.seed; d.ctr = 0;
    d.current_slice = 0; d.current_range = 1; d.direction = 1;
    d.active = 1;
}

// first-fit sub-allocation from a pool's arena
bool pool_alloc(dqmc_handle* h, size_t bytes, size_t* off) {
    bytes = align256(bytes);
    for (auto it = h->free_blocks.begin(); it != h->free_blocks.end(); ++it) {
        if (it->second >= bytes) {
            *off = it->first;
            const size_t rest = it->second - bytes, at = it->first + bytes;
            h->free_blocks.erase(it);
            if (rest) h->free_blocks[at] = rest;
            return true;
        }
    }
    return false;
}
void pool_free(dqmc_handle* h, size_t off, size_t bytes) {
    bytes = align256(bytes);
    auto it = h->free_blocks.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != h->free_blocks.end() && it->first + it->second == nx->first) {
        it->second += nx->second;
        h->free_blocks.erase(nx);
    }
    if (it != h->free_blocks.begin()) {
        auto pv = std::prev(it);
        if (pv->first + pv->second == it->first) {
            pv->second += it->second;
            h->free_blocks.erase(it);
        }
    }
}

}  // namespace

extern "C" {

const char* dqmc_last_error(void) { return g_last_error.c_str(); }
int dqmc_abi_version(void) { return DQMC_GB300_ABI_VERSION; }

int64_t dqmc_chain_bytes(const dqmc_chain_config* cfg, int precision) {
    if (!cfg) return -1;
    return (int64_t)layout_of(*cfg, precision).bytes;
}

int dqmc_create(int device, const dqmc_chain_config* chains, int n_chains, int precision,
                dqmc_handle** out) {
    if (!out || !chains || n_chains <= 0) return fail(DQMC_ERR_INVALID, "dqmc_create: bad arguments");
    *out = nullptr;
    if (precision != DQMC_PREC_FP64 && precision != DQMC_PREC_MIXED)
        return fail(DQMC_ERR_INVALID, "dqmc_create: unknown precision");
    for (int i = 0; i < n_chains; ++i) {
        if (int st = validate_config(chains[i], i)) return st;
        if (is_cplx(chains[i]) && precision != DQMC_PREC_FP64)
            return fail(DQMC_ERR_INVALID, "dqmc_create: complex chains run in FP64 only");
    }
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return fail(DQMC_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
    if (device < 0 || device >= ndev) return fail(DQMC_ERR_INVALID, "dqmc_create: bad device index");
    CUDA_TRY(cudaSetDevice(device), "cudaSetDevice");
    dqmc_handle* h = new dqmc_handle();
    h->device = device;
    h->precision = precision;
    h->cfg.assign(chains, chains + n_chains);
    for (int i = 0; i < n_chains; ++i) {
        h->n_max = std::max(h->n_max, (int)mat_n(chains[i]));
        h->tc = h->tc || tc_capable(chains[i], precision);
    }
    size_t total = 0;
    std::vector<size_t> base(n_chains);
    for (int i = 0; i < n_chains; ++i) {
        h->lay.push_back(layout_of(chains[i], precision));
        base[i] = total;
        total += h->lay.back().bytes;
    }
    e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete h; return cuda_fail(e, "cudaStreamCreate"); }
    h->stream = h->own_stream;
    e = cudaMalloc((void**)&h->arena, total);
    if (e != cudaSuccess) {
        cudaStreamDestroy(h->own_stream);
        delete h;
        return cuda_fail(e, "cudaMalloc chain workspace");
    }
    e = cudaMemsetAsync(h->arena, 0, total, h->stream);
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->d_chains, sizeof(DqmcChain) * n_chains);
    if (e != cudaSuccess) {
        cudaFree(h->arena);
        cudaStreamDestroy(h->own_stream);
        delete h;
        return cuda_fail(e, "cudaMalloc chain descriptors");
    }
    h->host.resize(n_chains);
    for (int i = 0; i < n_chains; ++i)
        fill_descriptor(h->host[i], chains[i], h->arena + base[i], h->lay[i], precision);
    int st = push_descriptors(h);
    if (st != DQMC_OK) { dqmc_destroy(h); return st; }
    *out = h;
    return DQMC_OK;
}

int dqmc_destroy(dqmc_handle* h) {
    if (!h) return DQMC_OK;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->arena) cudaFree(h->arena);
    for (double* p : h->ut_mem)
        if (p) cudaFree(p);
    for (double* p : h->td_mem)
        if (p) cudaFree(p);
    for (double* p : h->cb_mem)
        if (p) cudaFree(p);
    if (h->d_chains) cudaFree(h->d_chains);
    if (h->graph) cudaGraphExecDestroy(h->graph);
    if (h->pinned) cudaFreeHost(h->pinned);
    if (h->d_sync) cudaFree(h->d_sync);
    if (h->own_stream) cudaStreamDestroy(h->own_stream);
    delete h;
    return DQMC_OK;
}

int dqmc_set_small_chain_kernel(dqmc_handle* h, int enable) {
    if (!h) return fail(DQMC_ERR_INVALID, "null handle");
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    h->small_kernel = enable != 0;
    return DQMC_OK;
}

int dqmc_set_tensor_products(dqmc_handle* h, int chain, int mask) {
    if (!h) return fail(DQMC_ERR_INVALID, "null handle");
    if (mask < 0 || mask > (DQMC_TC_WRAPS | DQMC_TC_SLICES | DQMC_TC_GREENS))
        return fail(DQMC_ERR_INVALID, "dqmc_set_tensor_products: unknown mask");
    int lo = chain, hi = chain + 1;
    if (chain == -1) { lo = 0; hi = (int)h->cfg.size(); }
    else if (int st = check_chain(h, chain)) return st;
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    for (int i = lo; i < hi; ++i) h->host[i].tc_enable = mask;
    h->host_dirty = true;
    return DQMC_OK;
}

int dqmc_set_stream(dqmc_handle* h, void* cuda_stream) {
    if (!h) return fail(DQMC_ERR_INVALID, "null handle");
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    CUDA_TRY(cudaStreamSynchronize(h->stream), "synchronize");
    h->stream = cuda_stream ? (cudaStream_t)cuda_stream : h->own_stream;
    return DQMC_OK;
}

int dqmc_set_hopping(dqmc_handle* h, int chain, const double* a, const double* b, const double* c,
                     const double* d) {
    if (!h || !a || !b || !c || !d) return fail(DQMC_ERR_INVALID, "dqmc_set_hopping: null argument");
    int lo = chain, hi = chain + 1;
    if (chain == -1) { lo = 0; hi = (int)h->cfg.size(); }
    else if (int st = check_chain(h, chain)) return st;
    CUDA_TRY(cudaSetDevice(h->device), "cudaSetDevice");
    for (int i = lo; i < hi; ++i) {
        if (!h->host[i].active) continue;  // free pool slot
        const size_t nn = mat_n(h->cfg[i]) * mat_n(h->cfg[i]);
        if (chain == -1 && h->cfg[i].n_sites != h->cfg[lo].n_sites)
            return fail(DQMC_ERR_INVALID, "dqmc_set_hopping(-1): chains have different n_sites");
        const double* src[4] = {a, b, c, d};
        std::vector<double> rep;
        if (is_cplx(h->cfg[i])) {  // diag(A, A): the representation of the real matrix
            const size_t ns = h->cfg[i].n_sites;
            rep.resize(4 * nn);
            for (int m = 0; m < 4; ++m) {
                real_to_rep(ns, src[m], rep.data() + m * nn);
                src[m] = rep.data() + m * nn;
            }
        }
        double* dst[4] = {(double*)h->host[i].eT2, (double*)h->host[i].eT2inv,
                          (double*)h->host[i].eTh, (double*)h->host[i].eThinv};
        for (int m = 0; m < 4; ++m)
            CUDA_TRY(cudaMemcpyAsync(dst[m], src[m], nn * sizeof(double), cudaMemcpyHostToDevice,
                                     h->stream),
                     "upload hopping exponentials");
        // float pairs of exp(-dtau T) and exp(+dtau T): hi = fp32(x), lo = fp32(x - hi)
        std::vector<float2> split(2 * nn);
        for (int m = 0; m < 2; ++m)
            for (size_t e = 0; e < nn; ++e) {
                const double v = src[m][e];
                const float hi = (float)v;
                split[m * nn + e] = make_float2(hi, (float)(v - (double)hi));
            }
        CUDA_TRY(cudaMemcpyAsync((void*)h->host[i].eT2df, split.data(), 2 * nn * sizeof(float2),
                                 cudaMemcpyHostToDevice, h->stream),
                 "upload split hopping exponentials");
        CUDA_TRY(cudaStreamSynchronize(h->stream), "synchronize");
    }
    CUDA_TRY(cudaStreamSynchronize(h->stream), "synchronize");
    return DQMC_OK;
}

int dqmc_set_field(dqmc_handle* h, int chain, const int8_t* conf) {
    if (int st = check_chain(h, chain)) return st;
    if (!conf) return fail(DQMC_ERR_INVALID, "dqmc_set_field: null conf");
    const dqmc_chain_config& c = h->cfg[chain];
    const bool ghq = c.field >= 2;
    for (size_t i = 0; i < (size_t)c.n_sites * c.slices; ++i) {
        int v = conf[i];
        bool ok = ghq ? (v >= 1 && v <= 4) : (v == 1 || v == -1);
        if (!ok) return fail(DQMC_ERR_INVALID, "dqmc_set_field: value out of range for the field kind");
    }
    CUDA_TRY(cudaSetDevice(h->device), "cudaSetDevice");
    CUDA_TRY(cudaMemcpyAsync(h->host[chain].conf, conf, (size_t)c.n_sites * c.slices,
                             cudaMemcpyHostToDevice, h->stream),
             "upload field");
    CUDA_TRY(cudaStreamSynchronize(h->stream), "synchronize");
    return DQMC_OK;
}

int dqmc_get_field(dqmc_handle* h, int chain, int8_t* conf) {
    if (int st = check_chain(h, chain)) return st;
    if (!conf) return fail(DQMC_ERR_INVALID, "dqmc_get_field: null conf");
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    const dqmc_chain_config& c = h->cfg[chain];
    CUDA_TRY(cudaSetDevice(h->device), "cudaSetDevice");
    CUDA_TRY(cudaMemcpyAsync(conf, h->host[chain].conf, (size_t)c.n_sites * c.slices,
                             cudaMemcpyDeviceToHost, h->stream),
             "download field");
    CUDA_TRY(cudaStreamSynchronize(h->stream), "synchronize");
    return DQMC_OK;
}

int dqmc_init_random_field(dqmc_handle* h, int chain) {
    if (!h) return fail(DQMC_ERR_INVALID, "null handle");
    int lo = chain, hi = chain + 1;
    if (chain == -1) { lo = 0; hi = (int)h->cfg.size(); }
    else if (int st = check_chain(h, chain)) return st;
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    for (int i = lo; i < hi; ++i) {
        if (!h->host[i].active) continue;  // free pool slot
        const dqmc_chain_config& c = h->cfg[i];
        const size_t cnt = (size_t)c.n_sites * c.slices;
        std::vector<int8_t> conf(cnt);
        DqmcChain& d = h->host[i];
        for (size_t k = 0; k < cnt; ++k) {
            uint64_t w = dqmc_philox_word(d.key, (uint64_t)k);
            conf[k] = c.field >= 2 ? (int8_t)(1 + (int)(w >> 62)) : ((w >> 63) ? (int8_t)1 : (int8_t)-1);
        }
        d.ctr = cnt;
        h->host_dirty = true;
        if (int st = dqmc_set_field(h, i, conf.data())) return st;
    }
    return DQMC_OK;
}

int dqmc_set_rng(dqmc_handle* h, int chain, uint64_t key, uint64_t counter) {
    if (int st = check_chain(h, chain)) return st;
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    h->host[chain].key = key;
    h->host[chain].ctr = counter;
    h->host_dirty = true;
    return DQMC_OK;
}

int dqmc_get_rng(dqmc_handle* h, int chain, uint64_t* key, uint64_t* counter) {
    if (int st = check_chain(h, chain)) return st;
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    if (key) *key = h->host[chain].key;
    if (counter) *counter = h->host[chain].ctr;
    return DQMC_OK;
}

int dqmc_initialize_run(dqmc_handle* h) {
    if (!h) return fail(DQMC_ERR_INVALID, "null handle");
    return launch(h, DQMC_OP_BUILD, 0, 0, true);
}
int dqmc_build_stack(dqmc_handle* h) {
    if (!h) return fail(DQMC_ERR_INVALID, "null handle");
    return launch(h, DQMC_OP_BUILD_FWD, 0, 0, true);
}
int dqmc_propagate(dqmc_handle* h) {
    if (!h) return fail(DQMC_ERR_INVALID, "null handle");
    return launch(h, DQMC_OP_PROPAGATE, 0, 0, true);
}
int dqmc_sweep_spatial(dqmc_handle* h) {
    if (!h) return fail(DQMC_ERR_INVALID, "null handle");
    return launch(h, DQMC_OP_SWEEP_SPATIAL, 0, 0, true);
}

static void fill_stats(const DqmcChain& d, dqmc_stats* s) {
    s->accepted = d.accepted;
    s->proposals = d.proposals;
    s->propagation_errors = d.n_prop_err;
    s->negative_probability = d.n_neg_p;
    s->max_propagation_error = d.prop_err_max;
    s->max_reported_error = d.prop_err_reported;
    s->imaginary_probability = d.n_imag_p;
    s->max_imaginary_probability = d.max_imag_p;
    // MagnitudeStats min / mean / max (statistics.jl:26-28): 10^(log10 stats), 0 when empty
    auto mag = [](const double* ms, long long cnt, double* mn, double* mean, double* mx) {
        *mn = cnt > 0 ? pow(10.0, ms[1]) : 0.0;
        *mean = cnt > 0 ? pow(10.0, ms[2] / (double)cnt) : 0.0;
        if (mx) *mx = cnt > 0 ? pow(10.0, ms[0]) : 0.0;
    };
    mag(d.ms_prop, d.n_prop_err, &s->min_reported_error, &s->mean_reported_error, nullptr);
    mag(d.ms_neg, d.n_neg_p, &s->min_negative_probability, &s->mean_negative_probability,
        &s->max_negative_probability);
    mag(d.ms_imag, d.n_imag_p, &s->min_imaginary_probability, &s->mean_imaginary_probability,
        nullptr);
    s->current_slice = d.current_slice;
    s->current_range = d.current_range;
    s->direction = d.direction;
    s->status = d.status;
    s->near_ties = d.n_near_tie;
    s->min_tie_gap = d.min_tie_gap;
}

static int check_scheduled(dqmc_handle* h);

int dqmc_sweep(dqmc_handle* h, int n_sweeps, dqmc_stats* stats) {
    if (!h) return fail(DQMC_ERR_INVALID, "null handle");
    if (n_sweeps < 0) return fail(DQMC_ERR_INVALID, "dqmc_sweep: n_sweeps < 0");
    if (int st = check_scheduled(h)) return st;
    int st = launch(h, DQMC_OP_SWEEP, n_sweeps, 0, true);
    if (st != DQMC_OK) return st;
    if (stats)
        for (size_t i = 0; i < h->host.size(); ++i) fill_stats(h->host[i], stats + i);
    return DQMC_OK;
}

int dqmc_sweep_async(dqmc_handle* h, int n_sweeps) {
    if (!h) return fail(DQMC_ERR_INVALID, "null handle");
    if (n_sweeps < 0) return fail(DQMC_ERR_INVALID, "dqmc_sweep_async: n_sweeps < 0");
    if (int st = check_scheduled(h)) return st;
    return launch(h, DQMC_OP_SWEEP, n_sweeps, 0, false);
}

int dqmc_query(dqmc_handle* h) {
    if (!h) return fail(DQMC_ERR_INVALID, "null handle");
    if (!h->busy) return DQMC_OK;
    cudaError_t e = cudaStreamQuery(h->stream);
    if (e == cudaErrorNotReady) return DQMC_ERR_NOT_READY;
    if (e != cudaSuccess) return cuda_fail(e, "dqmc_query");
    return dqmc_synchronize(h);
}

int dqmc_synchronize(dqmc_handle* h) {
    if (!h) return fail(DQMC_ERR_INVALID, "null handle");
    if (!h->busy) return DQMC_OK;
    h->busy = false;
    CUDA_TRY(cudaSetDevice(h->device), "cudaSetDevice");
    CUDA_TRY(cudaStreamSynchronize(h->stream), "chain kernel");
    int st = pull_descriptors(h);
    if (st != DQMC_OK) return st;
    for (size_t i = 0; i < h->host.size(); ++i)
        if (h->host[i].status != 0)
            return fail(DQMC_ERR_NUMERICAL, "chain " + std::to_string(i) + " reported status " +
                                                 std::to_string(h->host[i].status));
    return DQMC_OK;
}

int dqmc_get_stats(dqmc_handle* h, int chain, dqmc_stats* out) {
    if (int st = check_chain(h, chain)) return st;
    if (!out) return fail(DQMC_ERR_INVALID, "dqmc_get_stats: null out");
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    fill_stats(h->host[chain], out);
    return DQMC_OK;
}

int dqmc_get_timers(dqmc_handle* h, int chain, uint64_t* out) {
    if (int st = check_chain(h, chain)) return st;
    if (!out) return fail(DQMC_ERR_INVALID, "dqmc_get_timers: null out");
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    for (int p = 0; p < 8; ++p) out[p] = h->host[chain].timers[p];
    return DQMC_OK;
}

// one matrix to the caller: as stored, or (complex chain, raw = false) as
// interleaved complex blocks
static int download_mat(dqmc_handle* h, int chain, const double* src, double* out,
                        bool raw = false) {
    const dqmc_chain_config& c = h->cfg[chain];
    const size_t bytes = mat_elems(c) * sizeof(double);
    if (raw || !is_cplx(c)) {
        CUDA_TRY(cudaMemcpyAsync(out, src, bytes, cudaMemcpyDeviceToHost, h->stream),
                 "download matrix");
        CUDA_TRY(cudaStreamSynchronize(h->stream), "synchronize");
        return DQMC_OK;
    }
    std::vector<double> rep(mat_elems(c));
    CUDA_TRY(cudaMemcpyAsync(rep.data(), src, bytes, cudaMemcpyDeviceToHost, h->stream),
             "download matrix");
    CUDA_TRY(cudaStreamSynchronize(h->stream), "synchronize");
    rep_to_complex(c, rep.data(), out);
    return DQMC_OK;
}

// run `op` for one chain only: launch over a one-element descriptor array
static int launch_one(dqmc_handle* h, int chain, int op, int arg0, int arg1) {
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    CUDA_TRY(cudaSetDevice(h->device), "cudaSetDevice");
    if (h->host_dirty) if (int st = push_descriptors(h)) return st;
    CUDA_TRY(dqmc_launch_chain_kernel(h->d_chains + chain, 1, op, arg0, arg1, h->stream,
                                      (int)mat_n(h->cfg[chain]), h->host[chain].tcs != nullptr,
                                      false),
             "chain kernel launch");
    CUDA_TRY(cudaStreamSynchronize(h->stream), "chain kernel");
    return pull_descriptors(h);
}

int dqmc_get_greens(dqmc_handle* h, int chain, int physical, double* out) {
    if (int st = check_chain(h, chain)) return st;
    if (!out) return fail(DQMC_ERR_INVALID, "dqmc_get_greens: null out");
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    CUDA_TRY(cudaSetDevice(h->device), "cudaSetDevice");
    if (physical) {
        if (int st = launch_one(h, chain, DQMC_OP_PHYSICAL, 0, 0)) return st;
        return download_mat(h, chain, h->host[chain].out, out);
    }
    return download_mat(h, chain, h->host[chain].G, out);
}

// chains first .. first+count-1: real, active, equal configurations, workspaces
// at one arena stride (so one strided copy moves all of them)
static bool uniform_range(dqmc_handle* h, int first, int count, size_t* stride) {
    const dqmc_chain_config& c0 = h->cfg[first];
    const char* g0 = (const char*)h->host[first].G;
    const size_t s = count > 1 ? (size_t)((const char*)h->host[first + 1].G - g0) : 0;
    for (int i = first; i < first + count; ++i) {
        const dqmc_chain_config& c = h->cfg[i];
        const DqmcChain& d = h->host[i];
        if (!d.active || is_cplx(c) || c.n_sites != c0.n_sites || c.n_flavors != c0.n_flavors ||
            c.slices != c0.slices || (const char*)d.G != g0 + (size_t)(i - first) * s ||
            (const char*)d.conf != (const char*)h->host[first].conf + (size_t)(i - first) * s ||
            (const char*)d.out != (const char*)h->host[first].out + (size_t)(i - first) * s)
            return false;
    }
    *stride = s;
    return count == 1 || s > 0;
}
static int check_range(dqmc_handle* h, int first, int count, const void* buf, const char* what) {
    if (!h) return fail(DQMC_ERR_INVALID, "null handle");
    if (!buf || count < 1 || first < 0 || first + count > (int)h->cfg.size())
        return fail(DQMC_ERR_INVALID, std::string(what) + ": bad range or null buffer");
    for (int i = first; i < first + count; ++i)
        if (int st = check_chain(h, i)) return st;
    return DQMC_OK;
}

int dqmc_get_greens_batch(dqmc_handle* h, int first, int count, int physical, double* out) {
    if (int st = check_range(h, first, count, out, "dqmc_get_greens_batch")) return st;
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    CUDA_TRY(cudaSetDevice(h->device), "cudaSetDevice");
    if (physical)
        if (int st = launch(h, DQMC_OP_PHYSICAL, 0, 0, true)) return st;
    size_t stride = 0;
    if (!uniform_range(h, first, count, &stride)) {
        size_t off = 0;
        for (int i = first; i < first + count; ++i) {
            if (int st = download_mat(h, i, physical ? h->host[i].out : h->host[i].G, out + off))
                return st;
            off += user_elems(h->cfg[i]);
        }
        return DQMC_OK;
    }
    const size_t bytes = mat_elems(h->cfg[first]) * sizeof(double);
    const void* src = physical ? (const void*)h->host[first].out : (const void*)h->host[first].G;
    CUDA_TRY(cudaMemcpy2DAsync(out, bytes, src, count > 1 ? stride : bytes, bytes, count,
                               cudaMemcpyDeviceToHost, h->stream),
             "download Green's functions");
    CUDA_TRY(cudaStreamSynchronize(h->stream), "synchronize");
    return DQMC_OK;
}

int dqmc_get_fields_batch(dqmc_handle* h, int first, int count, int8_t* out) {
    if (int st = check_range(h, first, count, out, "dqmc_get_fields_batch")) return st;
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    CUDA_TRY(cudaSetDevice(h->device), "cudaSetDevice");
    size_t stride = 0;
    if (!uniform_range(h, first, count, &stride)) {
        size_t off = 0;
        for (int i = first; i < first + count; ++i) {
            if (int st = dqmc_get_field(h, i, out + off)) return st;
            off += (size_t)h->cfg[i].n_sites * h->cfg[i].slices;
        }
        return DQMC_OK;
    }
    const size_t bytes = (size_t)h->cfg[first].n_sites * h->cfg[first].slices;
    CUDA_TRY(cudaMemcpy2DAsync(out, bytes, h->host[first].conf, count > 1 ? stride : bytes, bytes,
                               count, cudaMemcpyDeviceToHost, h->stream),
             "download fields");
    CUDA_TRY(cudaStreamSynchronize(h->stream), "synchronize");
    return DQMC_OK;
}

int dqmc_set_fields_batch(dqmc_handle* h, int first, int count, const int8_t* in) {
    if (int st = check_range(h, first, count, in, "dqmc_set_fields_batch")) return st;
    size_t stride = 0;
    if (!uniform_range(h, first, count, &stride)) {
        size_t off = 0;
        for (int i = first; i < first + count; ++i) {
            if (int st = dqmc_set_field(h, i, in + off)) return st;
            off += (size_t)h->cfg[i].n_sites * h->cfg[i].slices;
        }
        return DQMC_OK;
    }
    const dqmc_chain_config& c = h->cfg[first];
    const size_t bytes = (size_t)c.n_sites * c.slices;
    const bool ghq = c.field >= 2;
    for (size_t e = 0; e < bytes * count; ++e) {
        const int v = in[e];
        if (!(ghq ? (v >= 1 && v <= 4) : (v == 1 || v == -1)))
            return fail(DQMC_ERR_INVALID, "dqmc_set_fields_batch: value out of range for the field kind");
    }
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    CUDA_TRY(cudaSetDevice(h->device), "cudaSetDevice");
    CUDA_TRY(cudaMemcpy2DAsync(h->host[first].conf, count > 1 ? stride : bytes, in, bytes, bytes,
                               count, cudaMemcpyHostToDevice, h->stream),
             "upload fields");
    CUDA_TRY(cudaStreamSynchronize(h->stream), "synchronize");
    return DQMC_OK;
}

int dqmc_set_greens(dqmc_handle* h, int chain, const double* in) {
    if (int st = check_chain(h, chain)) return st;
    if (!in) return fail(DQMC_ERR_INVALID, "dqmc_set_greens: null in");
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    CUDA_TRY(cudaSetDevice(h->device), "cudaSetDevice");
    std::vector<double> rep;
    if (is_cplx(h->cfg[chain])) {
        rep.resize(mat_elems(h->cfg[chain]));
        complex_to_rep(h->cfg[chain], in, rep.data());
        in = rep.data();
    }
    CUDA_TRY(cudaMemcpyAsync(h->host[chain].G, in, mat_elems(h->cfg[chain]) * sizeof(double),
                             cudaMemcpyHostToDevice, h->stream),
             "upload greens");
    CUDA_TRY(cudaStreamSynchronize(h->stream), "synchronize");
    return DQMC_OK;
}

int dqmc_calculate_greens(dqmc_handle* h, int chain, int slice, int safe_mult, double* out) {
    if (int st = check_chain(h, chain)) return st;
    if (!out) return fail(DQMC_ERR_INVALID, "dqmc_calculate_greens: null out");
    if (slice < 0 || slice > h->cfg[chain].slices)
        return fail(DQMC_ERR_INVALID, "dqmc_calculate_greens: slice out of range 0..M");
    if (int st = launch_one(h, chain, DQMC_OP_GREENS_AT, slice, safe_mult)) return st;
    return download_mat(h, chain, h->host[chain].out, out);
}

int dqmc_get_stack(dqmc_handle* h, int chain, int which, int idx, double* out) {
    if (int st = check_chain(h, chain)) return st;
    const DqmcChain& d = h->host[chain];
    if (!out || which < 0 || which > 2 || idx < 1 || idx > d.nr + 1)
        return fail(DQMC_ERR_INVALID, "dqmc_get_stack: bad arguments");
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    CUDA_TRY(cudaSetDevice(h->device), "cudaSetDevice");
    const size_t ms = mat_elems(h->cfg[chain]);
    if (which == 2) {
        const size_t cnt = (size_t)d.nf * d.n;
        CUDA_TRY(cudaMemcpyAsync(out, d.dstack + (idx - 1) * cnt, cnt * sizeof(double),
                                 cudaMemcpyDeviceToHost, h->stream),
                 "download d_stack");
        CUDA_TRY(cudaStreamSynchronize(h->stream), "synchronize");
        return DQMC_OK;
    }
    const double* base = which == 0 ? d.ustack : d.tstack;
    return download_mat(h, chain, base + (idx - 1) * ms, out, true);
}

/* ---- equal-time measurements ---------------------------------------------- */

int dqmc_set_measurements(dqmc_handle* h, int chain, const dqmc_measure_config* cfg) {
    if (!h || !cfg) return fail(DQMC_ERR_INVALID, "dqmc_set_measurements: null argument");
    if (cfg->enable && cfg->measure_rate < 1)
        return fail(DQMC_ERR_INVALID, "dqmc_set_measurements: measure_rate < 1");
    if (!(cfg->U == cfg->U)) return fail(DQMC_ERR_INVALID, "dqmc_set_measurements: U is NaN");
    int lo = chain, hi = chain + 1;
    if (chain == -1) { lo = 0; hi = (int)h->cfg.size(); }
    else if (int st = check_chain(h, chain)) return st;
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    CUDA_TRY(cudaSetDevice(h->device), "cudaSetDevice");
    for (int i = lo; i < hi; ++i) {
        DqmcChain& d = h->host[i];
        if (!d.active) continue;  // free pool slot
        if (cfg->q_cos && chain == -1 && h->cfg[i].n_sites != h->cfg[lo].n_sites)
            return fail(DQMC_ERR_INVALID, "dqmc_set_measurements(-1): chains have different n_sites");
        if (cfg->enable && d.cplx)
            return fail(DQMC_ERR_INVALID, "dqmc_set_measurements: no device measurements on a "
                                          "complex chain (download its Green's function instead)");
        d.meas_enable = cfg->enable ? 1 : 0;
        if (cfg->measure_rate >= 1) d.meas_rate = cfg->measure_rate;
        d.meas_greens = cfg->greens_mean ? 1 : 0;
        d.meas_U = cfg->U;
        if (cfg->sweep >= 0) d.sweep = cfg->sweep;
        if (cfg->q_cos) {
            const size_t n = (size_t)d.n;
            double* q = (double*)((char*)d.meas + (h->lay[i].off_qcs - h->lay[i].off_meas));
            std::vector<double> buf(2 * n, 0.0);
            for (size_t k = 0; k < n; ++k) {
                buf[k] = cfg->q_cos[k];
                if (cfg->q_sin) buf[n + k] = cfg->q_sin[k];
            }
            CUDA_TRY(cudaMemcpyAsync(q, buf.data(), 2 * n * sizeof(double), cudaMemcpyHostToDevice,
                                     h->stream),
                     "upload structure-factor phases");
            CUDA_TRY(cudaStreamSynchronize(h->stream), "synchronize");
            d.qcs = q;
        } else {
            d.qcs = nullptr;
        }
    }
    h->host_dirty = true;
    return DQMC_OK;
}

int dqmc_reset_measurements(dqmc_handle* h, int chain) {
    if (!h) return fail(DQMC_ERR_INVALID, "null handle");
    int lo = chain, hi = chain + 1;
    if (chain == -1) { lo = 0; hi = (int)h->cfg.size(); }
    else if (int st = check_chain(h, chain)) return st;
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    CUDA_TRY(cudaSetDevice(h->device), "cudaSetDevice");
    for (int i = lo; i < hi; ++i) {
        const DqmcChain& d = h->host[i];
        if (!d.active) continue;
        CUDA_TRY(cudaMemsetAsync(d.meas, 0, DQMC_MEAS_DOUBLES(d.n, d.nf) * sizeof(double), h->stream),
                 "clear measurement accumulators");
    }
    CUDA_TRY(cudaStreamSynchronize(h->stream), "synchronize");
    return DQMC_OK;
}

int dqmc_get_measurements(dqmc_handle* h, int chain, dqmc_observables* out, double* occupation,
                          double* greens) {
    if (int st = check_chain(h, chain)) return st;
    if (!out) return fail(DQMC_ERR_INVALID, "dqmc_get_measurements: null out");
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    CUDA_TRY(cudaSetDevice(h->device), "cudaSetDevice");
    const DqmcChain& d = h->host[chain];
    const size_t nd = DQMC_MEAS_DOUBLES(d.n, d.nf);
    std::vector<double> m(nd);
    CUDA_TRY(cudaMemcpyAsync(m.data(), d.meas, nd * sizeof(double), cudaMemcpyDeviceToHost, h->stream),
             "download measurement accumulators");
    CUDA_TRY(cudaStreamSynchronize(h->stream), "synchronize");
    const double cnt = m[0];
    out->count = (int64_t)cnt;
    for (int k = 0; k < DQMC_MEAS_SCALARS; ++k) {
        const double* lv = m.data() + DQMC_MEAS_HEADER + (size_t)k * DQMC_MEAS_LEVELS * DQMC_MEAS_BIN_WORDS;
        out->mean[k] = lv[0] > 0 ? lv[1] : NAN;
        // highest level with >= 32 bins, else level 0 (LogBinner's std_error)
        int use = -1;
        for (int l = 0; l < DQMC_MEAS_LEVELS; ++l)
            if (lv[l * DQMC_MEAS_BIN_WORDS] >= 32.0) use = l;
        if (use < 0) use = 0;
        const double nb = lv[use * DQMC_MEAS_BIN_WORDS], m2 = lv[use * DQMC_MEAS_BIN_WORDS + 2];
        out->error[k] = nb >= 2.0 ? sqrt(m2 / (nb - 1.0) / nb) : INFINITY;
        out->error_level[k] = use;
    }
    const size_t nocc = (size_t)d.nf * d.n;
    if (occupation)
        for (size_t e = 0; e < nocc; ++e) occupation[e] = cnt > 0 ? m[DQMC_MEAS_OCC_OFF + e] / cnt : NAN;
    if (greens) {
        const size_t ng = (size_t)d.nf * d.n * d.n;
        for (size_t e = 0; e < ng; ++e)
            greens[e] = cnt > 0 ? m[DQMC_MEAS_OCC_OFF + nocc + e] / cnt : NAN;
    }
    return DQMC_OK;
}

/* ---- checkerboard decomposition ---------------------------------------------- */

int dqmc_set_checkerboard(dqmc_handle* h, int chain, int n_parts, const double* data) {
    if (!h) return fail(DQMC_ERR_INVALID, "null handle");
    int lo = chain, hi = chain + 1;
    if (chain == -1) { lo = 0; hi = (int)h->cfg.size(); }
    else if (int st = check_chain(h, chain)) return st;
    if (n_parts > DQMC_CB_MAXPARTS)
        return fail(DQMC_ERR_INVALID, "dqmc_set_checkerboard: more than 12 parts");
    if (n_parts >= 0 && !data) return fail(DQMC_ERR_INVALID, "dqmc_set_checkerboard: null data");
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    CUDA_TRY(cudaSetDevice(h->device), "cudaSetDevice");
    if (h->cb_mem.size() < h->host.size()) h->cb_mem.resize(h->host.size(), nullptr);
    for (int i = lo; i < hi; ++i) {
        DqmcChain& d = h->host[i];
        if (!d.active) continue;
        if (n_parts < 0) {  // back to the dense exponentials
            d.cb = nullptr;
            d.cbp = nullptr;
            d.cb_np = 0;
            continue;
        }
        const int n = d.ns;  // the caller's data: per site of the lattice
        if (chain == -1 && n != h->host[lo].ns)
            return fail(DQMC_ERR_INVALID, "dqmc_set_checkerboard(-1): chains have different n_sites");
        const size_t per = (size_t)n * (1 + 3 * (size_t)n_parts), cnt = 4 * per;
        for (size_t m = 0; m < 4; ++m) {
            const double* f = data + m * per;
            for (size_t e = 0; e < per; ++e)
                if (!std::isfinite(f[e]))
                    return fail(DQMC_ERR_INVALID, "dqmc_set_checkerboard: non-finite entry");
            for (int p = 0; p < n_parts; ++p) {
                const double* pt = f + n + (size_t)p * 3 * n + 2 * n;
                for (int k = 0; k < n; ++k) {
                    const double q = pt[k];
                    if (!(q == -1.0 || (q >= 0.0 && q < n && q == (double)(int)q)))
                        return fail(DQMC_ERR_INVALID, "dqmc_set_checkerboard: partner out of range");
                }
            }
        }
        // device layout: per factor D[dn] and per part c[dn], s[dn]; then the
        // partners as int32, per factor and part.  A complex chain's
        // representation needs diag(X, X): every site entry twice, partners
        // of the second copy shifted by n.
        const int dn = d.n, reps = dn / n;
        const size_t per_d = (size_t)dn * (1 + 2 * (size_t)n_parts);
        std::vector<double> dv(4 * per_d);
        std::vector<int32_t> pv(4 * (size_t)n_parts * dn);
        for (size_t m = 0; m < 4; ++m) {
            const double* f = data + m * per;
            double* g = dv.data() + m * per_d;
            for (int r = 0; r < reps; ++r)
                for (int k = 0; k < n; ++k) g[r * n + k] = f[k];
            for (int p = 0; p < n_parts; ++p) {
                const double* fp = f + n + (size_t)p * 3 * n;
                for (int r = 0; r < reps; ++r)
                    for (int k = 0; k < n; ++k) {
                        const int q = (int)fp[2 * n + k];
                        g[dn + (size_t)p * 2 * dn + r * n + k] = fp[k];
                        g[dn + (size_t)p * 2 * dn + dn + r * n + k] = fp[n + k];
                        pv[(m * n_parts + p) * (size_t)dn + r * n + k] = q < 0 ? -1 : q + r * n;
                    }
            }
        }
        (void)cnt;
        if (h->cb_mem[i]) { cudaFree(h->cb_mem[i]); h->cb_mem[i] = nullptr; }
        const size_t bytes = dv.size() * sizeof(double) + pv.size() * sizeof(int32_t);
        CUDA_TRY(cudaMalloc((void**)&h->cb_mem[i], bytes), "allocate checkerboard factors");
        CUDA_TRY(cudaMemcpyAsync(h->cb_mem[i], dv.data(), dv.size() * sizeof(double),
                                 cudaMemcpyHostToDevice, h->stream),
                 "upload checkerboard factors");
        int32_t* dp = reinterpret_cast<int32_t*>(h->cb_mem[i] + dv.size());
        if (!pv.empty())
            CUDA_TRY(cudaMemcpyAsync(dp, pv.data(), pv.size() * sizeof(int32_t),
                                     cudaMemcpyHostToDevice, h->stream),
                     "upload checkerboard partners");
        CUDA_TRY(cudaStreamSynchronize(h->stream), "synchronize");
        d.cb = h->cb_mem[i];
        d.cbp = dp;
        d.cb_np = n_parts;
    }
    h->host_dirty = true;
    return DQMC_OK;
}

/* ---- unequal-time Green's function ------------------------------------------ */

int dqmc_calculate_greens_kl(dqmc_handle* h, int chain, const int32_t* k, const int32_t* l,
                             int npairs, int physical, double* out) {
    if (int st = check_chain(h, chain)) return st;
    if (!k || !l || !out || npairs < 1)
        return fail(DQMC_ERR_INVALID, "dqmc_calculate_greens_kl: bad arguments");
    const int M = h->cfg[chain].slices;
    for (int p = 0; p < npairs; ++p)
        if (k[p] < 0 || k[p] > M || l[p] < 0 || l[p] > M)
            return fail(DQMC_ERR_INVALID, "dqmc_calculate_greens_kl: slices out of range 0..M");
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    CUDA_TRY(cudaSetDevice(h->device), "cudaSetDevice");
    DqmcChain& d = h->host[chain];
    if (h->ut_mem.size() < h->host.size()) h->ut_mem.resize(h->host.size(), nullptr);
    if (!h->ut_mem[chain]) {
        CUDA_TRY(cudaMalloc((void**)&h->ut_mem[chain],
                            DQMC_UT_DOUBLES(d.n, d.nf, d.nr) * sizeof(double)),
                 "allocate the unequal-time stack");
    }
    const size_t ms = (size_t)d.nf * d.n * d.n;
    std::vector<int32_t> kl(2 * (size_t)npairs);
    for (int p = 0; p < npairs; ++p) { kl[2 * p] = k[p]; kl[2 * p + 1] = l[p]; }
    int32_t* d_pairs = nullptr;
    double* d_out = nullptr;
    cudaError_t e = cudaMalloc((void**)&d_pairs, kl.size() * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc((void**)&d_out, ms * npairs * sizeof(double));
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_pairs, kl.data(), kl.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                            h->stream);
    int st = DQMC_OK;
    if (e != cudaSuccess) {
        st = cuda_fail(e, "dqmc_calculate_greens_kl: buffers");
    } else {
        d.ut = h->ut_mem[chain];
        d.ut_pairs = d_pairs;
        d.ut_out = d_out;
        h->host_dirty = true;
        st = launch_one(h, chain, DQMC_OP_GREENS_KL, npairs, physical ? 1 : 0);
        if (st == DQMC_OK && h->host[chain].status != 0)
            st = fail(DQMC_ERR_NUMERICAL, "chain " + std::to_string(chain) + " reported status " +
                                              std::to_string(h->host[chain].status));
        if (st == DQMC_OK) {
            const dqmc_chain_config& cc = h->cfg[chain];
            std::vector<double> rep;
            if (is_cplx(cc)) rep.resize(ms * npairs);
            e = cudaMemcpyAsync(is_cplx(cc) ? rep.data() : out, d_out, ms * npairs * sizeof(double),
                                cudaMemcpyDeviceToHost, h->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
            if (e != cudaSuccess) st = cuda_fail(e, "dqmc_calculate_greens_kl: download");
            else if (is_cplx(cc))
                for (int p = 0; p < npairs; ++p)
                    rep_to_complex(cc, rep.data() + (size_t)p * ms, out + (size_t)p * user_elems(cc));
        }
        h->host[chain].ut_pairs = nullptr;
        h->host[chain].ut_out = nullptr;
        h->host_dirty = true;
    }
    if (d_pairs) cudaFree(d_pairs);
    if (d_out) cudaFree(d_out);
    return st;
}

/* ---- global updates and replica exchange ----------------------------------- */

static int check_between_sweeps(dqmc_handle* h) {
    for (size_t i = 0; i < h->host.size(); ++i) {
        const DqmcChain& d = h->host[i];
        if (d.active && (d.current_slice != 1 || d.direction != 1))
            return fail(DQMC_ERR_INVALID, "chain " + std::to_string(i) +
                                              " is not between sweeps (initialize_run first; "
                                              "global moves need current_slice 1, direction +1)");
    }
    return DQMC_OK;
}

// global updates and replica exchange need the determinant's phase, which
// the real representation of a complex chain does not give
static int check_no_complex(dqmc_handle* h, const char* what) {
    for (size_t i = 0; i < h->host.size(); ++i)
        if (h->host[i].active && h->host[i].cplx)
            return fail(DQMC_ERR_INVALID, std::string(what) + ": chain " + std::to_string(i) +
                                              " is complex (no global updates on complex chains)");
    return DQMC_OK;
}

// sweeps with a scheduled global update must start between sweeps
static int check_scheduled(dqmc_handle* h) {
    bool any = false;
    for (const DqmcChain& d : h->host) any = any || (d.active && d.global_kind >= 0);
    if (!any) return DQMC_OK;
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    return check_between_sweeps(h);
}

int dqmc_global_update(dqmc_handle* h, int kind, int32_t* accepted) {
    if (!h) return fail(DQMC_ERR_INVALID, "null handle");
    if (kind != DQMC_GLOBAL_FLIP && kind != DQMC_GLOBAL_SHUFFLE)
        return fail(DQMC_ERR_INVALID, "dqmc_global_update: unknown kind");
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    if (int st = check_between_sweeps(h)) return st;
    if (int st = check_no_complex(h, "dqmc_global_update")) return st;
    std::vector<long long> before(h->host.size());
    for (size_t i = 0; i < h->host.size(); ++i) before[i] = h->host[i].g_accepted;
    if (int st = launch(h, DQMC_OP_GLOBAL, kind, 0, true)) return st;
    if (accepted)
        for (size_t i = 0; i < h->host.size(); ++i)
            accepted[i] = h->host[i].active ? (int32_t)(h->host[i].g_accepted - before[i]) : 0;
    return DQMC_OK;
}

int dqmc_set_global_schedule(dqmc_handle* h, int chain, int kind) {
    if (!h) return fail(DQMC_ERR_INVALID, "null handle");
    if (kind != -1 && kind != DQMC_GLOBAL_FLIP && kind != DQMC_GLOBAL_SHUFFLE)
        return fail(DQMC_ERR_INVALID, "dqmc_set_global_schedule: unknown kind");
    int lo = chain, hi = chain + 1;
    if (chain == -1) { lo = 0; hi = (int)h->cfg.size(); }
    else if (int st = check_chain(h, chain)) return st;
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    for (int i = lo; i < hi; ++i) {
        if (!h->host[i].active) continue;
        if (kind >= 0 && h->host[i].cplx)
            return fail(DQMC_ERR_INVALID, "dqmc_set_global_schedule: no global updates on a "
                                          "complex chain");
        h->host[i].global_kind = kind;
        h->host[i].sched_calls = 0;
    }
    h->host_dirty = true;
    return DQMC_OK;
}

int dqmc_replica_exchange(dqmc_handle* h, const int32_t* partner, int32_t* accepted) {
    if (!h || !partner) return fail(DQMC_ERR_INVALID, "dqmc_replica_exchange: null argument");
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    const int nc = (int)h->host.size();
    for (int i = 0; i < nc; ++i) {
        const int j = partner[i];
        if (j == -1) continue;
        if (j < 0 || j >= nc || j == i || partner[j] != i)
            return fail(DQMC_ERR_INVALID, "dqmc_replica_exchange: partners must pair chains "
                                          "(partner[partner[i]] == i)");
        if (!h->host[i].active || !h->host[j].active)
            return fail(DQMC_ERR_INVALID, "dqmc_replica_exchange: partner slot holds no chain");
        const dqmc_chain_config &a = h->cfg[i], &b = h->cfg[j];
        if (a.n_sites != b.n_sites || a.n_flavors != b.n_flavors || a.slices != b.slices ||
            a.field != b.field)
            return fail(DQMC_ERR_INVALID, "dqmc_replica_exchange: paired chains need the same "
                                          "n_sites, n_flavors, slices and field kind");
    }
    if (int st = check_between_sweeps(h)) return st;
    if (int st = check_no_complex(h, "dqmc_replica_exchange")) return st;
    std::vector<long long> before(nc);
    for (int i = 0; i < nc; ++i) {
        before[i] = h->host[i].g_accepted;
        h->host[i].partner = h->host[i].active ? partner[i] : -1;
    }
    h->host_dirty = true;
    int st = launch(h, DQMC_OP_REPLICA_WEIGHT, 0, 0, true);
    if (st == DQMC_OK) st = launch(h, DQMC_OP_REPLICA_ACCEPT, 0, 0, true);
    for (int i = 0; i < nc; ++i) h->host[i].partner = -1;
    h->host_dirty = true;
    if (st != DQMC_OK) return st;
    if (accepted)
        for (int i = 0; i < nc; ++i)
            accepted[i] = partner[i] >= 0 ? (int32_t)(h->host[i].g_accepted - before[i]) : 0;
    return DQMC_OK;
}

int dqmc_get_global_stats(dqmc_handle* h, int chain, int64_t* accepted, int64_t* proposals) {
    if (int st = check_chain(h, chain)) return st;
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    if (accepted) *accepted = h->host[chain].g_accepted;
    if (proposals) *proposals = h->host[chain].g_proposals;
    return DQMC_OK;
}

/* ---- time-displaced measurements on the device ----------------------------------- */

static int ensure_ut(dqmc_handle* h, int chain) {
    DqmcChain& d = h->host[chain];
    if (h->ut_mem.size() < h->host.size()) h->ut_mem.resize(h->host.size(), nullptr);
    if (!h->ut_mem[chain]) {
        CUDA_TRY(cudaMalloc((void**)&h->ut_mem[chain],
                            DQMC_UT_DOUBLES(d.n, d.nf, d.nr) * sizeof(double)),
                 "allocate the unequal-time stack");
    }
    d.ut = h->ut_mem[chain];
    return DQMC_OK;
}

int dqmc_set_td_measurements(dqmc_handle* h, int chain, const dqmc_td_config* cfg) {
    if (int st = check_chain(h, chain)) return st;
    if (!cfg) return fail(DQMC_ERR_INVALID, "dqmc_set_td_measurements: null config");
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    DqmcChain& d = h->host[chain];
    if (!cfg->enable) {
        d.td_enable = 0;
        h->host_dirty = true;
        return DQMC_OK;
    }
    if (d.cplx)
        return fail(DQMC_ERR_INVALID, "dqmc_set_td_measurements: real chains only (complex G: "
                                      "use dqmc_calculate_greens_kl)");
    const int n = d.n, P = cfg->n_slots;
    const int nf0 = cfg->n_form[0], nf1 = cfg->n_form[1], nc = cfg->n_current;
    if (cfg->measure_rate < 1 || P < 1 || nf0 < 0 || nf1 < 0 || nc < 0 || !cfg->pair_slot ||
        !(cfg->delta_tau > 0.0) || ((nf0 + nf1) > 0 && (!cfg->form_sites || !cfg->form_values)) ||
        (nc > 0 && (!cfg->current_sites || !cfg->current_values)))
        return fail(DQMC_ERR_INVALID, "dqmc_set_td_measurements: bad configuration");
    const TdLayout L = td_layout(n, d.nf, P, nf0 + nf1, nc);
    std::vector<double> buf(L.g, 0.0);  // everything before the Green's functions
    int32_t* slot = reinterpret_cast<int32_t*>(buf.data() + L.slot);
    for (size_t e = 0; e < (size_t)n * n; ++e) {
        const int v = cfg->pair_slot[e];
        if (v < 0 || v >= P) return fail(DQMC_ERR_INVALID, "dqmc_set_td_measurements: slot out of range");
        slot[e] = v;
    }
    for (int i = 0; i < n; ++i) {
        buf[L.q + i] = cfg->q_cos ? cfg->q_cos[i] : 1.0;
        buf[L.q + n + i] = cfg->q_sin ? cfg->q_sin[i] : 0.0;
    }
    for (int p = 0; p < nf0 + nf1; ++p) {
        const int a = cfg->form_sites[2 * p], b = cfg->form_sites[2 * p + 1];
        if (a < 0 || a >= n || b < 0 || b >= n)
            return fail(DQMC_ERR_INVALID, "dqmc_set_td_measurements: form-factor site out of range");
        buf[L.form + 3 * p] = a;
        buf[L.form + 3 * p + 1] = b;
        buf[L.form + 3 * p + 2] = cfg->form_values[p];
    }
    for (int p = 0; p < nc; ++p) {
        const int r = cfg->current_sites[2 * p], s2 = cfg->current_sites[2 * p + 1];
        if (r < 0 || r >= n || s2 < 0 || s2 >= n)
            return fail(DQMC_ERR_INVALID, "dqmc_set_td_measurements: current site out of range");
        buf[L.cur + 4 * p] = r;
        buf[L.cur + 4 * p + 1] = s2;
        buf[L.cur + 4 * p + 2] = cfg->current_values[2 * p];
        buf[L.cur + 4 * p + 3] = cfg->current_values[2 * p + 1];
    }
    CUDA_TRY(cudaSetDevice(h->device), "cudaSetDevice");
    if (int st = ensure_ut(h, chain)) return st;
    if (h->td_mem.size() < h->host.size()) h->td_mem.resize(h->host.size(), nullptr);
    // a new layout replaces the buffer and its accumulators
    const bool same = h->td_mem[chain] && d.td_P == P && d.td_nform0 == nf0 &&
                      d.td_nform1 == nf1 && d.td_ncur == nc;
    if (!same) {
        if (h->td_mem[chain]) cudaFree(h->td_mem[chain]);
        h->td_mem[chain] = nullptr;
        CUDA_TRY(cudaMalloc((void**)&h->td_mem[chain], L.total * sizeof(double)),
                 "allocate the time-displaced measurement buffer");
        CUDA_TRY(cudaMemsetAsync(h->td_mem[chain], 0, L.total * sizeof(double), h->stream),
                 "clear the time-displaced accumulators");
    }
    CUDA_TRY(cudaMemcpyAsync(h->td_mem[chain], buf.data(), L.g * sizeof(double),
                             cudaMemcpyHostToDevice, h->stream),
             "upload the time-displaced configuration");
    CUDA_TRY(cudaStreamSynchronize(h->stream), "synchronize");
    d.td = h->td_mem[chain];
    d.td_enable = 1;
    d.td_rate = cfg->measure_rate;
    d.td_P = P;
    d.td_nform0 = nf0;
    d.td_nform1 = nf1;
    d.td_ncur = nc;
    d.td_dtau = cfg->delta_tau;
    if (cfg->sweep >= 0) d.sweep = cfg->sweep;
    h->host_dirty = true;
    return DQMC_OK;
}

int dqmc_td_measure(dqmc_handle* h) {
    if (!h) return fail(DQMC_ERR_INVALID, "null handle");
    bool any = false;
    for (const DqmcChain& d : h->host) any = any || (d.active && d.td);
    if (!any) return fail(DQMC_ERR_INVALID, "dqmc_td_measure: no chain has time-displaced "
                                            "measurements set up");
    return launch(h, DQMC_OP_TD_MEASURE, 0, 0, true);
}

int dqmc_get_td_measurements(dqmc_handle* h, int chain, dqmc_td_observables* out, double* mean,
                             double* error) {
    if (int st = check_chain(h, chain)) return st;
    if (!out) return fail(DQMC_ERR_INVALID, "dqmc_get_td_measurements: null out");
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    const DqmcChain& d = h->host[chain];
    if (!d.td) return fail(DQMC_ERR_INVALID, "dqmc_get_td_measurements: not set up for this chain");
    CUDA_TRY(cudaSetDevice(h->device), "cudaSetDevice");
    const TdLayout L = td_layout(d.n, d.nf, d.td_P, d.td_nform0 + d.td_nform1, d.td_ncur);
    std::vector<double> m(L.total - L.acc);
    CUDA_TRY(cudaMemcpyAsync(m.data(), d.td + L.acc, m.size() * sizeof(double),
                             cudaMemcpyDeviceToHost, h->stream),
             "download the time-displaced accumulators");
    CUDA_TRY(cudaStreamSynchronize(h->stream), "synchronize");
    out->count = (int64_t)m[0];
    auto stats = [&](int k, double* mu, double* err, int32_t* lvl) {
        const double* lv = m.data() + DQMC_MEAS_HEADER + (size_t)k * DQMC_MEAS_LEVELS * DQMC_MEAS_BIN_WORDS;
        *mu = lv[0] > 0 ? lv[1] : NAN;
        int use = -1;
        for (int l = 0; l < DQMC_MEAS_LEVELS; ++l)
            if (lv[l * DQMC_MEAS_BIN_WORDS] >= 32.0) use = l;
        if (use < 0) use = 0;
        const double nb = lv[use * DQMC_MEAS_BIN_WORDS], m2 = lv[use * DQMC_MEAS_BIN_WORDS + 2];
        *err = nb >= 2.0 ? sqrt(m2 / (nb - 1.0) / nb) : INFINITY;
        if (lvl) *lvl = use;
    };
    for (int k = 0; k < DQMC_TD_SCALARS; ++k)
        stats(k, &out->mean[k], &out->error[k], &out->error_level[k]);
    const int nv = DQMC_TD_KINDS * d.td_P;
    for (int k = 0; k < nv; ++k) {
        double mu, err;
        stats(DQMC_TD_SCALARS + k, &mu, &err, nullptr);
        if (mean) mean[k] = mu;
        if (error) error[k] = err;
    }
    return DQMC_OK;
}

/* ---- checkpoint state --------------------------------------------------------- */

// Counters of a chain's checkpoint record, in order (integers stored as doubles,
// exact below 2^53): the DQMCAnalysis / acceptance counters, the MagnitudeStats
// accumulators, global-update and scheduler counts, the measurement settings.
#define DQMC_CKPT_HEADER 28

static void ckpt_pack(const DqmcChain& d, double* o) {
    o[0] = (double)d.accepted;     o[1] = (double)d.proposals;
    o[2] = (double)d.n_prop_err;   o[3] = (double)d.n_neg_p;
    o[4] = d.prop_err_max;         o[5] = d.prop_err_reported;
    o[6] = (double)d.n_imag_p;     o[7] = d.max_imag_p;
    for (int q = 0; q < 3; ++q) {
        o[8 + q] = d.ms_prop[q];
        o[11 + q] = d.ms_neg[q];
        o[14 + q] = d.ms_imag[q];
    }
    o[17] = (double)d.n_near_tie;  o[18] = d.min_tie_gap;
    o[19] = (double)d.g_accepted;  o[20] = (double)d.g_proposals;
    o[21] = (double)d.sched_calls; o[22] = (double)d.global_kind;
    o[23] = (double)d.sweep;       o[24] = (double)d.meas_enable;
    o[25] = (double)d.meas_rate;   o[26] = (double)d.meas_greens;
    o[27] = d.meas_U;
}

static void ckpt_unpack(DqmcChain& d, const double* o) {
    d.accepted = (long long)o[0];     d.proposals = (long long)o[1];
    d.n_prop_err = (long long)o[2];   d.n_neg_p = (long long)o[3];
    d.prop_err_max = o[4];            d.prop_err_reported = o[5];
    d.n_imag_p = (long long)o[6];     d.max_imag_p = o[7];
    for (int q = 0; q < 3; ++q) {
        d.ms_prop[q] = o[8 + q];
        d.ms_neg[q] = o[11 + q];
        d.ms_imag[q] = o[14 + q];
    }
    d.n_near_tie = (long long)o[17];  d.min_tie_gap = o[18];
    d.g_accepted = (long long)o[19];  d.g_proposals = (long long)o[20];
    d.sched_calls = (long long)o[21]; d.global_kind = (int)o[22];
    d.sweep = (long long)o[23];       d.meas_enable = (int)o[24];
    d.meas_rate = (int)o[25];         d.meas_greens = (int)o[26];
    d.meas_U = o[27];
}

int64_t dqmc_checkpoint_doubles(dqmc_handle* h, int chain) {
    if (check_chain(h, chain)) return -1;
    const DqmcChain& d = h->host[chain];
    return (int64_t)(DQMC_CKPT_HEADER + DQMC_MEAS_DOUBLES(d.n, d.nf));
}

int dqmc_get_checkpoint(dqmc_handle* h, int chain, double* out) {
    if (int st = check_chain(h, chain)) return st;
    if (!out) return fail(DQMC_ERR_INVALID, "dqmc_get_checkpoint: null out");
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    CUDA_TRY(cudaSetDevice(h->device), "cudaSetDevice");
    const DqmcChain& d = h->host[chain];
    ckpt_pack(d, out);
    CUDA_TRY(cudaMemcpyAsync(out + DQMC_CKPT_HEADER, d.meas,
                             DQMC_MEAS_DOUBLES(d.n, d.nf) * sizeof(double),
                             cudaMemcpyDeviceToHost, h->stream),
             "download measurement accumulators");
    CUDA_TRY(cudaStreamSynchronize(h->stream), "synchronize");
    return DQMC_OK;
}

int dqmc_set_checkpoint(dqmc_handle* h, int chain, const double* in) {
    if (int st = check_chain(h, chain)) return st;
    if (!in) return fail(DQMC_ERR_INVALID, "dqmc_set_checkpoint: null in");
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    const int gk = (int)in[22], rate = (int)in[25];
    if (!(gk == -1 || gk == DQMC_GLOBAL_FLIP || gk == DQMC_GLOBAL_SHUFFLE) || rate < 1 ||
        !(in[0] >= 0 && in[1] >= in[0]))
        return fail(DQMC_ERR_INVALID, "dqmc_set_checkpoint: not a checkpoint record");
    DqmcChain& d = h->host[chain];
    if (gk >= 0 && d.cplx)
        return fail(DQMC_ERR_INVALID, "dqmc_set_checkpoint: global updates on a complex chain");
    CUDA_TRY(cudaSetDevice(h->device), "cudaSetDevice");
    CUDA_TRY(cudaMemcpyAsync(d.meas, in + DQMC_CKPT_HEADER,
                             DQMC_MEAS_DOUBLES(d.n, d.nf) * sizeof(double),
                             cudaMemcpyHostToDevice, h->stream),
             "upload measurement accumulators");
    CUDA_TRY(cudaStreamSynchronize(h->stream), "synchronize");
    ckpt_unpack(d, in);
    h->host_dirty = true;
    return DQMC_OK;
}

/* ---- pools ------------------------------------------------------------------ */

int dqmc_pool_create(int device, int max_slots, int64_t budget_bytes, int precision,
                     dqmc_handle** out) {
    if (!out || max_slots <= 0 || budget_bytes <= 0)
        return fail(DQMC_ERR_INVALID, "dqmc_pool_create: bad arguments");
    *out = nullptr;
    if (precision != DQMC_PREC_FP64 && precision != DQMC_PREC_MIXED)
        return fail(DQMC_ERR_INVALID, "dqmc_pool_create: unknown precision");
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return fail(DQMC_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
    if (device < 0 || device >= ndev) return fail(DQMC_ERR_INVALID, "dqmc_pool_create: bad device");
    CUDA_TRY(cudaSetDevice(device), "cudaSetDevice");
    CUDA_TRY(dqmc_prepare_chain_kernels(), "kernel attributes");
    dqmc_handle* h = new dqmc_handle();
    h->device = device;
    h->precision = precision;
    h->pool = true;
    // a mixed pool may admit tensor-core-capable chains at any time (its
    // launch is captured once and replayed)
    h->tc = precision == DQMC_PREC_MIXED;
    h->budget = align256((size_t)budget_bytes);
    h->cfg.assign(max_slots, dqmc_chain_config{});
    h->lay.assign(max_slots, Layout{});
    h->host.assign(max_slots, DqmcChain{});
    h->slot_off.assign(max_slots, 0);
    h->slot_bytes.assign(max_slots, 0);
    e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete h; return cuda_fail(e, "cudaStreamCreate"); }
    h->stream = h->own_stream;
    e = cudaMalloc((void**)&h->arena, h->budget);
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->d_chains, sizeof(DqmcChain) * max_slots);
    if (e == cudaSuccess) e = cudaHostAlloc((void**)&h->pinned, sizeof(DqmcChain) * max_slots, 0);
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->d_sync, 4 * sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMemset(h->d_sync, 0, 4 * sizeof(unsigned int));
    if (e != cudaSuccess) {
        int st = cuda_fail(e, "dqmc_pool_create: allocation of the pool");
        dqmc_destroy(h);
        return st;
    }
    h->free_blocks[0] = h->budget;
    int st = push_descriptors(h);
    if (st != DQMC_OK) { dqmc_destroy(h); return st; }
    *out = h;
    return DQMC_OK;
}

int dqmc_pool_admit(dqmc_handle* h, const dqmc_chain_config* cfg, int* slot) {
    if (!h || !h->pool || !cfg || !slot) return fail(DQMC_ERR_INVALID, "dqmc_pool_admit: bad arguments");
    if (int st = validate_config(*cfg, -1)) return st;
    if (is_cplx(*cfg) && h->precision != DQMC_PREC_FP64)
        return fail(DQMC_ERR_INVALID, "dqmc_pool_admit: complex chains run in FP64 only");
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    int free_slot = -1;
    for (size_t i = 0; i < h->host.size(); ++i)
        if (!h->host[i].active) { free_slot = (int)i; break; }
    if (free_slot < 0) return fail(DQMC_ERR_NOT_READY, "dqmc_pool_admit: no free slot");
    const Layout L = layout_of(*cfg, h->precision);
    size_t off = 0;
    if (!pool_alloc(h, L.bytes, &off))
        return fail(DQMC_ERR_OOM, "dqmc_pool_admit: chain needs " + std::to_string(L.bytes) +
                                      " bytes, more than the pool's free budget allows");
    CUDA_TRY(cudaSetDevice(h->device), "cudaSetDevice");
    CUDA_TRY(cudaMemsetAsync(h->arena + off, 0, L.bytes, h->stream), "clear chain workspace");
    fill_descriptor(h->host[free_slot], *cfg, h->arena + off, L, h->precision);
    h->host[free_slot].needs_build = 1;
    h->host[free_slot].run_sync = h->d_sync;
    h->cfg[free_slot] = *cfg;
    h->lay[free_slot] = L;
    h->slot_off[free_slot] = off;
    h->slot_bytes[free_slot] = L.bytes;
    h->host_dirty = true;
    *slot = free_slot;
    return DQMC_OK;
}

int dqmc_pool_release(dqmc_handle* h, int slot) {
    if (int st = check_chain(h, slot)) return st;
    if (!h->pool) return fail(DQMC_ERR_INVALID, "dqmc_pool_release: not a pool");
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    pool_free(h, h->slot_off[slot], h->slot_bytes[slot]);
    if ((size_t)slot < h->ut_mem.size() && h->ut_mem[slot]) {
        cudaFree(h->ut_mem[slot]);
        h->ut_mem[slot] = nullptr;
    }
    if ((size_t)slot < h->td_mem.size() && h->td_mem[slot]) {
        cudaFree(h->td_mem[slot]);
        h->td_mem[slot] = nullptr;
    }
    if ((size_t)slot < h->cb_mem.size() && h->cb_mem[slot]) {
        cudaFree(h->cb_mem[slot]);
        h->cb_mem[slot] = nullptr;
    }
    memset(&h->host[slot], 0, sizeof(DqmcChain));
    h->cfg[slot] = dqmc_chain_config{};
    h->slot_bytes[slot] = 0;
    h->host_dirty = true;
    return DQMC_OK;
}

int dqmc_pool_set_flavour_split(dqmc_handle* h, int enable) {
    if (!h || !h->pool) return fail(DQMC_ERR_INVALID, "dqmc_pool_set_flavour_split: not a pool");
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    const bool on = enable != 0;
    if (on != h->flavour_split && h->graph) {  // the captured launch changes shape
        cudaGraphExecDestroy(h->graph);
        h->graph = nullptr;
    }
    h->flavour_split = on;
    return DQMC_OK;
}

int dqmc_pool_set_split_silence(dqmc_handle* h, int slot, int from_epoch) {
    if (int st = check_chain(h, slot)) return st;
    if (!h->pool) return fail(DQMC_ERR_INVALID, "dqmc_pool_set_split_silence: not a pool");
    if (from_epoch < 0) return fail(DQMC_ERR_INVALID, "dqmc_pool_set_split_silence: from_epoch < 0");
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    h->host[slot].x_silent_from = from_epoch;
    h->host_dirty = true;
    return DQMC_OK;
}

int dqmc_pool_set_quota(dqmc_handle* h, int slot, int64_t n_sweeps) {
    if (int st = check_chain(h, slot)) return st;
    if (n_sweeps < 0) return fail(DQMC_ERR_INVALID, "dqmc_pool_set_quota: n_sweeps < 0");
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    h->host[slot].visits_quota = n_sweeps * 2 * (int64_t)h->host[slot].M;
    h->host_dirty = true;
    return DQMC_OK;
}

int dqmc_pool_slot(dqmc_handle* h, int slot, int64_t* sweeps_done, int64_t* sweeps_left,
                   int32_t* active) {
    if (!h || slot < 0 || slot >= (int)h->host.size())
        return fail(DQMC_ERR_INVALID, "dqmc_pool_slot: slot out of range");
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    const DqmcChain& d = h->host[slot];
    const int64_t per = d.active ? 2 * (int64_t)d.M : 1;
    if (sweeps_done) *sweeps_done = d.active ? d.visits_done / per : 0;
    if (sweeps_left) *sweeps_left = d.active ? (d.visits_quota + per - 1) / per : 0;
    if (active) *active = d.active;
    return DQMC_OK;
}

int64_t dqmc_pool_free_bytes(dqmc_handle* h) {
    if (!h || !h->pool) return -1;
    int64_t s = 0;
    for (auto& kv : h->free_blocks) s += (int64_t)kv.second;
    return s;
}

int dqmc_pool_run(dqmc_handle* h, int budget_us, int use_graph) {
    if (!h || !h->pool) return fail(DQMC_ERR_INVALID, "dqmc_pool_run: not a pool");
    if (budget_us <= 0) return fail(DQMC_ERR_INVALID, "dqmc_pool_run: budget_us <= 0");
    if (!use_graph) {
        if (h->busy) if (int st = dqmc_synchronize(h)) return st;
        CUDA_TRY(cudaSetDevice(h->device), "cudaSetDevice");
        CUDA_TRY(cudaMemsetAsync(h->d_sync, 0, 4 * sizeof(unsigned int), h->stream),
                 "reset visit counters");
        return launch(h, DQMC_OP_RUN, budget_us, 0, true);
    }
    if (h->busy) if (int st = dqmc_synchronize(h)) return st;
    CUDA_TRY(cudaSetDevice(h->device), "cudaSetDevice");
    const size_t bytes = sizeof(DqmcChain) * h->host.size();
    if (!h->graph || h->graph_budget_us != budget_us) {
        if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
        // one replayable step: upload descriptors, time-sliced launch, download
        cudaGraph_t g = nullptr;
        CUDA_TRY(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
        cudaError_t e0 = cudaMemsetAsync(h->d_sync, 0, 4 * sizeof(unsigned int), h->stream);
        cudaError_t e1 = cudaMemcpyAsync(h->d_chains, h->pinned, bytes, cudaMemcpyHostToDevice, h->stream);
        if (e1 == cudaSuccess) e1 = e0;
        cudaError_t e2 = dqmc_launch_chain_kernel(h->d_chains, (int)h->host.size(), DQMC_OP_RUN,
                                                  budget_us, 0, h->stream, 0, h->tc,
                                                  h->flavour_split);
        cudaError_t e3 = cudaMemcpyAsync(h->pinned, h->d_chains, bytes, cudaMemcpyDeviceToHost, h->stream);
        cudaError_t e4 = cudaStreamEndCapture(h->stream, &g);
        if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess || e4 != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return cuda_fail(e4 != cudaSuccess ? e4 : (e1 != cudaSuccess ? e1 : (e2 != cudaSuccess ? e2 : e3)),
                             "graph capture of the pool step");
        }
        cudaError_t e5 = cudaGraphInstantiate(&h->graph, g, 0);
        cudaGraphDestroy(g);
        if (e5 != cudaSuccess) { h->graph = nullptr; return cuda_fail(e5, "graph instantiate"); }
        h->graph_budget_us = budget_us;
    }
    memcpy(h->pinned, h->host.data(), bytes);
    CUDA_TRY(cudaGraphLaunch(h->graph, h->stream), "graph launch");
    CUDA_TRY(cudaStreamSynchronize(h->stream), "pool step");
    memcpy(h->host.data(), h->pinned, bytes);
    h->host_dirty = false;
    for (size_t i = 0; i < h->host.size(); ++i)
        if (h->host[i].active && h->host[i].status != 0)
            return fail(DQMC_ERR_NUMERICAL, "slot " + std::to_string(i) + " reported status " +
                                                 std::to_string(h->host[i].status));
    return DQMC_OK;
}

}  // extern "C"

int dqmc_report_error(int code, const std::string& msg) { return fail(code, msg); }
