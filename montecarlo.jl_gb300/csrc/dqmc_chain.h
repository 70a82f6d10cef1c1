// Device-side description of one DQMC chain (one Markov chain of the
// reference's DQMC: field configuration, Green's function and UDT stack).
//
// Layout in HBM (all FP64 matrices column-major, n x n per flavour block,
// flavour block b of an nf-block matrix at offset b*n*n):
//   G, Gtmp, Ul, Ur, Tl, Tr, tmp1, tmp2, currU, out    nf*n*n each
//   ustack, tstack                                      (nr+1) * nf*n*n
//   dstack                                              (nr+1) * nf*n
//   Dl, Dr, tempv                                       nf*n
//   pivot                                               nf*n (int32, 1-based)
//   conf                                                n*M int8, site fastest
//   eT2, eT2inv, eTh, eThinv                            n*n each (one block,
//                                                       shared by both flavours)
#pragma once
#include <stdint.h>
#include <vector_types.h>

#define DQMC_MAX_CHUNKS 256

struct DqmcChain {
    // sizes
    int n, nf, M, k, kind, nr, check_prop, prec;
    // per-proposal tables computed on the host with the reference's
    // expressions (fields.jl:388-393, 440-449, 563-573, 627-637):
    //   Hirsch: index s_idx = (s > 0); GHQ: index (x_old-1)*4 + (x_new-1)
    double delta0[16], delta1[16], wboson[16];
    double gam[4];
    // interaction exponentials (fields.jl:380-386, 429-438, 548-560, 618-624)
    //   ev[f][v]: flavour block f, field value index v, power +1
    //   evinv[f][v]: power -1.  Hirsch v = (s > 0); GHQ v = x - 1.
    double ev[2][4], evinv[2][4];
    // chunk ranges (generate_chunks), 1-based inclusive
    int rfirst[DQMC_MAX_CHUNKS], rlast[DQMC_MAX_CHUNKS];
    // buffers
    int8_t* conf;
    const double *eT2, *eT2inv, *eTh, *eThinv;
    // eT2 and eT2inv split into float pairs (hi, lo) for the mixed path's
    // double-float products
    const float2 *eT2df, *eT2invdf;
    double *G, *Gtmp, *ustack, *tstack, *dstack, *Ul, *Ur, *Tl, *Tr, *Dl, *Dr, *tmp1, *tmp2,
        *currU, *tempv, *out;
    int* pivot;
    // RNG
    uint64_t key, ctr;
    // stack state (stack.jl:34-41)
    int current_slice, current_range, direction, pad0;
    // analysis (statistics.jl:9-51; stack.jl:644-653)
    double prop_err_max, prop_err_reported;
    long long n_prop_err, n_neg_p, accepted, proposals;
    int status, pad1;
    // SM cycles spent per phase (thread 0's clock64 around each phase), the
    // device counterpart of the reference's @bm / TimerOutputs sections
    // (helpers.jl:83-131): see DQMC_PHASE_*
    unsigned long long timers[8];
    // pool / time-sliced runs: slot in use, stack still to build, remaining
    // slice visits the chain may run, slice visits run so far
    int active, needs_build;
    long long visits_quota, visits_done;
    // equal-time measurements on the device (measure() in dqmc_chain_ops.cuh):
    // on/off, sweeps between measurements, accumulate the mean physical G,
    // the chain's sweep counter (the reference's mc.last_sweep), U for the
    // interaction energy, cos/sin(q.r_i) for S^z(q) (2n values, or NULL) and
    // the accumulator block (layout DQMC_MEAS_*)
    int meas_enable, meas_rate, meas_greens, pad2;
    long long sweep;
    double meas_U;
    const double* qcs;
    double* meas;
    // global updates (global_updates.jl) and replica exchange between chains
    // (parallel_updates.jl): temp_conf(field) (n*M), stack.tempvf (nf*n),
    // acceptance counters, the weight and uniform of the last replica-weight
    // step, the replica partner (-1: none), a global update scheduled before
    // every sweep but the first (-1: none; 0 flip, 1 shuffle) and the
    // scheduler calls made with it
    int8_t* temp_conf;
    double* tempvf;
    double alpha_field;
    long long g_accepted, g_proposals;
    double r_weight, r_prob;
    int partner, global_kind;
    long long sched_calls;
    // unequal-time Green's function (unequal_time_stack.jl): the chain's
    // forward / backward / inverse stacks and work matrices (layout in
    // ut_layout of dqmc_chain_ops.cuh; NULL until first used), and the (k, l)
    // pairs and output of the current request
    double* ut;
    const int* ut_pairs;
    double* ut_out;
    // checkerboard = true (stack.jl:240-246, linalg/checkerboard.jl): parts
    // per factor; the four factors exp(-dtau T), exp(+dtau T), exp(-dtau T/2),
    // exp(+dtau T/2), each D[n] then per part c[n], s[n] (cb), and per factor
    // and part the bond partner of each site (cbp, -1: none); NULL: the
    // dense exponentials
    int cb_np, pad3;
    const double* cb;
    const int* cbp;
    // complex chain (a complex field constant, the reference's ComplexF64
    // path): every matrix is the real 2 ns x 2 ns representation
    // [[Re, -Im], [Im, Re]] of the ns x ns complex one (n = 2 ns; the
    // adjoint of a complex matrix is the transpose of its representation),
    // ns = sites (= n on a real chain).  Imaginary parts of the proposal
    // tables and interaction exponentials, and the sign-problem statistics of
    // sweep_spatial (local_updates.jl:33-46): proposals with |imag(p)| > 1e-6
    // and the largest such |imag(p)|.
    int cplx, ns;
    double delta0i[16], delta1i[16], wbosoni[16];
    double evi[2][4], evinvi[2][4];
    long long n_imag_p;
    double max_imag_p;
    // MagnitudeStats (statistics.jl:9-36) of the recorded propagation errors
    // (> 1e-7), negative probabilities and imaginary probabilities: max, min
    // and sum of log10 |value| each (counts: n_prop_err, n_neg_p, n_imag_p)
    double ms_prop[3], ms_neg[3], ms_imag[3];
    // near ties of the Metropolis test `rand() < p` (local_updates.jl:53):
    // local proposals that drew a uniform u (p <= 1) with |u - p| < 1e-12,
    // where a rounding-level difference in p could change the decision, and
    // the smallest |u - p| of any drawn proposal (+inf before the first)
    long long n_near_tie;
    double min_tie_gap;
    // mixed chains with 96 <= n <= 256: which products run on the tensor
    // cores (tcgen05 split-precision products) instead of the FP32 pipe, a
    // mask of DQMC_TC_WRAPS, DQMC_TC_SLICES, DQMC_TC_GREENS
    int tc_enable, pad4;
    unsigned char* tcs;  // the tensor products' slice scratch (NULL: chain cannot use them)
    // time-displaced measurements on the device (td_measure in
    // dqmc_chain_ops.cuh): on/off, sweeps between measurements (on the sweep
    // counter `sweep`), slots of the by-distance arrays, bonds of the two pair
    // form factors, entries of the current operator, delta tau, and the buffer
    // (layout td_layout below)
    int td_enable, td_rate, td_P, td_nform0, td_nform1, td_ncur;
    double td_dtau;
    double* td;
    // pool launches: {chains that started visiting, chains past their time
    // budget} of the current launch (shared by the pool's chains, zeroed
    // before every launch); NULL outside pools
    unsigned int* run_sync;
    // test hook of a flavour-split chain's rendezvous time-out: from this
    // rendezvous epoch on, the second CTA no longer publishes its epoch, so
    // that the first one's bounded wait runs out (0: never)
    int x_silent_from, pad5;
};


// the near-tie window of DqmcChain::n_near_tie
#define DQMC_NEAR_TIE 1e-12
#ifdef __CUDACC__
// The decision `p > 1 || rand() < p` (local_updates.jl:53) with the uniform
// (w >> 11) 2^-53 built on the integer pipe: the 53-bit integer is exact in
// a double and the power-of-two scaling is exact, so these are the bits of
// the same double; the comparisons of non-negative doubles order like their
// bit patterns (NaN and negative p handled explicitly).  On GB300's narrow
// FP64 pipe this keeps the conversion and the comparisons off the serial
// decision chain.
__device__ __forceinline__ long long uniform_bits(uint64_t w) {
    const uint64_t m = w >> 11;
    if (m == 0) return 0;
    const int sh = __clzll((long long)m) - 11;  // the leading one to bit 52
    return (long long)(((uint64_t)(1022 - sh) << 52) | ((m << sh) & ((1ull << 52) - 1)));
}
__device__ __forceinline__ bool bits_nan(long long P) {
    return (P & 0x7FFFFFFFFFFFFFFFll) > 0x7FF0000000000000ll;
}
// p > 1.0
__device__ __forceinline__ bool above_one(double p) {
    const long long P = __double_as_longlong(p);
    return P > 0x3FF0000000000000ll && !bits_nan(P);
}
// p < 0.0
__device__ __forceinline__ bool below_zero(double p) {
    const long long P = __double_as_longlong(p);
    return P < 0 && (P & 0x7FFFFFFFFFFFFFFFll) != 0 && !bits_nan(P);
}
// u < p for a uniform's bits U (a double in [0, 1))
__device__ __forceinline__ bool uniform_below(long long U, double p) {
    const long long P = __double_as_longlong(p);
    return !bits_nan(P) && U < P;
}
// record the gap between a drawn uniform u and the probability p it is tested
// against (the decision itself is `u < p`)
__device__ __forceinline__ void note_tie(DqmcChain& c, double u, double p) {
    const double gap = fabs(u - p);
    if (gap < DQMC_NEAR_TIE) c.n_near_tie += 1;
    if (gap < c.min_tie_gap) c.min_tie_gap = gap;
}
#endif
#define DQMC_MS_PUSH(ms, v)                               \
    do {                                                  \
        const double l_ = log10(fabs(v));                 \
        if (l_ > (ms)[0]) (ms)[0] = l_;                   \
        if (l_ < (ms)[1]) (ms)[1] = l_;                   \
        (ms)[2] += l_;                                    \
    } while (0)
#define DQMC_CB_MAXPARTS 12

// Measurement accumulators of one chain (doubles):
//   [0] measurements taken, [1..3] unused
//   log binners: scalar k, level l at DQMC_MEAS_HEADER + (k * LEVELS + l) * 5:
//     {completed bins, Welford mean, Welford M2, pending value, pending flag}
//     (level l bins 2^l consecutive values)
//   occupation sums nf*n at DQMC_MEAS_OCC_OFF, then G sums nf*n*n
// Scalars: 0 density per site, 1 double occupancy, 2 interaction energy,
// 3 S^z(q).
#define DQMC_MEAS_SCALARS 4
#define DQMC_MEAS_LEVELS 32
#define DQMC_MEAS_HEADER 4
#define DQMC_MEAS_BIN_WORDS 5
#define DQMC_MEAS_OCC_OFF (DQMC_MEAS_HEADER + DQMC_MEAS_SCALARS * DQMC_MEAS_LEVELS * DQMC_MEAS_BIN_WORDS)
#define DQMC_MEAS_DOUBLES(n, nf) \
    ((size_t)DQMC_MEAS_OCC_OFF + (size_t)(nf) * (n) + (size_t)(nf) * (n) * (n))

// Time-displaced measurements: the susceptibilities (scalars) and the
// by-distance correlation arrays accumulated per measurement
#define DQMC_TD_SCALARS 8  // charge, spin x, y, z (at q), s, extended s, d pairing, current
#define DQMC_TD_KINDS 5    // by-distance arrays: charge, spin x, y, z, on-site pairing
// Offsets (in doubles) of a chain's time-displaced buffer: pair slots (n^2
// int32), q phases (cos, sin), form-factor bonds (a, b, F), current entries
// (r, s, re, im), the four physical Green's functions G(0,0), G(0,l), G(l,0),
// G(l,l), the by-distance sums of one measurement (5 P), and the log binners
// (header, then DQMC_TD_SCALARS + 5 P binners of DQMC_MEAS_LEVELS levels).
struct TdLayout {
    size_t slot, q, form, cur, g, stage, acc, total;
};
#ifdef __CUDACC__
__host__ __device__
#endif
inline TdLayout td_layout(int n, int nf, int P, int nform, int ncur) {
    TdLayout L;
    size_t o = 0;
    L.slot = o; o += ((size_t)n * n + 1) / 2;
    L.q = o; o += 2 * (size_t)n;
    L.form = o; o += 3 * (size_t)nform;
    L.cur = o; o += 4 * (size_t)ncur;
    L.g = o; o += 4 * (size_t)nf * n * n;
    L.stage = o; o += (size_t)DQMC_TD_KINDS * P;
    L.acc = o;
    o += DQMC_MEAS_HEADER +
         (size_t)(DQMC_TD_SCALARS + DQMC_TD_KINDS * (size_t)P) * DQMC_MEAS_LEVELS * DQMC_MEAS_BIN_WORDS;
    L.total = o;
    return L;
}

enum { DQMC_PHASE_SWEEP_SPATIAL = 0, DQMC_PHASE_WRAP = 1, DQMC_PHASE_SLICE_CHAIN = 2,
       DQMC_PHASE_UDT = 3, DQMC_PHASE_GREENS = 4, DQMC_PHASE_PROP_CHECK = 5,
       DQMC_PHASE_T_UPDATE = 6, DQMC_PHASE_OTHER = 7 };

enum { DQMC_OP_SWEEP = 0, DQMC_OP_BUILD = 1, DQMC_OP_GREENS_AT = 2, DQMC_OP_PHYSICAL = 3,
       DQMC_OP_BUILD_FWD = 4, DQMC_OP_PROPAGATE = 5, DQMC_OP_SWEEP_SPATIAL = 6,
       DQMC_OP_RUN = 7 /* time-sliced: arg0 = budget in microseconds */,
       DQMC_OP_GLOBAL = 8 /* arg0: 0 GlobalFlip, 1 GlobalShuffle */,
       DQMC_OP_REPLICA_WEIGHT = 9, DQMC_OP_REPLICA_ACCEPT = 10,
       DQMC_OP_GREENS_KL = 11 /* arg0 = number of (k, l) pairs */,
       DQMC_OP_TD_MEASURE = 12 };

// doubles of a chain's unequal-time workspace: forward and backward U, T
// ((nr + 1) each) and inverse U, T (nr each) of nf*n*n, their D vectors, and
// s.U, s.T, s.greens, s.D
#define DQMC_UT_DOUBLES(n, nf, nr)                                                   \
    ((size_t)(nf) * (n) * (n) * (4 * ((nr) + 1) + 2 * (nr) + 3) +                    \
     (size_t)(nf) * (n) * (2 * ((nr) + 1) + (nr) + 1))

// DqmcChain::prec values (same numbers as DQMC_PREC_* of the C ABI)
#define DQMC_PREC_FP64_ID 0
#define DQMC_PREC_MIXED_ID 1
