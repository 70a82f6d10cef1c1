/*
 * dqmc_gb300.h -- C ABI of the GB300 DQMC sweep library (libdqmc_gb300.so).
 *
 * The library replaces, for the determinant quantum Monte Carlo of
 * carstenbauer/MonteCarlo.jl, the hot path below the reference's plugin seam
 * `update(::AbstractUpdate, mc, model, field)`: the local sweep, the
 * Green's-function wraps, the slice-matrix chains and the UDT stabilisation
 * (the `DQMCStack` functions).  A host in any language (the reference's Julia
 * through `ccall`, Python through ctypes, C/C++) owns the model, lattice,
 * parameters and measurements, and calls these entry points.
 *
 * Conventions
 *   - Matrices are FP64, column-major, n x n per flavour block.  A chain with
 *     two flavour blocks (MagneticHirsch / MagneticGHQ fields) passes and
 *     receives 2*n*n doubles, block b at offset b*n*n: the reference's
 *     BlockDiagonal{Float64,2,Matrix{Float64}}.  One block is the reference's
 *     Matrix{Float64} (Density fields).
 *   - The field configuration is int8, n x M, column-major (site fastest),
 *     values +-1 (Hirsch) or 1..4 (Gauss-Hermite), as `field.conf`.
 *   - Slices and chunk indices are 1-based, as in the reference.
 *   - Host buffers are borrowed for the duration of the call; the handle owns
 *     all device memory.  Every call returns a status (DQMC_OK = 0); the text
 *     of the last error of the calling thread is `dqmc_last_error()`.  Nothing
 *     throws across the ABI.
 *   - A handle may not be used from two threads at once; distinct handles may.
 *     Synchronous calls return when their work is complete; *_async calls
 *     return at once and complete through dqmc_query / dqmc_synchronize.
 *   - The library has no CPU fallback: without a usable CUDA device every
 *     call that needs one returns DQMC_ERR_CUDA.
 *   - Complex chains (alpha_imag != 0: a field whose Hubbard-Stratonovich
 *     constant is complex because its kind does not match the sign of U, the
 *     reference's ComplexF64 path, fields.jl:294, 372, 421, 530, 600) exchange
 *     their Green's functions as complex n x n blocks, each entry two doubles
 *     (re, im) -- Julia's Matrix{ComplexF64} memory layout -- so 2*nf*n*n
 *     doubles per matrix.  Hopping matrices stay real n x n.
 */
#ifndef DQMC_GB300_H
#define DQMC_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DQMC_GB300_ABI_VERSION 10

/* status codes */
#define DQMC_OK 0
#define DQMC_ERR_INVALID 1   /* bad argument */
#define DQMC_ERR_CUDA 2      /* CUDA runtime error / no device */
#define DQMC_ERR_OOM 3       /* device allocation failed (or over the budget) */
#define DQMC_ERR_NUMERICAL 4 /* kernel reported a non-finite or invalid state */
#define DQMC_ERR_NOT_READY 5 /* asynchronous work still running */

/* field kinds (src/flavors/DQMC/fields.jl) */
#define DQMC_FIELD_DENSITY_HIRSCH 0  /* fields.jl:363-395 */
#define DQMC_FIELD_MAGNETIC_HIRSCH 1 /* fields.jl:412-451 */
#define DQMC_FIELD_DENSITY_GHQ 2     /* fields.jl:589-637 */
#define DQMC_FIELD_MAGNETIC_GHQ 3    /* fields.jl:519-573 */

/* arithmetic of the wraps and slice-matrix chains */
#define DQMC_PREC_FP64 0  /* everything FP64 (parity path) */
#define DQMC_PREC_MIXED 1 /* wraps, slice-matrix chains and the products of the Green's
                             reconstruction as double-float products on the FP32 pipe;
                             UDT factorisations, triangular solves, determinant ratios
                             and rank-1 updates in FP64 */

typedef struct dqmc_handle dqmc_handle;

/* One chain.  Mirrors what the reference derives in DQMC(model; beta, delta_tau,
 * safe_mult, field) (src/flavors/DQMC/DQMC.jl:32-64, parameters.jl:84-139). */
typedef struct {
    int32_t n_sites;       /* N = length(lattice(model)) */
    int32_t n_flavors;     /* unique_flavors(field, model): 1 or 2 */
    int32_t slices;        /* M = round(beta / delta_tau) */
    int32_t safe_mult;     /* parameters.safe_mult */
    int32_t field;         /* DQMC_FIELD_* */
    int32_t check_propagation_error; /* parameters.check_propagation_error */
    double alpha;          /* field.alpha (its real part for a complex alpha) */
    uint64_t seed;         /* key of the chain's Philox4x32-10 stream */
    double alpha_imag;     /* imaginary part of field.alpha; nonzero: complex chain
                              (FP64 only, n_sites <= 128; no device measurements,
                              global updates or replica exchange) */
} dqmc_chain_config;

/* Per-chain counters (DQMCAnalysis, statistics.jl:45-51; AcceptanceStatistics,
 * scheduler.jl:163-181). */
typedef struct {
    int64_t accepted;             /* accepted local moves since creation */
    int64_t proposals;            /* proposed local moves since creation */
    int64_t propagation_errors;   /* stabilisations with max|dG| > 1e-7 */
    int64_t negative_probability; /* proposals with p < 0 */
    double max_propagation_error; /* max over all stabilisations of max|dG| */
    double max_reported_error;    /* max of the errors counted above */
    /* status: 0 ok; 1 invalid chain (size out of range, or an operation the
     * chain was not set up for); 2 non-finite Green's function at a
     * stabilisation; 7 a tensor-core product's bounded wait ran out (the chain
     * continues on the FP32-pipe product); 9 the partner CTA of a
     * flavour-split chain stopped answering at a rendezvous.  A nonzero status
     * makes the call that ran the chain return DQMC_ERR_NUMERICAL. */
    int32_t current_slice, current_range, direction, status;
    int64_t imaginary_probability; /* proposals with |imag(p)| > 1e-6 (complex chains) */
    double max_imaginary_probability; /* max |imag(p)| of those */
    /* the rest of DQMCAnalysis' MagnitudeStats (statistics.jl:9-36): min and the
     * geometric mean (10^mean log10|v|) of the recorded propagation errors
     * (> 1e-7), of |p| of the negative probabilities (with their max) and of the
     * imaginary parts; 0 when nothing was recorded */
    double min_reported_error, mean_reported_error;
    double min_negative_probability, mean_negative_probability, max_negative_probability;
    double min_imaginary_probability, mean_imaginary_probability;
    /* near ties of the Metropolis test `rand() < p` (local_updates.jl:53):
     * local proposals whose drawn uniform u lay within 1e-12 of p (a
     * rounding-level difference in p could have changed the decision), and
     * the smallest |u - p| of any proposal that drew a uniform (+inf if none) */
    int64_t near_ties;
    double min_tie_gap;
} dqmc_stats;

/* ---- lifecycle ------------------------------------------------------------
 * Replaces: DQMC(model; ...) stack allocation, DQMCStack + initialize_stack
 * (src/flavors/DQMC/stack.jl:113-132, 160-206).  `precision` is DQMC_PREC_*. */
int dqmc_create(int device, const dqmc_chain_config* chains, int n_chains, int precision,
                dqmc_handle** out);
int dqmc_destroy(dqmc_handle* h);
const char* dqmc_last_error(void);
int dqmc_abi_version(void);
/* Run the handle's work on a caller-owned cudaStream_t (passed as void*);
 * NULL restores the handle's own stream.  Lets a host time or order the
 * library's launches with its own CUDA events and streams. */
int dqmc_set_stream(dqmc_handle* h, void* cuda_stream);
/* Sweeps of handles whose chains all have n_sites <= 32 (real, FP64, dense
 * hopping, no device measurements or scheduled global updates) run one warp
 * per chain, eight chains per CTA, instead of one CTA per chain (default
 * enable = 1; pools always use the CTA kernel).  Same state, workspace and
 * accept/reject decisions; sums in a different order (G agrees to rounding). */
int dqmc_set_small_chain_kernel(dqmc_handle* h, int enable);
/* Mixed-precision chains with 96 <= n_sites <= 256 (real, dense hopping) can
 * run products on the tensor cores: tcgen05 MMAs on BF16 digit slices of the
 * operands (six per operand, exact FP32 accumulation per digit level, 47 bits
 * relative to each row's / column's largest entry) instead of the
 * double-float products on the FP32 pipe.  mask: DQMC_TC_WRAPS (the ordinary
 * wraps of G), DQMC_TC_SLICES (the slice-matrix chains of the stack),
 * DQMC_TC_GREENS (the products of the Green's reconstruction); 0: none.
 * The default for new chains is DQMC_TC_DEFAULT.  chain = -1: all. */
#define DQMC_TC_WRAPS 1
#define DQMC_TC_SLICES 2
#define DQMC_TC_GREENS 4
#define DQMC_TC_DEFAULT (DQMC_TC_WRAPS | DQMC_TC_SLICES | DQMC_TC_GREENS)
int dqmc_set_tensor_products(dqmc_handle* h, int chain, int mask);
/* Device bytes one chain needs (stack + Green's function workspace). */
int64_t dqmc_chain_bytes(const dqmc_chain_config* cfg, int precision);

/* ---- inputs ---------------------------------------------------------------
 * Replaces: init_hopping_matrices (stack.jl:209-249).  The four matrices are
 * exp(-dtau T), exp(+dtau T), exp(-dtau T/2), exp(+dtau T/2), one n x n block
 * each (shared by both flavour blocks).  chain = -1 sets every chain. */
int dqmc_set_hopping(dqmc_handle* h, int chain, const double* exp_m_dtT, const double* exp_p_dtT,
                     const double* exp_m_half_dtT, const double* exp_p_half_dtT);
/* Replaces: field.conf access / copyto!(conf(field), c) (fields.jl:305-318). */
int dqmc_set_field(dqmc_handle* h, int chain, const int8_t* conf);
int dqmc_get_field(dqmc_handle* h, int chain, int8_t* conf);
/* Replaces: rand!(field) (fields.jl:330, 470), drawn from the chain's stream;
 * leaves the stream counter at n*M.  chain = -1: all chains. */
int dqmc_init_random_field(dqmc_handle* h, int chain);
/* Replaces: Random.seed! / the RNG state saved with a simulation (FileIO.jl:201-222). */
int dqmc_set_rng(dqmc_handle* h, int chain, uint64_t key, uint64_t counter);
int dqmc_get_rng(dqmc_handle* h, int chain, uint64_t* key, uint64_t* counter);

/* ---- stack ----------------------------------------------------------------
 * Replaces: reverse_build_stack + propagate in initialize_run (DQMC.jl:178-179,
 * stack.jl:284-308, 605-730), all chains. */
int dqmc_initialize_run(dqmc_handle* h);
/* Replaces: build_stack (stack.jl:257-281), all chains. */
int dqmc_build_stack(dqmc_handle* h);
/* Replaces: propagate (stack.jl:605-730), one step, all chains. */
int dqmc_propagate(dqmc_handle* h);
/* Replaces: sweep_spatial (local_updates.jl:23-60) at the current slice. */
int dqmc_sweep_spatial(dqmc_handle* h);

/* ---- the hot path -----------------------------------------------------------
 * Replaces: update(::LocalSweep, mc, model, field) (local_updates.jl:7-14, 82)
 * called n_sweeps times, for every chain of the handle in one launch.
 * stats (may be NULL) receives n_chains entries after the call. */
int dqmc_sweep(dqmc_handle* h, int n_sweeps, dqmc_stats* stats);
int dqmc_sweep_async(dqmc_handle* h, int n_sweeps);
int dqmc_query(dqmc_handle* h);       /* DQMC_OK when idle, DQMC_ERR_NOT_READY when busy */
int dqmc_synchronize(dqmc_handle* h);
int dqmc_get_stats(dqmc_handle* h, int chain, dqmc_stats* out);
/* Replaces: the @bm / TimerOutputs sections (src/helpers.jl:83-131).  out[8]:
 * SM cycles since creation spent in sweep_spatial, ordinary wraps, slice chains,
 * UDT decompositions, Green's reconstruction, propagation checks, T updates,
 * other. */
int dqmc_get_timers(dqmc_handle* h, int chain, uint64_t* out);

/* ---- outputs --------------------------------------------------------------
 * Replaces: mc.stack.greens (physical = 0) and greens!/_greens!
 * (greens.jl:94-125, physical = 1). */
int dqmc_get_greens(dqmc_handle* h, int chain, int physical, double* out);
int dqmc_set_greens(dqmc_handle* h, int chain, const double* in);
/* Chains first .. first+count-1 at once (one strided copy when they are real
 * chains of equal configuration with evenly spaced workspaces, as a fixed
 * handle's equal chains are; chain by chain otherwise): their Green's
 * functions back to back into out (physical = 1: greens!, computed for every
 * chain of the handle), their fields into / from n*M int8 each. */
int dqmc_get_greens_batch(dqmc_handle* h, int first, int count, int physical, double* out);
int dqmc_get_fields_batch(dqmc_handle* h, int first, int count, int8_t* out);
int dqmc_set_fields_batch(dqmc_handle* h, int first, int count, const int8_t* in);
/* Replaces: calculate_greens(mc, slice, output, field, safe_mult) (stack.jl:525-583).
 * safe_mult <= 0 uses the chain's own. */
int dqmc_calculate_greens(dqmc_handle* h, int chain, int slice, int safe_mult, double* out);
/* which: 0 u_stack, 1 t_stack (nf*n*n), 2 d_stack (nf*n); idx 1-based (stack.jl:13-15) */
int dqmc_get_stack(dqmc_handle* h, int chain, int which, int idx, double* out);
/* Replaces: calculate_greens(mc, k, l) / greens(mc, k, l) through the
 * UnequalTimeStack (unequal_time_stack.jl:124-178, 326-338, 400-697): the
 * unequal-time G(k, l) = <c(k dtau) c^dagger(l dtau)> of the chain's current
 * configuration for npairs pairs (0 <= k, l <= M), out: npairs * nf*n*n.
 * physical = 1 applies the _greens! transform (greens.jl:114-125).  The
 * forward, backward and inverse stacks are built once per call (the chain's
 * workspace for them, (4(nr+1) + 2nr + 3) nf n^2 doubles, is allocated on the
 * first call).  Overwrites the stack scratch Ul..Tr, curr_U, tmp1, tmp2,
 * pivot and tempv, as the reference's greens(mc, k, l) does. */
int dqmc_calculate_greens_kl(dqmc_handle* h, int chain, const int32_t* k, const int32_t* l,
                             int npairs, int physical, double* out);

/* ---- equal-time measurements on the device ----------------------------------
 * Replaces: the measurement step of run! (DQMC.jl:205-222: after every
 * measure_rate-th sweep past thermalisation) with the equal-time kernels the
 * reference evaluates on greens!(mc) (greens.jl:94-125): occupation
 * (occupation.jl:44-55), double occupancy and the interaction energy
 * (HubbardModel.jl:160-183), the z spin-density correlation
 * (spin_density.jl:182-227, tau = 0) reduced to S^z(q) for the caller's q,
 * and the equal-time G (constructors/greens.jl:39-40), binned as
 * BinningAnalysis' LogBinner does (generic.jl:57-69).  The values stay on the
 * device: no G download per measurement.  Measurements run inside dqmc_sweep,
 * dqmc_sweep_async and dqmc_pool_run whenever a chain completes a sweep whose
 * count (the chain's sweep counter after the sweep) is a multiple of
 * measure_rate. */
typedef struct {
    int32_t enable;        /* 1: measure; 0: stop measuring (accumulators are kept) */
    int32_t measure_rate;  /* >= 1 */
    int32_t greens_mean;   /* 1: also accumulate the physical G */
    int32_t reserved;
    int64_t sweep;         /* the chain's sweep counter now (mc.last_sweep); < 0 keeps it */
    double U;              /* the model's U (reference sign convention) */
    const double* q_cos;   /* n_sites values cos(q . r_i), or NULL: no S^z(q) */
    const double* q_sin;   /* n_sites values sin(q . r_i), or NULL (zeros) */
} dqmc_measure_config;

/* Scalars: 0 density per site, 1 double occupancy <n_up n_down> per site,
 * 2 interaction energy, 3 S^z(q) = (1/n) sum_ij cos(q.(r_i - r_j)) <m_z(i) m_z(j)>.
 * error[k]: standard error of the mean from the highest binning level with at
 * least 32 bins (level 0 when there is none; +inf below two measurements). */
typedef struct {
    int64_t count;
    double mean[4];
    double error[4];
    int32_t error_level[4];
} dqmc_observables;

/* chain = -1: every chain of the handle (q given: all chains need the same n_sites). */
int dqmc_set_measurements(dqmc_handle* h, int chain, const dqmc_measure_config* cfg);
/* Clear the accumulators (chain = -1: all). */
int dqmc_reset_measurements(dqmc_handle* h, int chain);
/* Means and binning errors; occupation (n_flavors*n, block-major, or NULL) and
 * greens (n_flavors*n*n physical G, or NULL) receive the means of those. */
int dqmc_get_measurements(dqmc_handle* h, int chain, dqmc_observables* out, double* occupation,
                          double* greens);

/* ---- checkerboard decomposition -------------------------------------------------
 * Replaces: DQMCParameters(checkerboard = true) (stack.jl:240-246,
 * linalg/checkerboard.jl:14-473): the hopping exponentials as products of
 * site-disjoint bond factors, applied in O(n^2) per factor instead of a dense
 * O(n^3) product.  Factor m (0 exp(-dtau T), 1 exp(+dtau T), 2 exp(-dtau T/2),
 * 3 exp(+dtau T/2)) is X = P_1 ... P_N D with N = n_parts; data holds, per
 * factor, D[n] then per part c[n] (cosh of the bond or 1), s[n] (sinh or 0)
 * and partner[n] (the bond's other site, -1: none).  The decomposition
 * (build_checkerboard's bond groups) is the host's: the Python package
 * builds it as the reference does.  n_parts < 0 returns to the dense
 * exponentials; chain = -1: all chains (same n_sites).  A chain with
 * checkerboard factors computes its slice products in FP64 on every
 * precision. */
int dqmc_set_checkerboard(dqmc_handle* h, int chain, int n_parts, const double* data);

/* ---- global updates and replica exchange -------------------------------------
 * Replaces: update(::GlobalFlip / ::GlobalShuffle, mc, model, field)
 * (global_updates.jl:188-203, 244-278: propose_conf!, propose_global_from_conf,
 * inv_det, accept_global!) for every chain of the handle in one launch.  The
 * chains must be between sweeps (current_slice 1, direction +1, as after
 * dqmc_initialize_run or a whole number of sweeps).  accepted (may be NULL)
 * receives n_chains 0/1 flags.  GlobalShuffle draws its permutation from the
 * chain's stream (Fisher-Yates, j = floor(w (i+1) / 2^64)). */
#define DQMC_GLOBAL_FLIP 0
#define DQMC_GLOBAL_SHUFFLE 1
int dqmc_global_update(dqmc_handle* h, int kind, int32_t* accepted);
/* Replaces: SimpleScheduler(LocalSweep(), GlobalFlip() or GlobalShuffle())
 * (scheduler.jl:258-289): from now on every dqmc_sweep call's sweeps run the
 * global update first, except the first sweep after this call.  kind = -1
 * turns it off.  chain = -1: all chains. */
int dqmc_set_global_schedule(dqmc_handle* h, int chain, int kind);
/* Replaces: update(::ReplicaExchange, ...) (parallel_updates.jl:116-150)
 * between chains of this handle (no MPI / Distributed.jl): partner[i] = j
 * pairs chain i with chain j (partner[j] = i; -1: not exchanging).  Each chain
 * weighs adopting its partner's configuration, the lower index's uniform
 * decides for the pair against the product of the two weights, and accepted
 * pairs swap configurations and rebuild their stacks.  Paired chains need the
 * same n_sites, n_flavors, slices and field kind (their U, mu, beta/dtau
 * hopping may differ).  accepted (may be NULL): n_chains 0/1 flags. */
int dqmc_replica_exchange(dqmc_handle* h, const int32_t* partner, int32_t* accepted);
/* accepted / proposed global and replica moves since creation */
int dqmc_get_global_stats(dqmc_handle* h, int chain, int64_t* accepted, int64_t* proposals);

/* ---- time-displaced measurements on the device ----------------------------------
 * Replaces: the TimeIntegral measurements of run! (generic.jl:337-366: the
 * unequal-time G(0,0), G(0,l), G(l,0), G(l,l) of the UnequalTimeStack for
 * l = 0..M with trapezoid weights) with the Wick kernels full_cdc_kernel
 * (charge_density.jl:65-112), full_sdc_x/y/z_kernel (spin_density.jl:100-227)
 * and pc_combined_kernel (pairing.jl:95-161), reduced by distance as
 * EachSitePairByDistance does (lattice_iterators.jl:160-260,
 * generic.jl:434-461, divided by the number of sites, :582-584), and the
 * susceptibilities charge_density_susceptibility,
 * spin_density_susceptibility (x, y, z at q), pairing_susceptibility (on
 * site, and with the extended-s and d-wave form factors of the caller's
 * bonds) and the uniform current_current_susceptibility of the caller's
 * current operator.  Everything is computed and log-binned on the device,
 * after every measure_rate-th sweep (the chain's sweep counter, shared with
 * the equal-time measurements) inside dqmc_sweep / dqmc_pool_run, or now
 * with dqmc_td_measure.  Real chains only. */
typedef struct {
    int32_t enable;          /* 1: measure; 0: stop measuring (accumulators are kept) */
    int32_t measure_rate;    /* >= 1 */
    int32_t n_slots;         /* P: length of each by-distance array (Ndir * B * B) */
    int32_t n_form[2];       /* bonds of the extended-s and d form factors (0: none) */
    int32_t n_current;       /* nonzero entries of the current operator (0: none) */
    double delta_tau;
    int64_t sweep;           /* the chain's sweep counter now; < 0 keeps it */
    const int32_t* pair_slot;     /* n_sites^2: by-distance slot of (src, trg) at src + n*trg */
    const double* q_cos;          /* n_sites cos(q . r_i) (NULL: q = 0) */
    const double* q_sin;          /* n_sites sin(q . r_i) (NULL: zeros) */
    const int32_t* form_sites;    /* 2 * (n_form[0] + n_form[1]) 0-based site pairs (a, b) */
    const double* form_values;    /* F_ab of those pairs */
    const int32_t* current_sites; /* 2 * n_current: (r, s) of the entries A[r, s] */
    const double* current_values; /* 2 * n_current: (re, im) of A[r, s] */
} dqmc_td_config;

/* Susceptibilities: 0 charge(q), 1 spin x(q), 2 spin y(q), 3 spin z(q),
 * 4 on-site s-wave pairing, 5 extended-s pairing, 6 d-wave pairing,
 * 7 uniform current (all (1/n) int_0^beta d tau); errors as for
 * dqmc_observables. */
typedef struct {
    int64_t count;
    double mean[8];
    double error[8];
    int32_t error_level[8];
} dqmc_td_observables;

/* A new configuration with other array sizes clears the accumulators. */
int dqmc_set_td_measurements(dqmc_handle* h, int chain, const dqmc_td_config* cfg);
/* One measurement of every chain that has them set up, now. */
int dqmc_td_measure(dqmc_handle* h);
/* mean / error (may be NULL): 5 * n_slots values, the by-distance arrays of
 * the charge, spin x, spin y, spin z and on-site pairing correlations, each
 * (Ndir, B, B) column-major. */
int dqmc_get_td_measurements(dqmc_handle* h, int chain, dqmc_td_observables* out, double* mean,
                             double* error);

/* ---- checkpoint state -----------------------------------------------------------
 * Replaces: the parts of a saved simulation that live with the chain
 * (flavors/DQMC/FileIO.jl:10-22: DQMCAnalysis, the scheduler, the
 * measurements' binners; field, RNG and parameters have their own calls):
 * the acceptance and DQMCAnalysis counters with their MagnitudeStats, the
 * near-tie counters, the global-update counts and schedule, the measurement
 * settings and the device measurement accumulators (log binners, occupation
 * and G sums), as one flat record of dqmc_checkpoint_doubles() doubles.
 * dqmc_set_checkpoint restores a record taken from a chain of the same
 * n_sites and n_flavors; the stack is not part of it (rebuild it with
 * dqmc_initialize_run, as the reference's resume! does). */
int64_t dqmc_checkpoint_doubles(dqmc_handle* h, int chain); /* < 0: bad chain */
int dqmc_get_checkpoint(dqmc_handle* h, int chain, double* out);
int dqmc_set_checkpoint(dqmc_handle* h, int chain, const double* in);

/* ---- pools: batched and served chains -------------------------------------
 * Replaces: a set of independent simulations driven one after another
 * (the reference's mpi_queue / pmap task farms, src/mpi.jl:26-168).  A pool
 * holds up to max_slots chains in one device arena of budget_bytes; chains
 * are admitted and released between launches while the others keep their
 * device-resident state (G, UDT stack, field), and one launch advances all of
 * them.  Per-chain calls (dqmc_set_hopping, dqmc_set_field,
 * dqmc_init_random_field, dqmc_get_greens, dqmc_get_stats, ...) take the slot
 * index as the chain index. */
int dqmc_pool_create(int device, int max_slots, int64_t budget_bytes, int precision,
                     dqmc_handle** out);
/* Admit a chain: DQMC_ERR_OOM when its workspace (dqmc_chain_bytes) does not
 * fit the free budget, DQMC_ERR_NOT_READY when no slot is free (retry after
 * a release).  The stack is built on the chain's first run. */
int dqmc_pool_admit(dqmc_handle* h, const dqmc_chain_config* cfg, int* slot);
int dqmc_pool_release(dqmc_handle* h, int slot);
/* Sweeps the slot may still run (one sweep = 2M slice visits). */
int dqmc_pool_set_quota(dqmc_handle* h, int slot, int64_t n_sweeps);
/* One time slice of every admitted chain: each runs slice visits until its
 * quota is used up or budget_us microseconds have passed (a chain finishes the
 * visit it is in); a chain past its budget keeps visiting while another chain
 * of the slice is not past its own (no SM idles waiting for a chain with long
 * visits).  use_graph = 1 replays the step (descriptor upload, launch,
 * download) as one captured CUDA graph. */
int dqmc_pool_run(dqmc_handle* h, int budget_us, int use_graph);
/* enable = 1: a two-flavour chain of the pool (at least 48 sites, real field,
 * dense hopping, no device measurements, global updates or replica exchange) runs its two
 * flavour blocks on two CTAs of a two-CTA cluster, i.e. on two SMs, which
 * roughly halves its time per sweep when SMs are free (served streams at light
 * load).  Results are bit-identical to the chain on one CTA.  Default 0. */
int dqmc_pool_set_flavour_split(dqmc_handle* h, int enable);
/* Test hook of the flavour split's failure path (no counterpart in the
 * reference).  The two CTAs of a split chain meet at rendezvous, each waiting
 * at most 2 s for its partner; after a time-out the chain's status becomes 9
 * (dqmc_pool_run returns DQMC_ERR_NUMERICAL naming the slot) and both CTAs
 * finish the launch without further waits.  from_epoch > 0 makes the second
 * CTA of the slot's chain stop announcing itself from that rendezvous on, so
 * that the wait runs out; 0 (the default) turns the hook off. */
int dqmc_pool_set_split_silence(dqmc_handle* h, int slot, int from_epoch);
int dqmc_pool_slot(dqmc_handle* h, int slot, int64_t* sweeps_done, int64_t* sweeps_left,
                   int32_t* active);
int64_t dqmc_pool_free_bytes(dqmc_handle* h);

/* ---- allocation-free Green's function ---------------------------------------
 * No counterpart in the reference: an addition for callers that cannot
 * allocate device memory when they need G -- hosts whose device memory budget
 * is owned by their own pool allocator, or latency-critical loops where
 * cudaMalloc / cudaFree would synchronise the device.  Computes the same
 * calculate_greens(mc, slice) as dqmc_calculate_greens, without a handle and
 * without allocating: all work matrices live in one fixed device array of the
 * library (about 0.53 MB per GPU, held until the process exits).
 *   d_hopping: device, 4 n x n FP64 blocks (the order of dqmc_set_hopping)
 *   d_conf:    device, n x M int8 field configuration
 *   d_out:     device, n_flavors*n*n FP64 result
 * Limit: n_flavors * n_sites^2 <= 8192; larger chains return DQMC_ERR_INVALID.
 * The work is queued on cuda_stream (NULL = legacy default stream); the result
 * is ready when that stream reaches it.  The first call on a device looks up
 * the array's address (make it before any stream capture) and keeps it for
 * the life of the process: do not call this entry point on a device after a
 * cudaDeviceReset (or any release and re-creation of its primary context) in
 * the same process.  All calls share the array: calls that overlap on the GPU
 * race and must be serialised. */
int dqmc_calculate_greens_noalloc(const dqmc_chain_config* cfg, const double* d_hopping,
                                  const int8_t* d_conf, int slice, int safe_mult, double* d_out,
                                  void* cuda_stream);

#ifdef __cplusplus
}
#endif
#endif
