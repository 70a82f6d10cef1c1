/*
 * dqmc_oracle.h -- CPU FP64 restatement of the DQMC local-sweep path of
 * carstenbauer/MonteCarlo.jl.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: tests/, the smoke
 * test and bench.py's CPU-baseline / reference arm may load it.  The product
 * library (libdqmc_gb300.so) never links or calls it.
 *
 * Every function names the reference file:line it restates.  Matrices are
 * column-major FP64, n x n per flavour block; a chain with nf = 2 flavour
 * blocks (MagneticHirsch / MagneticGHQ fields) stores block b at offset b*n*n,
 * which is the reference's BlockDiagonal{Float64,2,Matrix}.  nf = 1 is the
 * reference's dense Matrix{Float64} path (Density fields).
 */
#ifndef DQMC_ORACLE_H
#define DQMC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* field kinds: same numbering as include/dqmc_gb300.h */
enum { OC_DENSITY_HIRSCH = 0, OC_MAGNETIC_HIRSCH = 1, OC_DENSITY_GHQ = 2, OC_MAGNETIC_GHQ = 3 };

typedef struct OcChain OcChain;

/* Philox4x32-10 (Salmon et al., SC'11); out[4] */
void oc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* 64-bit word of draw number `ctr` of stream `key` */
uint64_t oc_rng_word(uint64_t key, uint64_t ctr);
double oc_word_to_uniform(uint64_t w);

/* generate_chunks, stack.jl:154-158.  Writes first/last (1-based, inclusive)
 * and returns the number of chunks. */
int oc_generate_chunks(int length, int max_chunk, int* first, int* last);

/* Create a chain.  eT2 = exp(-dtau T), eT2inv = exp(+dtau T), eTh = exp(-dtau T/2),
 * eThinv = exp(+dtau T/2) (n x n, one block; stack.jl:235-239).  alpha is the
 * field's alpha (fields.jl:370-376, 419-425, 529-530, 599-600). */
OcChain* oc_create(int n, int nf, int M, int safe_mult, int kind, double alpha,
                   const double* eT2, const double* eT2inv, const double* eTh,
                   const double* eThinv, uint64_t seed, int check_propagation_error);
void oc_destroy(OcChain* c);

/* rand!(field), fields.jl:330 / :470, from the chain's Philox stream (draws 0..n*M-1) */
void oc_init_random_conf(OcChain* c);
void oc_set_conf(OcChain* c, const int8_t* conf);
void oc_get_conf(const OcChain* c, int8_t* conf);
void oc_set_rng(OcChain* c, uint64_t key, uint64_t counter);
uint64_t oc_get_rng_counter(const OcChain* c);

void oc_build_stack(OcChain* c);          /* stack.jl:257-281 */
void oc_reverse_build_stack(OcChain* c);  /* stack.jl:284-308 */
void oc_propagate(OcChain* c);            /* stack.jl:605-730 */
/* sweep_spatial, local_updates.jl:23-60: returns accepted count */
int oc_sweep_spatial(OcChain* c);
/* local_sweep, local_updates.jl:7-14: nsweeps full sweeps, returns accepted count */
long oc_local_sweeps(OcChain* c, int nsweeps);
/* initialize_run's stack part, DQMC.jl:178-179 */
void oc_initialize_run(OcChain* c);

/* wrap_greens!, stack.jl:594-603 applied to an nf*n*n buffer */
void oc_wrap_greens(OcChain* c, double* gf, int curr_slice, int direction);
/* calculate_greens(mc, slice, output), stack.jl:525-583 */
void oc_calculate_greens_at(OcChain* c, int slice, double* out, int safe_mult);
/* _greens!, greens.jl:114-125 (effective -> physical) */
void oc_greens_physical(OcChain* c, const double* src, double* out);

void oc_get_greens(const OcChain* c, double* out);
void oc_set_greens(OcChain* c, const double* in);
/* state: current_slice, current_range (1-based), direction, n_ranges */
void oc_get_state(const OcChain* c, int* state4);
/* which = 0 u_stack, 1 t_stack (nf*n*n), 2 d_stack (nf*n); idx 1-based */
void oc_get_stack(const OcChain* c, int which, int idx, double* out);
/* analysis: [max propagation error over all stabilisations, count > 1e-7,
 *            max reported (>1e-7), negative-p count, accepted total,
 *            near ties (drawn uniforms within 1e-12 of p), smallest |u - p|] */
void oc_get_analysis(const OcChain* c, double* out7);

/* checkerboard = true (stack.jl:240-246, linalg/checkerboard.jl): the four
 * hopping factors as np parts each, data = 4 x (D[n], np x (cosh-or-1[n],
 * sinh-or-0[n], partner[n] (-1: none))), factors in the order exp(-dtau T),
 * exp(+dtau T), exp(-dtau T/2), exp(+dtau T/2) */
void oc_set_checkerboard(OcChain* c, int np, const double* data);

/* global updates (global_updates.jl), at current_slice 1, direction +1:
 * kind 0 GlobalFlip, 1 GlobalShuffle; returns 1 when accepted */
int oc_global_update(OcChain* c, int kind);
/* propose_global_from_conf for `proposal` (n*M): det ratio, Delta E_boson;
 * the chain's configuration is left unchanged (G, stacks are not) */
double oc_global_detratio(OcChain* c, const int8_t* proposal, double* dEb);
/* ReplicaExchange's local half (parallel_updates.jl:116-150): weight of
 * adopting partner_conf and one uniform draw */
void oc_replica_weight(OcChain* c, const int8_t* partner_conf, double* weight, double* prob);
/* accept_global! with partner_conf */
void oc_replica_accept(OcChain* c, const int8_t* partner_conf);
/* propose_local + accept_local! of site i (0-based) to value x_new at the
 * current slice; returns p = exp(-Delta E) detratio */
double oc_local_move_to(OcChain* c, int i, int x_new);
void oc_get_global_stats(const OcChain* c, long* accepted, long* proposals);

/* calculate_greens(mc, k, l) (unequal_time_stack.jl:326-338, 536-697): the
 * effective unequal-time G(k, l) for npairs (k, l) pairs, 0 <= k, l <= M,
 * into out (npairs * nf*n*n) */
void oc_greens_kl(OcChain* c, const int* k, const int* l, int npairs, double* out);

/* stand-alone linalg kernels for unit tests */
/* udt_AVX_pivot!, UDT.jl:216-309 (one n x n block) */
void oc_udt_pivot(int n, double* U, double* D, double* input, int64_t* pivot,
                  double* temp, int apply_pivot);
/* rdivp!, real.jl:198-226 (block_form = 0) / blockdiagonal.jl:286-324 (block_form = 1) */
void oc_rdivp(int n, double* A, const double* T, double* O, const int64_t* pivot, int block_form);
/* calculate_greens_AVX!, stack.jl:442-496, on nf blocks */
void oc_calculate_greens_avx(int n, int nf, double* Ul, double* Dl, double* Tl, double* Ur,
                             double* Dr, double* Tr, double* G);
/* update_greens!, fields.jl:271-286, for a given Delta per block and site i (0-based):
 * computes R, invRDelta and the rank-1 update in place. */
void oc_update_greens(int n, int nf, double* G, const double* delta, int i);

/* many independent chains on `threads` host threads; used for the CPU baseline.
 * Returns wall seconds. */
double oc_run_chains_threaded(OcChain** chains, int nchains, int nsweeps, int threads);

#ifdef __cplusplus
}
#endif
#endif
