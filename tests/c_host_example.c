/*
 * c_host_example.c -- a pure C host of libdqmc_gb300.so (no Python): the
 * pool calls of the serving loop for one attractive 4x4 Hubbard chain
 * (DensityHirschField, U = 4 in the reference's convention, beta = 2,
 * dtau = 0.1, safe_mult = 10), run for a few sweeps in 50 ms time slices.
 *
 * Exit codes: 0 done (prints sweeps, acceptance and the largest propagation
 * error), 3 no usable CUDA device (dqmc_pool_create's error is printed: the
 * library has no CPU fallback), 1 any other failure.
 *
 * Build: gcc -I include tests/c_host_example.c -L montecarlo.jl_gb300
 *        -ldqmc_gb300 -lm -o c_host_example
 */
#include <math.h>
#include <stdio.h>
#include <string.h>

#include "dqmc_gb300.h"

#define L 4
#define N (L * L)
#define SLICES 20

/* exp(s T) for the symmetric hopping matrix T by a Taylor series after
 * scaling by 2^-4 and squaring four times (||s T|| <= 0.4 here, so 30 terms
 * are exact to rounding). */
static void expm(double s, const double* T, double* out) {
    double A[N * N], term[N * N], tmp[N * N], R[N * N];
    const double scale = s / 16.0;
    for (int e = 0; e < N * N; ++e) {
        A[e] = scale * T[e];
        R[e] = (e % (N + 1) == 0) ? 1.0 : 0.0;
        term[e] = R[e];
    }
    for (int k = 1; k <= 30; ++k) {
        for (int j = 0; j < N; ++j)
            for (int i = 0; i < N; ++i) {
                double v = 0.0;
                for (int q = 0; q < N; ++q) v += term[q * N + i] * A[j * N + q];
                tmp[j * N + i] = v / k;
            }
        memcpy(term, tmp, sizeof term);
        for (int e = 0; e < N * N; ++e) R[e] += term[e];
    }
    for (int sq = 0; sq < 4; ++sq) {
        for (int j = 0; j < N; ++j)
            for (int i = 0; i < N; ++i) {
                double v = 0.0;
                for (int q = 0; q < N; ++q) v += R[q * N + i] * R[j * N + q];
                tmp[j * N + i] = v;
            }
        memcpy(R, tmp, sizeof tmp);
    }
    memcpy(out, R, sizeof R);
}

int main(void) {
    /* hopping matrix of the periodic L x L square lattice, t = 1, mu = 0:
     * T_ij = -t for nearest neighbours (site index x + L y) */
    static double T[N * N], eT2[N * N], eT2inv[N * N], eTh[N * N], eThinv[N * N];
    for (int y = 0; y < L; ++y)
        for (int x = 0; x < L; ++x) {
            const int i = x + L * y;
            const int nb[2] = {(x + 1) % L + L * y, x + L * ((y + 1) % L)};
            for (int d = 0; d < 2; ++d) {
                T[nb[d] * N + i] -= 1.0;
                T[i * N + nb[d]] -= 1.0;
            }
        }
    const double dtau = 0.1, U = 4.0;
    expm(-dtau, T, eT2);        /* exp(-dtau T) */
    expm(dtau, T, eT2inv);      /* exp(+dtau T) */
    expm(-0.5 * dtau, T, eTh);  /* exp(-dtau T / 2) */
    expm(0.5 * dtau, T, eThinv);

    dqmc_chain_config cfg;
    memset(&cfg, 0, sizeof cfg);
    cfg.n_sites = N;
    cfg.n_flavors = 1;
    cfg.slices = SLICES;
    cfg.safe_mult = 10;
    cfg.field = DQMC_FIELD_DENSITY_HIRSCH;
    cfg.check_propagation_error = 1;
    cfg.alpha = acosh(exp(0.5 * dtau * U)); /* DensityHirschField at U > 0 */
    cfg.seed = 11;

    dqmc_handle* pool = NULL;
    if (dqmc_pool_create(0, 8, 64LL << 20, DQMC_PREC_FP64, &pool) != DQMC_OK) {
        printf("dqmc_pool_create: %s\n", dqmc_last_error());
        return 3;
    }
    int slot = -1;
    if (dqmc_pool_admit(pool, &cfg, &slot) != DQMC_OK ||
        dqmc_set_hopping(pool, slot, eT2, eT2inv, eTh, eThinv) != DQMC_OK ||
        dqmc_init_random_field(pool, slot) != DQMC_OK || dqmc_pool_set_quota(pool, slot, 5) != DQMC_OK) {
        printf("admission: %s\n", dqmc_last_error());
        dqmc_destroy(pool);
        return 1;
    }
    int64_t done = 0, left = 1;
    for (int slices = 0; left > 0 && slices < 1000; ++slices) {
        if (dqmc_pool_run(pool, 50000, 1) != DQMC_OK ||
            dqmc_pool_slot(pool, slot, &done, &left, NULL) != DQMC_OK) {
            printf("run: %s\n", dqmc_last_error());
            dqmc_destroy(pool);
            return 1;
        }
    }
    dqmc_stats st;
    if (left != 0 || dqmc_get_stats(pool, slot, &st) != DQMC_OK || st.status != 0) {
        printf("unfinished or failed: %s\n", dqmc_last_error());
        dqmc_destroy(pool);
        return 1;
    }
    printf("sweeps %lld acceptance %.4f max_propagation_error %.3e\n", (long long)done,
           (double)st.accepted / (double)st.proposals, st.max_propagation_error);
    dqmc_pool_release(pool, slot);
    dqmc_destroy(pool);
    return 0;
}
