/*
 * dqmc_oracle.c -- CPU FP64 restatement of the DQMC local-sweep path of
 * carstenbauer/MonteCarlo.jl (TEST INFRASTRUCTURE ONLY; see dqmc_oracle.h).
 *
 * Reference files restated here (paths inside the reference project):
 *   src/flavors/DQMC/stack.jl, fields.jl, greens.jl,
 *   src/flavors/DQMC/linalg/{UDT,real,blockdiagonal,updates,fallbacks}.jl,
 *   src/flavors/DQMC/updates/local_updates.jl.
 * Loop orders of the matrix products are this file's own (the reference's
 * @turbo loops have no fixed summation order either); the sequence of
 * operations, chunking, pivoting and decisions follow the reference.
 *
 * The random stream is Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11),
 * which replaces Julia's global RNG: draw d of a chain with seed s is
 * philox(ctr = {d_lo, d_hi, 0, 0}, key = {s_lo, s_hi}); the 64-bit word is
 * (out0 << 32) | out1.  Draws are consumed in the reference's order.
 *
 * What pins this restatement: the reference's own known-answer recipes,
 * restated (the analytic U = 0 Green's function and the direct pivoted-QR
 * chain of test/testfunctions.jl, exact diagonalisation of test/ED on 2x2,
 * the global-update and rank-1 identities of test/updates.jl and
 * test/fields.jl), with the fixtures under tests/golden.  It is not pinned
 * against outputs of the reference itself: Julia is absent and the reference
 * ships no golden vectors.  Its accept/reject sequences follow this file's
 * Philox stream, so parity of decision sequences with the reference's Julia
 * RNG is unpinned.
 */
#include "dqmc_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* ------------------------------------------------------------------ RNG */

void oc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

uint64_t oc_rng_word(uint64_t key, uint64_t ctr) {
    uint32_t c[4] = {(uint32_t)ctr, (uint32_t)(ctr >> 32), 0u, 0u};
    uint32_t k[2] = {(uint32_t)key, (uint32_t)(key >> 32)};
    uint32_t o[4];
    oc_philox4x32_10(c, k, o);
    return ((uint64_t)o[0] << 32) | (uint64_t)o[1];
}

double oc_word_to_uniform(uint64_t w) { return (double)(w >> 11) * 0x1.0p-53; }

/* ------------------------------------------------------------------ chain */

struct OcChain {
    int n, nf, M, k, kind, nr, check_prop;
    int *rfirst, *rlast;          /* 1-based inclusive slice ranges (generate_chunks) */
    double alpha;
    double gam[4], eta[4];
    double *eT2, *eT2inv, *eTh, *eThinv;
    int8_t* conf;                 /* n x M, column-major (site fastest) */
    uint64_t key, ctr;
    double *u_stack, *t_stack, *d_stack;
    double *Ul, *Ur, *Tl, *Tr, *Dl, *Dr, *greens, *greens_temp, *tmp1, *tmp2, *curr_U, *eV;
    double *tempv, *scratch;
    int64_t* pivot;
    int current_slice, current_range, direction;
    double prop_err_all, prop_err_reported;
    long n_prop_err, n_neg_p, accepted;
    int cb_np;                    /* checkerboard parts per factor (0: dense exponentials) */
    double* cb;                   /* 4 factors x (D[n], parts x (c[n], s[n], partner[n])) */
    double *cbt0, *cbt1;          /* n x n scratch of the checkerboard products */
    int8_t* temp_conf;            /* temp_conf(field): the configuration before a global move */
    double* tempvf;               /* stack.tempvf: Dl of the current G during a global move */
    long g_accepted, g_proposals;
    long n_near_tie;              /* drawn uniforms within 1e-12 of p (local_updates.jl:53) */
    double min_tie_gap;           /* smallest |u - p| of a drawn uniform (+inf: none) */
};

int oc_generate_chunks(int length, int max_chunk, int* first, int* last) {
    /* N_chunks = cld(length, max_chunk); step = length / N_chunks;
       [round(Int,(i-1)*step)+1 : round(Int, i*step)]  (round half to even) */
    int nch = (length + max_chunk - 1) / max_chunk;
    double step = (double)length / (double)nch;
    for (int i = 1; i <= nch; ++i) {
        first[i - 1] = (int)nearbyint((double)(i - 1) * step) + 1;
        last[i - 1] = (int)nearbyint((double)i * step);
    }
    return nch;
}

#define NN(c) ((size_t)(c)->n * (size_t)(c)->n)
#define MATSZ(c) ((size_t)(c)->nf * NN(c))

static double* dalloc(size_t cnt) {
    double* p = (double*)calloc(cnt ? cnt : 1, sizeof(double));
    return p;
}

/* ---------------------------------------------------------- block algebra */

/* C = A * B, one n x n block, column-major (register-blocked, no aliasing). */
static void gemm_nn(int n, double* restrict C, const double* restrict A, const double* restrict B) {
    int j = 0;
    for (; j + 4 <= n; j += 4) {
        int i = 0;
        for (; i + 8 <= n; i += 8) {
            double acc[4][8];
            for (int q = 0; q < 4; ++q)
                for (int r = 0; r < 8; ++r) acc[q][r] = 0.0;
            for (int k = 0; k < n; ++k) {
                const double* a = A + (size_t)k * n + i;
                for (int q = 0; q < 4; ++q) {
                    double b = B[(size_t)(j + q) * n + k];
                    for (int r = 0; r < 8; ++r) acc[q][r] += a[r] * b;
                }
            }
            for (int q = 0; q < 4; ++q)
                for (int r = 0; r < 8; ++r) C[(size_t)(j + q) * n + i + r] = acc[q][r];
        }
        for (; i < n; ++i) {
            for (int q = 0; q < 4; ++q) {
                double s = 0.0;
                for (int k = 0; k < n; ++k) s += A[(size_t)k * n + i] * B[(size_t)(j + q) * n + k];
                C[(size_t)(j + q) * n + i] = s;
            }
        }
    }
    for (; j < n; ++j) {
        for (int i = 0; i < n; ++i) C[(size_t)j * n + i] = 0.0;
        for (int k = 0; k < n; ++k) {
            double b = B[(size_t)j * n + k];
            const double* a = A + (size_t)k * n;
            double* cc = C + (size_t)j * n;
            for (int i = 0; i < n; ++i) cc[i] += a[i] * b;
        }
    }
}

static void transpose(int n, double* restrict out, const double* restrict A) {
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) out[(size_t)i * n + j] = A[(size_t)j * n + i];
}

/* C = A^T * B  (real.jl:82-91, vmul!(C, adjoint(A), B)) */
static void gemm_tn(int n, double* C, const double* A, const double* B, double* scratch) {
    transpose(n, scratch, A);
    gemm_nn(n, C, scratch, B);
}
/* C = A * B^T  (real.jl:72-81, vmul!(C, A, adjoint(B))) */
static void gemm_nt(int n, double* C, const double* A, const double* B, double* scratch) {
    transpose(n, scratch, B);
    gemm_nn(n, C, A, scratch);
}
/* C = Diagonal(d) * B  (real.jl:27-37) */
static void diag_left(int n, double* C, const double* d, const double* B) {
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) C[(size_t)j * n + i] = d[i] * B[(size_t)j * n + i];
}
/* C = A * Diagonal(d)  (real.jl:16-26) */
static void diag_right(int n, double* C, const double* A, const double* d) {
    for (int j = 0; j < n; ++j) {
        double dj = d[j];
        for (int i = 0; i < n; ++i) C[(size_t)j * n + i] = A[(size_t)j * n + i] * dj;
    }
}
static void set_identity(int n, double* A) {
    memset(A, 0, sizeof(double) * (size_t)n * n);
    for (int i = 0; i < n; ++i) A[(size_t)i * n + i] = 1.0;
}

/* ------------------------------------------------------------------- UDT */

/* indmaxcolumn, UDT.jl:175-192 (0-based j) */
static int indmaxcolumn(int n, const double* A, int j, double* maxval) {
    double sq = 0.0;
    for (int k = j; k < n; ++k) sq += A[(size_t)j * n + k] * A[(size_t)j * n + k];
    int ii = j;
    for (int i = j + 1; i < n; ++i) {
        double mi = 0.0;
        const double* col = A + (size_t)i * n;
        for (int k = j; k < n; ++k) mi += col[k] * col[k];
        if (fabs(mi) > sq) { sq = mi; ii = i; }
    }
    *maxval = sq;
    return ii;
}

void oc_udt_pivot(int n, double* U, double* D, double* input, int64_t* pivot, double* temp,
                  int apply_pivot) {
    for (int i = 0; i < n; ++i) pivot[i] = i + 1;
    /* QR with column pivoting, UDT.jl:236-268 */
    for (int j = 0; j < n; ++j) {
        double normu;
        int jm = indmaxcolumn(n, input, j, &normu);
        if (jm != j) {
            int64_t tp = pivot[jm]; pivot[jm] = pivot[j]; pivot[j] = tp;
            double* a = input + (size_t)jm * n;
            double* b = input + (size_t)j * n;
            for (int i = 0; i < n; ++i) { double t = a[i]; a[i] = b[i]; b[i] = t; }
        }
        /* reflector!, UDT.jl:157-172 */
        double* x = input + (size_t)j * n;
        double tau;
        double xi1 = x[j];
        if (normu == 0.0) {
            tau = 0.0;
        } else {
            double nrm = sqrt(normu);
            double nu = copysign(nrm, xi1);
            xi1 += nu;
            x[j] = -nu;
            for (int i = j + 1; i < n; ++i) x[i] /= xi1;
            tau = xi1 / nu;
        }
        temp[j] = tau;
        /* reflectorApply!(M, tau, k, n), UDT.jl:53-70 */
        for (int jj = j + 1; jj < n; ++jj) {
            double* col = input + (size_t)jj * n;
            double vAj = col[j];
            for (int i = j + 1; i < n; ++i) vAj += x[i] * col[i];
            vAj = tau * vAj;
            col[j] -= vAj;
            for (int i = j + 1; i < n; ++i) col[i] -= x[i] * vAj;
        }
    }
    /* Calculate Q, UDT.jl:272-289 */
    set_identity(n, U);
    U[(size_t)(n - 1) * n + (n - 1)] -= temp[n - 1];
    for (int k = n - 2; k >= 0; --k) {
        const double* v = input + (size_t)k * n;
        for (int j = k; j < n; ++j) {
            double* u = U + (size_t)j * n;
            double vBj = u[k];
            for (int i = k + 1; i < n; ++i) vBj += v[i] * u[i];
            vBj = temp[k] * vBj;
            u[k] -= vBj;
            for (int i = k + 1; i < n; ++i) u[i] -= v[i] * vBj;
        }
    }
    /* D, UDT.jl:293-301 */
    for (int i = 0; i < n; ++i) {
        double xx = fabs(input[(size_t)i * n + i]);
        D[i] = (xx == 0.0) ? 1.0 : xx;
    }
    /* _apply_pivot!, UDT.jl:311-334 */
    if (apply_pivot) {
        for (int i = 0; i < n; ++i) {
            double d = 1.0 / D[i];
            for (int j = 0; j < i; ++j) temp[pivot[j] - 1] = 0.0;
            for (int j = i; j < n; ++j) temp[pivot[j] - 1] = d * input[(size_t)j * n + i];
            for (int j = 0; j < n; ++j) input[(size_t)j * n + i] = temp[j];
        }
    } else {
        for (int i = 0; i < n; ++i) {
            double d = 1.0 / D[i];
            for (int j = i; j < n; ++j) input[(size_t)j * n + i] = d * input[(size_t)j * n + i];
        }
    }
}

/* rdivp!: A <- A * T^{-1} (pivoted), real.jl:198-226 / blockdiagonal.jl:286-324 */
void oc_rdivp(int n, double* A, const double* T, double* O, const int64_t* pivot, int block_form) {
    for (int j = 0; j < n; ++j) {
        const double* src = A + (size_t)(pivot[j] - 1) * n;
        double* dst = O + (size_t)j * n;
        for (int i = 0; i < n; ++i) dst[i] = src[i];
    }
    for (int j = 0; j < n; ++j) {
        double tjj = T[(size_t)j * n + j];
        double inv = 1.0 / tjj;
        double* aj = A + (size_t)j * n;
        const double* oj = O + (size_t)j * n;
        for (int i = 0; i < n; ++i) aj[i] = oj[i];
        for (int k = 0; k < j; ++k) {
            double tkj = T[(size_t)j * n + k];
            const double* ak = A + (size_t)k * n;
            for (int i = 0; i < n; ++i) aj[i] -= ak[i] * tkj;
        }
        if (block_form)
            for (int i = 0; i < n; ++i) aj[i] = aj[i] * inv;
        else
            for (int i = 0; i < n; ++i) aj[i] = aj[i] / tjj;
    }
}

/* calculate_greens_AVX!, stack.jl:442-496; all operations act per flavour block.
 * finish = 0 stops after the second UDT: calculate_inv_greens_udt
 * (global_updates.jl:26-49), which leaves det(G) = 1/prod(Dr) up to phases. */
static void calc_greens_blocks_part(int n, int nf, double* Ul, double* Dl, double* Tl, double* Ur,
                                    double* Dr, double* Tr, double* G, int64_t* pivot, double* temp,
                                    double* scratch, int finish) {
    size_t nn = (size_t)n * n;
    for (int b = 0; b < nf; ++b) {
        double *ul = Ul + b * nn, *tl = Tl + b * nn, *ur = Ur + b * nn, *tr = Tr + b * nn,
               *g = G + b * nn;
        double *dl = Dl + b * n, *dr = Dr + b * n;
        int64_t* pv = pivot + b * n;
        double* tv = temp + b * n;
        gemm_nt(n, g, tl, tr, scratch);          /* G = Tl * Tr'          */
        diag_right(n, tr, g, dr);                /* Tr = G * Dr           */
        diag_left(n, g, dl, tr);                 /* G = Dl * Tr           */
        oc_udt_pivot(n, tr, dr, g, pv, tv, 0);   /* Tr, Dr, G = udt(G)    */
        gemm_nn(n, tl, ul, tr);                  /* Tl = Ul * Tr          */
        oc_rdivp(n, ur, g, ul, pv, nf > 1);      /* Ur = Ur * G^-1        */
        gemm_tn(n, tr, tl, ur, scratch);         /* Tr = Tl' * Ur         */
        for (int i = 0; i < n; ++i) tr[(size_t)i * n + i] += dr[i]; /* rvadd! */
        oc_udt_pivot(n, ul, dr, tr, pv, tv, 0);  /* Ul, Dr, Tr = udt(Tr)  */
        if (!finish) continue;
        oc_rdivp(n, ur, tr, g, pv, nf > 1);      /* Ur = Ur * Tr^-1       */
        gemm_nn(n, tr, tl, ul);                  /* Tr = Tl * Ul          */
        for (int i = 0; i < n; ++i) dl[i] = 1.0 / dr[i]; /* vinv!        */
        diag_right(n, ul, ur, dl);               /* Ul = Ur * Dl          */
        gemm_nt(n, g, ul, tr, scratch);          /* G = Ul * Tr'          */
    }
}

static void calc_greens_blocks(int n, int nf, double* Ul, double* Dl, double* Tl, double* Ur,
                               double* Dr, double* Tr, double* G, int64_t* pivot, double* temp,
                               double* scratch) {
    calc_greens_blocks_part(n, nf, Ul, Dl, Tl, Ur, Dr, Tr, G, pivot, temp, scratch, 1);
}

void oc_calculate_greens_avx(int n, int nf, double* Ul, double* Dl, double* Tl, double* Ur,
                             double* Dr, double* Tr, double* G) {
    int64_t* pivot = (int64_t*)calloc((size_t)nf * n, sizeof(int64_t));
    double* temp = dalloc((size_t)nf * n);
    double* scratch = dalloc((size_t)n * n);
    calc_greens_blocks(n, nf, Ul, Dl, Tl, Ur, Dr, Tr, G, pivot, temp, scratch);
    free(pivot); free(temp); free(scratch);
}

/* ------------------------------------------------------------ chain setup */

OcChain* oc_create(int n, int nf, int M, int safe_mult, int kind, double alpha,
                   const double* eT2, const double* eT2inv, const double* eTh,
                   const double* eThinv, uint64_t seed, int check_propagation_error) {
    OcChain* c = (OcChain*)calloc(1, sizeof(OcChain));
    c->min_tie_gap = INFINITY;
    c->n = n; c->nf = nf; c->M = M; c->k = safe_mult; c->kind = kind; c->alpha = alpha;
    c->check_prop = check_propagation_error;
    int maxch = (M + safe_mult - 1) / safe_mult;
    c->rfirst = (int*)calloc((size_t)maxch, sizeof(int));
    c->rlast = (int*)calloc((size_t)maxch, sizeof(int));
    c->nr = oc_generate_chunks(M, safe_mult, c->rfirst, c->rlast);
    /* GHQ tables, fields.jl:531-534 / 601-604 */
    double s6 = sqrt(6.0);
    c->gam[0] = 1.0 - s6 / 3.0; c->gam[1] = 1.0 + s6 / 3.0;
    c->gam[2] = 1.0 + s6 / 3.0; c->gam[3] = 1.0 - s6 / 3.0;
    c->eta[0] = -sqrt(6.0 + 2.0 * s6); c->eta[1] = -sqrt(6.0 - 2.0 * s6);
    c->eta[2] = sqrt(6.0 - 2.0 * s6);  c->eta[3] = sqrt(6.0 + 2.0 * s6);
    size_t nn = (size_t)n * n;
    c->eT2 = dalloc(nn); c->eT2inv = dalloc(nn); c->eTh = dalloc(nn); c->eThinv = dalloc(nn);
    memcpy(c->eT2, eT2, nn * sizeof(double));
    memcpy(c->eT2inv, eT2inv, nn * sizeof(double));
    memcpy(c->eTh, eTh, nn * sizeof(double));
    memcpy(c->eThinv, eThinv, nn * sizeof(double));
    c->conf = (int8_t*)calloc((size_t)n * M, 1);
    c->temp_conf = (int8_t*)calloc((size_t)n * M, 1);
    c->tempvf = dalloc((size_t)nf * n);
    c->key = seed; c->ctr = 0;
    size_t ms = (size_t)nf * nn;
    c->u_stack = dalloc(ms * (c->nr + 1));
    c->t_stack = dalloc(ms * (c->nr + 1));
    c->d_stack = dalloc((size_t)nf * n * (c->nr + 1));
    c->Ul = dalloc(ms); c->Ur = dalloc(ms); c->Tl = dalloc(ms); c->Tr = dalloc(ms);
    c->Dl = dalloc((size_t)nf * n); c->Dr = dalloc((size_t)nf * n);
    c->greens = dalloc(ms); c->greens_temp = dalloc(ms); c->tmp1 = dalloc(ms); c->tmp2 = dalloc(ms);
    c->curr_U = dalloc(ms);
    c->eV = dalloc((size_t)nf * n);
    c->tempv = dalloc((size_t)nf * n);
    c->scratch = dalloc(nn);
    c->pivot = (int64_t*)calloc((size_t)nf * n, sizeof(int64_t));
    /* initialize_stack, stack.jl:187-192 */
    for (int b = 0; b < nf; ++b) {
        set_identity(n, c->Ul + b * nn); set_identity(n, c->Ur + b * nn);
        set_identity(n, c->Tl + b * nn); set_identity(n, c->Tr + b * nn);
    }
    for (int i = 0; i < nf * n; ++i) { c->Dl[i] = 1.0; c->Dr[i] = 1.0; }
    return c;
}

void oc_destroy(OcChain* c) {
    if (!c) return;
    free(c->rfirst); free(c->rlast);
    free(c->eT2); free(c->eT2inv); free(c->eTh); free(c->eThinv); free(c->conf);
    free(c->temp_conf); free(c->tempvf);
    free(c->cb); free(c->cbt0); free(c->cbt1);
    free(c->u_stack); free(c->t_stack); free(c->d_stack);
    free(c->Ul); free(c->Ur); free(c->Tl); free(c->Tr); free(c->Dl); free(c->Dr);
    free(c->greens); free(c->greens_temp); free(c->tmp1); free(c->tmp2); free(c->curr_U);
    free(c->eV); free(c->tempv); free(c->scratch); free(c->pivot);
    free(c);
}

static inline uint64_t next_word(OcChain* c) { return oc_rng_word(c->key, c->ctr++); }

void oc_init_random_conf(OcChain* c) {
    size_t cnt = (size_t)c->n * c->M;
    int ghq = (c->kind == OC_DENSITY_GHQ || c->kind == OC_MAGNETIC_GHQ);
    for (size_t i = 0; i < cnt; ++i) {
        uint64_t w = next_word(c);
        if (ghq) c->conf[i] = (int8_t)(1 + (int)(w >> 62));
        else c->conf[i] = (w >> 63) ? (int8_t)1 : (int8_t)-1;
    }
}
void oc_set_conf(OcChain* c, const int8_t* conf) { memcpy(c->conf, conf, (size_t)c->n * c->M); }
void oc_get_conf(const OcChain* c, int8_t* conf) { memcpy(conf, c->conf, (size_t)c->n * c->M); }
void oc_set_rng(OcChain* c, uint64_t key, uint64_t counter) { c->key = key; c->ctr = counter; }
uint64_t oc_get_rng_counter(const OcChain* c) { return c->ctr; }

/* interaction_matrix_exp!, fields.jl:380-386, 429-438, 548-560, 618-624 */
static void interaction_matrix_exp(OcChain* c, int slice, double power, double* eV) {
    int n = c->n;
    const int8_t* s = c->conf + (size_t)(slice - 1) * n;
    double a = c->alpha;
    switch (c->kind) {
    case OC_DENSITY_HIRSCH:
        for (int i = 0; i < n; ++i) eV[i] = exp(power * a * (double)s[i]);
        break;
    case OC_MAGNETIC_HIRSCH:
        for (int i = 0; i < n; ++i) eV[i] = exp(power * a * (double)s[i]);
        for (int i = 0; i < n; ++i) eV[i + n] = exp(-power * a * (double)s[i]);
        break;
    case OC_DENSITY_GHQ:
        for (int i = 0; i < n; ++i) eV[i] = exp(+power * a * c->eta[s[i] - 1]);
        break;
    default: /* OC_MAGNETIC_GHQ */
        for (int i = 0; i < n; ++i) eV[i] = exp(+power * a * c->eta[s[i] - 1]);
        for (int i = 0; i < n; ++i) eV[i + n] = exp(-power * a * c->eta[s[i] - 1]);
        break;
    }
}

/* ---- checkerboard products (linalg/checkerboard.jl:272-473) ----------------
 * Factor m (0 exp(-dtau T), 1 exp(+dtau T), 2 exp(-dtau T/2), 3 exp(+dtau T/2))
 * is X = P_1 ... P_N D; mode 0: X A, 1: A X, 2: X^T A = D P_N ... P_1 A.  One
 * pass per part: row (or column) i takes c_i times itself plus s_i times its
 * partner's, D fused into the first (mode 0) or last (modes 1, 2) pass. */
void oc_set_checkerboard(OcChain* c, int np, const double* data) {
    size_t per = (size_t)c->n * (1 + 3 * (size_t)np);
    free(c->cb);
    c->cb_np = np;
    c->cb = dalloc(4 * per);
    memcpy(c->cb, data, 4 * per * sizeof(double));
    if (!c->cbt0) { c->cbt0 = dalloc(NN(c)); c->cbt1 = dalloc(NN(c)); }
}
static void cb_apply(OcChain* c, int m, int mode, double* out, const double* in) {
    const int n = c->n, np = c->cb_np;
    const double* D = c->cb + (size_t)m * n * (1 + 3 * (size_t)np);
    const double* P = D + n;
    const double* src = in;
    double* bufs[2] = {c->cbt0, c->cbt1};
    if (np == 0) {
        for (int k = 0; k < n; ++k)
            for (int i = 0; i < n; ++i)
                c->cbt0[i + (size_t)k * n] = (mode == 1) ? in[i + (size_t)k * n] * D[k]
                                                         : D[i] * in[i + (size_t)k * n];
        memcpy(out, c->cbt0, NN(c) * sizeof(double));
        return;
    }
    for (int step = 0; step < np; ++step) {
        /* mode 0 applies P_N first; modes 1, 2 apply P_1 first */
        const int part = (mode == 0) ? np - 1 - step : step;
        const double* cc = P + (size_t)part * 3 * n;
        const double* ss = cc + n;
        const double* pt = ss + n;
        const int first = (step == 0), last = (step == np - 1);
        double* dst = bufs[step & 1];
        for (int k = 0; k < n; ++k)
            for (int i = 0; i < n; ++i) {
                double y;
                if (mode == 1) {  /* columns */
                    const int q = (int)pt[k];
                    const double v = src[i + (size_t)k * n];
                    y = (q >= 0) ? fma(src[i + (size_t)q * n], ss[k], v * cc[k]) : v;
                    if (last) y = y * D[k];
                } else {          /* rows */
                    const int q = (int)pt[i];
                    double v = src[i + (size_t)k * n];
                    double w = (q >= 0) ? src[q + (size_t)k * n] : 0.0;
                    if (mode == 0 && first) {
                        v = D[i] * v;
                        if (q >= 0) w = D[q] * w;
                    }
                    y = (q >= 0) ? fma(ss[i], w, cc[i] * v) : v;
                    if (mode == 2 && last) y = D[i] * y;
                }
                dst[i + (size_t)k * n] = y;
            }
        src = dst;
    }
    memcpy(out, src, NN(c) * sizeof(double));
}

/* slice matrices, stack.jl:319-367 (hopping exponentials are Hermitian-wrapped,
 * so vmul! multiplies with the transposed data: fallbacks.jl:67-68); with a
 * checkerboard decomposition the exponentials are applied as its products */
static void mult_slice_left(OcChain* c, int slice, double* M) {
    int n = c->n; size_t nn = NN(c);
    interaction_matrix_exp(c, slice, 1.0, c->eV);
    for (int b = 0; b < c->nf; ++b) {
        diag_left(n, c->tmp1 + b * nn, c->eV + b * n, M + b * nn);
        if (c->cb) cb_apply(c, 0, 0, M + b * nn, c->tmp1 + b * nn);
        else gemm_tn(n, M + b * nn, c->eT2, c->tmp1 + b * nn, c->scratch);
    }
}
static void mult_slice_right(OcChain* c, int slice, double* M) {
    int n = c->n; size_t nn = NN(c);
    interaction_matrix_exp(c, slice, 1.0, c->eV);
    for (int b = 0; b < c->nf; ++b) {
        if (c->cb) cb_apply(c, 0, 1, c->tmp1 + b * nn, M + b * nn);
        else gemm_nt(n, c->tmp1 + b * nn, M + b * nn, c->eT2, c->scratch);
        diag_right(n, M + b * nn, c->tmp1 + b * nn, c->eV + b * n);
    }
}
static void mult_slice_inv_right(OcChain* c, int slice, double* M) {
    int n = c->n; size_t nn = NN(c);
    interaction_matrix_exp(c, slice, -1.0, c->eV);
    for (int b = 0; b < c->nf; ++b) {
        diag_right(n, c->tmp1 + b * nn, M + b * nn, c->eV + b * n);
        if (c->cb) cb_apply(c, 1, 1, M + b * nn, c->tmp1 + b * nn);
        else gemm_nt(n, M + b * nn, c->tmp1 + b * nn, c->eT2inv, c->scratch);
    }
}
static void mult_slice_inv_left(OcChain* c, int slice, double* M) {
    int n = c->n; size_t nn = NN(c);
    interaction_matrix_exp(c, slice, -1.0, c->eV);
    for (int b = 0; b < c->nf; ++b) {
        if (c->cb) cb_apply(c, 1, 0, c->tmp1 + b * nn, M + b * nn);
        else gemm_tn(n, c->tmp1 + b * nn, c->eT2inv, M + b * nn, c->scratch);
        diag_left(n, M + b * nn, c->eV + b * n, c->tmp1 + b * nn);
    }
}
static void mult_daggered_slice_left(OcChain* c, int slice, double* M) {
    int n = c->n; size_t nn = NN(c);
    interaction_matrix_exp(c, slice, 1.0, c->eV);
    for (int b = 0; b < c->nf; ++b) {
        if (c->cb) cb_apply(c, 0, 2, c->tmp1 + b * nn, M + b * nn);
        else gemm_tn(n, c->tmp1 + b * nn, c->eT2, M + b * nn, c->scratch);
        diag_left(n, M + b * nn, c->eV + b * n, c->tmp1 + b * nn);
    }
}

static double* ustk(OcChain* c, int idx) { return c->u_stack + (size_t)(idx - 1) * MATSZ(c); }
static double* tstk(OcChain* c, int idx) { return c->t_stack + (size_t)(idx - 1) * MATSZ(c); }
static double* dstk(OcChain* c, int idx) { return c->d_stack + (size_t)(idx - 1) * c->nf * c->n; }

static void mat_identity(OcChain* c, double* A) {
    for (int b = 0; b < c->nf; ++b) set_identity(c->n, A + b * NN(c));
}
static void vec_ones(OcChain* c, double* d) {
    for (int i = 0; i < c->nf * c->n; ++i) d[i] = 1.0;
}
static void mat_copy(OcChain* c, double* dst, const double* src) {
    memcpy(dst, src, MATSZ(c) * sizeof(double));
}
static void vec_copy(OcChain* c, double* dst, const double* src) {
    memcpy(dst, src, (size_t)c->nf * c->n * sizeof(double));
}

/* udt_AVX_pivot! on all blocks (blockdiagonal.jl:352-370) */
static void udt_blocks(OcChain* c, double* U, double* D, double* input, int apply) {
    for (int b = 0; b < c->nf; ++b)
        oc_udt_pivot(c->n, U + b * NN(c), D + b * c->n, input + b * NN(c), c->pivot + b * c->n,
                     c->tempv + b * c->n, apply);
}
static void gemm_blocks(OcChain* c, double* C, const double* A, const double* B) {
    for (int b = 0; b < c->nf; ++b) gemm_nn(c->n, C + b * NN(c), A + b * NN(c), B + b * NN(c));
}
static void diag_right_blocks(OcChain* c, double* C, const double* A, const double* d) {
    for (int b = 0; b < c->nf; ++b) diag_right(c->n, C + b * NN(c), A + b * NN(c), d + b * c->n);
}

/* add_slice_sequence_left, stack.jl:377-393 */
static void add_slice_sequence_left(OcChain* c, int idx) {
    mat_copy(c, c->curr_U, ustk(c, idx));
    for (int s = c->rfirst[idx - 1]; s <= c->rlast[idx - 1]; ++s) mult_slice_left(c, s, c->curr_U);
    diag_right_blocks(c, c->tmp1, c->curr_U, dstk(c, idx));
    udt_blocks(c, ustk(c, idx + 1), dstk(c, idx + 1), c->tmp1, 1);
    gemm_blocks(c, tstk(c, idx + 1), c->tmp1, tstk(c, idx));
}
/* add_slice_sequence_right, stack.jl:402-416 */
static void add_slice_sequence_right(OcChain* c, int idx) {
    mat_copy(c, c->curr_U, ustk(c, idx + 1));
    for (int s = c->rlast[idx - 1]; s >= c->rfirst[idx - 1]; --s)
        mult_daggered_slice_left(c, s, c->curr_U);
    diag_right_blocks(c, c->tmp1, c->curr_U, dstk(c, idx + 1));
    udt_blocks(c, ustk(c, idx), dstk(c, idx), c->tmp1, 1);
    gemm_blocks(c, tstk(c, idx), c->tmp1, tstk(c, idx + 1));
}

/* calculate_greens(mc), stack.jl:509-516 */
static void calculate_greens(OcChain* c, double* out) {
    calc_greens_blocks(c->n, c->nf, c->Ul, c->Dl, c->Tl, c->Ur, c->Dr, c->Tr, out, c->pivot,
                       c->tempv, c->scratch);
}

void oc_build_stack(OcChain* c) {
    mat_identity(c, ustk(c, 1)); vec_ones(c, dstk(c, 1)); mat_identity(c, tstk(c, 1));
    for (int i = 1; i <= c->nr; ++i) add_slice_sequence_left(c, i);
    c->current_slice = c->M + 1;
    c->current_range = c->nr;
    c->direction = -1;
    mat_copy(c, c->Ul, ustk(c, c->nr + 1)); vec_copy(c, c->Dl, dstk(c, c->nr + 1));
    mat_copy(c, c->Tl, tstk(c, c->nr + 1));
    mat_identity(c, c->Ur); vec_ones(c, c->Dr); mat_identity(c, c->Tr);
    calculate_greens(c, c->greens);
}

void oc_reverse_build_stack(OcChain* c) {
    mat_identity(c, ustk(c, c->nr + 1)); vec_ones(c, dstk(c, c->nr + 1));
    mat_identity(c, tstk(c, c->nr + 1));
    for (int i = c->nr; i >= 1; --i) add_slice_sequence_right(c, i);
    c->current_slice = 0;
    c->current_range = 1;
    c->direction = 1;
    mat_identity(c, c->Ul); vec_ones(c, c->Dl); mat_identity(c, c->Tl);
    mat_copy(c, c->Ur, ustk(c, 1)); vec_copy(c, c->Dr, dstk(c, 1)); mat_copy(c, c->Tr, tstk(c, 1));
    calculate_greens(c, c->greens);
}

void oc_wrap_greens(OcChain* c, double* gf, int curr_slice, int direction) {
    if (direction == -1) {
        mult_slice_inv_left(c, curr_slice - 1, gf);
        mult_slice_right(c, curr_slice - 1, gf);
    } else {
        mult_slice_left(c, curr_slice, gf);
        mult_slice_inv_right(c, curr_slice, gf);
    }
}

static void record_prop_error(OcChain* c) {
    double mx = 0.0;
    size_t ms = MATSZ(c);
    for (size_t i = 0; i < ms; ++i) {
        double d = fabs(c->greens_temp[i] - c->greens[i]);
        if (d > mx || d != d) mx = d;
    }
    if (mx > c->prop_err_all || mx != mx) c->prop_err_all = mx;
    if (mx > 1e-7) {
        c->n_prop_err++;
        if (mx > c->prop_err_reported) c->prop_err_reported = mx;
    }
}

void oc_propagate(OcChain* c) {
    c->current_slice += c->direction;
    if (c->direction == 1) {
        if (c->current_slice == 1) {
            mat_identity(c, ustk(c, 1)); vec_ones(c, dstk(c, 1)); mat_identity(c, tstk(c, 1));
        } else if (c->current_slice - 1 == c->rlast[c->current_range - 1]) {
            int idx = c->current_range;
            mat_copy(c, c->Ur, ustk(c, idx + 1)); vec_copy(c, c->Dr, dstk(c, idx + 1));
            mat_copy(c, c->Tr, tstk(c, idx + 1));
            add_slice_sequence_left(c, idx);
            mat_copy(c, c->Ul, ustk(c, idx + 1)); vec_copy(c, c->Dl, dstk(c, idx + 1));
            mat_copy(c, c->Tl, tstk(c, idx + 1));
            if (c->check_prop) mat_copy(c, c->greens_temp, c->greens);
            oc_wrap_greens(c, c->greens_temp, c->current_slice - 1, 1);
            calculate_greens(c, c->greens);
            if (c->check_prop) record_prop_error(c);
            if (c->current_range == c->nr) {
                c->direction = -1;
                oc_propagate(c);
            } else {
                c->current_range += 1;
            }
        } else {
            oc_wrap_greens(c, c->greens, c->current_slice - 1, 1);
        }
    } else {
        if (c->current_slice == c->M) {
            mat_identity(c, ustk(c, c->nr + 1)); vec_ones(c, dstk(c, c->nr + 1));
            mat_identity(c, tstk(c, c->nr + 1));
            oc_wrap_greens(c, c->greens, c->current_slice + 1, -1);
        } else if (c->current_slice + 1 == c->rfirst[c->current_range - 1]) {
            int idx = c->current_range;
            mat_copy(c, c->Ul, ustk(c, idx)); vec_copy(c, c->Dl, dstk(c, idx));
            mat_copy(c, c->Tl, tstk(c, idx));
            add_slice_sequence_right(c, idx);
            mat_copy(c, c->Ur, ustk(c, idx)); vec_copy(c, c->Dr, dstk(c, idx));
            mat_copy(c, c->Tr, tstk(c, idx));
            if (c->check_prop) mat_copy(c, c->greens_temp, c->greens);
            calculate_greens(c, c->greens);
            if (c->check_prop) record_prop_error(c);
            if (c->current_range == 1) {
                c->direction = 1;
                oc_propagate(c);
            } else {
                oc_wrap_greens(c, c->greens, c->current_slice + 1, -1);
                c->current_range -= 1;
            }
        } else {
            oc_wrap_greens(c, c->greens, c->current_slice + 1, -1);
        }
    }
}

void oc_initialize_run(OcChain* c) {
    oc_reverse_build_stack(c);
    oc_propagate(c);
}

/* update_greens!, fields.jl:271-286 with vldiv22!/vsub!/vmul!/vsubkron!
 * (fields.jl:176-209, linalg/updates.jl:7-11, 48-54, 92-97) on one block */
static void update_block(int n, double* G, double R, double delta, int i, double* IG, double* Gr) {
    double invRD = delta / R;
    for (int j = 0; j < n; ++j) IG[j] = -G[(size_t)i * n + j];
    IG[i] += 1.0;
    for (int j = 0; j < n; ++j) Gr[j] = invRD * G[(size_t)j * n + i];
    for (int l = 0; l < n; ++l) {
        double r = Gr[l];
        double* g = G + (size_t)l * n;
        for (int k = 0; k < n; ++k) g[k] -= IG[k] * r;
    }
}

void oc_update_greens(int n, int nf, double* G, const double* delta, int i) {
    double* IG = dalloc((size_t)n);
    double* Gr = dalloc((size_t)n);
    for (int b = 0; b < nf; ++b) {
        double* g = G + (size_t)b * n * n;
        double R = 1.0 + delta[b] * (1.0 - g[(size_t)i * n + i]);
        update_block(n, g, R, delta[b], i, IG, Gr);
    }
    free(IG); free(Gr);
}

/* sweep_spatial, local_updates.jl:23-60 with propose_local / accept_local!
 * (fields.jl:340-344, 388-393, 440-449, 497-503, 563-573, 627-637) */
int oc_sweep_spatial(OcChain* c) {
    int n = c->n, nf = c->nf;
    size_t nn = NN(c);
    int slice = c->current_slice;
    int8_t* s = c->conf + (size_t)(slice - 1) * n;
    double* IG = c->tempv;         /* n-vectors: reuse workspace not live here */
    double* Gr = c->scratch;
    int accepted = 0;
    static const int8_t choices[4][3] = {{2, 3, 4}, {1, 3, 4}, {1, 2, 4}, {1, 2, 3}};
    for (int i = 0; i < n; ++i) {
        double delta[2], R[2], detratio, dEb, p;
        int x_new = 0;
        double* g0 = c->greens;
        double* g1 = c->greens + nn;
        switch (c->kind) {
        case OC_DENSITY_HIRSCH:
            dEb = -2.0 * c->alpha * (double)s[i];
            delta[0] = exp(dEb) - 1.0;
            R[0] = 1.0 + delta[0] * (1.0 - g0[(size_t)i * n + i]);
            detratio = R[0] * R[0];
            p = exp(-dEb) * detratio;
            break;
        case OC_MAGNETIC_HIRSCH:
            dEb = -2.0 * c->alpha * (double)s[i];
            delta[0] = exp(+dEb) - 1.0;
            delta[1] = exp(-dEb) - 1.0;
            R[0] = 1.0 + delta[0] * (1.0 - g0[(size_t)i * n + i]);
            R[1] = 1.0 + delta[1] * (1.0 - g1[(size_t)i * n + i]);
            detratio = R[0] * R[1];
            p = exp(-0.0) * detratio;
            break;
        case OC_DENSITY_GHQ: {
            int x_old = s[i];
            uint64_t w = next_word(c);
            int r = (int)(((unsigned __int128)w * 3u) >> 64);
            x_new = choices[x_old - 1][r];
            dEb = c->alpha * (c->eta[x_new - 1] - c->eta[x_old - 1]);
            double er = exp(dEb);
            delta[0] = er - 1.0;
            R[0] = 1.0 + delta[0] * (1.0 - g0[(size_t)i * n + i]);
            detratio = R[0] * R[0];
            detratio = detratio * c->gam[x_new - 1] / c->gam[x_old - 1];
            p = exp(-dEb) * detratio;
            break;
        }
        default: { /* OC_MAGNETIC_GHQ */
            int x_old = s[i];
            uint64_t w = next_word(c);
            int r = (int)(((unsigned __int128)w * 3u) >> 64);
            x_new = choices[x_old - 1][r];
            double er = exp(c->alpha * (c->eta[x_new - 1] - c->eta[x_old - 1]));
            delta[0] = er - 1.0;
            delta[1] = 1.0 / er - 1.0;
            R[0] = 1.0 + delta[0] * (1.0 - g0[(size_t)i * n + i]);
            R[1] = 1.0 + delta[1] * (1.0 - g1[(size_t)i * n + i]);
            detratio = R[0] * R[1];
            detratio = detratio * c->gam[x_new - 1] / c->gam[x_old - 1];
            p = exp(-0.0) * detratio;
            break;
        }
        }
        if (p < 0.0) c->n_neg_p++;
        int acc = 0;
        if (p > 1.0) acc = 1;
        else {
            const double u = oc_word_to_uniform(next_word(c));
            acc = u < p;
            const double gap = fabs(u - p);
            if (gap < 1e-12) c->n_near_tie++;
            if (gap < c->min_tie_gap) c->min_tie_gap = gap;
        }
        if (acc) {
            for (int b = 0; b < nf; ++b)
                update_block(n, c->greens + b * nn, R[b], delta[b], i, IG, Gr);
            if (c->kind == OC_DENSITY_HIRSCH || c->kind == OC_MAGNETIC_HIRSCH) s[i] = (int8_t)(-s[i]);
            else s[i] = (int8_t)x_new;
            accepted++;
        }
    }
    c->accepted += accepted;
    return accepted;
}

long oc_local_sweeps(OcChain* c, int nsweeps) {
    long acc = 0;
    for (int s = 0; s < nsweeps; ++s)
        for (int t = 0; t < 2 * c->M; ++t) {
            acc += oc_sweep_spatial(c);
            oc_propagate(c);
        }
    return acc;
}

/* the UDT chains of calculate_greens(mc, slice, ...) (stack.jl:525-583) and of
 * inv_det (global_updates.jl:65-133): Ur,Dr,Tr = B(slice+1)'...B(M)' and
 * Ul,Dl,Tl = B(slice)...B(1), stabilised every safe_mult slices */
static void udt_chains_from_scratch(OcChain* c, int slice, int safe_mult) {
    mat_identity(c, c->curr_U); mat_identity(c, c->Ur); vec_ones(c, c->Dr); mat_identity(c, c->Tr);
    if (slice + 1 <= c->M) {
        for (int k = c->M; k >= slice + 1; --k) {
            mult_daggered_slice_left(c, k, c->curr_U);
            if (k % safe_mult == 0) {
                diag_right_blocks(c, c->tmp1, c->curr_U, c->Dr);
                udt_blocks(c, c->curr_U, c->Dr, c->tmp1, 1);
                mat_copy(c, c->tmp2, c->Tr);
                gemm_blocks(c, c->Tr, c->tmp1, c->tmp2);
            }
        }
        diag_right_blocks(c, c->tmp1, c->curr_U, c->Dr);
        udt_blocks(c, c->Ur, c->Dr, c->tmp1, 1);
        mat_copy(c, c->tmp2, c->Tr);
        gemm_blocks(c, c->Tr, c->tmp1, c->tmp2);
    }
    mat_identity(c, c->curr_U); mat_identity(c, c->Ul); vec_ones(c, c->Dl); mat_identity(c, c->Tl);
    if (slice >= 1) {
        for (int k = 1; k <= slice; ++k) {
            mult_slice_left(c, k, c->curr_U);
            if (k % safe_mult == 0) {
                diag_right_blocks(c, c->tmp1, c->curr_U, c->Dl);
                udt_blocks(c, c->curr_U, c->Dl, c->tmp1, 1);
                mat_copy(c, c->tmp2, c->Tl);
                gemm_blocks(c, c->Tl, c->tmp1, c->tmp2);
            }
        }
        diag_right_blocks(c, c->tmp1, c->curr_U, c->Dl);
        udt_blocks(c, c->Ul, c->Dl, c->tmp1, 1);
        mat_copy(c, c->tmp2, c->Tl);
        gemm_blocks(c, c->Tl, c->tmp1, c->tmp2);
    }
}

/* calculate_greens(mc, slice, output, field, safe_mult), stack.jl:525-583 */
void oc_calculate_greens_at(OcChain* c, int slice, double* out, int safe_mult) {
    if (safe_mult <= 0) safe_mult = c->k;
    udt_chains_from_scratch(c, slice, safe_mult);
    calculate_greens(c, out);
}

/* ------------------------------------------------------------ global updates */

/* inv_det, global_updates.jl:65-133: the stack of the current configuration
 * from scratch, then calculate_inv_greens_udt into greens_temp; returns Dr
 * (det(G) = 1 / prod(Dr), phases ignored as the reference does) */
static const double* inv_det(OcChain* c, int slice) {
    udt_chains_from_scratch(c, slice, c->k);
    calc_greens_blocks_part(c->n, c->nf, c->Ul, c->Dl, c->Tl, c->Ur, c->Dr, c->Tr, c->greens_temp,
                            c->pivot, c->tempv, c->scratch, 0);
    return c->Dr;
}

/* energy_boson, fields.jl:395, 451, 544, 614 */
static double energy_boson(const OcChain* c, const int8_t* conf) {
    if (c->kind == OC_MAGNETIC_HIRSCH || c->kind == OC_MAGNETIC_GHQ) return 0.0;
    long sum = 0;
    for (size_t i = 0; i < (size_t)c->n * c->M; ++i) sum += conf[i];
    return c->alpha * (double)sum;
}

/* propose_global_from_conf, global_updates.jl:137-166, with conf = the
 * proposal and old = the configuration it replaces: det ratio and
 * Delta E_boson = E(conf) - E(old) */
static double propose_global(OcChain* c, const int8_t* old, double* dEb) {
    const int cnt = c->nf * c->n;
    memcpy(c->tempvf, c->Dl, (size_t)cnt * sizeof(double));
    const double* Dr = inv_det(c, c->current_slice - 1);
    double detratio = 1.0;
    for (int i = 0; i < cnt; ++i) detratio *= c->tempvf[i] * Dr[i];
    *dEb = energy_boson(c, c->conf) - energy_boson(c, old);
    if (c->nf == 1) detratio = detratio * detratio;
    return detratio;
}

/* accept_global!, global_updates.jl:169-185: full rebuild */
static void accept_global(OcChain* c) {
    oc_reverse_build_stack(c);
    oc_propagate(c);
}

double oc_global_detratio(OcChain* c, const int8_t* proposal, double* dEb) {
    const size_t cnt = (size_t)c->n * c->M;
    memcpy(c->temp_conf, c->conf, cnt);
    memcpy(c->conf, proposal, cnt);
    double r = propose_global(c, c->temp_conf, dEb);
    memcpy(c->conf, c->temp_conf, cnt);
    return r;
}

/* global_update (global_updates.jl:188-203) after propose_conf! of
 * GlobalFlip (:244-256: s -> -s, GHQ x -> 5 - x) or GlobalShuffle
 * (:270-278: a Fisher-Yates shuffle of the whole configuration drawing
 * j = floor(w (i+1) / 2^64) from the chain's stream for i = nM-1 ... 1) */
int oc_global_update(OcChain* c, int kind) {
    const size_t cnt = (size_t)c->n * c->M;
    const int ghq = (c->kind == OC_DENSITY_GHQ || c->kind == OC_MAGNETIC_GHQ);
    memcpy(c->temp_conf, c->conf, cnt);
    if (kind == 0) {
        for (size_t i = 0; i < cnt; ++i) c->conf[i] = ghq ? (int8_t)(5 - c->conf[i]) : (int8_t)(-c->conf[i]);
    } else {
        for (size_t i = cnt - 1; i >= 1; --i) {
            uint64_t w = next_word(c);
            size_t j = (size_t)(((unsigned __int128)w * (unsigned __int128)(i + 1)) >> 64);
            int8_t t = c->conf[i]; c->conf[i] = c->conf[j]; c->conf[j] = t;
        }
    }
    double dEb;
    double detratio = propose_global(c, c->temp_conf, &dEb);
    double p = fabs(exp(-dEb) * detratio);
    int acc = (p > 1.0) ? 1 : (oc_word_to_uniform(next_word(c)) < p);
    c->g_proposals++;
    if (acc) {
        accept_global(c);
        c->g_accepted++;
    } else {
        memcpy(c->conf, c->temp_conf, cnt);
    }
    return acc;
}

/* the local half of ReplicaExchange (parallel_updates.jl:116-150): the
 * weight exp(-Delta E) * detratio of adopting the partner's configuration and
 * one uniform draw; the configuration is left unchanged */
void oc_replica_weight(OcChain* c, const int8_t* partner_conf, double* weight, double* prob) {
    double dEb;
    double detratio = oc_global_detratio(c, partner_conf, &dEb);
    *weight = exp(-dEb) * detratio;
    *prob = oc_word_to_uniform(next_word(c));
}

/* accept_global! with the partner's configuration */
void oc_replica_accept(OcChain* c, const int8_t* partner_conf) {
    memcpy(c->conf, partner_conf, (size_t)c->n * c->M);
    accept_global(c);
    c->g_accepted++;
}

/* a local move of site i (0-based) at the current slice to field value
 * x_new (the reference's propose_local + accept_local!, fields.jl:340-344,
 * 388-393, 440-449, 497-503, 563-573, 627-637); returns p = exp(-dE) detratio */
double oc_local_move_to(OcChain* c, int i, int x_new) {
    int n = c->n;
    size_t nn = NN(c);
    int8_t* s = c->conf + (size_t)(c->current_slice - 1) * n;
    double delta[2] = {0.0, 0.0}, R[2] = {1.0, 1.0}, detratio, dEb, p;
    double* g0 = c->greens;
    double* g1 = c->greens + nn;
    int x_old = s[i];
    switch (c->kind) {
    case OC_DENSITY_HIRSCH:
        dEb = -2.0 * c->alpha * (double)s[i];
        delta[0] = exp(dEb) - 1.0;
        R[0] = 1.0 + delta[0] * (1.0 - g0[(size_t)i * n + i]);
        detratio = R[0] * R[0];
        p = exp(-dEb) * detratio;
        break;
    case OC_MAGNETIC_HIRSCH:
        dEb = -2.0 * c->alpha * (double)s[i];
        delta[0] = exp(+dEb) - 1.0;
        delta[1] = exp(-dEb) - 1.0;
        R[0] = 1.0 + delta[0] * (1.0 - g0[(size_t)i * n + i]);
        R[1] = 1.0 + delta[1] * (1.0 - g1[(size_t)i * n + i]);
        detratio = R[0] * R[1];
        p = detratio;
        break;
    case OC_DENSITY_GHQ:
        dEb = c->alpha * (c->eta[x_new - 1] - c->eta[x_old - 1]);
        delta[0] = exp(dEb) - 1.0;
        R[0] = 1.0 + delta[0] * (1.0 - g0[(size_t)i * n + i]);
        detratio = R[0] * R[0] * c->gam[x_new - 1] / c->gam[x_old - 1];
        p = exp(-dEb) * detratio;
        break;
    default: {
        double er = exp(c->alpha * (c->eta[x_new - 1] - c->eta[x_old - 1]));
        delta[0] = er - 1.0;
        delta[1] = 1.0 / er - 1.0;
        R[0] = 1.0 + delta[0] * (1.0 - g0[(size_t)i * n + i]);
        R[1] = 1.0 + delta[1] * (1.0 - g1[(size_t)i * n + i]);
        detratio = R[0] * R[1] * c->gam[x_new - 1] / c->gam[x_old - 1];
        p = detratio;
        break;
    }
    }
    for (int b = 0; b < c->nf; ++b)
        update_block(n, c->greens + b * nn, R[b], delta[b], i, c->tempv, c->scratch);
    s[i] = (int8_t)x_new;
    return p;
}

void oc_get_global_stats(const OcChain* c, long* accepted, long* proposals) {
    *accepted = c->g_accepted;
    *proposals = c->g_proposals;
}

/* _greens!, greens.jl:114-125: eThalfplus * (G * eThalfminus) */
void oc_greens_physical(OcChain* c, const double* src, double* out) {
    int n = c->n;
    size_t nn = NN(c);
    double* tmp = dalloc(nn);
    for (int b = 0; b < c->nf; ++b) {
        if (c->cb) {
            cb_apply(c, 2, 1, tmp, src + b * nn);
            cb_apply(c, 3, 0, out + b * nn, tmp);
        } else {
            gemm_nt(n, tmp, src + b * nn, c->eTh, c->scratch);
            gemm_tn(n, out + b * nn, c->eThinv, tmp, c->scratch);
        }
    }
    free(tmp);
}

void oc_get_greens(const OcChain* c, double* out) { memcpy(out, c->greens, MATSZ(c) * sizeof(double)); }
void oc_set_greens(OcChain* c, const double* in) { memcpy(c->greens, in, MATSZ(c) * sizeof(double)); }

void oc_get_state(const OcChain* c, int* st) {
    st[0] = c->current_slice; st[1] = c->current_range; st[2] = c->direction; st[3] = c->nr;
}

void oc_get_stack(const OcChain* c, int which, int idx, double* out) {
    OcChain* cc = (OcChain*)c;
    if (which == 0) memcpy(out, ustk(cc, idx), MATSZ(c) * sizeof(double));
    else if (which == 1) memcpy(out, tstk(cc, idx), MATSZ(c) * sizeof(double));
    else memcpy(out, dstk(cc, idx), (size_t)c->nf * c->n * sizeof(double));
}

void oc_get_analysis(const OcChain* c, double* out) {
    out[0] = c->prop_err_all;
    out[1] = (double)c->n_prop_err;
    out[2] = c->prop_err_reported;
    out[3] = (double)c->n_neg_p;
    out[4] = (double)c->accepted;
    out[5] = (double)c->n_near_tie;
    out[6] = c->min_tie_gap;
}

/* ---------------------------------------------------- threaded baseline */

typedef struct {
    OcChain** chains;
    int first, count, nsweeps;
} OcWork;

static void* oc_worker(void* arg) {
    OcWork* w = (OcWork*)arg;
    for (int i = 0; i < w->count; ++i) oc_local_sweeps(w->chains[w->first + i], w->nsweeps);
    return NULL;
}

double oc_run_chains_threaded(OcChain** chains, int nchains, int nsweeps, int threads) {
    if (threads < 1) threads = 1;
    if (threads > nchains) threads = nchains;
    pthread_t* th = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
    OcWork* wk = (OcWork*)calloc((size_t)threads, sizeof(OcWork));
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    int base = nchains / threads, rem = nchains % threads, pos = 0;
    for (int t = 0; t < threads; ++t) {
        wk[t].chains = chains; wk[t].first = pos; wk[t].count = base + (t < rem ? 1 : 0);
        wk[t].nsweeps = nsweeps;
        pos += wk[t].count;
        pthread_create(&th[t], NULL, oc_worker, &wk[t]);
    }
    for (int t = 0; t < threads; ++t) pthread_join(th[t], NULL);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    free(th); free(wk);
    return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}

/* ------------------------------------------------- unequal-time Green's function
 * calculate_greens(mc, k, l) through the UnequalTimeStack
 * (unequal_time_stack.jl:124-178, 326-338, 354-697), the stacks rebuilt from
 * the current configuration at every call (the reference rebuilds them when
 * the configuration has changed since the last call). */

typedef struct {
    int nr;
    double *fu, *fd, *ft;   /* forward  B_{n*k} ... B_1, nr+1 entries */
    double *bu, *bd, *bt;   /* backward B_{n*k+1}^T ... B_M^T, nr+1 entries */
    double *iu, *id, *it;   /* inverse chunks, nr entries */
    double *U, *D, *T, *G;  /* s.U, s.D, s.T, s.greens */
} OcUt;

static OcUt ut_alloc(OcChain* c) {
    OcUt s;
    size_t ms = MATSZ(c), vs = (size_t)c->nf * c->n;
    s.nr = c->nr;
    s.fu = dalloc(ms * (c->nr + 1)); s.ft = dalloc(ms * (c->nr + 1)); s.fd = dalloc(vs * (c->nr + 1));
    s.bu = dalloc(ms * (c->nr + 1)); s.bt = dalloc(ms * (c->nr + 1)); s.bd = dalloc(vs * (c->nr + 1));
    s.iu = dalloc(ms * c->nr); s.it = dalloc(ms * c->nr); s.id = dalloc(vs * c->nr);
    s.U = dalloc(ms); s.T = dalloc(ms); s.G = dalloc(ms); s.D = dalloc(vs);
    return s;
}
static void ut_free(OcUt* s) {
    free(s->fu); free(s->ft); free(s->fd); free(s->bu); free(s->bt); free(s->bd);
    free(s->iu); free(s->it); free(s->id); free(s->U); free(s->T); free(s->G); free(s->D);
}
#define UTM(p, c, idx) ((p) + (size_t)((idx) - 1) * MATSZ(c))
#define UTV(p, c, idx) ((p) + (size_t)((idx) - 1) * (size_t)(c)->nf * (c)->n)

/* build_stack(mc, ::UnequalTimeStack), unequal_time_stack.jl:124-178 */
static void ut_build(OcChain* c, OcUt* s) {
    const int nr = c->nr;
    mat_identity(c, UTM(s->fu, c, 1)); vec_ones(c, UTV(s->fd, c, 1)); mat_identity(c, UTM(s->ft, c, 1));
    mat_identity(c, UTM(s->bu, c, nr + 1)); vec_ones(c, UTV(s->bd, c, nr + 1));
    mat_identity(c, UTM(s->bt, c, nr + 1));
    for (int idx = 1; idx <= nr; ++idx) {
        mat_copy(c, c->curr_U, UTM(s->fu, c, idx));
        for (int sl = c->rfirst[idx - 1]; sl <= c->rlast[idx - 1]; ++sl) mult_slice_left(c, sl, c->curr_U);
        diag_right_blocks(c, c->tmp1, c->curr_U, UTV(s->fd, c, idx));
        udt_blocks(c, UTM(s->fu, c, idx + 1), UTV(s->fd, c, idx + 1), c->tmp1, 1);
        gemm_blocks(c, UTM(s->ft, c, idx + 1), c->tmp1, UTM(s->ft, c, idx));
    }
    for (int idx = nr; idx >= 1; --idx) {
        mat_copy(c, c->curr_U, UTM(s->bu, c, idx + 1));
        for (int sl = c->rlast[idx - 1]; sl >= c->rfirst[idx - 1]; --sl)
            mult_daggered_slice_left(c, sl, c->curr_U);
        diag_right_blocks(c, c->tmp1, c->curr_U, UTV(s->bd, c, idx + 1));
        udt_blocks(c, UTM(s->bu, c, idx), UTV(s->bd, c, idx), c->tmp1, 1);
        gemm_blocks(c, UTM(s->bt, c, idx), c->tmp1, UTM(s->bt, c, idx + 1));
    }
    for (int idx = 1; idx <= nr; ++idx) {
        double* it = UTM(s->it, c, idx);
        mat_identity(c, it);
        for (int sl = c->rlast[idx - 1]; sl >= c->rfirst[idx - 1]; --sl) mult_slice_inv_left(c, sl, it);
        udt_blocks(c, UTM(s->iu, c, idx), UTV(s->id, c, idx), it, 1);
    }
}

/* _find_range_with_value, unequal_time_stack.jl:354-390: 1-based chunk
 * holding slice val; 0 below, nr + 1 above */
static int find_range(const OcChain* c, int val) {
    if (val < 1) return 0;
    if (val > c->rlast[c->nr - 1]) return c->nr + 1;
    for (int i = 0; i < c->nr; ++i)
        if (c->rfirst[i] <= val && val <= c->rlast[i]) return i + 1;
    return c->nr + 1;
}

static void gemm_nt_blocks(OcChain* c, double* C, const double* A, const double* B) {
    for (int b = 0; b < c->nf; ++b) gemm_nt(c->n, C + b * NN(c), A + b * NN(c), B + b * NN(c), c->scratch);
}
static void gemm_tn_blocks(OcChain* c, double* C, const double* A, const double* B) {
    for (int b = 0; b < c->nf; ++b) gemm_tn(c->n, C + b * NN(c), A + b * NN(c), B + b * NN(c), c->scratch);
}
static void diag_left_blocks(OcChain* c, double* C, const double* d, const double* B) {
    for (int b = 0; b < c->nf; ++b) diag_left(c->n, C + b * NN(c), d + b * c->n, B + b * NN(c));
}
static void rdivp_blocks(OcChain* c, double* A, const double* T, double* O) {
    for (int b = 0; b < c->nf; ++b)
        oc_rdivp(c->n, A + b * NN(c), T + b * NN(c), O + b * NN(c), c->pivot + b * c->n, c->nf > 1);
}
static void vmaxinv(OcChain* c, double* v, const double* w) {  /* real.jl:164-170 */
    for (int i = 0; i < c->nf * c->n; ++i) v[i] = 1.0 / (w[i] > 1.0 ? w[i] : 1.0);
}
static void vmin1(OcChain* c, double* v, const double* w) {    /* real.jl:143-149 */
    for (int i = 0; i < c->nf * c->n; ++i) v[i] = (w[i] < 1.0 ? w[i] : 1.0);
}
static void mat_add(OcChain* c, double* A, const double* B) {  /* rvadd!, real.jl:123-127 */
    for (size_t e = 0; e < MATSZ(c); ++e) A[e] += B[e];
}
static void mat_diag(OcChain* c, double* A, const double* d) { /* copyto!(A, Diagonal(d)) */
    memset(A, 0, MATSZ(c) * sizeof(double));
    for (int b = 0; b < c->nf; ++b)
        for (int i = 0; i < c->n; ++i) A[b * NN(c) + (size_t)i * c->n + i] = d[b * c->n + i];
}

/* compute_inverse_udt_block!, unequal_time_stack.jl:400-463:
 * U D T = B_{low+1}^-1 ... B_high^-1 */
static void ut_inverse_block(OcChain* c, OcUt* s, int low, int high) {
    const int lower = find_range(c, low) + 1, upper = find_range(c, high + 1) - 1;
    mat_identity(c, s->U); vec_ones(c, s->D); mat_identity(c, s->T);
    for (int idx = lower; idx <= upper; ++idx) {
        gemm_blocks(c, c->tmp1, s->T, UTM(s->iu, c, idx));
        diag_left_blocks(c, c->tmp2, s->D, c->tmp1);
        diag_right_blocks(c, c->tmp1, c->tmp2, UTV(s->id, c, idx));
        udt_blocks(c, c->tmp2, s->D, c->tmp1, 1);
        gemm_blocks(c, s->T, c->tmp1, UTM(s->it, c, idx));
        gemm_blocks(c, c->tmp1, s->U, c->tmp2);
        mat_copy(c, s->U, c->tmp1);
    }
    const int lower_slice = lower <= c->nr ? c->rfirst[lower - 1] : c->rlast[c->nr - 1] + 1;
    const int upper_slice = upper > 0 ? c->rlast[upper - 1] : 0;
    const int top = (lower_slice - 1 < high) ? lower_slice - 1 : high;
    for (int sl = top; sl >= low + 1; --sl) mult_slice_inv_left(c, sl, s->U);
    if (top >= low + 1) {
        diag_right_blocks(c, c->tmp1, s->U, s->D);
        udt_blocks(c, s->U, s->D, c->tmp1, 1);
        gemm_blocks(c, c->tmp2, c->tmp1, s->T);
        mat_copy(c, s->T, c->tmp2);
    }
    const int from = (upper_slice + 1 > top + 1) ? upper_slice + 1 : top + 1;
    for (int sl = from; sl <= high; ++sl) mult_slice_inv_right(c, sl, s->T);
}

/* compute_forward_udt_block!, :474-497: Ul Dl Tl = B_slice ... B_1 */
static void ut_forward_block(OcChain* c, OcUt* s, int slice) {
    int idx = find_range(c, slice) - 1;
    if (idx < 0) idx = 0;
    mat_copy(c, c->Tl, UTM(s->fu, c, idx + 1));
    const int target = idx > 0 ? c->rlast[idx - 1] + 1 : 1;
    for (int l = target; l <= slice; ++l) mult_slice_left(c, l, c->Tl);
    diag_right_blocks(c, c->tmp1, c->Tl, UTV(s->fd, c, idx + 1));
    udt_blocks(c, c->Ul, c->Dl, c->tmp1, 1);
    gemm_blocks(c, c->Tl, c->tmp1, UTM(s->ft, c, idx + 1));
}

/* compute_backward_udt_block!, :509-533: (Ur Dr Tr)^T = B_M ... B_{slice+1} */
static void ut_backward_block(OcChain* c, OcUt* s, int slice) {
    const int idx = find_range(c, slice) + 1;
    mat_copy(c, c->Ur, UTM(s->bu, c, idx));
    const int target = idx <= c->nr ? c->rfirst[idx - 1] - 1 : c->rlast[c->nr - 1];
    for (int l = target; l >= slice + 1; --l) mult_daggered_slice_left(c, l, c->Ur);
    diag_right_blocks(c, c->tmp1, c->Ur, UTV(s->bd, c, idx));
    udt_blocks(c, c->Ur, c->Dr, c->tmp1, 1);
    gemm_blocks(c, c->Tr, c->tmp1, UTM(s->bt, c, idx));
}

/* calculate_greens_full1!, :536-619 (slice1 >= slice2) */
static void ut_full1(OcChain* c, OcUt* s, int slice1, int slice2) {
    ut_inverse_block(c, s, slice2, slice1);
    ut_forward_block(c, s, slice2);
    ut_backward_block(c, s, slice1);
    gemm_nt_blocks(c, s->G, c->Tl, c->Tr);
    diag_right_blocks(c, c->tmp1, s->G, c->Dr);
    diag_left_blocks(c, s->G, c->Dl, c->tmp1);
    udt_blocks(c, c->Tr, c->Dr, s->G, 0);
    gemm_blocks(c, c->Tl, c->Ul, c->Tr);
    rdivp_blocks(c, c->Ur, s->G, c->Ul);
    gemm_tn_blocks(c, c->Tr, s->U, c->Tl);
    vmaxinv(c, c->Dl, s->D);
    diag_left_blocks(c, c->tmp1, c->Dl, c->Tr);
    vmin1(c, c->Dl, c->Dr);
    diag_right_blocks(c, c->Tr, c->tmp1, c->Dl);
    gemm_blocks(c, c->Tl, s->T, c->Ur);
    vmin1(c, c->Dl, s->D);
    diag_left_blocks(c, c->tmp1, c->Dl, c->Tl);
    vmaxinv(c, c->Dl, c->Dr);
    diag_right_blocks(c, c->Tl, c->tmp1, c->Dl);
    mat_add(c, c->Tl, c->Tr);
    udt_blocks(c, c->Tr, c->Dl, c->Tl, 0);
    vmaxinv(c, c->Dr, c->Dr);
    mat_diag(c, c->Ul, c->Dr);
    rdivp_blocks(c, c->Ul, c->Tl, c->tmp1);
    for (int i = 0; i < c->nf * c->n; ++i) c->Dl[i] = 1.0 / c->Dl[i];
    diag_right_blocks(c, c->tmp1, c->Ul, c->Dl);
    gemm_nt_blocks(c, c->Ul, c->tmp1, c->Tr);
    vmaxinv(c, c->Dl, s->D);
    diag_right_blocks(c, s->G, c->Ul, c->Dl);
    gemm_nt_blocks(c, c->Tr, s->G, s->U);
    gemm_blocks(c, s->G, c->Ur, c->Tr);
}

/* calculate_greens_full2!, :621-697 (slice1 < slice2) */
static void ut_full2(OcChain* c, OcUt* s, int slice1, int slice2) {
    ut_inverse_block(c, s, slice1, slice2);
    ut_forward_block(c, s, slice1);
    ut_backward_block(c, s, slice2);
    gemm_nt_blocks(c, s->G, c->Tl, c->Tr);
    diag_left_blocks(c, c->tmp1, c->Dl, s->G);
    diag_right_blocks(c, s->G, c->tmp1, c->Dr);
    udt_blocks(c, c->Tr, c->Dr, s->G, 0);
    gemm_blocks(c, c->Tl, c->Ul, c->Tr);
    gemm_tn_blocks(c, c->Ul, s->U, c->Tl);
    vmaxinv(c, c->Dl, s->D);
    diag_left_blocks(c, s->U, c->Dl, c->Ul);
    vmin1(c, c->Dl, c->Dr);
    diag_right_blocks(c, c->Ul, s->U, c->Dl);
    gemm_blocks(c, s->U, s->T, c->Ur);
    rdivp_blocks(c, s->U, s->G, c->Ur);
    vmin1(c, c->Dl, s->D);
    diag_left_blocks(c, c->Ur, c->Dl, s->U);
    vmaxinv(c, c->Dl, c->Dr);
    diag_right_blocks(c, c->Tr, c->Ur, c->Dl);
    mat_add(c, c->Tr, c->Ul);
    udt_blocks(c, c->Ul, c->Dl, c->Tr, 0);
    vmin1(c, c->Dr, c->Dr);
    mat_diag(c, s->U, c->Dr);
    rdivp_blocks(c, s->U, c->Tr, c->Ur);
    for (int i = 0; i < c->nf * c->n; ++i) c->Dl[i] = 1.0 / c->Dl[i];
    diag_right_blocks(c, c->Ur, s->U, c->Dl);
    gemm_nt_blocks(c, s->U, c->Ur, c->Ul);
    vmin1(c, s->D, s->D);
    diag_right_blocks(c, c->Ur, s->U, s->D);
    gemm_blocks(c, c->Tr, c->Ur, s->T);
    gemm_blocks(c, s->G, c->Tl, c->Tr);
    for (size_t e = 0; e < MATSZ(c); ++e) s->G[e] = -s->G[e];
}

/* calculate_greens(mc, slice1, slice2), :326-338: the effective G(k, l) for
 * npairs pairs (one stack build) */
void oc_greens_kl(OcChain* c, const int* k, const int* l, int npairs, double* out) {
    OcUt s = ut_alloc(c);
    ut_build(c, &s);
    for (int p = 0; p < npairs; ++p) {
        if (k[p] >= l[p]) ut_full1(c, &s, k[p], l[p]);
        else ut_full2(c, &s, k[p], l[p]);
        memcpy(out + (size_t)p * MATSZ(c), s.G, MATSZ(c) * sizeof(double));
    }
    ut_free(&s);
}
