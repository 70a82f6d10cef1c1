// Host-side builders of a chain descriptor: stabilisation chunks and the
// proposal / interaction exponential tables.  Shared by the C-ABI
// translation units.
#pragma once
#include <math.h>

#include "../../include/dqmc_gb300.h"
#include "dqmc_chain.h"

namespace dqmc_host {

// generate_chunks (stack.jl:154-158)
inline int generate_chunks(int length, int max_chunk, int* first, int* last) {
    int nch = (length + max_chunk - 1) / max_chunk;
    double step = (double)length / (double)nch;
    for (int i = 1; i <= nch; ++i) {
        first[i - 1] = (int)nearbyint((double)(i - 1) * step) + 1;
        last[i - 1] = (int)nearbyint((double)i * step);
    }
    return nch;
}

// Tables of the proposal / interaction exponentials, computed with the
// reference's expressions in the reference's operation order.
inline void fill_tables(DqmcChain& d, int kind, double alpha) {
    const double s6 = sqrt(6.0);
    const double gam[4] = {1.0 - s6 / 3.0, 1.0 + s6 / 3.0, 1.0 + s6 / 3.0, 1.0 - s6 / 3.0};
    const double eta[4] = {-sqrt(6.0 + 2.0 * s6), -sqrt(6.0 - 2.0 * s6), sqrt(6.0 - 2.0 * s6),
                           sqrt(6.0 + 2.0 * s6)};
    for (int i = 0; i < 4; ++i) d.gam[i] = gam[i];
    for (int i = 0; i < 16; ++i) { d.delta0[i] = 0.0; d.delta1[i] = 0.0; d.wboson[i] = 0.0; }
    for (int f = 0; f < 2; ++f)
        for (int v = 0; v < 4; ++v) { d.ev[f][v] = 0.0; d.evinv[f][v] = 0.0; }
    const double a = alpha;
    switch (kind) {
    case DQMC_FIELD_DENSITY_HIRSCH:
        for (int v = 0; v < 2; ++v) {
            double s = v ? 1.0 : -1.0;
            d.ev[0][v] = exp(1.0 * a * s);      // fields.jl:383
            d.evinv[0][v] = exp(-1.0 * a * s);
            double dE = -2.0 * a * s;           // fields.jl:389-390
            d.delta0[v] = exp(dE) - 1;
            d.wboson[v] = exp(-dE);             // local_updates.jl:31
        }
        break;
    case DQMC_FIELD_MAGNETIC_HIRSCH:
        for (int v = 0; v < 2; ++v) {
            double s = v ? 1.0 : -1.0;
            d.ev[0][v] = exp(1.0 * a * s);      // fields.jl:432
            d.ev[1][v] = exp(-1.0 * a * s);     // fields.jl:435
            d.evinv[0][v] = exp(-1.0 * a * s);
            d.evinv[1][v] = exp(-(-1.0) * a * s);
            double dE = -2.0 * a * s;           // fields.jl:441-443
            d.delta0[v] = exp(+dE) - 1.0;
            d.delta1[v] = exp(-dE) - 1.0;
            d.wboson[v] = exp(-0.0);
        }
        break;
    case DQMC_FIELD_DENSITY_GHQ:
        for (int v = 0; v < 4; ++v) {
            d.ev[0][v] = exp(+1.0 * a * eta[v]); // fields.jl:621
            d.evinv[0][v] = exp(+(-1.0) * a * eta[v]);
        }
        for (int xo = 0; xo < 4; ++xo)
            for (int xn = 0; xn < 4; ++xn) {
                if (xo == xn) continue;
                double dE = a * (eta[xn] - eta[xo]); // fields.jl:631-633
                double er = exp(dE);
                d.delta0[xo * 4 + xn] = er - 1.0;
                d.wboson[xo * 4 + xn] = exp(-dE);
            }
        break;
    default: /* DQMC_FIELD_MAGNETIC_GHQ */
        for (int v = 0; v < 4; ++v) {
            d.ev[0][v] = exp(+1.0 * a * eta[v]);    // fields.jl:553
            d.ev[1][v] = exp(-1.0 * a * eta[v]);    // fields.jl:556
            d.evinv[0][v] = exp(+(-1.0) * a * eta[v]);
            d.evinv[1][v] = exp(-(-1.0) * a * eta[v]);
        }
        for (int xo = 0; xo < 4; ++xo)
            for (int xn = 0; xn < 4; ++xn) {
                if (xo == xn) continue;
                double er = exp(a * (eta[xn] - eta[xo])); // fields.jl:567-569
                d.delta0[xo * 4 + xn] = er - 1.0;
                d.delta1[xo * 4 + xn] = 1 / er - 1.0;
                d.wboson[xo * 4 + xn] = exp(-0.0);
            }
        break;
    }
}

// Complex arithmetic in the operation order of Julia's Complex{Float64}
// (Real * Complex scales both parts; exp(z) = e^re (cos im, sin im), or
// (e^re, im) when im == 0; 1/z by Smith's method, R. L. Smith, "Algorithm
// 116: Complex division", CACM 5 (1962) 435).
struct Cx {
    double re, im;
};
inline Cx cx_scale(Cx z, double x) { return {x * z.re, x * z.im}; }
inline Cx cx_exp(Cx z) {
    const double er = exp(z.re);
    if (z.im == 0.0) return {er, z.im};
    return {er * cos(z.im), er * sin(z.im)};
}
inline Cx cx_minus1(Cx z) { return {z.re - 1.0, z.im}; }
inline Cx cx_neg(Cx z) { return {-z.re, -z.im}; }
inline Cx cx_inv(Cx w) {
    const double c = w.re, d = w.im;
    if (fabs(d) <= fabs(c)) {
        const double r = d / c, t = 1.0 / (c + d * r);
        return {t, -r * t};
    }
    const double r = c / d, t = 1.0 / (d + c * r);
    return {r * t, -t};
}

// The same tables for a complex field constant alpha = (ar, ai) (the
// reference's AbstractHirschField{ComplexF64} / AbstractGHQField{ComplexF64},
// fields.jl:372, 383, 389-390, 421, 432-443, 530, 553-569, 600, 621-633):
// real parts into delta0 / delta1 / wboson / ev / evinv, imaginary parts into
// the *i arrays.  The bosonic weight of the magnetic fields is exp(-0.0) = 1.
inline void fill_tables_complex(DqmcChain& d, int kind, double ar, double ai) {
    fill_tables(d, kind, 0.0);  // gamma; zeroes the real tables
    for (int i = 0; i < 16; ++i) { d.delta0i[i] = 0.0; d.delta1i[i] = 0.0; d.wbosoni[i] = 0.0; }
    for (int f = 0; f < 2; ++f)
        for (int v = 0; v < 4; ++v) { d.evi[f][v] = 0.0; d.evinvi[f][v] = 0.0; }
    const double s6 = sqrt(6.0);
    const double eta[4] = {-sqrt(6.0 + 2.0 * s6), -sqrt(6.0 - 2.0 * s6), sqrt(6.0 - 2.0 * s6),
                           sqrt(6.0 + 2.0 * s6)};
    const Cx a{ar, ai}, one{1.0, 0.0};
    auto put = [](double* re, double* im, int i, Cx z) { re[i] = z.re; im[i] = z.im; };
    switch (kind) {
    case DQMC_FIELD_DENSITY_HIRSCH:
        for (int v = 0; v < 2; ++v) {
            const double s = v ? 1.0 : -1.0;
            put(d.ev[0], d.evi[0], v, cx_exp(cx_scale(cx_scale(a, 1.0), s)));
            put(d.evinv[0], d.evinvi[0], v, cx_exp(cx_scale(cx_scale(a, -1.0), s)));
            const Cx dE = cx_scale(cx_scale(a, -2.0), s);
            put(d.delta0, d.delta0i, v, cx_minus1(cx_exp(dE)));
            put(d.wboson, d.wbosoni, v, cx_exp(cx_neg(dE)));
        }
        break;
    case DQMC_FIELD_MAGNETIC_HIRSCH:
        for (int v = 0; v < 2; ++v) {
            const double s = v ? 1.0 : -1.0;
            put(d.ev[0], d.evi[0], v, cx_exp(cx_scale(cx_scale(a, 1.0), s)));
            put(d.ev[1], d.evi[1], v, cx_exp(cx_scale(cx_scale(a, -1.0), s)));
            put(d.evinv[0], d.evinvi[0], v, cx_exp(cx_scale(cx_scale(a, -1.0), s)));
            put(d.evinv[1], d.evinvi[1], v, cx_exp(cx_scale(cx_scale(a, 1.0), s)));
            const Cx dE = cx_scale(cx_scale(a, -2.0), s);
            put(d.delta0, d.delta0i, v, cx_minus1(cx_exp(dE)));
            put(d.delta1, d.delta1i, v, cx_minus1(cx_exp(cx_neg(dE))));
            put(d.wboson, d.wbosoni, v, one);
        }
        break;
    case DQMC_FIELD_DENSITY_GHQ:
        for (int v = 0; v < 4; ++v) {
            put(d.ev[0], d.evi[0], v, cx_exp(cx_scale(cx_scale(a, 1.0), eta[v])));
            put(d.evinv[0], d.evinvi[0], v, cx_exp(cx_scale(cx_scale(a, -1.0), eta[v])));
        }
        for (int xo = 0; xo < 4; ++xo)
            for (int xn = 0; xn < 4; ++xn) {
                if (xo == xn) continue;
                const Cx dE = cx_scale(a, eta[xn] - eta[xo]);
                put(d.delta0, d.delta0i, xo * 4 + xn, cx_minus1(cx_exp(dE)));
                put(d.wboson, d.wbosoni, xo * 4 + xn, cx_exp(cx_neg(dE)));
            }
        break;
    default: /* DQMC_FIELD_MAGNETIC_GHQ */
        for (int v = 0; v < 4; ++v) {
            put(d.ev[0], d.evi[0], v, cx_exp(cx_scale(cx_scale(a, 1.0), eta[v])));
            put(d.ev[1], d.evi[1], v, cx_exp(cx_scale(cx_scale(a, -1.0), eta[v])));
            put(d.evinv[0], d.evinvi[0], v, cx_exp(cx_scale(cx_scale(a, -1.0), eta[v])));
            put(d.evinv[1], d.evinvi[1], v, cx_exp(cx_scale(cx_scale(a, 1.0), eta[v])));
        }
        for (int xo = 0; xo < 4; ++xo)
            for (int xn = 0; xn < 4; ++xn) {
                if (xo == xn) continue;
                const Cx er = cx_exp(cx_scale(a, eta[xn] - eta[xo]));
                put(d.delta0, d.delta0i, xo * 4 + xn, cx_minus1(er));
                put(d.delta1, d.delta1i, xo * 4 + xn, cx_minus1(cx_scale(cx_inv(er), 1.0)));
                put(d.wboson, d.wbosoni, xo * 4 + xn, one);
            }
        break;
    }
}

}  // namespace dqmc_host
