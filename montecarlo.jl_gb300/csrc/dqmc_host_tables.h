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

}  // namespace dqmc_host
