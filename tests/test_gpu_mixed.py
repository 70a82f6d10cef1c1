"""Mixed-precision path: wraps, slice-matrix chains and the reconstruction's
products in split FP32; UDT factorisations, triangular solves, determinant
ratios and rank-1 updates in FP64.  Every result is
compared with the FP64 oracle; the target is max |dG| <= 1e-6."""
import numpy as np
import pytest

from _util import FIELD_U, chain_config, make_setup, maxdiff, oracle_chain

pytestmark = pytest.mark.gpu

TOL_MIXED = 1e-6


def _mixed_pair(pkg, lib, oracle, field, L, beta, safe_mult=10, seed=3):
    model, param, fld, exps = make_setup(pkg, L=L, U=FIELD_U[field], beta=beta,
                                         safe_mult=safe_mult, field=getattr(pkg, field))
    h = lib.Handle([chain_config(lib, model, param, fld, seed)], precision=lib.PREC_MIXED)
    h.set_hopping(-1, exps)
    oc = oracle_chain(oracle, model, param, fld, exps, seed)
    return h, oc, param


@pytest.mark.parametrize("field,L,beta", [("MagneticHirschField", 8, 8.0),
                                          ("DensityHirschField", 6, 4.0),
                                          ("MagneticGHQField", 4, 2.0)])
def test_mixed_calculate_greens_vs_fp64_oracle(pkg, lib, oracle, field, L, beta):
    h, oc, param = _mixed_pair(pkg, lib, oracle, field, L, beta)
    h.init_random_field(0)
    oc.init_random_conf()
    worst = 0.0
    for sl in (0, 1, param.slices // 2, param.slices):
        worst = max(worst, maxdiff(h.calculate_greens(0, sl), oc.calculate_greens_at(sl)))
    print(f"max |dG| calculate_greens mixed vs FP64 oracle: {worst:.2e}")
    assert worst <= TOL_MIXED


def test_mixed_every_stabilisation_vs_fp64_oracle(pkg, lib, oracle):
    """Step the mixed chain through two full sweeps with the oracle's field
    configuration replayed, comparing G with the oracle after every
    stabilisation (chunk boundary) and every wrap."""
    h, oc, param = _mixed_pair(pkg, lib, oracle, "MagneticHirschField", 8, 8.0)
    h.init_random_field(0)
    oc.init_random_conf()
    h.initialize_run()
    oc.initialize_run()
    worst_stab, worst_wrap = 0.0, 0.0
    for _ in range(2 * 2 * param.slices):
        oc.sweep_spatial()
        # replay the oracle's decisions: same field, G re-derived by the update
        h.set_field(0, oc.get_conf())
        h.set_greens(0, oc.greens())
        st_before = oc.state()
        oc.propagate()
        h.propagate()
        d = maxdiff(h.greens(0), oc.greens())
        st = oc.state()
        chunk_boundary = st["current_range"] != st_before["current_range"] or \
            st["direction"] != st_before["direction"]
        if chunk_boundary:
            worst_stab = max(worst_stab, d)
        else:
            worst_wrap = max(worst_wrap, d)
    print(f"max |dG| mixed vs FP64: stabilisations {worst_stab:.2e}, wraps {worst_wrap:.2e}")
    assert worst_stab <= TOL_MIXED
    assert worst_wrap <= TOL_MIXED


def test_mixed_sweeps_track_fp64(pkg, lib, oracle):
    """Free-running mixed sweeps: the propagation error the chain reports at
    every stabilisation stays below 1e-6 and G matches a from-scratch FP64 G
    for the chain's own field configuration."""
    h, oc, param = _mixed_pair(pkg, lib, oracle, "MagneticHirschField", 8, 8.0, seed=11)
    h.init_random_field(0)
    h.initialize_run()
    st = h.sweep(3)[0]
    print(f"mixed propagation error max {st['max_propagation_error']:.2e}")
    assert st["max_propagation_error"] <= TOL_MIXED
    oc.set_conf(h.get_field(0))
    G = h.greens(0)
    Gref = oc.calculate_greens_at(st["current_slice"] - 1)
    assert maxdiff(G, Gref) <= TOL_MIXED


def test_mixed_16x16_beta10_every_stabilisation(pkg, lib, oracle):
    """The mixed-precision workload itself: 16x16 repulsive Hubbard (n = 256,
    two flavours), beta = 10, M = 100, safe_mult = 10.  G of the mixed path
    from scratch at every stabilisation slice (chunk boundary) against FP64:
    the FP64 oracle at three of them, the FP64 GPU path (itself pinned to the
    oracle at 1e-10) at all eleven."""
    model, param, fld, exps = make_setup(pkg, L=16, U=-4.0, beta=10.0, safe_mult=10,
                                         field=pkg.MagneticHirschField)
    cfg = [chain_config(lib, model, param, fld, 4)]
    hm = lib.Handle(cfg, precision=lib.PREC_MIXED)
    hd = lib.Handle(cfg, precision=lib.PREC_FP64)
    oc = oracle_chain(oracle, model, param, fld, exps, 4)
    for h in (hm, hd):
        h.set_hopping(-1, exps)
        h.init_random_field(0)
    oc.init_random_conf()
    assert np.array_equal(hm.get_field(0), oc.get_conf())
    bounds = sorted({0, param.slices} | {b for _, b in pkg.generate_chunks(param.slices, 10)})
    assert len(bounds) == 11
    worst_oracle, worst_fp64 = 0.0, 0.0
    for sl in bounds:
        gm = hm.calculate_greens(0, sl)
        worst_fp64 = max(worst_fp64, maxdiff(gm, hd.calculate_greens(0, sl)))
        if sl in (0, 50, 100):
            worst_oracle = max(worst_oracle, maxdiff(gm, oc.calculate_greens_at(sl)))
    print(f"16x16 beta=10: max |dG| mixed vs FP64 oracle {worst_oracle:.2e}, "
          f"vs FP64 GPU at every stabilisation {worst_fp64:.2e}")
    assert worst_oracle <= TOL_MIXED
    assert worst_fp64 <= TOL_MIXED


@pytest.mark.parametrize("L", [12, 16])
def test_mixed_two_flavour_honeycomb_large(pkg, lib, L):
    """Two-flavour mixed chains with nf * n above 512 (honeycomb, n = 288 and
    512; the largest lattices of the served stream): the double-float wraps
    stage one flavour block's diagonal at a time.  A free sweep keeps the
    propagation error and G within the bound of the FP64 path (itself pinned
    to the oracle at 1e-10) for the chain's own configuration."""
    model, param, fld, exps = make_setup(pkg, L=L, lattice="honeycomb", U=-4.0, beta=1.0,
                                         safe_mult=5, field=pkg.MagneticHirschField)
    assert fld.unique_flavors == 2 and len(model.l) == 2 * L * L
    cfg = [chain_config(lib, model, param, fld, 9)]
    hm = lib.Handle(cfg, precision=lib.PREC_MIXED)
    hd = lib.Handle(cfg, precision=lib.PREC_FP64)
    for h in (hm, hd):
        h.set_hopping(-1, exps)
        h.init_random_field(0)
    hm.initialize_run()
    st = hm.sweep(1)[0]
    assert st["status"] == 0
    assert st["max_propagation_error"] <= TOL_MIXED
    assert st["accepted"] > 0
    hd.set_field(0, hm.get_field(0))
    d = maxdiff(hm.greens(0), hd.calculate_greens(0, st["current_slice"] - 1))
    print(f"honeycomb L={L} (n={len(model.l)}) mixed vs FP64 max |dG| {d:.2e}")
    assert d <= TOL_MIXED
    hm.close()
    hd.close()
