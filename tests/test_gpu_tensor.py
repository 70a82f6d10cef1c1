"""Tensor-core split-precision products (tcgen05) of the mixed path.

Mixed chains with 96 <= n <= 256 run their wraps, slice-matrix chains and
reconstruction products as BF16 digit-slice MMAs on the tensor cores with
exact FP32 accumulation per digit level (about 46 correct bits).  Checked
against the FP64 oracle (max |dG| <= 1e-6, the mixed path's bound) and
against the same chain with the double-float FP32-pipe products (the two
products agree to ~1e-13 relative, so Green's functions to ~1e-9)."""
import numpy as np
import pytest

from _util import FIELD_U, chain_config, make_setup, maxdiff, oracle_chain

pytestmark = pytest.mark.gpu

TOL_MIXED = 1e-6


def _handles(pkg, lib, field, L, beta, safe_mult=10, seed=3):
    model, param, fld, exps = make_setup(pkg, L=L, U=FIELD_U[field], beta=beta,
                                         safe_mult=safe_mult, field=getattr(pkg, field))
    cfg = [chain_config(lib, model, param, fld, seed)]
    ht = lib.Handle(cfg, precision=lib.PREC_MIXED)
    ht.set_tensor_products(True)
    hd = lib.Handle(cfg, precision=lib.PREC_MIXED)
    hd.set_tensor_products(False)
    for h in (ht, hd):
        h.set_hopping(-1, exps)
        h.init_random_field(0)
    return ht, hd, model, param, fld, exps


@pytest.mark.parametrize("field,L,beta", [("DensityHirschField", 10, 4.0),
                                          ("MagneticHirschField", 12, 4.0)])
def test_tensor_calculate_greens(pkg, lib, oracle, field, L, beta):
    ht, hd, model, param, fld, exps = _handles(pkg, lib, field, L, beta)
    oc = oracle_chain(oracle, model, param, fld, exps, 3)
    oc.init_random_conf()
    assert np.array_equal(ht.get_field(0), oc.get_conf())
    worst_o, worst_d = 0.0, 0.0
    for sl in (0, 1, param.slices // 2, param.slices):
        gt = ht.calculate_greens(0, sl)
        worst_o = max(worst_o, maxdiff(gt, oc.calculate_greens_at(sl)))
        worst_d = max(worst_d, maxdiff(gt, hd.calculate_greens(0, sl)))
    print(f"n={L * L}: tensor vs FP64 oracle {worst_o:.2e}, vs double-float products {worst_d:.2e}")
    assert worst_o <= TOL_MIXED
    assert worst_d <= 1e-8


def test_tensor_sweeps_track_fp64(pkg, lib, oracle):
    """Free-running mixed sweeps on the tensor path (12 x 12, beta = 4):
    propagation error within the bound at every stabilisation, and the final
    G equals the FP64 oracle's from-scratch G of the chain's configuration."""
    ht, hd, model, param, fld, exps = _handles(pkg, lib, "DensityHirschField", 12, 4.0,
                                               safe_mult=5, seed=8)
    ht.initialize_run()
    st = ht.sweep(2)[0]
    print(f"tensor path propagation error max {st['max_propagation_error']:.2e}")
    assert st["status"] == 0
    assert st["max_propagation_error"] <= TOL_MIXED
    oc = oracle_chain(oracle, model, param, fld, exps, 8)
    oc.set_conf(ht.get_field(0))
    assert maxdiff(ht.greens(0), oc.calculate_greens_at(st["current_slice"] - 1)) <= TOL_MIXED


def test_tensor_switch_is_per_handle(pkg, lib):
    """With the tensor products off the chain reproduces the double-float
    path exactly (same operations); on, it differs only at rounding level."""
    ht, hd, model, param, fld, exps = _handles(pkg, lib, "DensityHirschField", 10, 2.0)
    h2 = lib.Handle([chain_config(lib, model, param, fld, 3)], precision=lib.PREC_MIXED)
    h2.set_tensor_products(False)
    h2.set_hopping(-1, exps)
    h2.init_random_field(0)
    a, b, c = (h.calculate_greens(0, 7) for h in (hd, h2, ht))
    assert np.array_equal(a, b)
    assert 0.0 < maxdiff(a, c) <= 1e-8


@pytest.mark.parametrize("tensor", [False, True])
def test_mixed_large_sweeps_track_fp64(pkg, lib, oracle, tensor):
    """Mixed chains with n > 64 keep G as float pairs in its global buffer
    between stabilisations (delayed updates and wraps in double-float): free
    sweeps on a 10 x 10 two-flavour lattice, with and without the tensor
    products, stay within the bound of the FP64 oracle."""
    model, param, fld, exps = make_setup(pkg, L=10, U=-4.0, beta=4.0, safe_mult=5,
                                         field=pkg.MagneticHirschField)
    h = lib.Handle([chain_config(lib, model, param, fld, 21)], precision=lib.PREC_MIXED)
    h.set_tensor_products(tensor)
    h.set_hopping(-1, exps)
    h.init_random_field(0)
    h.initialize_run()
    st = h.sweep(2)[0]
    print(f"n=100 mixed (tensor={tensor}) propagation error max {st['max_propagation_error']:.2e}")
    assert st["status"] == 0
    assert st["max_propagation_error"] <= TOL_MIXED
    assert st["accepted"] > 0
    oc = oracle_chain(oracle, model, param, fld, exps, 21)
    oc.set_conf(h.get_field(0))
    assert maxdiff(h.greens(0), oc.calculate_greens_at(st["current_slice"] - 1)) <= TOL_MIXED


def test_tune_tensor_probe(pkg, lib):
    """The autotuner times a 12 x 12 two-flavour mixed chain with and without
    the tensor-core products in one probe launch and caches the faster."""
    from montecarlo_gb300 import autotune
    m = pkg.HubbardModel(pkg.SquareLattice(12), U=-4.0)
    spec = [(m, pkg.MagneticHirschField, 2.0, 0.1, 5)]
    key = autotune.tensor_key(*spec[0][:4])
    autotune._TC_CACHE.pop(key, None)
    choice, ratio = autotune.tune_tensor(spec, ks=[5])
    assert ratio[0] == ratio[0] and ratio[0] > 0
    assert choice[0] == (ratio[0] > 1.0)
    assert autotune._TC_CACHE[key] == choice[0]
    autotune._TC_CACHE.pop(key, None)
