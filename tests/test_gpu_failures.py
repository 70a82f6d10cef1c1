"""Failure detection without a GPU fault: failures are made on the host
(invalid inputs, non-finite matrices) and must come back as error statuses
with the context still usable."""
import numpy as np
import pytest

from _util import chain_config, make_setup

pytestmark = pytest.mark.gpu


def test_nan_hopping_reports_numerical_error(pkg, lib):
    model, param, fld, exps = make_setup(pkg, L=4, U=4.0, beta=1.0, safe_mult=5)
    h = lib.Handle([chain_config(lib, model, param, fld, 3)])
    bad = [e.copy() for e in exps]
    bad[0][0, 0] = np.nan
    h.set_hopping(0, bad)
    h.init_random_field(0)
    with pytest.raises(lib.DQMCError) as ei:
        h.initialize_run()
        h.sweep(1)
    assert ei.value.code == 4
    h.close()
    # the device is still usable afterwards
    h2 = lib.Handle([chain_config(lib, model, param, fld, 3)])
    h2.set_hopping(0, exps)
    h2.init_random_field(0)
    h2.initialize_run()
    h2.sweep(1)
    assert np.isfinite(h2.greens(0)).all()
    h2.close()


def test_invalid_inputs_rejected(pkg, lib):
    model, param, fld, exps = make_setup(pkg, L=4, U=4.0, beta=1.0, safe_mult=5)
    h = lib.Handle([chain_config(lib, model, param, fld, 3)])
    with pytest.raises(lib.DQMCError) as ei:
        h.set_field(0, np.full((16, param.slices), 3, dtype=np.int8))  # not +-1
    assert ei.value.code == 1
    with pytest.raises(lib.DQMCError):
        h.calculate_greens(0, param.slices + 1)
    with pytest.raises(lib.DQMCError):
        h.greens(5)
    h.close()


def test_autotuner_respects_tolerance(pkg, lib):
    specs = []
    for U, beta in ((2.0, 2.0), (8.0, 8.0)):
        model = pkg.HubbardModel(pkg.SquareLattice(6), U=U)
        specs.append((model, model.choose_field(), beta, 0.1, 7))
    from montecarlo_gb300 import autotune
    ks, errs = autotune.tune_safe_mult(specs, tol=1e-6)
    assert all(e <= 0.5e-6 for e in errs), (ks, errs)
    assert ks[0] >= ks[1]  # weak coupling, short beta stabilises less often
