"""Golden fixtures (tests/golden/, made by tests/golden/make_golden.py from the
reference's known-answer recipes): the analytic U = 0 Green's function, exact
diagonalisation of the 2x2 model, and a fixed oracle trajectory that the CUDA
path must reproduce."""
import os

import numpy as np
import pytest

from _util import chain_config, maxdiff

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    return np.load(os.path.join(GOLDEN, name))


def test_oracle_matches_analytic_u0_fixture(pkg, oracle):
    d = _load("analytic_u0.npz")
    for name in ("square4", "chain6"):
        T, beta, G = d[name + "_T"], float(d[name + "_beta"]), d[name + "_G"]
        n = T.shape[0]
        param = pkg.DQMCParameters.make(beta=beta, delta_tau=0.1, safe_mult=5)
        exps = pkg.hopping_exponentials(T, param.delta_tau)
        c = oracle.OracleChain(n, 1, param.slices, 5, 0, 0.0, exps, 1)
        c.init_random_conf()
        for sl in (0, 3, param.slices):
            got = c.greens_physical(c.calculate_greens_at(sl))[0]
            assert maxdiff(got, G) < 1e-12, (name, sl)


def test_ed_matches_fixture(pkg):
    import ed
    d = _load("ed_2x2.npz")
    for U, key in ((-1.0, "Um"), (1.0, "Up")):
        model = pkg.HubbardModel(pkg.SquareLattice(2), U=U, mu=0.0)
        E = ed.HubbardED(4, model.l.bonds(), 1.0, U, 0.0, 1.0)
        assert maxdiff(E.greens(), d[key + "_G"]) < 1e-12
        assert maxdiff(E.double_occupancy(), d[key + "_docc"]) < 1e-12
        assert maxdiff(E.sdc_z(), d[key + "_sdcz"]) < 1e-12
        ph = np.cos(model.l.positions() @ np.array([np.pi, np.pi]))
        chi = [E.susceptibility_grid(k, ph, 0.1) for k in pkg.CORRELATIONS]
        assert maxdiff(chi, d[key + "_chi"]) < 1e-12


def _trajectory_setup(pkg):
    model = pkg.HubbardModel(pkg.SquareLattice(4), U=4.0)
    param = pkg.DQMCParameters.make(beta=1.0, delta_tau=0.1, safe_mult=5)
    fld = pkg.DensityHirschField(param, model)
    exps = pkg.hopping_exponentials(model.hopping_matrix(), param.delta_tau)
    return model, param, fld, exps


def test_oracle_reproduces_trajectory_fixture(pkg, oracle):
    d = _load("oracle_trajectory.npz")
    model, param, fld, exps = _trajectory_setup(pkg)
    c = oracle.OracleChain(16, 1, param.slices, 5, fld.kind, fld.alpha, exps, 7)
    c.init_random_conf()
    c.initialize_run()
    c.sweeps(2)
    assert np.array_equal(c.get_conf(), d["conf"])
    assert c.rng_counter() == int(d["counter"])
    assert c.analysis()["accepted"] == int(d["accepted"])
    assert maxdiff(c.greens(), d["G"]) < 1e-12


@pytest.mark.gpu
def test_cuda_path_reproduces_trajectory_fixture(pkg, lib):
    d = _load("oracle_trajectory.npz")
    model, param, fld, exps = _trajectory_setup(pkg)
    h = lib.Handle([chain_config(lib, model, param, fld, 7)])
    h.set_hopping(-1, exps)
    h.init_random_field(0)
    h.initialize_run()
    st = h.sweep(2)[0]
    assert np.array_equal(h.get_field(0), d["conf"])
    assert h.get_rng(0)[1] == int(d["counter"])
    assert st["accepted"] == int(d["accepted"])
    assert maxdiff(h.greens(0), d["G"]) < 1e-10


def test_complex_oracle_reproduces_trajectory_fixture(pkg):
    import sys
    sys.path.insert(0, GOLDEN)
    import complex_oracle as CO
    from make_golden import complex_trajectory
    d = _load("complex_trajectory.npz")
    got = complex_trajectory(pkg, CO)
    assert np.array_equal(got["conf0"], d["conf0"])
    assert np.array_equal(got["conf"], d["conf"])
    for k in ("counter", "accepted", "n_imag"):
        assert int(got[k]) == int(d[k]), k
    assert int(d["n_imag"]) > 0
    assert maxdiff(got["G"], d["G"]) < 1e-12
