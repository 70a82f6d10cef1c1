"""checkerboard = true: the hopping exponentials as products of site-disjoint
bond factors (linalg/checkerboard.jl) on the GPU against the oracle with the
same factors: G to 1e-10, sweeps replayed bit-exactly."""
import numpy as np
import pytest

from _util import FIELD_U, chain_config, make_setup, maxdiff, oracle_chain

pytestmark = pytest.mark.gpu

TOL_G = 1e-10


def _cb_pair(pkg, lib, oracle, field, L, lattice="square", beta=2.0, k=5, seed=41,
             precision=None):
    from montecarlo_gb300 import model as M
    model, param, fld, exps = make_setup(pkg, L=L, lattice=lattice, U=FIELD_U[field], beta=beta,
                                         safe_mult=k, field=getattr(pkg, field))
    data, npart = M.checkerboard_pack(
        M.checkerboard_exponentials(model.hopping_matrix(), model.l, param.delta_tau))
    h = lib.Handle([chain_config(lib, model, param, fld, seed)],
                   precision=lib.PREC_FP64 if precision is None else precision)
    h.set_hopping(-1, exps)
    h.set_checkerboard(0, data, npart)
    o = oracle_chain(oracle, model, param, fld, exps, seed)
    o.set_checkerboard(data, npart)
    return h, o, param


@pytest.mark.parametrize("field,L,lattice", [("DensityHirschField", 3, "square"),
                                             ("MagneticHirschField", 3, "square"),
                                             ("MagneticHirschField", 8, "square"),
                                             ("MagneticGHQField", 2, "honeycomb"),
                                             ("DensityHirschField", 10, "square")])
def test_checkerboard_replays_oracle(pkg, lib, oracle, field, L, lattice):
    h, o, param = _cb_pair(pkg, lib, oracle, field, L, lattice)
    h.init_random_field(0)
    o.init_random_conf()
    for sl in (0, 4, param.slices):
        assert maxdiff(h.calculate_greens(0, sl), o.calculate_greens_at(sl)) < TOL_G, sl
    h.initialize_run()
    o.initialize_run()
    for _ in range(2):
        h.sweep(1)
        o.sweeps(1)
        assert np.array_equal(h.get_field(0), o.get_conf())
        assert h.get_rng(0)[1] == o.rng_counter()
        assert maxdiff(h.greens(0), o.greens()) < TOL_G
    assert maxdiff(h.greens(0, physical=True), o.greens_physical(o.greens())) < TOL_G


def test_checkerboard_mixed_chain_is_fp64(pkg, lib, oracle):
    """A chain with checkerboard factors computes its slice products in FP64
    on either precision: the two precisions give the same bits."""
    h1, _, _ = _cb_pair(pkg, lib, oracle, "MagneticHirschField", 8, seed=5)
    h2, _, _ = _cb_pair(pkg, lib, oracle, "MagneticHirschField", 8, seed=5,
                        precision=lib.PREC_MIXED)
    for h in (h1, h2):
        h.init_random_field(0)
        h.initialize_run()
        h.sweep(2)
    assert np.array_equal(h1.get_field(0), h2.get_field(0))
    assert np.array_equal(h1.greens(0), h2.greens(0))


def test_dqmc_checkerboard_run(pkg):
    model = pkg.HubbardModel(pkg.SquareLattice(4), U=-4.0)
    mc = pkg.DQMC(model, beta=2.0, delta_tau=0.1, safe_mult=10, seed=3, thermalization=5,
                  sweeps=20, measure_rate=1, checkerboard=True)
    assert pkg.run(mc) == pkg.ExitCode.SUCCESS
    assert mc.analysis["max_propagation_error"] < 1e-6
    assert 0.0 < mc.observables()["double_occupancy"][0] < 0.25
