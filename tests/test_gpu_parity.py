"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

Tolerances: the reference's calculate_greens parity target is 1e-10 absolute
in FP64 for a given field configuration; accept/reject decisions, field
configurations and RNG counters must be bit-identical under the replayed
Philox stream.
"""
import numpy as np
import pytest

from _util import FIELD_U, FIELDS, chain_config, make_setup, maxdiff, oracle_chain

pytestmark = pytest.mark.gpu

TOL_G = 1e-10


def _pair(pkg, lib, oracle, field, L=4, lattice="square", beta=2.0, safe_mult=5, seed=11, U=None):
    fcls = getattr(pkg, field)
    U = FIELD_U[field] if U is None else U
    model, param, fld, exps = make_setup(pkg, L=L, lattice=lattice, U=U, beta=beta,
                                         safe_mult=safe_mult, field=fcls)
    h = lib.Handle([chain_config(lib, model, param, fld, seed)])
    h.set_hopping(-1, exps)
    oc = oracle_chain(oracle, model, param, fld, exps, seed)
    return h, oc, model, param, fld


@pytest.mark.parametrize("field", FIELDS)
def test_calculate_greens_matches_oracle(pkg, lib, oracle, field):
    h, oc, model, param, fld = _pair(pkg, lib, oracle, field)
    h.init_random_field(0)
    oc.init_random_conf()
    assert np.array_equal(h.get_field(0), oc.get_conf())
    for sl in (0, 1, 7, 10, param.slices):
        g_gpu = h.calculate_greens(0, sl)
        g_cpu = oc.calculate_greens_at(sl)
        assert maxdiff(g_gpu, g_cpu) < TOL_G, (sl, maxdiff(g_gpu, g_cpu))
    # safe_mult override (calculate_greens(mc, slice, ..., safe_mult))
    assert maxdiff(h.calculate_greens(0, 3, 2), oc.calculate_greens_at(3, 2)) < TOL_G


@pytest.mark.parametrize("field", FIELDS)
def test_initialize_run_stack_and_greens(pkg, lib, oracle, field):
    h, oc, model, param, fld = _pair(pkg, lib, oracle, field)
    h.init_random_field(0)
    oc.init_random_conf()
    h.initialize_run()
    oc.initialize_run()
    st = h.stats(0)
    ost = oc.state()
    assert (st["current_slice"], st["current_range"], st["direction"]) == \
        (ost["current_slice"], ost["current_range"], ost["direction"])
    assert maxdiff(h.greens(0), oc.greens()) < TOL_G
    for idx in range(1, ost["n_ranges"] + 2):
        # u/t stacks may differ by pivot ties only in degenerate cases; compare the products
        U, D, T = h.stack(0, 0, idx), h.stack(0, 2, idx), h.stack(0, 1, idx)
        Uo, Do, To = oc.stack(0, idx), oc.stack(2, idx), oc.stack(1, idx)
        for b in range(fld.unique_flavors):
            A = U[b] @ np.diag(D[b]) @ T[b]
            Ao = Uo[b] @ np.diag(Do[b]) @ To[b]
            assert maxdiff(A, Ao) <= 1e-10 * max(1.0, np.abs(Ao).max())
    assert maxdiff(h.greens(0, physical=True), oc.greens_physical(oc.greens())) < TOL_G


@pytest.mark.parametrize("field", FIELDS)
def test_sweeps_replay_bit_exact(pkg, lib, oracle, field):
    h, oc, model, param, fld = _pair(pkg, lib, oracle, field, beta=2.0, safe_mult=5, seed=2024)
    h.init_random_field(0)
    oc.init_random_conf()
    h.initialize_run()
    oc.initialize_run()
    for _ in range(3):
        st = h.sweep(1)[0]
        acc = oc.sweeps(1)
        assert np.array_equal(h.get_field(0), oc.get_conf())
        assert h.get_rng(0)[1] == oc.rng_counter()
        assert st["accepted"] == oc.analysis()["accepted"]
        assert maxdiff(h.greens(0), oc.greens()) < TOL_G
    assert acc > 0


def test_build_stack_and_propagate_steps(pkg, lib, oracle):
    h, oc, model, param, fld = _pair(pkg, lib, oracle, "MagneticHirschField", beta=2.0,
                                     safe_mult=5)
    h.init_random_field(0)
    oc.init_random_conf()
    h.build_stack()
    oc.build_stack()
    assert maxdiff(h.greens(0), oc.greens()) < TOL_G
    # walk through both directions, including every stabilisation and flip
    for step in range(2 * param.slices + 3):
        h.propagate()
        oc.propagate()
        st, ost = h.stats(0), oc.state()
        assert (st["current_slice"], st["current_range"], st["direction"]) == \
            (ost["current_slice"], ost["current_range"], ost["direction"]), step
        assert maxdiff(h.greens(0), oc.greens()) < TOL_G, step


def test_sweep_spatial_rank1(pkg, lib, oracle):
    h, oc, model, param, fld = _pair(pkg, lib, oracle, "DensityHirschField", seed=5)
    h.init_random_field(0)
    oc.init_random_conf()
    h.initialize_run()
    oc.initialize_run()
    for _ in range(4):
        h.sweep_spatial()
        oc.sweep_spatial()
        assert np.array_equal(h.get_field(0), oc.get_conf())
        assert maxdiff(h.greens(0), oc.greens()) < TOL_G
        h.propagate()
        oc.propagate()


@pytest.mark.parametrize("lattice,L,field", [("honeycomb", 2, "MagneticHirschField"),
                                             ("square", 8, "MagneticHirschField"),
                                             ("chain", 6, "DensityGHQField")])
def test_other_lattices(pkg, lib, oracle, lattice, L, field):
    h, oc, model, param, fld = _pair(pkg, lib, oracle, field, L=L, lattice=lattice, beta=1.0,
                                     safe_mult=4, seed=77)
    h.init_random_field(0)
    oc.init_random_conf()
    h.initialize_run()
    oc.initialize_run()
    h.sweep(1)
    oc.sweeps(1)
    assert np.array_equal(h.get_field(0), oc.get_conf())
    assert maxdiff(h.greens(0), oc.greens()) < TOL_G


def test_uneven_batch_one_launch(pkg, lib, oracle):
    """Chains of different size, field and length advance in one launch, each
    exactly as it would alone."""
    specs = [(4, "DensityHirschField", 2.0, 3), (6, "MagneticHirschField", 1.0, 4),
             (2, "MagneticGHQField", 1.5, 5), (5, "DensityGHQField", 1.0, 7)]
    cfgs, ocs, setups = [], [], []
    for i, (L, field, beta, k) in enumerate(specs):
        model, param, fld, exps = make_setup(pkg, L=L, U=FIELD_U[field], beta=beta, safe_mult=k,
                                             field=getattr(pkg, field))
        cfgs.append(chain_config(lib, model, param, fld, 100 + i))
        ocs.append(oracle_chain(oracle, model, param, fld, exps, 100 + i))
        setups.append(exps)
    h = lib.Handle(cfgs)
    for i, exps in enumerate(setups):
        h.set_hopping(i, exps)
    h.init_random_field(-1)
    for oc in ocs:
        oc.init_random_conf()
        oc.initialize_run()
    h.initialize_run()
    h.sweep(2)
    for i, oc in enumerate(ocs):
        oc.sweeps(2)
        assert np.array_equal(h.get_field(i), oc.get_conf()), i
        assert maxdiff(h.greens(i), oc.greens()) < TOL_G, i


def test_async_sweep_and_query(pkg, lib, oracle):
    h, oc, model, param, fld = _pair(pkg, lib, oracle, "DensityHirschField")
    h.init_random_field(0)
    h.initialize_run()
    h.sweep_async(2)
    while not h.query():
        pass
    st = h.stats(0)
    assert st["proposals"] == 2 * 2 * param.slices * len(model.l)


@pytest.mark.parametrize("lattice,L,field", [("square", 10, "DensityHirschField"),
                                             ("honeycomb", 6, "MagneticHirschField")])
def test_large_n_delayed_updates(pkg, lib, oracle, lattice, L, field):
    """n > 64: G stays in global memory and the rank-1 updates are applied in
    delayed blocks; decisions and fields still replay the oracle exactly."""
    h, oc, model, param, fld = _pair(pkg, lib, oracle, field, L=L, lattice=lattice, beta=1.0,
                                     safe_mult=5, seed=31)
    assert len(model.l) > 64
    h.init_random_field(0)
    oc.init_random_conf()
    h.initialize_run()
    oc.initialize_run()
    h.sweep(1)
    oc.sweeps(1)
    assert np.array_equal(h.get_field(0), oc.get_conf())
    assert maxdiff(h.greens(0), oc.greens()) < TOL_G


def test_max_size_16x16_two_flavours(pkg, lib, oracle):
    """The largest lattice of the workloads (16x16, n = 256, two flavours):
    G from scratch at several slices, then one full sweep replayed bit-exactly
    (G in global memory, delayed rank-16 updates)."""
    h, oc, model, param, fld = _pair(pkg, lib, oracle, "MagneticHirschField", L=16, beta=2.0,
                                     safe_mult=10, seed=9)
    assert len(model.l) == 256
    h.init_random_field(0)
    oc.init_random_conf()
    for sl in (0, 10, param.slices):
        assert maxdiff(h.calculate_greens(0, sl), oc.calculate_greens_at(sl)) < TOL_G, sl
    h.initialize_run()
    oc.initialize_run()
    h.sweep(1)
    oc.sweeps(1)
    assert np.array_equal(h.get_field(0), oc.get_conf())
    assert h.get_rng(0)[1] == oc.rng_counter()
    assert maxdiff(h.greens(0), oc.greens()) < TOL_G


def test_max_size_honeycomb_512_sites(pkg, lib, oracle):
    """The largest chain the library takes (n_sites = 512: the honeycomb
    L = 16 of the served stream), two flavours, short beta: G from scratch
    and one sweep replayed bit-exactly against the oracle."""
    h, oc, model, param, fld = _pair(pkg, lib, oracle, "MagneticHirschField", L=16,
                                     lattice="honeycomb", beta=0.5, safe_mult=5, seed=12)
    assert len(model.l) == 512
    h.init_random_field(0)
    oc.init_random_conf()
    for sl in (0, 3, param.slices):
        g = h.calculate_greens(0, sl)
        assert maxdiff(g, oc.calculate_greens_at(sl)) < TOL_G, sl
    h.initialize_run()
    oc.initialize_run()
    h.sweep(1)
    oc.sweeps(1)
    assert np.array_equal(h.get_field(0), oc.get_conf())
    assert h.get_rng(0)[1] == oc.rng_counter()
    assert maxdiff(h.greens(0), oc.greens()) < TOL_G


def test_negative_probability_magnitude_stats(pkg, lib, oracle):
    """A sign problem (repulsive U away from half filling): the device counts
    the same negative probabilities as the oracle and reports the
    MagnitudeStats min <= geometric mean <= max of |p| (statistics.jl:9-36)."""
    from _util import chain_config, make_setup, oracle_chain
    model, param, fld, exps = make_setup(pkg, L=4, U=-8.0, mu=1.0, beta=4.0, safe_mult=5,
                                         field=pkg.MagneticHirschField)
    h = lib.Handle([chain_config(lib, model, param, fld, 21)])
    h.set_hopping(-1, exps)
    h.init_random_field(0)
    oc = oracle_chain(oracle, model, param, fld, exps, 21)
    oc.init_random_conf()
    h.initialize_run()
    oc.initialize_run()
    st = h.sweep(3)[0]
    oc.sweeps(3)
    assert np.array_equal(h.get_field(0), oc.get_conf())
    n_neg = oc.analysis()["negative_probability"]
    assert st["negative_probability"] == n_neg > 0
    assert 0 < st["min_negative_probability"] <= st["mean_negative_probability"] \
        <= st["max_negative_probability"] * (1 + 1e-12)
