"""Global updates (GlobalFlip, GlobalShuffle, global_updates.jl) and replica
exchange between chains of one handle (ReplicaExchange, parallel_updates.jl)
on the GPU against the oracle under the replayed Philox stream: accepted
flags, configurations and stream counters bit-identical, G to 1e-10."""
import numpy as np
import pytest

from _util import FIELD_U, FIELDS, chain_config, make_setup, maxdiff, oracle_chain

pytestmark = pytest.mark.gpu

TOL_G = 1e-10


def _pairs(pkg, lib, oracle, specs, seed0=60):
    cfgs, ocs, exps_l = [], [], []
    for j, (L, field, U, mu, beta) in enumerate(specs):
        model, param, fld, exps = make_setup(pkg, L=L, U=U, mu=mu, beta=beta, safe_mult=5,
                                             field=getattr(pkg, field))
        cfgs.append(chain_config(lib, model, param, fld, seed0 + j))
        ocs.append(oracle_chain(oracle, model, param, fld, exps, seed0 + j))
        exps_l.append(exps)
    h = lib.Handle(cfgs)
    for j, e in enumerate(exps_l):
        h.set_hopping(j, e)
    h.init_random_field(-1)
    h.initialize_run()
    for o in ocs:
        o.init_random_conf()
        o.initialize_run()
    return h, ocs


def _same(h, ocs):
    for j, o in enumerate(ocs):
        assert np.array_equal(h.get_field(j), o.get_conf()), j
        assert h.get_rng(j)[1] == o.rng_counter(), j
        assert maxdiff(h.greens(j), o.greens()) < TOL_G, j


@pytest.mark.parametrize("field", FIELDS)
def test_global_flip_and_shuffle_replay_oracle(pkg, lib, oracle, field):
    """A flip of a magnetic field is an exact symmetry (up <-> down): its
    determinant ratio is 1 up to rounding, so whether p > 1 (no uniform drawn)
    depends on the last bit.  For those moves the test checks the move itself
    and re-aligns the stream position; every other move replays bit-exactly."""
    mu = 0.3 if field.startswith("Density") else 0.0
    magnetic = field.startswith("Magnetic")
    specs = [(4, field, FIELD_U[field], mu, 2.0), (3, field, FIELD_U[field], mu, 1.0)]
    h, ocs = _pairs(pkg, lib, oracle, specs)
    for k in range(4):
        kind = k % 2
        acc = h.global_update(kind)
        for j, o in enumerate(ocs):
            oacc = o.global_update(kind)
            if magnetic and kind == 0:
                cur = o.get_conf().astype(np.int16)
                flipped = (5 - cur) if "GHQ" in field else -cur
                d, _ = o.global_detratio(flipped.astype(np.int8))  # a flip back: ratio 1
                assert abs(d - 1.0) < 1e-9
                assert bool(acc[j]) and oacc
                h.set_rng(j, h.get_rng(j)[0], o.rng_counter())
            else:
                assert bool(acc[j]) == oacc, (k, j)
        _same(h, ocs)
        h.sweep(1)
        for o in ocs:
            o.sweeps(1)
        _same(h, ocs)
    for j, o in enumerate(ocs):
        assert h.global_stats(j) == o.global_stats()


def test_scheduled_global_update_in_the_sweep_launch(pkg, lib, oracle):
    """SimpleScheduler(LocalSweep(), GlobalFlip()): a global move before every
    sweep but the first, inside one launch, equals the explicit sequence."""
    spec = [(4, "DensityHirschField", 4.0, 0.5, 2.0)]
    h, ocs = _pairs(pkg, lib, oracle, spec, seed0=90)
    h.set_global_schedule(lib.GLOBAL_FLIP)
    h.sweep(5)
    o = ocs[0]
    for s in range(5):
        if s > 0:
            o.global_update(0)
        o.sweeps(1)
    _same(h, ocs)
    assert h.global_stats(0) == o.global_stats() and o.global_stats()[1] == 4
    h.set_global_schedule(None)
    h.sweep(1)
    o.sweeps(1)
    _same(h, ocs)


def test_replica_exchange_replays_oracle(pkg, lib, oracle):
    """Pairs of chains at different U exchange configurations (parallel
    tempering in U on one GPU): weights, the lower index's uniform and the
    swap replay the oracle."""
    specs = [(4, "MagneticHirschField", -4.0, 0.0, 2.0), (4, "MagneticHirschField", -2.5, 0.0, 2.0),
             (4, "DensityHirschField", 4.0, 0.3, 2.0), (4, "DensityHirschField", 3.0, 0.3, 2.0)]
    h, ocs = _pairs(pkg, lib, oracle, specs, seed0=120)
    partners = [1, 0, 3, 2]
    n_acc = 0
    for k in range(4):
        h.sweep(1)
        for o in ocs:
            o.sweeps(1)
        acc = h.replica_exchange(partners)
        confs = [o.get_conf() for o in ocs]
        wp = [o.replica_weight(confs[partners[j]]) for j, o in enumerate(ocs)]
        for a in (0, 2):
            b = partners[a]
            w = wp[a][0] * wp[b][0]
            ok = wp[a][1] < w
            assert bool(acc[a]) == ok and bool(acc[b]) == ok, (k, a)
            if ok:
                ocs[a].replica_accept(confs[b])
                ocs[b].replica_accept(confs[a])
                n_acc += 1
        _same(h, ocs)
    assert n_acc > 0


def test_global_update_needs_chains_between_sweeps(pkg, lib):
    model, param, fld, exps = make_setup(pkg, L=2, U=4.0, beta=1.0)
    h = lib.Handle([chain_config(lib, model, param, fld, 5)])
    h.set_hopping(0, exps)
    h.init_random_field(0)
    h.initialize_run()
    h.propagate()  # now at slice 2
    with pytest.raises(lib.DQMCError) as e:
        h.global_update(lib.GLOBAL_FLIP)
    assert e.value.code == 1
    with pytest.raises(lib.DQMCError):
        h.replica_exchange([0])


def test_parallel_tempering_in_u(pkg, lib):
    """Four replicas of the 4x4 repulsive model at U = 2, 3, 4, 5 exchange
    configurations with their neighbours every sweep; the device
    observables order with U (double occupancy falls as U grows)."""
    reps = [(pkg.HubbardModel(pkg.SquareLattice(4), U=-u), 2.0, 0.1, 10, 300 + j)
            for j, u in enumerate((2.0, 3.0, 4.0, 5.0))]
    out = pkg.run_tempering(reps, rounds=60, thermalization=20)
    assert len(out["exchange_acceptance"]) == 3
    assert all(0.0 <= a <= 1.0 for a in out["exchange_acceptance"])
    assert sum(out["exchanges_tried"]) == 90
    assert sum(a for a, _ in out["global_stats"]) > 0
    docc = [o["double_occupancy"][0] for o in out["observables"]]
    assert docc[0] > docc[-1]
    assert all(o["count"] == 60 for o in out["observables"])
