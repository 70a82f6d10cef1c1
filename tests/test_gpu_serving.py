"""Pools: HBM-budget admission, time-sliced launches, continuous batching.

A chain advanced in a pool over many time slices must be bit-identical to the
same chain swept by a plain handle, and a request must give the same result
served alone and in a mix of other requests."""
import numpy as np
import pytest

from _util import FIELD_U, chain_config, make_setup, maxdiff, oracle_chain

pytestmark = pytest.mark.gpu


def test_pool_budget_admission(pkg, lib):
    model, param, fld, exps = make_setup(pkg, L=4, U=4.0, beta=1.0, safe_mult=5)
    cfg = chain_config(lib, model, param, fld, 1)
    need = lib.chain_bytes(cfg)
    pool = lib.Pool(4, int(2.5 * need) + 512)
    a = pool.admit(cfg)
    b = pool.admit(cfg)
    assert a is not None and b is not None and a != b
    assert pool.admit(cfg) is None  # over budget
    free_before = pool.free_bytes()
    pool.release(a)
    assert pool.free_bytes() > free_before
    c = pool.admit(cfg)
    assert c is not None
    pool.close()


@pytest.mark.parametrize("use_graph", [False, True])
def test_pool_time_slices_equal_plain_sweeps(pkg, lib, oracle, use_graph):
    model, param, fld, exps = make_setup(pkg, L=6, U=-4.0, beta=2.0, safe_mult=5)
    cfg = chain_config(lib, model, param, fld, 42)
    h = lib.Handle([cfg])
    h.set_hopping(0, exps)
    h.init_random_field(0)
    h.initialize_run()
    h.sweep(3)
    pool = lib.Pool(3, 3 * lib.chain_bytes(cfg) + 4096)
    slot = pool.admit(cfg)
    pool.set_hopping(slot, exps)
    pool.init_random_field(slot)
    pool.set_quota(slot, 3)
    runs = 0
    while pool.slot(slot)[1] > 0:
        pool.run(200, use_graph)  # 0.2 ms slices: many launches per sweep
        runs += 1
    assert runs > 3
    assert pool.slot(slot)[0] == 3
    assert np.array_equal(pool.get_field(slot), h.get_field(0))
    assert np.array_equal(pool.greens(slot), h.greens(0))
    assert pool.get_rng(slot) == h.get_rng(0)
    oc = oracle_chain(oracle, model, param, fld, exps, 42)
    oc.init_random_conf()
    oc.initialize_run()
    oc.sweeps(3)
    assert np.array_equal(pool.get_field(slot), oc.get_conf())
    assert maxdiff(pool.greens(slot), oc.greens()) < 1e-10
    pool.close()


def test_request_alone_equals_request_in_mix(pkg, lib):
    reqs = [pkg.Request(0, "square", 4, 4.0, 2.0, 30, 11),
            pkg.Request(1, "honeycomb", 2, -3.0, 4.0, 20, 12),
            pkg.Request(2, "square", 6, 2.0, 2.0, 25, 13, arrival=0.0),
            pkg.Request(3, "square", 4, -6.0, 1.0, 40, 14)]
    alone = pkg.Server(max_slots=2, budget_bytes=64 << 20, quantum_us=500)
    r_alone = alone.serve([reqs[0]], realtime=False)["results"][0]
    alone.close()
    mix = pkg.Server(max_slots=3, budget_bytes=64 << 20, quantum_us=300)
    out = mix.serve(reqs, realtime=False)
    mix.close()
    assert out["unfinished"] == 0 and len(out["results"]) == 4
    r_mix = out["results"][0]
    assert np.array_equal(r_alone.conf, r_mix.conf)
    assert np.array_equal(r_alone.greens, r_mix.greens)
    assert r_alone.stats["accepted"] == r_mix.stats["accepted"]
    assert out["p50_block_s"] is not None and out["p99_block_s"] >= out["p50_block_s"]


def test_uneven_ensemble_time_sliced(pkg, lib):
    specs = [(4, 4.0, 2.0), (6, 3.0, 4.0), (8, 6.0, 1.0), (3, 2.0, 2.0)]
    ce = []
    for i, (L, U, beta) in enumerate(specs):
        model, param, fld, exps = make_setup(pkg, L=L, U=U, beta=beta, safe_mult=10)
        ce.append((chain_config(lib, model, param, fld, 500 + i), exps))
    out = pkg.run_ensemble(ce, seconds=0.5, quantum_us=20000)
    assert out["sweeps"] > 0 and all(s > 0 for s in out["per_chain"])
    # smaller chains do more sweeps in the same slices
    assert out["per_chain"][3] > out["per_chain"][2]
    assert out["max_propagation_error"] < 1e-6


@pytest.mark.parametrize("use_graph", [False, True])
def test_pool_time_slice_is_work_conserving(pkg, lib, use_graph):
    """A chain past its time budget keeps visiting while another chain of the
    launch is not (here: a 12 x 12 chain still building its stack), instead
    of leaving its SM idle; alone, a chain stops at the first visit past the
    budget (1 microsecond: exactly one visit)."""
    small = make_setup(pkg, L=4, U=4.0, beta=1.0, safe_mult=5)
    big = make_setup(pkg, L=12, U=4.0, beta=2.0, safe_mult=5)

    def admit(pool, setup, seed):
        model, param, fld, exps = setup
        s = pool.admit(chain_config(lib, model, param, fld, seed))
        pool.set_hopping(s, exps)
        pool.init_random_field(s)
        pool.set_quota(s, 1000)
        return s

    alone = lib.Pool(2, 64 << 20)
    s0 = admit(alone, small, 3)
    alone.run(1, use_graph)
    assert alone.stats(s0)["proposals"] == 16  # one visit of the 16 sites
    alone.close()

    pool = lib.Pool(2, 1 << 30)
    sb = admit(pool, big, 4)
    ss = admit(pool, small, 3)
    pool.run(1, use_graph)
    visits_big = pool.stats(sb)["proposals"] // 144
    visits_small = pool.stats(ss)["proposals"] // 16
    assert visits_big >= 1
    assert visits_small >= 10, (visits_small, visits_big)
    pool.close()


@pytest.mark.parametrize("prec,L", [("fp64", 4), ("fp64", 8), ("fp64", 10), ("mixed", 8),
                                    ("mixed", 12)])
def test_flavour_split_chain_equals_one_cta(pkg, lib, prec, L):
    """A two-flavour chain whose flavour blocks run on the two CTAs of a
    two-CTA cluster (n = 64: shared-memory QR and G; n = 100: G in global
    memory with delayed updates; mixed n = 144: tensor-core products and
    float-pair G) gives bit-identical fields, Green's function and counters
    to the chain on one CTA; a one-flavour chain in the same pool, and a
    two-flavour chain too small to split (n = 16), run on one CTA of their
    pair."""
    split_equals_one_cta(pkg, lib, prec, L)


def split_equals_one_cta(pkg, lib, prec, L):
    precision = lib.PREC_MIXED if prec == "mixed" else lib.PREC_FP64
    two = make_setup(pkg, L=L, U=-4.0, beta=2.0 if L <= 8 else 1.0, safe_mult=5,
                     field=pkg.MagneticHirschField)
    one = make_setup(pkg, L=4, U=4.0, beta=1.0, safe_mult=5, field=pkg.DensityHirschField)
    assert two[2].unique_flavors == 2 and one[2].unique_flavors == 1
    out = []
    for fsplit in (False, True):
        pool = lib.Pool(4, 1 << 30, precision=precision)
        pool.set_flavour_split(fsplit)
        slots = []
        for (model, param, fld, exps), seed in ((two, 21), (one, 22)):
            s = pool.admit(chain_config(lib, model, param, fld, seed))
            pool.set_hopping(s, exps)
            pool.init_random_field(s)
            pool.set_quota(s, 2)
            slots.append(s)
        pool.run(30_000_000, True)  # one slice covers both sweeps of both chains
        res = []
        for s in slots:
            done, left, _ = pool.slot(s)
            assert (done, left) == (2, 0)
            st = pool.stats(s)
            assert st["status"] == 0
            res.append((pool.get_field(s), pool.greens(s), st))
        out.append(res)
        pool.close()
    for (f0, g0, s0), (f1, g1, s1) in zip(out[0], out[1]):
        assert np.array_equal(f0, f1)
        assert np.array_equal(g0, g1)
        for k in ("accepted", "proposals", "near_ties", "max_propagation_error"):
            assert s0[k] == s1[k], k


def test_flavour_split_rendezvous_time_out(pkg, lib):
    """The two CTAs of a flavour-split chain wait at most 2 s for each other
    at a rendezvous.  When the second CTA stops announcing itself (the test
    hook: a flag that nothing sets any more), the first one's wait runs out:
    the chain reports status 9, dqmc_pool_run fails naming the slot, the
    launch ends within seconds (both CTAs finish without further waits), and
    the device stays usable: the next pools on it give bit-identical results
    split and unsplit."""
    import time

    two = make_setup(pkg, L=8, U=-4.0, beta=2.0, safe_mult=5, field=pkg.MagneticHirschField)
    model, param, fld, exps = two
    pool = lib.Pool(2, 1 << 30, precision=lib.PREC_FP64)
    pool.set_flavour_split(True)
    s = pool.admit(chain_config(lib, model, param, fld, 31))
    pool.set_hopping(s, exps)
    pool.init_random_field(s)
    pool.set_quota(s, 2)
    pool.set_split_silence(s, 5)
    t0 = time.perf_counter()
    with pytest.raises(lib.DQMCError) as err:
        pool.run(30_000_000, True)
    elapsed = time.perf_counter() - t0
    assert "status 9" in str(err.value), str(err.value)
    assert elapsed < 30.0, elapsed
    assert pool.stats(s)["status"] == 9
    pool.close()
    split_equals_one_cta(pkg, lib, "fp64", 8)
