"""The warp-per-chain sweep kernel of small lattices (n <= 32) against the
CTA-per-chain kernel and the oracle: field configurations, RNG counters and
accepted counts bit-identical, G to 1e-10, for both field families, one and
two flavour blocks, n from 4 to 32."""
import numpy as np
import pytest

from _util import FIELD_U, chain_config, make_setup, maxdiff, oracle_chain

pytestmark = pytest.mark.gpu

CASES = [("DensityHirschField", 2, "square"), ("MagneticHirschField", 3, "square"),
         ("MagneticHirschField", 4, "square"), ("DensityGHQField", 4, "square"),
         ("MagneticGHQField", 3, "honeycomb"), ("DensityHirschField", 5, "square"),
         ("MagneticHirschField", 4, "honeycomb")]


@pytest.mark.parametrize("field,L,lattice", CASES)
def test_warp_kernel_replays_oracle_and_cta_kernel(pkg, lib, oracle, field, L, lattice):
    model, param, fld, exps = make_setup(pkg, L=L, lattice=lattice, U=FIELD_U[field], beta=2.0,
                                         safe_mult=5, field=getattr(pkg, field))
    n = len(model.l)
    assert n <= 32
    hs = []
    for small in (True, False):
        h = lib.Handle([chain_config(lib, model, param, fld, 100 + j) for j in range(11)])
        h.set_small_chain_kernel(small)
        h.set_hopping(-1, exps)
        h.init_random_field(-1)
        h.initialize_run()
        hs.append(h)
    oc = oracle_chain(oracle, model, param, fld, exps, 100)
    oc.init_random_conf()
    oc.initialize_run()
    for _ in range(3):
        sts = [h.sweep(1) for h in hs]
        oc.sweeps(1)
        for j in range(11):
            assert np.array_equal(hs[0].get_field(j), hs[1].get_field(j)), j
            assert hs[0].get_rng(j) == hs[1].get_rng(j)
            assert sts[0][j]["accepted"] == sts[1][j]["accepted"]
            assert maxdiff(hs[0].greens(j), hs[1].greens(j)) < 1e-10
        assert np.array_equal(hs[0].get_field(0), oc.get_conf())
        assert hs[0].get_rng(0)[1] == oc.rng_counter()
        assert maxdiff(hs[0].greens(0), oc.greens()) < 1e-10
    st = sts[0][0]
    assert (st["current_slice"], st["current_range"], st["direction"]) == \
        tuple(oc.state()[k] for k in ("current_slice", "current_range", "direction"))
    assert st["max_propagation_error"] < 1e-8
    assert sum(hs[0].timers(0).values()) > 0


def test_warp_kernel_mixed_batch_and_async(pkg, lib):
    """Uneven chains (n = 4, 9, 16) in one warp-kernel launch, queued
    asynchronously, equal the same chains swept one handle each."""
    setups = [make_setup(pkg, L=L, U=-4.0, beta=1.0 + 0.5 * L, safe_mult=4) for L in (2, 3, 4)]
    cfgs = [chain_config(lib, m, p, f, 7 + i) for i, (m, p, f, e) in enumerate(setups)]
    h = lib.Handle(cfgs)
    for i, (m, p, f, e) in enumerate(setups):
        h.set_hopping(i, e)
    h.init_random_field(-1)
    h.initialize_run()
    for _ in range(3):
        h.sweep_async(1)
    h.synchronize()
    for i, (m, p, f, e) in enumerate(setups):
        h1 = lib.Handle([cfgs[i]])
        h1.set_hopping(0, e)
        h1.init_random_field(0)
        h1.initialize_run()
        h1.sweep(3)
        assert np.array_equal(h.get_field(i), h1.get_field(0))
        assert maxdiff(h.greens(i), h1.greens(0)) < 1e-12


def test_batched_transfers_equal_per_chain(pkg, lib):
    """dqmc_get_greens_batch / dqmc_get_fields_batch / dqmc_set_fields_batch
    (one strided copy for equal chains, chain by chain otherwise) move the
    same bytes as the per-chain calls."""
    for Ls in ((4, 4, 4, 4, 4), (2, 4, 3)):
        setups = [make_setup(pkg, L=L, U=-4.0, beta=2.0, safe_mult=5) for L in Ls]
        cfgs = [chain_config(lib, m, p, f, 50 + i) for i, (m, p, f, e) in enumerate(setups)]
        h = lib.Handle(cfgs)
        for i, s in enumerate(setups):
            h.set_hopping(i, s[3])
        sizes = [len(m.l) * p.slices for m, p, f, e in setups]
        rng = np.random.default_rng(len(Ls))
        conf = rng.choice(np.array([-1, 1], dtype=np.int8), size=sum(sizes))
        h.set_fields_batch(0, len(Ls), conf)
        back = np.zeros_like(conf)
        h.fields_batch_into(0, len(Ls), back)
        assert np.array_equal(back, conf)
        h.initialize_run()
        h.sweep(1)
        nf = [f.unique_flavors * len(m.l) ** 2 for m, p, f, e in setups]
        for physical in (False, True):
            g = np.zeros(sum(nf))
            h.greens_batch_into(0, len(Ls), g, physical=physical)
            off = 0
            for i in range(len(Ls)):
                one = np.zeros(nf[i])
                h.greens_into(i, one, physical=physical)
                assert np.array_equal(g[off:off + nf[i]], one)
                off += nf[i]
        f = np.zeros(sum(sizes), dtype=np.int8)
        h.fields_batch_into(0, len(Ls), f)
        off = 0
        for i in range(len(Ls)):
            assert np.array_equal(f[off:off + sizes[i]], h.get_field(i).ravel(order="F"))
            off += sizes[i]
        # a sub-range
        g = np.zeros(sum(nf))
        h.greens_batch_into(0, len(Ls), g)
        g2 = np.zeros(nf[1] + nf[2])
        h.greens_batch_into(1, 2, g2)
        assert np.array_equal(g2, g[nf[0]:nf[0] + nf[1] + nf[2]])
        h.close()
