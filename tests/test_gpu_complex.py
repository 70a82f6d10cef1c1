"""Complex chains (a field kind that does not match the sign of U: the
reference's ComplexF64 path) on the GPU against the complex oracle.

The device keeps each complex n x n matrix as its real 2n x 2n
representation; the C ABI exchanges interleaved complex blocks.  Bars as for
real chains: Green's functions to 1e-10 relative to max(1, |G|) in FP64;
field configurations, RNG counters, accepted counts and the sign-problem
counters bit-identical under the replayed Philox stream.  n = 4 and 16 run
with G resident in shared memory (representation 8 and 32), n = 36 with G in
global memory and delayed updates (representation 72).
"""
import numpy as np
import pytest

import complex_oracle as CO
from _util import chain_config, maxdiff

pytestmark = pytest.mark.gpu

TOL_G = 1e-10
MISMATCH_U = {"DensityHirschField": -4.0, "MagneticHirschField": 4.0, "DensityGHQField": -4.0,
              "MagneticGHQField": 4.0}


def _rel(a, b):
    return maxdiff(a, b) / max(1.0, float(np.abs(b).max()))


def _pair(pkg, lib, field, L=4, mu=0.3, beta=2.0, k=5, seed=31, exps=None, lattice="square"):
    lat = pkg.SquareLattice(L) if lattice == "square" else pkg.Honeycomb(L)
    model = pkg.HubbardModel(lat, U=MISMATCH_U[field], mu=mu)
    param = pkg.DQMCParameters.make(beta=beta, delta_tau=0.1, safe_mult=k)
    fld = getattr(pkg, field)(param, model)
    assert fld.is_complex
    hop = pkg.hopping_exponentials(model.hopping_matrix(), param.delta_tau)
    h = lib.Handle([chain_config(lib, model, param, fld, seed)])
    h.set_hopping(-1, hop)
    c = CO.ComplexChain(len(model.l), fld.unique_flavors, param.slices, param.safe_mult, fld.kind,
                        fld.alpha, hop if exps is None else exps, seed)
    h.init_random_field(0)
    c.set_conf(h.get_field(0))
    c.set_rng(seed, h.get_rng(0)[1])
    return h, c, model, param, fld


CASES = [(f, L) for f in MISMATCH_U for L in (2, 4)] + [("DensityHirschField", 6),
                                                       ("MagneticHirschField", 6),
                                                       ("MagneticGHQField", 6)]


@pytest.mark.parametrize("field,L", CASES)
def test_complex_calculate_greens_matches_oracle(pkg, lib, field, L):
    h, c, model, param, fld = _pair(pkg, lib, field, L=L)
    for sl in (0, 1, 7, 10, param.slices):
        g = h.calculate_greens(0, sl)
        assert g.dtype == np.complex128
        assert _rel(g, c.calculate_greens_at(sl)) < TOL_G, sl


@pytest.mark.parametrize("field,L", CASES)
def test_complex_sweeps_replay_bit_exact(pkg, lib, field, L):
    h, c, model, param, fld = _pair(pkg, lib, field, L=L, seed=2024 + L)
    h.initialize_run()
    c.initialize_run()
    assert _rel(h.greens(0), c.G) < TOL_G
    for _ in range(2):
        st = h.sweep(1)[0]
        c.sweeps(1)
        assert np.array_equal(h.get_field(0), c.conf)
        assert h.get_rng(0)[1] == c.ctr
        assert st["accepted"] == c.accepted and st["proposals"] == c.proposals
        assert st["imaginary_probability"] == c.n_imag_p
        assert st["negative_probability"] == c.n_neg_p
        assert _rel(h.greens(0), c.G) < 1e-9
    if field.startswith("Density"):  # away from half filling: a sign problem
        assert st["imaginary_probability"] > 0
        assert abs(st["max_imaginary_probability"] - c.max_imag_p) <= 1e-9 * c.max_imag_p
    # the device projects G back onto the representation subspace after each
    # wrap: its propagation error stays at the complex oracle's level
    assert st["max_propagation_error"] <= 10 * c.prop_err_max + 1e-13
    assert _rel(h.greens(0, physical=True), c.greens_physical(c.G)) < 1e-9


@pytest.mark.parametrize("field", ["DensityHirschField", "MagneticGHQField"])
def test_complex_unequal_time(pkg, lib, field):
    h, c, model, param, fld = _pair(pkg, lib, field, L=2, beta=1.0, k=4)
    h.initialize_run()
    h.sweep(1)
    c.set_conf(h.get_field(0))
    M = param.slices
    pairs = [(0, 0), (M, M), (3, 0), (0, 3), (M - 1, 2), (2, M - 1), (M, 0), (0, M), (5, 5)]
    for (k, l), g in zip(pairs, h.greens_kl(0, pairs)):
        assert _rel(g, CO.direct_greens_kl(c, k, l)) < 1e-9, (k, l)
    assert _rel(h.greens_kl(0, [(4, 4)])[0], h.calculate_greens(0, 4)) < 1e-12


@pytest.mark.parametrize("field", ["DensityHirschField", "MagneticHirschField"])
def test_complex_checkerboard(pkg, lib, field):
    from montecarlo_gb300 import model as M
    lat = pkg.SquareLattice(4)
    T = pkg.HubbardModel(lat, U=MISMATCH_U[field], mu=0.3).hopping_matrix()
    cbf = M.checkerboard_exponentials(T, lat, 0.1)
    dense = [M.checkerboard_matrix(D, parts) for D, parts in cbf]
    h, c, model, param, fld = _pair(pkg, lib, field, L=4, exps=dense, seed=77)
    h.set_checkerboard(0, *M.checkerboard_pack(cbf))
    h.initialize_run()
    c.initialize_run()
    assert _rel(h.greens(0), c.G) < TOL_G
    h.sweep(1)
    c.sweeps(1)
    assert np.array_equal(h.get_field(0), c.conf)
    assert _rel(h.greens(0), c.G) < 1e-9


def test_complex_set_greens_round_trip_and_rejections(pkg, lib):
    h, c, model, param, fld = _pair(pkg, lib, "DensityHirschField", L=2)
    h.initialize_run()
    G = h.greens(0)
    h.set_greens(0, G * 0.5)
    assert maxdiff(h.greens(0), G * 0.5) == 0.0
    cfg = chain_config(lib, model, param, fld, 1)
    with pytest.raises(lib.DQMCError):
        lib.Handle([cfg], precision=lib.PREC_MIXED)
    with pytest.raises(lib.DQMCError):
        h.global_update(lib.GLOBAL_FLIP)
    with pytest.raises(lib.DQMCError):
        h.set_global_schedule(lib.GLOBAL_FLIP, 0)
    with pytest.raises(lib.DQMCError):
        h.set_measurements(0, enable=True, U=model.U)


def test_dqmc_run_with_complex_field(pkg):
    model = pkg.HubbardModel(pkg.SquareLattice(2), U=-4.0, mu=0.3)
    mc = pkg.DQMC(model, field=pkg.DensityHirschField, beta=1.0, thermalization=3, sweeps=4,
                  measure_rate=2, seed=5)
    assert mc.field.is_complex
    assert mc.run() == pkg.ExitCode.SUCCESS
    G = mc.greens()
    assert G.dtype == np.complex128 and G.shape == (1, 4, 4)
    n_imag, max_imag = mc.analysis["imaginary_probability"]
    assert n_imag >= 0 and max_imag >= 0.0
    assert mc.analysis["max_propagation_error"] < 1e-6


def test_complex_chain_in_a_pool_equals_plain_sweeps(pkg, lib):
    """A complex chain admitted to a pool beside a real one, time-sliced with
    graph replays, ends where a plain handle's sweeps end (bit-for-bit)."""
    h, c, model, param, fld = _pair(pkg, lib, "DensityHirschField", L=4, seed=88)
    h.initialize_run()
    h.sweep(2)
    cfg = chain_config(lib, model, param, fld, 88)
    rmodel = pkg.HubbardModel(pkg.SquareLattice(4), U=-4.0)
    rfld = pkg.MagneticHirschField(param, rmodel)
    rcfg = chain_config(lib, rmodel, param, rfld, 89)
    hop = pkg.hopping_exponentials(model.hopping_matrix(), param.delta_tau)
    pool = lib.Pool(2, lib.chain_bytes(cfg) + lib.chain_bytes(rcfg) + 8192)
    slots = [pool.admit(cfg), pool.admit(rcfg)]
    for s in slots:
        pool.set_hopping(s, hop)
        pool.init_random_field(s)
        pool.set_quota(s, 2)
    while any(pool.slot(s)[1] > 0 for s in slots):
        pool.run(300, True)
    assert np.array_equal(pool.get_field(slots[0]), h.get_field(0))
    assert np.array_equal(pool.greens(slots[0]), h.greens(0))
    assert pool.get_rng(slots[0]) == h.get_rng(0)
    pool.close()


def test_complex_propagation_error_at_oracle_level_8x8(pkg, lib):
    """The 8x8 lattice at beta = 8 (the plain benchmark's lattice and U, with
    the complex density-channel field): the device's propagation errors stay
    at the complex oracle's level over two sweeps, decisions replay."""
    model = pkg.HubbardModel(pkg.SquareLattice(8), U=-4.0)
    param = pkg.DQMCParameters.make(beta=8.0, delta_tau=0.1, safe_mult=10)
    fld = pkg.DensityHirschField(param, model)
    hop = pkg.hopping_exponentials(model.hopping_matrix(), param.delta_tau)
    h = lib.Handle([chain_config(lib, model, param, fld, 100 + j) for j in range(8)])
    h.set_hopping(-1, hop)
    h.init_random_field(-1)
    c = CO.ComplexChain(64, 1, param.slices, 10, fld.kind, fld.alpha, hop, 100)
    c.set_conf(h.get_field(0))
    c.set_rng(100, h.get_rng(0)[1])
    h.initialize_run()
    c.initialize_run()
    st = h.sweep(2)
    c.sweeps(2)
    assert np.array_equal(h.get_field(0), c.conf)
    assert st[0]["max_propagation_error"] <= 10 * c.prop_err_max + 1e-13
    assert max(s["max_propagation_error"] for s in st) < 1e-9
    assert all(s["imaginary_probability"] == 0 for s in st)   # real weights at half filling


def test_complex_max_size_128_sites(pkg, lib):
    """The largest complex chain (n_sites = 128, the honeycomb L = 8;
    representation 256, G in global memory): G from scratch and one sweep
    replayed against the complex oracle."""
    h, c, model, param, fld = _pair(pkg, lib, "DensityHirschField", L=8, lattice="honeycomb",
                                    beta=0.5, k=5, seed=13)
    assert len(model.l) == 128
    for sl in (0, 3, param.slices):
        assert _rel(h.calculate_greens(0, sl), c.calculate_greens_at(sl)) < TOL_G, sl
    h.initialize_run()
    c.initialize_run()
    st = h.sweep(1)[0]
    c.sweeps(1)
    assert np.array_equal(h.get_field(0), c.conf)
    assert st["accepted"] == c.accepted
    assert _rel(h.greens(0), c.G) < 1e-9


def test_magnitude_stats_of_the_sign_problem(pkg, lib):
    """DQMCAnalysis' MagnitudeStats on the device: counts equal the oracle's,
    max equals the oracle's max, and min <= geometric mean <= max."""
    h, c, model, param, fld = _pair(pkg, lib, "DensityHirschField", L=4, mu=0.5, seed=3)
    h.initialize_run()
    c.initialize_run()
    st = h.sweep(2)[0]
    c.sweeps(2)
    assert st["imaginary_probability"] == c.n_imag_p > 0
    assert abs(st["max_imaginary_probability"] - c.max_imag_p) <= 1e-9 * c.max_imag_p
    assert 0 < st["min_imaginary_probability"] <= st["mean_imaginary_probability"] \
        <= st["max_imaginary_probability"] * (1 + 1e-12)
    if st["negative_probability"] > 0:
        assert 0 < st["min_negative_probability"] <= st["mean_negative_probability"] \
            <= st["max_negative_probability"] * (1 + 1e-12)
    else:
        assert st["max_negative_probability"] == 0.0
    assert st["propagation_errors"] == 0 and st["mean_reported_error"] == 0.0
