"""On-device equal-time measurements (density, double occupancy,
interaction energy, S^z(q), occupations, mean physical G, log binning)
against the host kernels of montecarlo_gb300.measurements applied to the
downloaded physical G of an identical chain, and against exact
diagonalisation on the 2x2 lattice."""
import numpy as np
import pytest

from _util import FIELD_U, chain_config, make_setup

pytestmark = pytest.mark.gpu

SPECS = [(4, "MagneticHirschField", 2.0), (4, "DensityHirschField", 2.0),
         (3, "MagneticGHQField", 1.0)]


def _handles(pkg, lib, specs, seed0=40):
    cfgs, exps_l, models = [], [], []
    for j, (L, field, beta) in enumerate(specs):
        model, param, fld, exps = make_setup(pkg, L=L, U=FIELD_U[field], beta=beta, safe_mult=5,
                                             field=getattr(pkg, field))
        cfgs.append(chain_config(lib, model, param, fld, seed0 + j))
        exps_l.append(exps)
        models.append(model)
    hs = [lib.Handle(cfgs), lib.Handle(cfgs)]
    for h in hs:
        for j, e in enumerate(exps_l):
            h.set_hopping(j, e)
        h.init_random_field(-1)
        h.initialize_run()
    return hs, models


def _phases(model, q=np.pi):
    pos = model.l.positions()
    ph = pos @ np.full(pos.shape[1], q)
    return np.cos(ph), np.sin(ph)


def _host_values(pkg, G, model, q):
    corr = pkg.spin_density_correlation_z(G)
    occ = pkg.occupation_kernel(G)
    dens = float(np.sum(1.0 - np.array([np.diag(g) for g in G]))) / G.shape[1]
    if G.shape[0] == 1:
        dens *= 2.0
    return [dens, float(np.mean(pkg.double_occupancy_kernel(G))),
            pkg.interaction_energy(G, model.U),
            pkg.structure_factor(corr, model.l.positions(), q)], occ


@pytest.mark.parametrize("n_sweeps,rate", [(12, 1), (140, 1), (30, 3)])
def test_device_measurements_match_host_kernels(pkg, lib, n_sweeps, rate):
    hs, models = _handles(pkg, lib, SPECS)
    hd, hh = hs
    for j, m in enumerate(models):
        hd.set_measurements(j, enable=True, rate=rate, greens=True, sweep=0, U=m.U,
                            q=_phases(m))
    hd.sweep(n_sweeps)  # one launch, measuring inside
    binners = [[pkg.LogBinner() for _ in range(4)] for _ in models]
    occs = [[] for _ in models]
    Gs = [[] for _ in models]
    for s in range(1, n_sweeps + 1):
        hh.sweep(1)
        if s % rate:
            continue
        for j, m in enumerate(models):
            G = hh.greens(j, physical=True)
            vals, occ = _host_values(pkg, G, m, (np.pi,) * m.l.positions().shape[1])
            for k in range(4):
                binners[j][k].push(vals[k])
            occs[j].append(occ)
            Gs[j].append(G)
    for j, m in enumerate(models):
        # the two chains are the same chain: measuring does not disturb it
        assert np.array_equal(hd.get_field(j), hh.get_field(j))
        out = hd.measurements(j)
        assert out["count"] == n_sweeps // rate
        for k, name in enumerate(lib.OBSERVABLES):
            mean, err = out[name]
            assert abs(mean - float(binners[j][k].mean())) <= 1e-11 * max(1.0, abs(mean)), name
            he = float(binners[j][k].std_error())
            assert abs(err - he) <= 1e-8 * max(he, 1e-300) + 1e-14, (name, err, he)
        assert np.max(np.abs(out["occupation"] - np.mean(occs[j], axis=0))) < 1e-12
        assert np.max(np.abs(out["greens"] - np.mean(Gs[j], axis=0))) < 1e-12


def test_measurements_off_and_reset(pkg, lib):
    hs, models = _handles(pkg, lib, SPECS[:1])
    h = hs[0]
    m = models[0]
    h.set_measurements(0, enable=True, rate=2, U=m.U, sweep=0)
    h.sweep(4)
    assert h.measurements(0)["count"] == 2
    h.set_measurements(0, enable=False)
    h.sweep(4)
    assert h.measurements(0)["count"] == 2
    h.reset_measurements(0)
    out = h.measurements(0)
    assert out["count"] == 0 and np.isnan(out["density"][0])
    # no q: S^z(q) is reported as 0
    h.set_measurements(0, enable=True, rate=1, U=m.U)
    h.sweep(2)
    out = h.measurements(0)
    assert out["count"] == 2 and out["sz_structure_factor"][0] == 0.0
    with pytest.raises(lib.DQMCError):
        h.set_measurements(0, enable=True, rate=0)


def test_pool_runs_measure(pkg, lib):
    """Time-sliced pool launches measure at the same sweeps as dqmc_sweep."""
    model, param, fld, exps = make_setup(pkg, L=4, U=-4.0, beta=2.0, safe_mult=5,
                                         field=pkg.MagneticHirschField)
    cfg = chain_config(lib, model, param, fld, 77)
    pool = lib.Pool(4, 64 << 20)
    slot = pool.admit(cfg)
    pool.set_hopping(slot, exps)
    pool.init_random_field(slot)
    pool.set_measurements(slot, enable=True, rate=1, greens=True, sweep=0, U=model.U,
                          q=_phases(model))
    pool.set_quota(slot, 6)
    while pool.slot(slot)[1] > 0:
        pool.run(2000)
    h = lib.Handle([cfg])
    h.set_hopping(0, exps)
    h.init_random_field(0)
    h.initialize_run()
    h.set_measurements(0, enable=True, rate=1, greens=True, sweep=0, U=model.U, q=_phases(model))
    h.sweep(6)
    a, b = pool.measurements(slot), h.measurements(0)
    assert a["count"] == b["count"] == 6
    for name in lib.OBSERVABLES:
        assert a[name][0] == b[name][0], name
    assert np.array_equal(a["greens"], b["greens"])


@pytest.mark.parametrize("U,mu", [(-1.0, 0.0), (1.0, 1.0)])
def test_device_observables_match_ed_2x2(pkg, lib, U, mu):
    """DQMC.run with only the device accumulators (no G download per
    measurement) against exact diagonalisation (test/ED/ED_tests.jl:400-460:
    beta = 1, dtau = 0.1, atol 3.05 dtau^2)."""
    import ed
    DT = 0.1
    ATOL = 3.05 * DT ** 2
    model = pkg.HubbardModel(pkg.SquareLattice(2), U=U, mu=mu)
    E = ed.HubbardED(4, model.l.bonds(), 1.0, U, mu, 1.0)
    mc = pkg.DQMC(model, beta=1.0, delta_tau=DT, safe_mult=10, seed=29, thermalization=500,
                  sweeps=4000, measure_rate=1)
    assert pkg.run(mc) == pkg.ExitCode.SUCCESS
    out = mc.observables()
    assert out["count"] == 4000
    Ged = E.greens()
    docc, docc_err = out["double_occupancy"]
    assert abs(docc - E.double_occupancy().mean()) <= ATOL + 5 * docc_err
    n_ed = float(np.sum([1.0 - np.diag(g) for g in Ged])) / 4 * (2.0 / len(Ged))
    dens, dens_err = out["density"]
    assert abs(dens - n_ed) <= ATOL + 5 * dens_err + 1e-12
    S_ed = pkg.structure_factor(E.sdc_z(), model.l.positions(), (np.pi, np.pi))
    S, S_err = out["sz_structure_factor"]
    assert abs(S - S_ed) <= ATOL + 5 * S_err + 1e-12
    nf = out["greens"].shape[0]  # one block: spin-degenerate, both ED blocks equal it
    for b in range(len(Ged)):
        assert np.all(np.abs(out["greens"][min(b, nf - 1)] - Ged[b]) <= ATOL + 0.03)
