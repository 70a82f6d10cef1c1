"""Observables against exact diagonalisation on the 2x2 lattice (the
reference's ED tests, test/ED/ED_tests.jl:400-460: beta = 1, dtau = 0.1,
atol 3.05 dtau^2).  The oracle run is CPU-only; the GPU run goes through the
DQMC / run API and the CUDA library."""
import numpy as np
import pytest

DT = 0.1
ATOL = 3.05 * DT ** 2


def _ed(pkg, U, mu):
    import ed
    model = pkg.HubbardModel(pkg.SquareLattice(2), U=U, mu=mu)
    return model, ed.HubbardED(4, model.l.bonds(), 1.0, U, mu, 1.0)


def _check(pkg, G_mean, G_err, docc, docc_err, sdc, sdc_err, E):
    Ged = E.greens()
    nf = G_mean.shape[0]
    for b in range(nf):
        assert np.all(np.abs(G_mean[b] - Ged[b]) <= ATOL + 5 * G_err[b] + 1e-12)
    assert abs(docc - E.double_occupancy().mean()) <= ATOL + 5 * docc_err
    assert np.all(np.abs(sdc - E.sdc_z()) <= ATOL + 5 * sdc_err + 1e-12)


@pytest.mark.parametrize("U,mu", [(-1.0, 0.0), (1.0, 1.0)])
def test_oracle_matches_ed_2x2(oracle, pkg, U, mu):
    model, E = _ed(pkg, U, mu)
    param = pkg.DQMCParameters.make(beta=1.0, delta_tau=DT, safe_mult=10)
    fld = model.choose_field()(param, model)
    exps = pkg.hopping_exponentials(model.hopping_matrix(), DT)
    c = oracle.OracleChain(4, fld.unique_flavors, param.slices, 10, fld.kind, fld.alpha, exps, 17)
    c.init_random_conf()
    c.initialize_run()
    c.sweeps(500)
    bG, bd, bs = pkg.LogBinner(), pkg.LogBinner(), pkg.LogBinner()
    for _ in range(4000):
        c.sweeps(1)
        G = c.greens_physical(c.greens())
        bG.push(G)
        bd.push(np.mean(pkg.double_occupancy_kernel(G)))
        bs.push(pkg.spin_density_correlation_z(G))
    _check(pkg, bG.mean(), bG.std_error(), float(bd.mean()), float(bd.std_error()),
           bs.mean(), bs.std_error(), E)


@pytest.mark.gpu
@pytest.mark.parametrize("U,mu", [(-1.0, 0.0), (1.0, 1.0)])
def test_gpu_dqmc_run_matches_ed_2x2(pkg, lib, U, mu):
    model, E = _ed(pkg, U, mu)
    mc = pkg.DQMC(model, beta=1.0, delta_tau=DT, safe_mult=10, seed=23, thermalization=500,
                  sweeps=4000, measure_rate=1)
    mc["G"] = pkg.greens_measurement(mc, model)
    mc["docc"] = pkg.double_occupancy(mc, model)
    mc["sdcz"] = pkg.spin_density_correlation(mc, model)
    assert pkg.run(mc) == pkg.ExitCode.SUCCESS
    _check(pkg, mc["G"].mean(), mc["G"].std_error(), float(mc["docc"].mean()),
           float(mc["docc"].std_error()), mc["sdcz"].mean(), mc["sdcz"].std_error(), E)
    assert mc.analysis["negative_probability"] == 0


def test_ed_grid_integral_converges_to_the_continuous_one(pkg):
    """The trapezoid time integral on the DQMC grid (susceptibility_grid)
    approaches the exact spectral integral as dtau -> 0 (error ~ dtau^2)."""
    import ed
    model = pkg.HubbardModel(pkg.SquareLattice(2), U=-1.0, mu=0.0)
    E = ed.HubbardED(4, model.l.bonds(), 1.0, -1.0, 0.0, 1.0)
    F = pkg.pair_form_factor(model.l, "s*")
    exact = E.susceptibility("pair_field", F)
    e1 = abs(E.susceptibility_grid("pair_field", F, 0.1) - exact)
    e2 = abs(E.susceptibility_grid("pair_field", F, 0.05) - exact)
    assert e2 < e1 / 3.5 and e1 < 0.2
