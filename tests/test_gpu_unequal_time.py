"""Unequal-time Green's function G(k, l) (calculate_greens(mc, k, l) through
the UnequalTimeStack) on the GPU against the oracle, FP64, 1e-10."""
import numpy as np
import pytest

from _util import FIELD_U, chain_config, make_setup, maxdiff, oracle_chain

pytestmark = pytest.mark.gpu

TOL_G = 1e-10


@pytest.mark.parametrize("L,field,beta,k", [(4, "DensityHirschField", 2.0, 5),
                                            (4, "MagneticHirschField", 2.0, 5),
                                            (8, "MagneticHirschField", 2.0, 10),
                                            (3, "MagneticGHQField", 1.5, 4),
                                            (10, "DensityHirschField", 1.0, 5)])
def test_greens_kl_matches_oracle(pkg, lib, oracle, L, field, beta, k):
    model, param, fld, exps = make_setup(pkg, L=L, U=FIELD_U[field], beta=beta, safe_mult=k,
                                         field=getattr(pkg, field))
    h = lib.Handle([chain_config(lib, model, param, fld, 17)])
    h.set_hopping(-1, exps)
    h.init_random_field(0)
    h.initialize_run()
    h.sweep(1)
    o = oracle_chain(oracle, model, param, fld, exps, 17)
    o.set_conf(h.get_field(0))
    M = param.slices
    pairs = [(0, 0), (M, M), (3, 0), (0, 3), (M - 1, 2), (2, M - 1), (M, 0), (0, M), (7, 7),
             (M // 2, M // 3)]
    g_gpu = h.greens_kl(0, pairs)
    g_cpu = o.greens_kl(pairs)
    for p, a, b in zip(pairs, g_gpu, g_cpu):
        assert maxdiff(a, b) < TOL_G, (p, maxdiff(a, b))
    # physical form and equal-time consistency on the GPU itself
    gp = h.greens_kl(0, [(4, 4)], physical=True)[0]
    eq = h.calculate_greens(0, 4)
    assert maxdiff(h.greens_kl(0, [(4, 4)])[0], eq) < 1e-12
    assert maxdiff(gp, o.greens_physical(o.calculate_greens_at(4))) < TOL_G


def test_greens_kl_does_not_disturb_the_chain(pkg, lib, oracle):
    """Sweeps after an unequal-time request replay the oracle exactly."""
    model, param, fld, exps = make_setup(pkg, L=4, U=-4.0, beta=2.0, safe_mult=5,
                                         field=pkg.MagneticHirschField)
    h = lib.Handle([chain_config(lib, model, param, fld, 23)])
    h.set_hopping(-1, exps)
    h.init_random_field(0)
    h.initialize_run()
    o = oracle_chain(oracle, model, param, fld, exps, 23)
    o.init_random_conf()
    o.initialize_run()
    h.sweep(1)
    o.sweeps(1)
    h.greens_kl(0, [(5, 1), (1, 5)])
    h.sweep(1)
    o.sweeps(1)
    assert np.array_equal(h.get_field(0), o.get_conf())
    assert maxdiff(h.greens(0), o.greens()) < TOL_G
    with pytest.raises(lib.DQMCError):
        h.greens_kl(0, [(param.slices + 1, 0)])


@pytest.mark.parametrize("U", [-1.0, 1.0])
def test_spin_susceptibility_matches_ed_2x2(pkg, lib, U):
    """chi_z(pi, pi) from the time-displaced Green's functions (TimeIntegral
    of the z spin-density correlation) against exact diagonalisation on 2x2
    at beta = 1, dtau = 0.1 (atol 3.05 dtau^2 as the reference's ED tests,
    plus five binning errors)."""
    import ed
    DT = 0.1
    model = pkg.HubbardModel(pkg.SquareLattice(2), U=U, mu=0.0)
    E = ed.HubbardED(4, model.l.bonds(), 1.0, U, 0.0, 1.0)
    pos = model.l.positions()
    chi_ed = E.susceptibility_z(np.cos(pos @ np.array([np.pi, np.pi])))
    mc = pkg.DQMC(model, beta=1.0, delta_tau=DT, safe_mult=10, seed=44, thermalization=200,
                  sweeps=0, measure_rate=1)
    pkg.run(mc)
    b = pkg.LogBinner()
    for _ in range(1500):
        mc.handle.sweep(1)
        b.push(mc.spin_susceptibility())
    chi, err = float(b.mean()), float(b.std_error())
    assert abs(chi - chi_ed) <= 3.05 * DT ** 2 + 5 * err, (chi, chi_ed, err)


@pytest.mark.parametrize("U,mu", [(-1.0, 0.0), (1.0, 0.2)])
def test_all_susceptibilities_match_ed_2x2(pkg, lib, U, mu):
    """Charge and spin x / y / z susceptibilities at (pi, pi) and the on-site
    s-wave pairing susceptibility, all from the same time-displaced Green's
    functions of each sweep, against exact diagonalisation (2x2, beta = 1,
    dtau = 0.1; repulsive at half filling, attractive at mu = 0.2: no sign
    problem; atol 3.05 dtau^2 plus five binning errors)."""
    import ed
    DT = 0.1
    model = pkg.HubbardModel(pkg.SquareLattice(2), U=U, mu=mu)
    E = ed.HubbardED(4, model.l.bonds(), 1.0, U, mu, 1.0)
    pos = model.l.positions()
    phases = np.cos(pos @ np.array([np.pi, np.pi]))
    # ED integrated on the same imaginary-time grid with the same trapezoid
    # weights (as the reference's ED tests do): only the Trotter error and the
    # statistics remain
    want = {k: E.susceptibility_grid(k, phases, DT) for k in pkg.CORRELATIONS}
    for ff in ("s*", "d"):  # extended-s and d-wave pair fields
        want["pairing_" + ff] = E.susceptibility_grid("pair_field",
                                                      pkg.pair_form_factor(model.l, ff), DT)
    mc = pkg.DQMC(model, beta=1.0, delta_tau=DT, safe_mult=10, seed=45, thermalization=200,
                  sweeps=0, measure_rate=1)
    pkg.run(mc)
    bins = {k: pkg.LogBinner() for k in want}
    for _ in range(1200):
        mc.handle.sweep(1)
        chi = mc.susceptibilities()
        for k in want:
            bins[k].push(chi[k])
    for k in want:
        # the Trotter error of a susceptibility scales with its size: the
        # reference's atol 3.05 dtau^2 for values up to 1, relative above
        chi, err = float(bins[k].mean()), float(bins[k].std_error())
        tol = 3.05 * DT ** 2 * max(1.0, abs(want[k])) + 5 * err
        assert abs(chi - want[k]) <= tol, (k, chi, want[k], err)


@pytest.mark.parametrize("U,mu", [(-2.0, 0.0), (2.0, 0.3)])
def test_current_susceptibility_matches_ed_chain4(pkg, lib, U, mu):
    """Uniform current-current susceptibility (bond currents of cc_kernel)
    and the others on a 4-site chain against exact diagonalisation
    (beta = 1, dtau = 0.1; atol 3.05 dtau^2 plus five binning errors)."""
    import ed
    DT = 0.1
    model = pkg.HubbardModel(pkg.Chain(4), U=U, mu=mu)
    E = ed.HubbardED(4, model.l.bonds(), 1.0, U, mu, 1.0)
    J = pkg.current_operator(model.hopping_matrix(), model.l)
    phases = np.cos(np.pi * model.l.positions()[:, 0])
    want = {k: E.susceptibility_grid(k, phases, DT) for k in pkg.CORRELATIONS}
    want["current"] = E.susceptibility_grid("current", J, DT)
    mc = pkg.DQMC(model, beta=1.0, delta_tau=DT, safe_mult=10, seed=46, thermalization=200,
                  sweeps=0, measure_rate=1, structure_factor_q=[np.pi])
    pkg.run(mc)
    bins = {k: pkg.LogBinner() for k in want}
    for _ in range(1200):
        mc.handle.sweep(1)
        for k, v in mc.susceptibilities().items():
            bins[k].push(v)
    for k in want:
        chi, err = float(bins[k].mean()), float(bins[k].std_error())
        assert abs(chi - want[k]) <= 3.05 * DT ** 2 + 5 * err, (k, chi, want[k], err)
