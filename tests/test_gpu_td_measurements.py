"""Time-displaced measurements on the device (TimeIntegral, generic.jl:337-366).

The device contracts G(0,0), G(0,l), G(l,0), G(l,l) of the UnequalTimeStack
into the charge, spin x / y / z and pairing correlations, reduces them by
distance (EachSitePairByDistance) and integrates the susceptibilities, all
inside the launch; nothing is downloaded per measurement.  Checked against
the host contractions of the same Green's functions (downloaded with
greens_kl for the test only) at 1e-11, and against exact diagonalisation
through the DQMC API."""
import numpy as np
import pytest

from _util import chain_config, make_setup

pytestmark = pytest.mark.gpu

TOL = 1e-11


def _host_reference(pkg, h, model, param, arrays):
    """Susceptibilities and by-distance arrays of the chain's current
    configuration from downloaded unequal-time Green's functions."""
    M = param.slices
    pairs = [(0, 0)]
    for l in range(M + 1):
        pairs += [(l, l), (0, l), (l, 0)]
    Gs = h.greens_kl(0, pairs, physical=True)
    by_l = [(Gs[0], Gs[2 + 3 * l], Gs[3 + 3 * l], Gs[1 + 3 * l]) for l in range(M + 1)]
    phases = (arrays["q_cos"], arrays["q_sin"])
    J = pkg.current_operator(model.hopping_matrix(), model.l)
    pf = {}
    if len(model.l.unitcell.lattice_vectors) >= 2:
        pf = {k: pkg.pair_form_factor(model.l, k) for k in ("s*", "d")}
    chi = pkg.susceptibilities(by_l, phases, param.delta_tau, current=J, pair_fields=pf)
    n, P = len(model.l), arrays["n_slots"]
    slot = model.l.pair_distance_index()
    bd = np.zeros((5, P))
    for l, (G00, G0l, Gl0, Gll) in enumerate(by_l):
        C = pkg.time_displaced_correlations(G00, G0l, Gl0, Gll, l == 0)
        w = (0.5 if l in (0, M) else 1.0) * param.delta_tau
        for k, name in enumerate(["charge", "spin_x", "spin_y", "spin_z", "pairing"]):
            bd[k] += w * pkg.by_distance(C[name], slot, P)
    return chi, bd


def _rel(a, b):
    return abs(a - b) / max(1.0, abs(b))


@pytest.mark.parametrize("lattice,L,U,field", [
    ("square", 4, -4.0, "MagneticHirschField"),
    ("square", 4, 4.0, "DensityHirschField"),
    ("honeycomb", 2, -4.0, "MagneticHirschField"),
    ("chain", 6, 4.0, "DensityGHQField")])
def test_td_measure_equals_host_contractions(pkg, lib, lattice, L, U, field):
    model, param, fld, exps = make_setup(pkg, L=L, lattice=lattice, U=U, beta=1.0,
                                         safe_mult=5, field=getattr(pkg, field))
    arrays = pkg.td_arrays(model, q=[np.pi] * len(model.l.unitcell.lattice_vectors))
    h = lib.Handle([chain_config(lib, model, param, fld, 31)])
    h.set_hopping(-1, exps)
    h.init_random_field(0)
    h.initialize_run()
    h.sweep(1)
    h.set_td_measurements(0, arrays, param.delta_tau)
    h.td_measure()
    dev = h.td_measurements(0, arrays["n_slots"])
    assert dev["count"] == 1
    chi, bd = _host_reference(pkg, h, model, param, arrays)
    for name in lib.TD_SCALARS:
        if name in chi:
            assert _rel(dev[name][0], chi[name]) < TOL, (name, dev[name][0], chi[name])
    assert np.max(np.abs(dev["by_distance"] - bd)) < TOL * max(1.0, np.abs(bd).max())


def test_td_measurements_inside_sweeps(pkg, lib):
    """Measured after every sweep inside the sweep launch: three
    measurements whose means equal the host values of the three
    configurations."""
    model, param, fld, exps = make_setup(pkg, L=4, U=-4.0, beta=1.0, safe_mult=5,
                                         field=pkg.MagneticHirschField)
    arrays = pkg.td_arrays(model)
    h = lib.Handle([chain_config(lib, model, param, fld, 32)])
    h.set_hopping(-1, exps)
    h.init_random_field(0)
    h.initialize_run()
    h.set_td_measurements(0, arrays, param.delta_tau, rate=1, sweep=0)
    host = []
    for _ in range(3):
        h.sweep(1)
        host.append(_host_reference(pkg, h, model, param, arrays))
    dev = h.td_measurements(0, arrays["n_slots"])
    assert dev["count"] == 3
    for name in ("charge", "spin_z", "pairing", "pairing_d", "current"):
        want = np.mean([c[name] for c, _ in host])
        assert _rel(dev[name][0], want) < TOL, (name, dev[name][0], want)
    want_bd = np.mean([b for _, b in host], axis=0)
    assert np.max(np.abs(dev["by_distance"] - want_bd)) < TOL * max(1.0, np.abs(want_bd).max())


def test_td_measurements_match_ed_2x2(pkg, lib):
    """DQMC(...; time_displaced = true) on the 2x2 attractive model at
    beta = 1: every device susceptibility (the current one is checked on the
    chain against the host contractions above) agrees with exact diagonalisation
    on the same imaginary-time grid (atol 3.05 dtau^2, relative above 1, plus
    five binning errors, as the host-contraction tests)."""
    import ed
    DT = 0.1
    U, mu = -1.0, 0.0
    model = pkg.HubbardModel(pkg.SquareLattice(2), U=U, mu=mu)
    E = ed.HubbardED(4, model.l.bonds(), 1.0, U, mu, 1.0)
    pos = model.l.positions()
    phases = np.cos(pos @ np.array([np.pi, np.pi]))
    want = {k: E.susceptibility_grid(k, phases, DT) for k in pkg.CORRELATIONS}
    for ff in ("s*", "d"):
        want["pairing_" + ff] = E.susceptibility_grid("pair_field",
                                                      pkg.pair_form_factor(model.l, ff), DT)
    mc = pkg.DQMC(model, beta=1.0, delta_tau=DT, safe_mult=10, seed=47, thermalization=200,
                  sweeps=1200, measure_rate=1, time_displaced=True)
    pkg.run(mc)
    got = mc.time_displaced_observables()
    assert got["count"] == 1200
    for k, v in want.items():
        chi, err = got[k]
        tol = 3.05 * DT ** 2 * max(1.0, abs(v)) + 5 * err
        assert abs(chi - v) <= tol, (k, chi, v, err)
