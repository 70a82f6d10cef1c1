"""The time-displaced correlation kernels of the susceptibility measurements
(charge, spin x / y / z, on-site pairing: the reference's full_cdc_kernel,
full_sdc_x/y/z_kernel, pc_combined_kernel) pinned exactly on the CPU.

At U = 0 the slice matrices have no Trotter error and no field, so the
oracle's unequal-time Green's functions G(k, l) are the free ones and every
Wick contraction must equal exact diagonalisation's <A(l dtau) B(0)> to
rounding, at every l."""
import numpy as np
import pytest

from _util import make_setup, oracle_chain


@pytest.mark.parametrize("field", ["DensityHirschField", "MagneticHirschField"])
@pytest.mark.parametrize("mu", [0.0, 0.3])
def test_time_displaced_correlations_exact_at_u0(pkg, oracle, field, mu):
    import ed
    from montecarlo_gb300.measurements import CORRELATIONS, time_displaced_correlations
    model, param, fld, exps = make_setup(pkg, L=2, U=0.0, mu=mu, beta=1.0, safe_mult=5,
                                         field=getattr(pkg, field))
    o = oracle_chain(oracle, model, param, fld, exps, 3)
    o.init_random_conf()
    E = ed.HubbardED(4, model.l.bonds(), 1.0, 0.0, mu, param.beta)
    pos = model.l.positions()
    phases = np.cos(pos @ np.array([np.pi, np.pi]))
    M = param.slices
    pairs = [(0, 0)]
    for l in range(M + 1):
        pairs += [(l, l), (0, l), (l, 0)]
    Gs = [o.greens_physical(g) for g in o.greens_kl(pairs)]
    for l in range(M + 1):
        C = time_displaced_correlations(Gs[0], Gs[2 + 3 * l], Gs[3 + 3 * l], Gs[1 + 3 * l], l == 0)
        tau = l * param.delta_tau
        for kind in CORRELATIONS:
            A, B = E.operators(kind, phases)
            if kind == "pairing":
                want = E.correlation(A, B, tau) + E.correlation(B, A, tau)
                got = C[kind].sum()
            else:
                want = E.correlation(A, B, tau)
                got = phases @ C[kind] @ phases
            assert abs(got - want) < 1e-10, (kind, l, got, want)



@pytest.mark.parametrize("field", ["DensityHirschField", "MagneticHirschField"])
def test_current_and_bilinear_correlations_exact_at_u0(pkg, oracle, field):
    """The uniform current J_x (bond currents of cc_kernel) and a generic
    bilinear through bilinear_correlation equal ED at every tau (4-site
    chain, U = 0), and the bilinear form reproduces the charge kernel."""
    import ed
    from montecarlo_gb300.measurements import (bilinear_correlation, current_operator,
                                               time_displaced_correlations)
    model, param, fld, exps = make_setup(pkg, L=4, lattice="chain", U=0.0, mu=0.3, beta=1.0,
                                         safe_mult=5, field=getattr(pkg, field))
    o = oracle_chain(oracle, model, param, fld, exps, 3)
    o.init_random_conf()
    E = ed.HubbardED(4, model.l.bonds(), 1.0, 0.0, 0.3, param.beta)
    J = current_operator(model.hopping_matrix(), model.l)
    assert np.abs(J).max() > 0.5 and np.allclose(J, J.conj().T)
    Jop = E.operators("bilinear", J)
    rng = np.random.default_rng(1)
    Bm = rng.standard_normal((4, 4))
    Bop = E.operators("bilinear", Bm)
    ph = np.cos(np.pi * model.l.positions()[:, 0])
    M = param.slices
    pairs = [(0, 0)]
    for l in range(M + 1):
        pairs += [(l, l), (0, l), (l, 0)]
    Gs = [o.greens_physical(g) for g in o.greens_kl(pairs)]
    for l in range(M + 1):
        q = (Gs[0], Gs[2 + 3 * l], Gs[3 + 3 * l], Gs[1 + 3 * l])
        tau = l * param.delta_tau
        got = bilinear_correlation(J, J, *q, l == 0)
        assert abs(got - E.correlation(*Jop, tau)) < 1e-10, (l, got)
        got = bilinear_correlation(Bm, Bm.T, *q, l == 0)
        assert abs(got - E.correlation(Bop[0], Bop[1], tau)) < 1e-10, l
        C = time_displaced_correlations(*q, l == 0)["charge"]
        D = np.diag(ph)
        assert abs(ph @ C @ ph - bilinear_correlation(D, D, *q, l == 0)) < 1e-12


@pytest.mark.parametrize("kind", ["s", "s*", "d"])
def test_pair_fields_exact_at_u0(pkg, oracle, kind):
    """Pair fields with a form factor (on-site s, extended s, d) through
    pair_correlation equal ED's <Delta(tau) Delta^+> + <Delta^+(tau) Delta> at
    every tau (2x2 lattice, U = 0, both block structures); the on-site form
    factor reproduces the on-site pairing kernel."""
    import ed
    from montecarlo_gb300.measurements import (pair_correlation, pair_form_factor,
                                               time_displaced_correlations)
    for field in ("DensityHirschField", "MagneticHirschField"):
        model, param, fld, exps = make_setup(pkg, L=2, U=0.0, mu=0.3, beta=1.0, safe_mult=5,
                                             field=getattr(pkg, field))
        o = oracle_chain(oracle, model, param, fld, exps, 3)
        o.init_random_conf()
        E = ed.HubbardED(4, model.l.bonds(), 1.0, 0.0, 0.3, param.beta)
        F = pair_form_factor(model.l, kind)
        assert np.abs(F).sum() > 0
        D, Dd = E.operators("pair_field", F)
        M = param.slices
        pairs = [(0, 0)]
        for l in range(M + 1):
            pairs += [(l, l), (0, l), (l, 0)]
        Gs = [o.greens_physical(g) for g in o.greens_kl(pairs)]
        for l in range(M + 1):
            q = (Gs[0], Gs[2 + 3 * l], Gs[3 + 3 * l], Gs[1 + 3 * l])
            tau = l * param.delta_tau
            want = E.correlation(D, Dd, tau) + E.correlation(Dd, D, tau)
            got = pair_correlation(F, *q, l == 0)
            assert abs(got - want) < 1e-10, (field, kind, l, got, want)
            if kind == "s":
                C = time_displaced_correlations(*q, l == 0)["pairing"]
                assert abs(got - C.sum()) < 1e-12


def test_form_factors_and_current_operator_structure(pkg):
    """Form factors: s = I; s* has every nearest-neighbour bond (row sums =
    coordination); d is +1 along the first lattice vector and -1 along the
    second (row sums 0 on the square lattice); all symmetric.  The current
    operator is Hermitian, antisymmetric in the bond direction and zero on
    a lattice whose +x and -x neighbours coincide (L = 2)."""
    from montecarlo_gb300.measurements import current_operator, pair_form_factor
    lat = pkg.SquareLattice(4)
    assert np.array_equal(pair_form_factor(lat, "s"), np.eye(16))
    ss, d = pair_form_factor(lat, "s*"), pair_form_factor(lat, "d")
    assert np.array_equal(ss, ss.T) and np.array_equal(d, d.T)
    assert np.all(ss.sum(axis=1) == 4) and np.all(d.sum(axis=1) == 0)
    assert np.all(np.abs(d).sum(axis=1) == 4)
    with pytest.raises(ValueError):
        pair_form_factor(lat, "p")
    T = pkg.HubbardModel(lat, U=1.0).hopping_matrix()
    J = current_operator(T, lat)
    assert np.allclose(J, J.conj().T) and np.allclose(J.real, 0)
    Jy = current_operator(T, lat, direction=[0.0, 1.0])
    assert np.abs(J).sum() == np.abs(Jy).sum() > 0 and not np.allclose(J, Jy)
    lat2 = pkg.SquareLattice(2)
    assert np.allclose(current_operator(pkg.HubbardModel(lat2, U=1.0).hopping_matrix(), lat2), 0)
