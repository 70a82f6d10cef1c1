"""The complex-field oracle (oracle/complex_oracle.py) pinned on the CPU.

A field whose kind does not match the sign of U has a complex constant alpha
(fields.jl:294, 372, 421, 530, 600): the reference then runs its ComplexF64
path (linalg/complex.jl).  Pins, in the reference's own test patterns:

* alpha: the branch Julia's acosh / sqrt pick from the signed zero of
  c * ComplexF64(U), and cosh(alpha) = exp(c U) (Hirsch), alpha^2 = c U (GHQ);
* udt_AVX_pivot! for complex matrices reconstructs its input with a unitary U
  (test/linalg.jl:97-132);
* calculate_greens(mc, slice) and the stack during a sweep agree with the
  independent slice-matrix chain (flavortests_DQMC.jl:243-301,
  test/testfunctions.jl);
* the local-update ratio is the determinant ratio, and the rank-1 update
  gives the Green's function of the new configuration (fields.jl tests,
  test/fields.jl:133-246);
* exact enumeration: the complex Hubbard-Stratonovich field reproduces, to
  rounding, the Green's function average of the real field of the other
  channel (both are exact decompositions of the same Trotterised model).
"""
import itertools
import math

import numpy as np
import pytest

import complex_oracle as CO
from _util import maxdiff

FIELDS = ["DensityHirschField", "MagneticHirschField", "DensityGHQField", "MagneticGHQField"]
# reference sign convention: the mismatched sign of U makes alpha complex
MISMATCH_U = {"DensityHirschField": -4.0, "MagneticHirschField": 4.0, "DensityGHQField": -4.0,
              "MagneticGHQField": 4.0}


def _setup(pkg, field, L=4, U=None, mu=0.0, beta=2.0, safe_mult=5, dt=0.1, lattice="square"):
    U = MISMATCH_U[field] if U is None else U
    lat = pkg.SquareLattice(L) if lattice == "square" else pkg.Chain(L)
    model = pkg.HubbardModel(lat, U=U, mu=mu)
    param = pkg.DQMCParameters.make(beta=beta, delta_tau=dt, safe_mult=safe_mult)
    fld = getattr(pkg, field)(param, model)
    exps = pkg.hopping_exponentials(model.hopping_matrix(), param.delta_tau)
    c = CO.ComplexChain(len(model.l), fld.unique_flavors, param.slices, param.safe_mult, fld.kind,
                        fld.alpha, exps, 5)
    return model, param, fld, exps, c


def _random_conf(c, ghq, seed):
    rng = np.random.default_rng(seed)
    if ghq:
        return rng.integers(1, 5, size=(c.n, c.M)).astype(np.int8)
    return (2 * rng.integers(0, 2, size=(c.n, c.M)) - 1).astype(np.int8)


def test_complex_alpha_branches(pkg):
    dt = 0.1
    param = pkg.DQMCParameters.make(beta=1.0, delta_tau=dt)
    for field, sign in (("DensityHirschField", 1), ("MagneticHirschField", -1),
                        ("DensityGHQField", 1), ("MagneticGHQField", -1)):
        U = MISMATCH_U[field]
        model = pkg.HubbardModel(pkg.SquareLattice(2), U=U)
        fld = getattr(pkg, field)(param, model)
        a = fld.alpha
        assert isinstance(a, complex) and fld.is_complex and a.real == 0.0
        assert math.copysign(1.0, a.imag) == sign
        c = 0.5 * dt if field.startswith("Density") else -0.5 * dt
        if "Hirsch" in field:
            assert abs(np.cosh(a) - math.exp(c * U)) < 1e-15
        else:
            assert abs(a * a - c * U) < 1e-15
        # matched sign: real alpha, as before
        matched = getattr(pkg, field)(param, pkg.HubbardModel(pkg.SquareLattice(2), U=-U))
        assert isinstance(matched.alpha, float) and not matched.is_complex


@pytest.mark.parametrize("n", [1, 2, 7, 16])
@pytest.mark.parametrize("apply_pivot", [True, False])
def test_complex_udt_reconstruction(n, apply_pivot):
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    A = A * np.exp(rng.uniform(-8, 8, n))[None, :]  # graded columns
    U, D, T, piv = CO.udt_pivot(A, apply_pivot)
    assert maxdiff(U.conj().T @ U, np.eye(n)) < 1e-13
    if apply_pivot:
        got = U @ np.diag(D) @ T
        assert maxdiff(got, A) < 1e-12 * np.abs(A).max()
    else:
        got = U @ np.diag(D) @ np.triu(T)
        assert maxdiff(got, A[:, piv]) < 1e-12 * np.abs(A).max()
        assert np.allclose(np.abs(np.diag(T)), 1.0)
    assert np.all(np.diff(D) <= 1e-12 * D.max())  # pivoted: non-increasing


@pytest.mark.parametrize("field", FIELDS)
def test_complex_calculate_greens_vs_direct_chain(pkg, field):
    model, param, fld, exps, c = _setup(pkg, field, mu=0.3)
    assert fld.is_complex
    c.set_conf(_random_conf(c, fld.ghq, 3))
    for sl in (0, 1, 7, 10, param.slices):
        G = c.calculate_greens_at(sl)
        Gd = CO.direct_greens(c, sl)
        assert maxdiff(G, Gd) < 1e-12 * max(1.0, np.abs(Gd).max()), sl
        assert np.abs(G.imag).max() > 1e-3  # genuinely complex


@pytest.mark.parametrize("field", ["DensityHirschField", "MagneticHirschField"])
def test_complex_stack_vs_direct_over_a_sweep(pkg, field):
    model, param, fld, exps, c = _setup(pkg, field, mu=0.5)
    c.set_conf(_random_conf(c, False, 4))
    c.initialize_run()
    for _ in range(2 * c.M + 3):
        Gd = CO.direct_greens(c, c.current_slice - 1)
        assert maxdiff(c.G, Gd) < 1e-11 * max(1.0, np.abs(Gd).max())
        c.propagate()
    assert c.prop_err_max < 1e-10


@pytest.mark.parametrize("field", FIELDS)
def test_complex_ratio_is_determinant_ratio(pkg, field):
    model, param, fld, exps, c = _setup(pkg, field, L=2, mu=0.4, beta=1.0)
    c.set_conf(_random_conf(c, fld.ghq, 5))
    c.initialize_run()
    for _ in range(5):
        c.propagate()
    sl = c.current_slice
    for j in range(c.n):
        old = c.conf.copy()
        xold = int(old[j, sl - 1])
        xnew = (xold % 4) + 1 if fld.ghq else 0
        t = (xold - 1) * 4 + (xnew - 1) if fld.ghq else (1 if xold > 0 else 0)
        p, R, dl = c.ratio(j, t, xnew, xold)
        G0 = CO.direct_greens(c, sl - 1)
        G_before = c.G.copy()
        c.accept(j, R, dl, xnew)
        G1 = CO.direct_greens(c, sl - 1)
        # det(I + B') / det(I + B) = det G / det G' per block (squared for nf = 1)
        det = 1.0 + 0j
        for b in range(c.nf):
            det *= np.linalg.det(G0[b]) / np.linalg.det(G1[b])
        if c.nf == 1:
            det = det * det
        a = complex(fld.alpha)
        if fld.kind == CO.DENSITY_HIRSCH:   # exp(-dE_boson), dE = -2 alpha s
            det *= np.exp(2 * a * xold)
        elif fld.kind == CO.DENSITY_GHQ:
            det *= np.exp(-a * (CO.ETA[xnew - 1] - CO.ETA[xold - 1]))
        if fld.ghq:
            det *= CO.GAMMA[xnew - 1] / CO.GAMMA[xold - 1]
        assert abs(p - det) < 1e-10 * max(1.0, abs(det)), (j, p, det)
        assert maxdiff(c.G, G1) < 1e-11 * max(1.0, np.abs(G1).max())
        assert maxdiff(G_before, G0) < 1e-11 * max(1.0, np.abs(G0).max())


@pytest.mark.parametrize("mu", [0.0, 0.4])
@pytest.mark.parametrize("U", [-4.0, 4.0])
def test_complex_enumeration_matches_real_field(pkg, U, mu):
    """Sum over all 2^(n M) Hirsch configurations of a 2-site chain, M = 4:
    the density- and magnetic-channel fields (one of them complex at either
    sign of U) give the same Green's function average."""
    means = []
    for field in ("DensityHirschField", "MagneticHirschField"):
        model, param, fld, exps, c = _setup(pkg, field, L=2, U=U, mu=mu, beta=0.4,
                                            safe_mult=10, lattice="chain")
        num, den = 0.0, 0.0
        for bits in itertools.product((-1, 1), repeat=c.n * c.M):
            conf = np.array(bits, dtype=np.int8).reshape((c.n, c.M), order="F")
            c.set_conf(conf)
            G = CO.direct_greens(c, 0)
            w = np.exp(-complex(fld.alpha) * conf.sum()) if fld.kind == CO.DENSITY_HIRSCH else 1.0
            for b in range(c.nf):
                w = w / np.linalg.det(G[b])
            if c.nf == 1:
                w = w / np.linalg.det(G[0])
            num = num + w * G[0]
            den = den + w
        means.append(num / den)
    assert maxdiff(means[0], means[1]) < 1e-12
    assert np.abs(means[0].imag).max() < 1e-12


def test_complex_sweeps_sign_problem_statistics(pkg):
    model, param, fld, exps, c = _setup(pkg, "DensityHirschField", mu=0.5)
    c.set_conf(_random_conf(c, False, 6))
    c.initialize_run()
    c.sweeps(2)
    assert c.n_imag_p > 0 and c.max_imag_p > 1e-6
    assert 0 < c.accepted < c.proposals == 2 * 2 * c.M * c.n
    Gd = CO.direct_greens(c, c.current_slice - 1)
    assert maxdiff(c.G, Gd) < 1e-10 * max(1.0, np.abs(Gd).max())


def test_direct_greens_kl_matches_real_oracle(pkg, oracle):
    """The defining products of G(k, l) reproduce the real oracle's
    UnequalTimeStack result on a real chain, which pins their convention."""
    from _util import make_setup, oracle_chain
    model, param, fld, exps = make_setup(pkg, L=2, U=4.0, beta=1.0, safe_mult=5,
                                         field=pkg.DensityHirschField)
    o = oracle_chain(oracle, model, param, fld, exps, 9)
    o.init_random_conf()
    c = CO.ComplexChain(len(model.l), 1, param.slices, param.safe_mult, fld.kind, fld.alpha,
                        exps, 9)
    c.set_conf(o.get_conf())
    M = param.slices
    pairs = [(0, 0), (3, 1), (1, 3), (M, 0), (0, M), (M - 1, 2), (2, M - 1)]
    for (k, l), g in zip(pairs, o.greens_kl(pairs)):
        assert maxdiff(CO.direct_greens_kl(c, k, l).real, g) < 1e-11, (k, l)
