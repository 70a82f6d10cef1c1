"""The CPU oracle against the known answers the reference's own tests pin.

* Philox4x32-10 against the published Random123 known-answer vectors.
* generate_chunks bounds (test/flavortests_DQMC.jl:244-262).
* U = 0: the equal-time G equals the analytic [1 + e^{-beta T}]^-1
  (test/flavortests_DQMC.jl:355-385, tolerance 1e-12).
* The stack's G equals an independent pivoted-QR chain
  (calculate_greens_and_logdet, test/flavortests_DQMC.jl:282-294, 303-311).
* 10 wraps agree with the recomputed G to 1e-9 (test/flavortests_DQMC.jl:296-301).
* build_stack and reverse_build_stack meet in the same state
  (test/flavortests_DQMC.jl:313-342).
* udt_AVX_pivot! reconstructs its input; rdivp! equals A P^T / T
  (test/linalg.jl:97-132, 240-261, 100 eps).
* update_greens! equals the dense Sherman-Morrison formula (test/fields.jl:133-246).
* Local sweeps produce no negative probabilities and no propagation errors
  (test/fields.jl:248-261).
"""
import numpy as np
import pytest

from _util import FIELD_U, FIELDS, make_setup, maxdiff, oracle_chain


def test_philox_known_answers(oracle):
    assert oracle.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert oracle.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [
        0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert oracle.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344],
                         [0xA4093822, 0x299F31D0]) == [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_generate_chunks(oracle, pkg):
    rng = np.random.default_rng(0)
    for _ in range(200):
        slices = int(rng.integers(1, 101))
        k = int(rng.integers(1, 13))
        ch = oracle.generate_chunks(slices, k)
        assert ch == pkg.generate_chunks(slices, k)
        assert ch[0][0] == 1 and ch[-1][1] == slices
        for (a, b), (c, _) in zip(ch, ch[1:]):
            assert c == b + 1
        for a, b in ch:
            assert 1 <= b - a + 1 <= k


@pytest.mark.parametrize("L,mu", [(7, 0.0), (8, 1.0)])
@pytest.mark.parametrize("beta", [1.0, 10.0])
def test_analytic_greens_u0(oracle, pkg, L, mu, beta):
    model, param, fld, exps = make_setup(pkg, L=L, U=0.0, mu=mu, beta=beta, safe_mult=5)
    c = oracle_chain(oracle, model, param, fld, exps, 1)
    c.init_random_conf()
    c.initialize_run()
    c.sweeps(2)
    G = c.greens_physical(c.greens())[0]
    Ga = oracle.analytic_greens(model.hopping_matrix(), beta)
    assert np.allclose(G, Ga, atol=1e-12, rtol=1e-12)


def _dense_B(pkg, model, fld, exps, conf, block):
    eta = np.array([-np.sqrt(6 + 2 * np.sqrt(6)), -np.sqrt(6 - 2 * np.sqrt(6)),
                    np.sqrt(6 - 2 * np.sqrt(6)), np.sqrt(6 + 2 * np.sqrt(6))])
    sign = 1.0 if block == 0 else -1.0
    out = []
    for l in range(conf.shape[1]):
        x = fld.alpha * (eta[conf[:, l] - 1] if fld.ghq else conf[:, l].astype(float))
        out.append(exps[0] * np.exp(sign * x)[None, :])
    return out


@pytest.mark.parametrize("field", FIELDS)
def test_calculate_greens_vs_direct_chain(oracle, pkg, field):
    model, param, fld, exps = make_setup(pkg, L=4, U=FIELD_U[field], beta=4.0, safe_mult=10,
                                         field=getattr(pkg, field))
    c = oracle_chain(oracle, model, param, fld, exps, 7)
    c.init_random_conf()
    conf = c.get_conf()
    # Hirsch fields are well conditioned here; the GHQ fields' larger couplings cost accuracy in
    # the direct chain too (both are stabilised QR chains)
    tol = 1e-12 if not fld.ghq else 1e-9
    for sl in (0, 1, 9, 10, 23, param.slices):
        G = c.calculate_greens_at(sl)
        for b in range(fld.unique_flavors):
            Bs = _dense_B(pkg, model, fld, exps, conf, b)
            Gd = oracle.direct_greens(Bs, sl, param.safe_mult)
            assert maxdiff(G[b], Gd) < tol * max(1.0, np.abs(Gd).max()), (sl, b)


def test_stack_greens_and_wraps(oracle, pkg):
    """flavortests_DQMC.jl:282-301 with a chain lattice (HubbardModel(8, 1)), beta = 5."""
    model = pkg.HubbardModel(8, 1)
    param = pkg.DQMCParameters.make(beta=5.0, delta_tau=0.1, safe_mult=1)
    fld = model.choose_field()(param, model)
    exps = pkg.hopping_exponentials(model.hopping_matrix(), param.delta_tau)
    c = oracle_chain(oracle, model, param, fld, exps, 3)
    c.init_random_conf()
    c.build_stack()
    c.propagate()
    cs = c.state()["current_slice"]
    G = c.calculate_greens_at(cs)
    G = c.wrap_greens(G, cs + 1, -1)
    assert np.allclose(G, c.greens(), atol=1e-12)
    assert maxdiff(c.calculate_greens_at(cs - 1), c.greens()) < 1e-12
    Gw = c.greens()
    for k in range(10):
        Gw = c.wrap_greens(Gw, cs - k, -1)
    assert maxdiff(c.calculate_greens_at(cs - 11), Gw) < 1e-9


def test_build_vs_reverse_build(oracle, pkg):
    """flavortests_DQMC.jl:313-342."""
    model = pkg.HubbardModel(8, 1)
    param = pkg.DQMCParameters.make(beta=5.0, delta_tau=0.1, safe_mult=10)
    fld = model.choose_field()(param, model)
    exps = pkg.hopping_exponentials(model.hopping_matrix(), param.delta_tau)
    c1 = oracle_chain(oracle, model, param, fld, exps, 9)
    c1.init_random_conf()
    c1.build_stack()
    c1.propagate()
    for _ in range(param.slices):
        c1.propagate()
    c2 = oracle_chain(oracle, model, param, fld, exps, 9)
    c2.set_conf(c1.get_conf())
    c2.reverse_build_stack()
    c2.propagate()
    assert c1.state() == c2.state()
    assert np.allclose(c1.greens(), c2.greens(), atol=1e-12)
    for which in (0, 1, 2):
        for idx in range(1, c1.state()["n_ranges"] + 2):
            assert np.allclose(c1.stack(which, idx), c2.stack(which, idx), atol=1e-10)


@pytest.mark.parametrize("n", [1, 2, 7, 16, 33])
@pytest.mark.parametrize("apply_pivot", [True, False])
def test_udt_pivot_reconstruction(oracle, n, apply_pivot):
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n))
    U, D, T, piv = oracle.udt_pivot(A, apply_pivot)
    assert np.allclose(U.T @ U, np.eye(n), atol=100 * np.finfo(float).eps * n)
    if apply_pivot:
        assert np.allclose(U @ np.diag(D) @ T, A, atol=100 * np.finfo(float).eps * n)
    else:
        R = np.triu(T)
        P = np.eye(n)[:, piv - 1]
        assert np.allclose(U @ np.diag(D) @ R, A @ P, atol=100 * np.finfo(float).eps * n)
        # rdivp!: A * (R P^T)^-1 for both forms
        X = rng.standard_normal((n, n))
        want = X @ np.linalg.inv(R @ P.T)
        for bf in (False, True):
            got = oracle.rdivp(X, T, piv, block_form=bf)
            assert np.allclose(got, want, atol=1e-10 * max(1, np.abs(want).max()))
    assert np.all(D > 0)


@pytest.mark.parametrize("nf", [1, 2])
def test_update_greens_sherman_morrison(oracle, nf):
    """G' = [I + (I + Delta e_i e_i^T) (G^-1 - I)]^-1 for a single-site change."""
    rng = np.random.default_rng(nf)
    n = 9
    G = np.stack([np.linalg.inv(np.eye(n) + rng.standard_normal((n, n)) * 0.3) for _ in range(nf)])
    delta = rng.uniform(-0.7, 1.5, nf)
    i = 4
    got = oracle.update_greens(G, delta, i)
    for b in range(nf):
        E = np.eye(n)
        E[i, i] += delta[b]
        # G = (I + A)^-1 ;  A -> A (I + Delta e_i e_i^T)
        A = np.linalg.inv(G[b]) - np.eye(n)
        want = np.linalg.inv(np.eye(n) + A @ E)
        assert np.allclose(got[b], want, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("field", FIELDS)
def test_sweeps_no_sign_problem_no_propagation_errors(oracle, pkg, field):
    model, param, fld, exps = make_setup(pkg, L=4, U=FIELD_U[field], beta=2.0, safe_mult=5,
                                         field=getattr(pkg, field))
    c = oracle_chain(oracle, model, param, fld, exps, 21)
    c.init_random_conf()
    c.initialize_run()
    acc = c.sweeps(5)
    a = c.analysis()
    assert a["negative_probability"] == 0
    assert a["propagation_error_count"] == 0
    assert 0 < acc < 5 * 2 * param.slices * len(model.l)
    st = c.state()
    assert maxdiff(c.greens(), c.calculate_greens_at(st["current_slice"] - 1)) < 1e-10


def test_replay_determinism(oracle, pkg):
    """Same seed -> identical field trajectory; the stream counter advances
    exactly by the draws the reference's order implies."""
    model, param, fld, exps = make_setup(pkg, L=4, U=4.0, beta=1.0, safe_mult=5)
    a = oracle_chain(oracle, model, param, fld, exps, 5)
    b = oracle_chain(oracle, model, param, fld, exps, 5)
    for c in (a, b):
        c.init_random_conf()
        assert c.rng_counter() == len(model.l) * param.slices
        c.initialize_run()
        c.sweeps(3)
    assert np.array_equal(a.get_conf(), b.get_conf())
    assert np.array_equal(a.greens(), b.greens())
    # Hirsch fields draw one uniform per proposal with p <= 1 only
    props = 3 * 2 * param.slices * len(model.l)
    assert len(model.l) * param.slices < a.rng_counter() <= len(model.l) * param.slices + props


@pytest.mark.parametrize("U,mu,field", [(1.0, 0.5, "DensityHirschField"),
                                        (1.0, 0.5, "DensityGHQField"),
                                        (-1.0, 0.0, "MagneticHirschField"),
                                        (-1.0, 0.0, "MagneticGHQField")])
def test_global_update_equals_product_of_local_updates(oracle, pkg, U, mu, field):
    """The backbone check of the reference's global and parallel updates
    (test/updates.jl:186-236): the probability of a global move to a shuffled
    configuration equals the product of the local-move probabilities along a
    path of single-site moves to the same configuration, and both end in the
    same configuration, slice and Green's function."""
    model, param, fld, exps = make_setup(pkg, L=2, U=U, mu=mu, beta=2.0,
                                         field=getattr(pkg, field))
    rng = np.random.default_rng(8)
    ghq = "GHQ" in field
    for trial in range(5):
        conf0 = (rng.integers(1, 5, size=(4, param.slices)) if ghq else
                 rng.choice([-1, 1], size=(4, param.slices))).astype(np.int8)
        o1 = oracle_chain(oracle, model, param, fld, exps, 3 + trial)
        o2 = oracle_chain(oracle, model, param, fld, exps, 3 + trial)
        for o in (o1, o2):
            o.set_conf(conf0)
            o.initialize_run()
        target = np.asfortranarray(rng.permuted(conf0.ravel(order="F")).reshape(conf0.shape,
                                                                                order="F"))
        detratio, dE = o1.global_detratio(target)
        global_p = abs(np.exp(-dE) * detratio)
        o1.replica_accept(target)
        local_p = 1.0
        for _ in range(param.slices):
            t = o2.state()["current_slice"]
            cur = o2.get_conf()
            for i in range(4):
                if cur[i, t - 1] != target[i, t - 1]:
                    local_p *= o2.local_move_to(i, int(target[i, t - 1]))
            o2.propagate()
        for _ in range(param.slices):
            o2.propagate()
        assert abs(local_p - global_p) <= 1.5e-8 * abs(global_p), (local_p, global_p)
        assert np.array_equal(o1.get_conf(), o2.get_conf())
        assert o1.state()["current_slice"] == o2.state()["current_slice"]
        assert maxdiff(o1.greens(), o2.greens()) < 1e-10


@pytest.mark.parametrize("field", FIELDS)
def test_global_flip_and_shuffle_keep_stack_consistent(oracle, pkg, field):
    """Global moves (accepted or rejected) leave a valid chain: G equals the
    from-scratch G of the resulting configuration, rejected moves restore the
    configuration, and local sweeps continue without propagation errors."""
    model, param, fld, exps = make_setup(pkg, L=2, U=FIELD_U[field], beta=2.0, safe_mult=5,
                                         field=getattr(pkg, field))
    o = oracle_chain(oracle, model, param, fld, exps, 21)
    o.init_random_conf()
    o.initialize_run()
    n_acc = 0
    for k in range(12):
        before = o.get_conf()
        acc = o.global_update(k % 2)
        n_acc += acc
        if not acc:
            assert np.array_equal(o.get_conf(), before)
        assert o.state()["current_slice"] == 1 and o.state()["direction"] == 1
        assert maxdiff(o.greens(), o.calculate_greens_at(0)) < 1e-9
        o.sweeps(1)
    assert o.global_stats() == (n_acc, 12)
    assert o.analysis()["propagation_error_reported"] < 1e-6


def _slice_B(exps, fld_kind, alpha, conf_col, nf, n):
    """B_l = exp(-dtau T) exp(V_l) per flavour block (the slice matrix of
    multiply_slice_matrix_left!, stack.jl:319-327)."""
    eT2 = np.asarray(exps[0])
    s = conf_col.astype(float)
    if fld_kind in (0, 1):
        v = [np.exp(alpha * s), np.exp(-alpha * s)]
    else:
        eta = np.array([-np.sqrt(6 + 2 * np.sqrt(6)), -np.sqrt(6 - 2 * np.sqrt(6)),
                        np.sqrt(6 - 2 * np.sqrt(6)), np.sqrt(6 + 2 * np.sqrt(6))])
        e = eta[conf_col.astype(int) - 1]
        v = [np.exp(alpha * e), np.exp(-alpha * e)]
    return [eT2 @ np.diag(v[b]) for b in range(nf)]


@pytest.mark.parametrize("field", ["DensityHirschField", "MagneticHirschField", "MagneticGHQField"])
def test_unequal_time_greens_known_answers(oracle, pkg, field):
    """The reference's unequal-time checks (test/DQMC/unequal_time_stack.jl:84-103):
    G(k, k) equals the equal-time G, G(k, 0) = -G(k, M); and the defining
    relations G(k, l) = B_k...B_{l+1} G(l) (k > l), G(k, l) = -(1 - G(k))
    (B_l...B_{k+1})^-1 (k < l) on a short chain."""
    model, param, fld, exps = make_setup(pkg, L=2, U=FIELD_U[field], beta=1.2, safe_mult=4,
                                         field=getattr(pkg, field))
    o = oracle_chain(oracle, model, param, fld, exps, 12)
    o.init_random_conf()
    o.initialize_run()
    M = param.slices
    pairs = [(k, k) for k in range(M + 1)] + [(k, 0) for k in range(M)] + \
            [(k, M) for k in range(M)] + [(7, 2), (2, 7), (11, 4), (3, 9), (M, 1), (0, M)]
    G = dict(zip(pairs, o.greens_kl(pairs)))
    eq = {k: o.calculate_greens_at(k) for k in range(M + 1)}
    for k in range(M + 1):
        assert maxdiff(G[(k, k)], eq[k]) < 1e-12, k
    for k in range(M):
        assert maxdiff(G[(k, 0)], -G[(k, M)]) < 1e-12, k
    conf = o.get_conf()
    nf, n = fld.unique_flavors, 4
    Bs = [None] + [_slice_B(exps, fld.kind, fld.alpha, conf[:, t - 1], nf, n) for t in range(1, M + 1)]
    for (k, l) in [(7, 2), (11, 4), (M, 1)]:
        for b in range(nf):
            P = np.eye(n)
            for t in range(l + 1, k + 1):
                P = Bs[t][b] @ P
            assert maxdiff(G[(k, l)][b], P @ eq[l][b]) < 1e-10, (k, l)
    for (k, l) in [(2, 7), (3, 9), (0, M)]:
        for b in range(nf):
            P = np.eye(n)
            for t in range(k + 1, l + 1):
                P = Bs[t][b] @ P
            ref = -(np.eye(n) - eq[k][b]) @ np.linalg.inv(P)
            assert maxdiff(G[(k, l)][b], ref) < 1e-10, (k, l)


def test_checkerboard_groups_and_factors(pkg):
    """build_checkerboard: site-disjoint groups that cover every bond once;
    the factors invert each other exactly and approximate exp(f T) to the
    Trotter order (exactly where the groups commute, as on 4x4)."""
    from scipy.linalg import expm
    from montecarlo_gb300 import model as M
    for lat in (pkg.SquareLattice(4), pkg.SquareLattice(3), pkg.SquareLattice(8), pkg.Honeycomb(2),
                pkg.Chain(6)):
        T = pkg.HubbardModel(lat, U=1.0, mu=0.3).hopping_matrix()
        groups = M.checkerboard_groups(lat)
        seen = set()
        for g in groups:
            sites = [s for b in g for s in b]
            assert len(sites) == len(set(sites))
            for s, t in g:
                seen.add((min(s, t), max(s, t)))
        nz = {(i, j) for i in range(len(T)) for j in range(i + 1, len(T)) if T[i, j] != 0}
        assert nz <= seen
        X = [M.checkerboard_matrix(*f) for f in M.checkerboard_exponentials(T, lat, 0.1)]
        assert np.abs(X[0] @ X[1] - np.eye(len(T))).max() < 1e-14
        assert np.abs(X[2] @ X[3] - np.eye(len(T))).max() < 1e-14
        assert np.abs(X[0] - expm(-0.1 * T)).max() < 0.02
    T = pkg.HubbardModel(pkg.SquareLattice(4), U=1.0).hopping_matrix()
    X0 = M.checkerboard_matrix(*M.checkerboard_exponentials(T, pkg.SquareLattice(4), 0.1)[0])
    assert np.abs(X0 - expm(-0.1 * T)).max() < 1e-14


@pytest.mark.parametrize("field", ["DensityHirschField", "MagneticHirschField"])
def test_checkerboard_chain_vs_direct(oracle, pkg, field):
    """With checkerboard = true the stack uses the factor products: G from the
    oracle's stack equals the direct QR chain of the dense checkerboard slice
    matrices (3x3: the groups do not commute, so this differs from the dense
    exponential path)."""
    from montecarlo_gb300 import model as M
    model, param, fld, exps = make_setup(pkg, L=3, U=FIELD_U[field], beta=2.0, safe_mult=5,
                                         field=getattr(pkg, field))
    T = model.hopping_matrix()
    cb = M.checkerboard_exponentials(T, model.l, param.delta_tau)
    X = [M.checkerboard_matrix(*f) for f in cb]
    cexps = [X[0], X[1], X[2], X[3]]
    c = oracle_chain(oracle, model, param, fld, exps, 31)
    c.set_checkerboard(*M.checkerboard_pack(cb))
    c.init_random_conf()
    conf = c.get_conf()
    for sl in (0, 3, 10, param.slices):
        G = c.calculate_greens_at(sl)
        for b in range(fld.unique_flavors):
            Bs = _dense_B(pkg, model, fld, cexps, conf, b)
            Gd = oracle.direct_greens(Bs, sl, param.safe_mult)
            assert maxdiff(G[b], Gd) < 1e-12 * max(1.0, np.abs(Gd).max()), (sl, b)
    c.initialize_run()
    c.sweeps(2)
    assert c.analysis()["propagation_error_reported"] < 1e-8
    Gp = c.greens_physical(c.greens())
    for b in range(fld.unique_flavors):
        ref = X[3] @ c.greens()[b] @ X[2]
        assert maxdiff(Gp[b], ref) < 1e-13
