"""Measurement kernels and the log binner (CPU)."""
import numpy as np


def test_logbinner_error_matches_ar1(pkg):
    """For an AR(1) series x_t = phi x_{t-1} + e_t the standard error of the
    mean is sigma_x sqrt((1 + phi) / ((1 - phi) N)); the binning estimate
    must land within 20 % of it."""
    rng = np.random.default_rng(0)
    phi, N = 0.8, 2 ** 16
    x = np.zeros(N)
    e = rng.standard_normal(N)
    for t in range(1, N):
        x[t] = phi * x[t - 1] + e[t]
    b = pkg.LogBinner()
    for v in x:
        b.push(v)
    sig = 1.0 / np.sqrt(1 - phi ** 2)
    want = sig * np.sqrt((1 + phi) / ((1 - phi) * N))
    assert abs(float(b.std_error()) / want - 1) < 0.2
    assert abs(float(b.tau()) - 0.5 * (1 + phi) / (1 - phi)) < 0.25 * (1 + phi) / (1 - phi)


def test_kernels_on_u0_greens(oracle, pkg):
    """At U = 0 the kernels reduce to closed forms of the analytic G."""
    model = pkg.HubbardModel(pkg.SquareLattice(4), U=0.0)
    G0 = oracle.analytic_greens(model.hopping_matrix(), 2.0)
    occ = pkg.occupation_kernel([G0])
    assert np.allclose(occ, 0.5, atol=1e-12)  # half filling
    docc = pkg.double_occupancy_kernel([G0, G0])
    assert np.allclose(docc, 0.25, atol=1e-12)
    C1 = pkg.spin_density_correlation_z([G0])
    C2 = pkg.spin_density_correlation_z([G0, G0])
    assert np.allclose(C1, C2, atol=1e-12)  # repeating and block forms agree
    pos = model.l.positions()
    S = pkg.structure_factor(C1, pos, (np.pi, np.pi))
    assert S > 0
    assert abs(pkg.interaction_energy([G0], 1.0)) < 1e-12


def test_lattice_conventions(pkg):
    """Site numbering x + Lx(y-1) + LxLy(b-1) and T = -t per directed bond
    (lattice.jl:240-373, HubbardModel.jl:112-124)."""
    sq = pkg.SquareLattice(4)
    T = pkg.HubbardModel(sq, U=1.0, mu=0.5).hopping_matrix()
    assert np.array_equal(T, T.T)
    assert np.allclose(np.diag(T), -0.5)
    assert np.all(np.sum(T != 0, axis=1) == 5)
    assert T[1, 0] == -1.0 and T[4, 0] == -1.0 and T[3, 0] == -1.0 and T[12, 0] == -1.0
    T2 = pkg.HubbardModel(pkg.SquareLattice(2), U=1.0).hopping_matrix()
    assert T2[1, 0] == -2.0  # +-x land on the same neighbour for L = 2
    hc = pkg.Honeycomb(3)
    Th = pkg.HubbardModel(hc, U=1.0).hopping_matrix()
    assert len(hc) == 18 and np.all(np.sum(Th != 0, axis=1) == 3)
    assert np.all(Th[:9, :9] == 0) and np.all(Th[9:, 9:] == 0)  # bipartite A/B blocks
    assert len(pkg.Chain(5)) == 5 and len(pkg.CubicLattice(2)) == 8


def test_parameters(pkg):
    """DQMCParameters (parameters.jl:84-139, test/flavortests_DQMC.jl:4-18)."""
    p = pkg.DQMCParameters.make(beta=4.0, delta_tau=0.1)
    assert p.slices == 40
    p = pkg.DQMCParameters.make(beta=5.0)
    assert p.delta_tau == 0.1 and p.slices == 50
    p = pkg.DQMCParameters.make(beta=2.0, slices=20)
    assert abs(p.delta_tau - 0.1) < 1e-15
    p = pkg.DQMCParameters.make(delta_tau=0.05, slices=10)
    assert abs(p.beta - 0.5) < 1e-15
    import pytest
    with pytest.raises(ValueError):
        pkg.DQMCParameters.make(beta=1.0, delta_tau=0.1, slices=11)


def test_field_alpha_and_flavours(pkg):
    """fields.jl:370-376, 419-425, 529-530, 599-600 and the sign rule of
    choose_field (HubbardModel.jl:83)."""
    import math
    import pytest
    p = pkg.DQMCParameters.make(beta=1.0, delta_tau=0.1)
    att = pkg.HubbardModel(pkg.SquareLattice(2), U=4.0)
    rep = pkg.HubbardModel(pkg.SquareLattice(2), U=-4.0)
    assert att.choose_field() is pkg.DensityHirschField
    assert rep.choose_field() is pkg.MagneticHirschField
    assert pkg.DensityHirschField(p, att).alpha == math.acosh(math.exp(0.5 * 0.1 * 4.0))
    assert pkg.MagneticHirschField(p, rep).alpha == math.acosh(math.exp(0.5 * 0.1 * 4.0))
    assert pkg.DensityGHQField(p, att).alpha == math.sqrt(0.2)
    assert pkg.MagneticGHQField(p, rep).alpha == math.sqrt(0.2)
    assert pkg.MagneticHirschField(p, rep).unique_flavors == 2
    # field/U mismatch: the complex path, alpha = i acos(exp(-0.2))
    assert pkg.DensityHirschField(p, rep).alpha == complex(0.0, 2 * math.atan2(
        math.sqrt(1 - math.exp(-0.2)), math.sqrt(1 + math.exp(-0.2))))


def test_config_recorder_roundtrip(pkg):
    """compress / decompress (fields.jl:331-334, 472-484) for both field families."""
    from montecarlo_gb300.dqmc import ConfigRecorder
    rng = np.random.default_rng(1)
    for ghq, values in ((False, np.array([-1, 1], dtype=np.int8)),
                        (True, np.array([1, 2, 3, 4], dtype=np.int8))):
        rec = ConfigRecorder(rate=2)
        confs = [np.asfortranarray(rng.choice(values, size=(7, 5))) for _ in range(6)]
        for s, c in enumerate(confs, start=1):
            rec.push(c, s, ghq=ghq)
        assert len(rec) == 3
        for i, c in enumerate(confs[1::2]):
            assert np.array_equal(rec[i], c)


def test_neighbour_partners(pkg):
    """Replica-exchange rounds pair neighbours, alternating even and odd pairs."""
    assert pkg.neighbour_partners(5, False).tolist() == [1, 0, 3, 2, -1]
    assert pkg.neighbour_partners(5, True).tolist() == [-1, 2, 1, 4, 3]


def test_time_displaced_kernel_reduces_to_equal_time(pkg):
    """With all four Green's functions equal to G and l = 0 the time-displaced
    kernel is the equal-time one."""
    rng = np.random.default_rng(4)
    for nf in (1, 2):
        G = rng.normal(size=(nf, 5, 5)) * 0.1 + 0.5 * np.eye(5)
        C0 = pkg.time_displaced_sdc_z(G, G, G, G, True)
        C1 = pkg.spin_density_correlation_z(G)
        assert np.max(np.abs(C0 - C1)) < 1e-14
