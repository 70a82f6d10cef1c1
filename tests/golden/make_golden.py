"""Generate the golden fixtures of tests/test_golden.py (run from the repository root:
``python tests/golden/make_golden.py``).

The reference (Julia) cannot run here, so the fixtures come from the
reference's own known-answer recipes, restated:

* ``analytic_u0.npz``: the U = 0 equal-time Green's function
  U diag(1 / (1 + e^{-beta lambda})) U^-1 of the hopping matrix
  (test/testfunctions.jl:128-165) for a 4x4 lattice at mu = 0.5, beta = 2 and a
  6-site chain at mu = -0.3, beta = 5;
* ``ed_2x2.npz``: exact diagonalisation of the 2x2 Hubbard model
  (test/ED/ED.jl restated in oracle/ed.py) at U = +-1, beta = 1: the Green's
  function, double occupancies, the z spin-density correlation, and the
  susceptibilities integrated on the dtau = 0.1 grid;
* ``oracle_trajectory.npz``: the CPU oracle's state after two sweeps of a 4x4
  DensityHirschField chain (U = 4, beta = 1, seed 7): field configuration, RNG
  counter, accepted count and G -- a regression fixture for the oracle and the
  CUDA path, which must reproduce the configuration bit for bit.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle")]


def main():
    import __graft_entry__ as g
    pkg = g.load_package()
    import ed
    import oracle as O
    O.build()

    out = {}
    for name, lat, mu, beta in (("square4", pkg.SquareLattice(4), 0.5, 2.0),
                                ("chain6", pkg.Chain(6), -0.3, 5.0)):
        T = pkg.HubbardModel(lat, U=0.0, mu=mu).hopping_matrix()
        out[name + "_T"] = T
        out[name + "_beta"] = np.array(beta)
        out[name + "_G"] = O.analytic_greens(T, beta)
    np.savez_compressed(os.path.join(HERE, "analytic_u0.npz"), **out)

    out = {}
    for U in (-1.0, 1.0):
        model = pkg.HubbardModel(pkg.SquareLattice(2), U=U, mu=0.0)
        E = ed.HubbardED(4, model.l.bonds(), 1.0, U, 0.0, 1.0)
        key = "Um" if U < 0 else "Up"
        out[key + "_G"] = E.greens()
        out[key + "_docc"] = E.double_occupancy()
        out[key + "_sdcz"] = E.sdc_z()
        ph = np.cos(model.l.positions() @ np.array([np.pi, np.pi]))
        out[key + "_chi"] = np.array([E.susceptibility_grid(k, ph, 0.1) for k in pkg.CORRELATIONS])
    np.savez_compressed(os.path.join(HERE, "ed_2x2.npz"), **out)

    model = pkg.HubbardModel(pkg.SquareLattice(4), U=4.0)
    param = pkg.DQMCParameters.make(beta=1.0, delta_tau=0.1, safe_mult=5)
    fld = pkg.DensityHirschField(param, model)
    exps = pkg.hopping_exponentials(model.hopping_matrix(), param.delta_tau)
    c = O.OracleChain(16, 1, param.slices, 5, fld.kind, fld.alpha, exps, 7)
    c.init_random_conf()
    c.initialize_run()
    c.sweeps(2)
    np.savez_compressed(os.path.join(HERE, "oracle_trajectory.npz"), conf=c.get_conf(),
                        counter=np.array(c.rng_counter(), dtype=np.uint64),
                        accepted=np.array(c.analysis()["accepted"]), G=c.greens())

    # the complex (field / sign(U) mismatch) oracle: 4x4, DensityHirschField at
    # repulsive U, mu = 0.3, two sweeps from a fixed configuration
    import complex_oracle as CO
    cx = complex_trajectory(pkg, CO)
    np.savez_compressed(os.path.join(HERE, "complex_trajectory.npz"), **cx)


def complex_trajectory(pkg, CO):
    model = pkg.HubbardModel(pkg.SquareLattice(4), U=-4.0, mu=0.3)
    param = pkg.DQMCParameters.make(beta=1.0, delta_tau=0.1, safe_mult=5)
    fld = pkg.DensityHirschField(param, model)
    exps = pkg.hopping_exponentials(model.hopping_matrix(), param.delta_tau)
    c = CO.ComplexChain(16, 1, param.slices, 5, fld.kind, fld.alpha, exps, 11)
    rng = np.random.default_rng(11)
    conf0 = (2 * rng.integers(0, 2, size=(16, param.slices)) - 1).astype(np.int8)
    c.set_conf(conf0)
    c.initialize_run()
    c.sweeps(2)
    return dict(conf0=conf0, conf=c.conf, counter=np.array(c.ctr, dtype=np.uint64),
                accepted=np.array(c.accepted), n_imag=np.array(c.n_imag_p), G=c.G)


if __name__ == "__main__":
    main()
