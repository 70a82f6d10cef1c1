"""Shared helpers of the test-suite: matched GPU / oracle chains."""
import numpy as np


def make_setup(pkg, L=4, lattice="square", U=4.0, mu=0.0, beta=2.0, delta_tau=0.1, safe_mult=10,
               field=None):
    if lattice == "square":
        lat = pkg.SquareLattice(L)
    elif lattice == "honeycomb":
        lat = pkg.Honeycomb(L)
    elif lattice == "chain":
        lat = pkg.Chain(L)
    else:
        raise ValueError(lattice)
    model = pkg.HubbardModel(lat, U=U, mu=mu)
    param = pkg.DQMCParameters.make(beta=beta, delta_tau=delta_tau, safe_mult=safe_mult)
    fcls = field if field is not None else model.choose_field()
    fld = fcls(param, model)
    exps = pkg.hopping_exponentials(model.hopping_matrix(), param.delta_tau)
    return model, param, fld, exps


def chain_config(lib, model, param, fld, seed, check_prop=1):
    a = complex(fld.alpha)
    return lib.ChainConfig(len(model.l), fld.unique_flavors, param.slices, param.safe_mult,
                           fld.kind, check_prop, a.real, seed, a.imag)


def oracle_chain(oracle, model, param, fld, exps, seed, check_prop=True):
    return oracle.OracleChain(len(model.l), fld.unique_flavors, param.slices, param.safe_mult,
                              fld.kind, fld.alpha, exps, seed, check_prop)


FIELDS = ["DensityHirschField", "MagneticHirschField", "DensityGHQField", "MagneticGHQField"]
# reference sign convention: Density fields want U > 0, Magnetic fields U < 0
FIELD_U = {"DensityHirschField": 4.0, "MagneticHirschField": -4.0, "DensityGHQField": 4.0,
           "MagneticGHQField": -4.0}


def maxdiff(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))))
