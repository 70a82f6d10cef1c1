"""Hubbard model, parameters and Hubbard-Stratonovich fields (host side).

Mirrors src/models/HubbardModel.jl, src/flavors/DQMC/parameters.jl and the
field constructors of src/flavors/DQMC/fields.jl.  Sign convention is the
reference's: ``U > 0`` is attractive (DensityHirschField), ``U < 0`` is
repulsive (MagneticHirschField) -- HubbardModel.jl:15-16, 83.
"""
from __future__ import annotations

import cmath
import math
import warnings
from dataclasses import dataclass
from typing import Optional

import numpy as np

from .lattices import Lattice, choose_lattice

# field kind numbering shared with include/dqmc_gb300.h
DENSITY_HIRSCH = 0
MAGNETIC_HIRSCH = 1
DENSITY_GHQ = 2
MAGNETIC_GHQ = 3


class HubbardModel:
    """``HubbardModel(l; U, mu, t)`` / ``HubbardModel(L, dims; ...)``
    (HubbardModel.jl:23-46)."""

    def __init__(self, l: Optional[Lattice] = None, dims: int = 2, L: int = 2,
                 U: float = 1.0, mu: float = 0.0, t: float = 1.0, *args):
        if isinstance(l, int):  # HubbardModel(L, dims; kwargs...)
            L, dims, l = l, (dims if not args else args[0]), None
        if l is None:
            l = choose_lattice(dims, L)
        if U < 0.0 and mu != 0.0:
            warnings.warn(
                f"A repulsive Hubbard model with chemical potential mu = {mu} will have a sign problem!")
        self.t = float(t)
        self.mu = float(mu)
        self.U = float(U)
        self.l = l

    def __repr__(self):
        kind = "repulsive" if self.U < 0 else "attractive"
        return (f"{kind} Hubbard model\n\tParameters t = {self.t}, mu = {self.mu}, U = {self.U}\n"
                f"\t{self.l.name} with {len(self.l)} sites")

    @property
    def lattice(self) -> Lattice:
        return self.l

    def choose_field(self):
        """HubbardModel.jl:83."""
        return MagneticHirschField if self.U < 0.0 else DensityHirschField

    def hopping_matrix(self) -> np.ndarray:
        """T = diag(-mu) - t * sum over directed bonds (HubbardModel.jl:112-124)."""
        n = len(self.l)
        T = np.zeros((n, n))
        T[np.diag_indices(n)] = -self.mu
        for fr, to in self.l.bonds(True):
            T[to, fr] += -self.t
        return T


def AttractiveHubbardModel(*args, **kw):
    return HubbardModel(*args, **kw)


def RepulsiveHubbardModel(*args, **kw):
    """HubbardModel.jl:49-53: flips the sign of U."""
    kw = dict(kw)
    kw["U"] = -kw.get("U", 1.0)
    return HubbardModel(*args, **kw)


@dataclass
class DQMCParameters:
    """parameters.jl:84-139."""

    thermalization: int = 100
    sweeps: int = 100
    silent: bool = False
    check_sign_problem: bool = True
    check_propagation_error: bool = True
    safe_mult: int = 10
    delta_tau: float = 0.1
    beta: float = 1.0
    slices: int = 10
    measure_rate: int = 10
    print_rate: int = 10
    checkerboard: bool = False

    @classmethod
    def make(cls, thermalization=100, sweeps=100, silent=False, check_sign_problem=True,
             check_propagation_error=True, safe_mult=10, measure_rate=10, warn_round=True,
             print_rate=None, checkerboard=False, **kw):
        if print_rate is None:
            print_rate = max(10, (thermalization + sweeps) // 100)
        keys = set(kw)
        if keys == {"beta"}:
            kw = dict(beta=kw["beta"], delta_tau=0.1)
            keys = set(kw)
        if keys == {"delta_tau", "beta", "slices"}:
            dt, beta = kw["delta_tau"], kw["beta"]
            slices = _round_half_even(beta / dt)
            if slices != kw["slices"]:
                raise ValueError(f"Given slices ({kw['slices']}) does not match calculated slices "
                                 f"beta/delta_tau ~ {slices}")
        elif keys == {"beta", "slices"}:
            beta, slices = kw["beta"], kw["slices"]
            dt = beta / slices
        elif keys == {"delta_tau", "slices"}:
            dt, slices = kw["delta_tau"], kw["slices"]
            beta = dt * slices
        elif keys == {"delta_tau", "beta"}:
            dt, beta = kw["delta_tau"], kw["beta"]
            slices = _round_half_even(beta / dt)
            if warn_round and not math.isclose(slices, beta / dt, rel_tol=1.5e-8):
                warnings.warn(f"beta/delta_tau = {beta / dt} not an integer. Rounded to {slices}")
        else:
            raise ValueError(f"Invalid keyword arguments to DQMCParameters {kw}")
        return cls(thermalization, sweeps, silent, check_sign_problem, check_propagation_error,
                   safe_mult, float(dt), float(beta), int(slices), measure_rate, print_rate,
                   bool(checkerboard))


def _round_half_even(x: float) -> int:
    return int(round(x))  # Python rounds half to even, like Julia's round


class _Field:
    kind = -1
    unique_flavors = 1
    ghq = False

    def __init__(self, param: DQMCParameters, model: HubbardModel, U: Optional[float] = None):
        U = model.U if U is None else U
        self.alpha = self._alpha(param.delta_tau, U)
        self.n = len(model.l)
        self.slices = param.slices
        self.conf = np.zeros((self.n, self.slices), dtype=np.int8, order="F")

    @staticmethod
    def _real(x: complex, what: str = ""):
        """maybe_to_float (fields.jl:294): real when the imaginary part is
        below 10 eps of the real part, else the complex value (the
        reference's ComplexF64 field path)."""
        if isinstance(x, complex):
            if abs(x.imag) < 10 * np.spacing(abs(x.real)):
                return x.real
            return x
        return float(x)

    @property
    def is_complex(self) -> bool:
        return isinstance(self.alpha, complex)

    def energy_boson(self, conf=None):
        return 0.0


def _acosh_complex(z: complex) -> complex:
    """acosh of a complex number with Kahan's formula (W. Kahan, "Branch cuts
    for complex elementary functions", 1987), the one Julia's acosh(::Complex)
    uses: the sign of a zero imaginary part selects the branch."""
    zm1 = cmath.sqrt(complex(z.real - 1.0, z.imag))
    zp1 = cmath.sqrt(complex(z.real + 1.0, z.imag))
    xi = math.asinh((zm1.conjugate() * zp1).real)
    eta = 2.0 * math.atan2(zm1.imag, zp1.real)
    return complex(xi, eta)


def _hirsch_alpha(c: float, U: float):
    """acosh(exp(c * ComplexF64(U))) with the signed zero of c * (U + 0im)."""
    x = math.exp(c * U)
    if x >= 1.0:
        return math.acosh(x)
    z = cmath.exp(complex(c * U, c * 0.0))
    return _Field._real(_acosh_complex(complex(z.real, math.copysign(0.0, c))))


def _ghq_alpha(c: float, U: float):
    """sqrt(c * ComplexF64(U)) with the signed zero of c * (U + 0im)."""
    x = c * U
    if x >= 0:
        return math.sqrt(x)
    return _Field._real(cmath.sqrt(complex(x, c * 0.0)))


class DensityHirschField(_Field):
    """fields.jl:363-395: alpha = acosh(exp(0.5 dtau U))."""

    kind = DENSITY_HIRSCH

    def _alpha(self, dt, U):
        return _hirsch_alpha(0.5 * dt, U)

    def energy_boson(self, conf=None):
        conf = self.conf if conf is None else conf
        return self.alpha * float(np.sum(conf))


class MagneticHirschField(_Field):
    """fields.jl:412-451: alpha = acosh(exp(-0.5 dtau U))."""

    kind = MAGNETIC_HIRSCH
    unique_flavors = 2

    def _alpha(self, dt, U):
        return _hirsch_alpha(-0.5 * dt, U)


class DensityGHQField(_Field):
    """fields.jl:589-637: alpha = sqrt(0.5 dtau U)."""

    kind = DENSITY_GHQ
    ghq = True

    def _alpha(self, dt, U):
        return _ghq_alpha(0.5 * dt, U)


class MagneticGHQField(_Field):
    """fields.jl:519-573: alpha = sqrt(-0.5 dtau U)."""

    kind = MAGNETIC_GHQ
    unique_flavors = 2
    ghq = True

    def _alpha(self, dt, U):
        return _ghq_alpha(-0.5 * dt, U)


def hopping_exponentials(T: np.ndarray, delta_tau: float):
    """The four hopping exponentials of init_hopping_matrices (stack.jl:209-249):
    exp(-dtau T), exp(+dtau T), exp(-dtau T / 2), exp(+dtau T / 2).

    The reference's ``exp`` of a Hermitian matrix is an eigendecomposition
    followed by copying the upper triangle into the lower one, so each result
    is exactly symmetric; this does the same with numpy's ``eigh``.
    """
    if not np.array_equal(T, T.T):
        if not np.allclose(T, T.T, rtol=math.sqrt(np.finfo(float).eps)):
            raise ValueError("The hopping matrix is not approximately Hermitian.")
        warnings.warn("The hopping matrix is not exactly Hermitian.")
    lam, V = np.linalg.eigh(T)

    def ex(c):
        E = (V * np.exp(c * lam)) @ V.T
        iu = np.triu_indices(E.shape[0], 1)
        E[(iu[1], iu[0])] = E[iu]
        return np.asfortranarray(E)

    return ex(-delta_tau), ex(+delta_tau), ex(-0.5 * delta_tau), ex(+0.5 * delta_tau)


def generate_chunks(length: int, max_chunk: int):
    """stack.jl:154-158 (1-based inclusive (first, last) pairs)."""
    n = -(-length // max_chunk)
    step = length / n
    return [(_round_half_even((i - 1) * step) + 1, _round_half_even(i * step)) for i in range(1, n + 1)]


# ---- checkerboard decomposition of the hopping exponentials ------------------

def _is_reversal(b1, b2) -> bool:
    """lattice.jl:48-51."""
    return (b1.frm == b2.to and b1.to == b2.frm and
            all(a == -b for a, b in zip(b1.uc_shift, b2.uc_shift)))


def checkerboard_groups(lattice):
    """build_checkerboard (linalg/checkerboard.jl:14-140): bond groups in
    which every site occurs at most once, one bond direction per group, as
    0-based (src, trg) pairs, in the reference's order.

    Per directed unit-cell bond (the first of each reversal pair,
    lattice.jl:126-134) the bonds of all Bravais cells form a base group
    (duplicates and reversals within it dropped); a base group that chains
    (some bond starts where the first one ends) is split greedily into up to
    three site-disjoint groups.  The reference's filter of bonds repeated
    across base groups compares tuples with pairs and so never removes any;
    that is kept (no cross-group filter)."""
    uc = lattice.unitcell
    directed = []
    for i, b in enumerate(uc.bonds):
        if not any(_is_reversal(b, uc.bonds[j]) for j in directed):
            directed.append(i)
    nb = int(np.prod(lattice.Ls))
    out = []
    for j in directed:
        group = [lattice._shift_bravais(src, uc.bonds[j]) for src in range(1, nb + 1)]
        i = 0
        while i < len(group) - 1:
            s, t = group[i]
            k = i + 1
            while k < len(group):
                if group[k] == (s, t) or group[k] == (t, s):
                    del group[k]
                else:
                    k += 1
            i += 1
        s0, t0 = group[0]
        if any(g[0] == t0 for g in group):
            parts, used = [[], [], []], [set(), set(), set()]
            for s, t in group:
                for p in range(3):
                    if s not in used[p] and t not in used[p]:
                        parts[p].append((s, t))
                        used[p].update((s, t))
                        break
                else:
                    raise RuntimeError("Failed to distribute bonds into groups.")
            groups = [g for g in parts if g]
        else:
            groups = [group]
        out.extend([[(s - 1, t - 1) for s, t in g] for g in groups])
    return out


def checkerboard_factor(T: np.ndarray, groups, factor: float):
    """CheckerboardDecomposed(T, lattice, factor) (checkerboard.jl:203-270)
    of one flavour block: exp(factor T) ~ P_1 P_2 ... P_N D with
    D = exp(factor diag(T)) and, per group, P = 1 + (cosh(v) - 1) on the
    bond's two sites and sinh(v) between them (v = factor T[src, trg]); the
    parts are reversed for factor > 0 (the inverse's order).  Returns
    (D, [(c, s, partner), ...]) with per-site c (cosh or 1), s (sinh or 0)
    and partner site (-1: none)."""
    n = T.shape[0]
    D = np.exp(factor * np.diag(T))
    parts = []
    for g in groups:
        c, s, partner = np.ones(n), np.zeros(n), np.full(n, -1, dtype=np.int64)
        for src, trg in g:
            v = factor * T[src, trg]
            c[src] = c[trg] = math.cosh(v)
            s[src] = s[trg] = math.sinh(v)
            partner[src], partner[trg] = trg, src
        parts.append((c, s, partner))
    if factor > 0.0:
        parts.reverse()
    return D, parts


def checkerboard_matrix(D, parts) -> np.ndarray:
    """Dense form P_1 ... P_N D of a checkerboard factor (for tests)."""
    n = len(D)
    X = np.diag(D)
    for c, s, partner in reversed(parts):
        P = np.diag(c)
        for i in range(n):
            if partner[i] >= 0:
                P[i, partner[i]] = s[i]
        X = P @ X
    return X


def checkerboard_exponentials(T: np.ndarray, lattice, delta_tau: float):
    """The four hopping exponentials of init_hopping_matrices with
    checkerboard = true (stack.jl:240-246): factors -dtau, +dtau, -dtau/2,
    +dtau/2."""
    groups = checkerboard_groups(lattice)
    return [checkerboard_factor(T, groups, f)
            for f in (-delta_tau, +delta_tau, -0.5 * delta_tau, +0.5 * delta_tau)]


def checkerboard_pack(cb_factors):
    """Flat FP64 layout of the four checkerboard factors, as
    dqmc_set_checkerboard takes them: per factor D[n], then per part
    c[n], s[n], partner[n] (-1: none).  Returns (data, parts per factor)."""
    n_parts = len(cb_factors[0][1])
    out = []
    for D, parts in cb_factors:
        if len(parts) != n_parts:
            raise ValueError("all checkerboard factors need the same number of parts")
        out.append(np.asarray(D, dtype=np.float64))
        for c, s, partner in parts:
            out += [np.asarray(c, dtype=np.float64), np.asarray(s, dtype=np.float64),
                    np.asarray(partner, dtype=np.float64)]
    return np.ascontiguousarray(np.concatenate(out)), n_parts
