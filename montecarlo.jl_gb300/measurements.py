"""Equal-time measurements on the physical Green's function, and log binning.

Kernels follow src/flavors/DQMC/measurements/constructors/*.jl with the
reference's greens-matrix conventions: ``G[b]`` is flavour block b of the
physical equal-time G = <c_i c_j^dagger> (greens.jl:94-125); one block means
the spin-degenerate (DiagonallyRepeatingMatrix) case, two blocks the
BlockDiagonal case of the MagneticHirsch / MagneticGHQ fields.

``LogBinner`` restates the binning error analysis of BinningAnalysis.jl (the
reference's observable container, generic.jl:57-69): values are averaged in
bins of size 2^k; the error of the mean at level k is sqrt(var_k / n_k); the
reported error uses the highest level with at least 32 bins.
"""
from __future__ import annotations

import numpy as np


class LogBinner:
    """Running log binning of scalar or array observables."""

    def __init__(self, min_bins: int = 32):
        self.values = []
        self.min_bins = min_bins

    def push(self, v):
        self.values.append(np.array(v, dtype=np.float64, copy=True))

    def __len__(self):
        return len(self.values)

    def mean(self):
        return np.mean(np.stack(self.values), axis=0)

    def _levels(self):
        x = np.stack(self.values)
        out = []
        k = 0
        while True:
            b = 2 ** k
            nb = x.shape[0] // b
            if nb < 2:
                break
            m = x[: nb * b].reshape((nb, b) + x.shape[1:]).mean(axis=1)
            out.append((k, nb, np.sqrt(np.var(m, axis=0, ddof=1) / nb)))
            k += 1
        return out

    def std_error(self):
        levels = self._levels()
        if not levels:
            return np.full(np.shape(self.values[0]), np.inf)
        ok = [lv for lv in levels if lv[1] >= self.min_bins]
        return (ok[-1] if ok else levels[0])[2]

    def tau(self):
        """Integrated autocorrelation time estimate from the binning ratio."""
        levels = self._levels()
        if not levels:
            return np.nan
        e0 = levels[0][2]
        e = self.std_error()
        with np.errstate(divide="ignore", invalid="ignore"):
            return 0.5 * ((e / e0) ** 2 - 1.0)


def greens_kernel(G):
    """greens_kernel (constructors/greens.jl:39-40): G itself."""
    return np.array(G)


def occupation_kernel(G):
    """<n_{i,flv}> = 1 - G_ii per flavour block (occupation.jl:44-55)."""
    return np.stack([1.0 - np.diag(g) for g in G])


def double_occupancy(G):
    """<n_{i,up} n_{i,down}> per site.  Spin-diagonal G: the Wick contraction
    has no up-down exchange term, so it is (1 - G^up_ii)(1 - G^down_ii); one
    block means G^up = G^down."""
    up = 1.0 - np.diag(G[0])
    dn = 1.0 - np.diag(G[-1])
    return up * dn


def interaction_energy(G, U):
    """interaction_energy_kernel (HubbardModel.jl:160-183) with the reference's
    U: -U sum (G_ii - 1/2)^2 (one block) or -U sum (G^1_ii - 1/2)(G^2_ii - 1/2)."""
    a = np.diag(G[0]) - 0.5
    b = np.diag(G[-1]) - 0.5
    return -U * float(np.sum(a * b))


def spin_density_correlation_z(G):
    """Equal-time <m_z(i) m_z(j)> with m_z = n_up - n_down, all site pairs
    (full_sdc_z_kernel, spin_density.jl:182-227, at tau = 0)."""
    n = G[0].shape[0]
    eye = np.eye(n)
    if len(G) == 1:
        g = G[0]
        return 2.0 * (eye - g.T) * g
    g1, g2 = G
    o1 = 1.0 - np.diag(g1)
    o2 = 1.0 - np.diag(g2)
    dis = np.outer(o1, o1) - np.outer(o1, o2) - np.outer(o2, o1) + np.outer(o2, o2)
    exch = (eye - g1.T) * g1 + (eye - g2.T) * g2
    return dis + exch


def structure_factor(corr, positions, q):
    """S(q) = (1/N) sum_ij exp(i q (r_i - r_j)) C_ij for an N x N correlation."""
    r = np.asarray(positions, dtype=float)
    ph = np.exp(1j * (r @ np.asarray(q, dtype=float)))
    return float(np.real(np.conj(ph) @ corr @ ph) / len(r))


def time_displaced_sdc_z(G00, G0l, Gl0, Gll, at_zero):
    """<m_z(i, tau) m_z(j, 0)> for all site pairs from the four Green's
    functions G(0,0), G(0,l), G(l,0), G(l,l) (full_sdc_z_kernel,
    spin_density.jl:182-227); ``at_zero``: l == 0 (the delta of the
    time-ordered contraction)."""
    n = G00.shape[1]
    idm = np.eye(n) if at_zero else np.zeros((n, n))
    if G00.shape[0] == 1:
        return 2.0 * (idm - G0l[0].T) * Gl0[0]
    ml = np.diag(Gll[1]) - np.diag(Gll[0])      # (1 - G1_ii) - (1 - G2_ii)
    m0 = np.diag(G00[1]) - np.diag(G00[0])
    exch = sum((idm - G0l[b].T) * Gl0[b] for b in range(2))
    return np.outer(ml, m0) + exch


CORRELATIONS = ("charge", "spin_x", "spin_y", "spin_z", "pairing")


def time_displaced_correlations(G00, G0l, Gl0, Gll, at_zero):
    """<A_i(l dtau) B_j(0)> for all site pairs, from G(0,0), G(0,l), G(l,0),
    G(l,l), for the Wick-expanded kernels of the reference (BlockDiagonal
    spin blocks, or one block repeated for both spins):

    * "charge": full_cdc_kernel (charge_density.jl:65-112), n = n_up + n_dn;
    * "spin_x", "spin_y": full_sdc_x/y_kernel (spin_density.jl:100-169);
    * "spin_z": full_sdc_z_kernel (spin_density.jl:182-227);
    * "pairing": pc_combined_kernel (pairing.jl:95-161) on site
      (Delta_i = c_i,up c_i,dn): <Delta_i(tau) Delta_j^+(0)> + <Delta_i^+(tau) Delta_j(0)>.

    ``at_zero``: l == 0 (the delta of the time-ordered contraction)."""
    n = G00.shape[1]
    idm = np.eye(n) if at_zero else np.zeros((n, n))
    out = {}
    if G00.shape[0] == 1:
        g00, g0l, gl0, gll = G00[0], G0l[0], Gl0[0], Gll[0]
        ex = (idm - g0l.T) * gl0
        out["charge"] = 4.0 * np.outer(1.0 - np.diag(gll), 1.0 - np.diag(g00)) + 2.0 * ex
        out["spin_x"] = out["spin_y"] = out["spin_z"] = 2.0 * ex
        out["pairing"] = gl0 * gl0 + (idm - g0l.T) * (idm - g0l.T)
        return out
    occ_l = [1.0 - np.diag(Gll[b]) for b in range(2)]
    occ_0 = [1.0 - np.diag(G00[b]) for b in range(2)]
    ex = [(idm - G0l[b].T) * Gl0[b] for b in range(2)]
    out["charge"] = sum(np.outer(occ_l[a], occ_0[b]) for a in range(2) for b in range(2)) + \
        ex[0] + ex[1]
    out["spin_x"] = out["spin_y"] = (idm - G0l[0].T) * Gl0[1] + (idm - G0l[1].T) * Gl0[0]
    ml = occ_l[0] - occ_l[1]
    m0 = occ_0[0] - occ_0[1]
    out["spin_z"] = np.outer(ml, m0) + ex[0] + ex[1]
    out["pairing"] = Gl0[0] * Gl0[1] + (idm - G0l[1].T) * (idm - G0l[0].T)
    return out


def current_operator(T, lattice, direction=None):
    """Single-particle matrix A of the paramagnetic current J = sum_sigma
    sum_ab A_ab c^+_a c_b along ``direction`` (default: the first lattice
    vector): the sum over directed bonds (s -> t) whose displacement points
    along +direction of the reference's bond current
    j(s, t) = i T[s, t] c^+_t c_s - i T[t, s] c^+_s c_t (cc_kernel,
    current_current.jl:44-61) with T the hopping matrix."""
    uc = lattice.unitcell
    vecs = np.asarray(uc.lattice_vectors, dtype=float)
    sites = np.asarray(uc.sites, dtype=float)
    e = vecs[0] if direction is None else np.asarray(direction, dtype=float)
    nbu = len(uc.bonds)
    n = T.shape[0]
    A = np.zeros((n, n), dtype=np.complex128)
    for k, (s, t) in enumerate(lattice.bonds()):
        b = uc.bonds[k % nbu]
        disp = sites[b.to - 1] - sites[b.frm - 1] + np.asarray(b.uc_shift, dtype=float) @ vecs
        if disp @ e > 1e-12:
            A[t, s] += 1j * T[s, t]
            A[s, t] += -1j * T[t, s]
    return A


def pair_form_factor(lattice, kind="s"):
    """Form-factor matrix F of the pair field Delta = sum_ab F[a, b] c_a,up c_b,dn:
    "s" on-site (F = I), "s*" extended s-wave (1 on every nearest-neighbour
    bond) and "d" (d_x2-y2: +1 on bonds along the first lattice vector, -1
    along the second) -- the reference's pairing quads of
    EachLocalQuadByDistance (pairing.jl:1-52) contracted with these form
    factors."""
    n = len(lattice)
    if kind == "s":
        return np.eye(n)
    uc = lattice.unitcell
    vecs = np.asarray(uc.lattice_vectors, dtype=float)
    sites = np.asarray(uc.sites, dtype=float)
    nbu = len(uc.bonds)
    F = np.zeros((n, n))
    for k, (a, b) in enumerate(lattice.bonds()):
        bond = uc.bonds[k % nbu]
        disp = sites[bond.to - 1] - sites[bond.frm - 1] + np.asarray(bond.uc_shift, float) @ vecs
        if kind == "s*":
            F[a, b] += 1.0
        elif kind == "d":
            if abs(abs(disp @ vecs[0]) - vecs[0] @ vecs[0]) < 1e-9 and abs(disp @ vecs[1]) < 1e-9:
                F[a, b] += 1.0
            elif abs(abs(disp @ vecs[1]) - vecs[1] @ vecs[1]) < 1e-9 and abs(disp @ vecs[0]) < 1e-9:
                F[a, b] -= 1.0
        else:
            raise ValueError(f"unknown pairing form factor {kind!r}")
    return F


def pair_correlation(F, G00, G0l, Gl0, Gll, at_zero):
    """<Delta(l dtau) Delta^+(0)> + <Delta^+(l dtau) Delta(0)> for the pair field
    Delta = sum_ab F[a, b] c_a,up c_b,dn (pc_combined_kernel, pairing.jl:95-161,
    summed with the form factor): sum(conj(F) o (Gl0_up^T F Gl0_dn)) +
    sum(conj(F) o (X_up^T F X_dn)), X = id - G0l; one block serves both spins."""
    up, dn = (0, 0) if G00.shape[0] == 1 else (0, 1)
    n = G00.shape[1]
    idm = np.eye(n) if at_zero else np.zeros((n, n))
    Fc = np.conj(F)
    t1 = np.sum(Fc * (Gl0[up].T @ F @ Gl0[dn]))
    t2 = np.sum(Fc * ((idm - G0l[up]).T @ F @ (idm - G0l[dn])))
    return t1 + t2


def bilinear_correlation(A, B, G00, G0l, Gl0, Gll, at_zero):
    """<O_A(l dtau) O_B(0)> for spin-summed bilinears O_A = sum_sigma sum_ab
    A_ab c^+_a c_b (Wick's theorem with G(0,0), G(0,l), G(l,0), G(l,l); one
    block counts for both spins): tr[A (I - Gll)] tr[B (I - G00)] +
    tr[A Gl0 B (id - G0l)], summed over spin blocks."""
    n = G00.shape[1]
    eye = np.eye(n)
    rep = 2.0 if G00.shape[0] == 1 else 1.0
    nb = G00.shape[0]
    t1 = rep * sum(np.trace(A @ (eye - Gll[b])) for b in range(nb))
    t2 = rep * sum(np.trace(B @ (eye - G00[b])) for b in range(nb))
    idm = eye if at_zero else 0.0 * eye
    ex = rep * sum(np.trace(A @ Gl0[b] @ B @ (idm - G0l[b])) for b in range(nb))
    return t1 * t2 + ex


def td_arrays(model, q=None, current_direction=None):
    """Inputs of the device time-displaced measurements for ``model``'s
    lattice: the by-distance slot of every site pair (src + n trg order, the
    reference's EachSitePairByDistance), cos / sin (q . r_i) (q defaults to
    (pi, pi, ...)), the extended-s and d pair form factors as (a, b, F) bond
    lists (lattices with at least two lattice vectors) and the uniform
    current operator along ``current_direction`` as (r, s, A_rs) entries."""
    lat = model.l
    n = len(lat)
    slot = lat.pair_distance_index()
    pos = lat.positions()
    qv = np.full(pos.shape[1], np.pi) if q is None else np.asarray(q, dtype=float)
    ph = pos @ qv
    sites, vals, nform = [], [], [0, 0]
    if len(lat.unitcell.lattice_vectors) >= 2:
        for f, kind in enumerate(("s*", "d")):
            F = pair_form_factor(lat, kind)
            a, b = np.nonzero(F)
            sites += [np.stack([a, b], axis=1).ravel()]
            vals += [F[a, b]]
            nform[f] = len(a)
    A = current_operator(model.hopping_matrix(), lat, current_direction)
    r, c = np.nonzero(A)
    return {"n_slots": int(slot.max()) + 1, "pair_slot": slot.ravel(order="F"),
            "q_cos": np.cos(ph), "q_sin": np.sin(ph), "n_form": nform,
            "form_sites": np.concatenate(sites) if sites else None,
            "form_values": np.concatenate(vals) if vals else None,
            "n_current": len(r),
            "current_sites": np.stack([r, c], axis=1).ravel() if len(r) else None,
            "current_values": np.stack([A[r, c].real, A[r, c].imag], axis=1).ravel()
            if len(r) else None, "n_sites": n}


def by_distance(C, slot, n_slots):
    """The reference's EachSitePairByDistance reduction of a correlation
    matrix C[src, trg]: sum over the pairs of every slot, divided by the
    number of sites (generic.jl:434-461, 582-584)."""
    out = np.zeros(n_slots)
    np.add.at(out, np.asarray(slot).ravel(), np.asarray(C).ravel())
    return out / C.shape[0]


def susceptibilities(greens_by_l, phases, delta_tau, kinds=CORRELATIONS, current=None,
                     pair_fields=None):
    """chi_K(q) = (1/n) sum_l w_l sum_ij e^{i q (r_i - r_j)} C_K(i, j; l dtau)
    for the correlations K of ``time_displaced_correlations``, with the
    TimeIntegral's trapezoid weights (generic.jl:337-366) and real phases
    (cos(q.r_i), sin(q.r_i)); the pairing susceptibility is summed without
    phases (the q = 0 on-site s-wave channel).  The reference's
    charge_density_susceptibility, spin_density_susceptibility(:x/:y/:z)
    and pairing_susceptibility with an on-site lattice iterator.  With
    ``current`` (a ``current_operator`` matrix) also "current": the uniform
    current-current susceptibility (1/n) int <J(tau) J(0)> dtau, the q = 0
    sum of the reference's current_current_susceptibility.  ``pair_fields``
    ({name: F}, see ``pair_form_factor``) adds "pairing_<name>" per form factor."""
    c, s = phases
    n = len(c)
    ones = np.ones(n)
    M = len(greens_by_l) - 1
    chi = {k: 0.0 for k in kinds}
    if current is not None:
        chi["current"] = 0.0
    for name in (pair_fields or {}):
        chi["pairing_" + name] = 0.0
    for l, (G00, G0l, Gl0, Gll) in enumerate(greens_by_l):
        C = time_displaced_correlations(G00, G0l, Gl0, Gll, l == 0)
        w = (0.5 if l in (0, M) else 1.0) * delta_tau
        for k in kinds:
            if k == "pairing":
                chi[k] += w * float(np.real(ones @ C[k] @ ones))
            else:
                chi[k] += w * float(np.real(c @ C[k] @ c + s @ C[k] @ s))
        if current is not None:
            chi["current"] += w * float(np.real(
                bilinear_correlation(current, current, G00, G0l, Gl0, Gll, l == 0)))
        for name, F in (pair_fields or {}).items():
            chi["pairing_" + name] += w * float(np.real(
                pair_correlation(F, G00, G0l, Gl0, Gll, l == 0)))
    return {k: v / n for k, v in chi.items()}


def spin_susceptibility_z(greens_by_l, phases, delta_tau):
    """chi_z(q) = (1/n) sum_l w_l sum_ij e^{i q (r_i - r_j)} <m_z(i, l dtau) m_z(j, 0)>
    with the trapezoid weights of the reference's TimeIntegral
    (generic.jl:337-366: 0.5 dtau at l = 0 and l = M, dtau otherwise) and real
    phases (cos(q.r_i), sin(q.r_i)).  greens_by_l[l] = (G00, G0l, Gl0, Gll)."""
    c, s = phases
    M = len(greens_by_l) - 1
    chi = 0.0
    for l, (G00, G0l, Gl0, Gll) in enumerate(greens_by_l):
        C = time_displaced_sdc_z(G00, G0l, Gl0, Gll, l == 0)
        w = (0.5 if l in (0, M) else 1.0) * delta_tau
        chi += w * float(c @ C @ c + s @ C @ s)
    return chi / len(c)


MEASUREMENTS = {
    "greens": greens_kernel,
    "occupation": occupation_kernel,
    "double_occupancy": double_occupancy,
    "spin_density_correlation_z": spin_density_correlation_z,
}
