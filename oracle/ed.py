"""Exact diagonalisation of the Hubbard model on small lattices (numpy).

TEST INFRASTRUCTURE ONLY: the known-answer check the reference's ED tests
make (test/ED/ED.jl, HamiltonMatrix :68-121, calculate_Greens_matrix :515,
energy :539) restated: the grand-canonical Hamiltonian
    H = -t sum_{directed bonds, sigma} c^dag_{to,sigma} c_{from,sigma}
        + U_phys sum_i (n_{i,up} - 1/2)(n_{i,down} - 1/2) - mu sum_{i,sigma} n_{i,sigma}
with U_phys = -U (the reference's sign convention, ED.jl:71), Jordan-Wigner
fermions, and thermal expectation values at inverse temperature beta.
"""
from __future__ import annotations

import numpy as np


def _ops(nmodes):
    """Annihilation operators of nmodes fermionic modes (Jordan-Wigner)."""
    a = np.array([[0.0, 1.0], [0.0, 0.0]])  # |0><1| acting on a mode
    z = np.diag([1.0, -1.0])
    eye = np.eye(2)
    ops = []
    for m in range(nmodes):
        mats = [z] * m + [a] + [eye] * (nmodes - m - 1)
        o = mats[0]
        for x in mats[1:]:
            o = np.kron(o, x)
        ops.append(o)
    return ops


class HubbardED:
    def __init__(self, n_sites, bonds, t, U_ref, mu, beta):
        self.n = n_sites
        self.beta = beta
        modes = 2 * n_sites  # mode 2*i + s
        self.c = _ops(modes)
        c = self.c
        dim = 2 ** modes
        H = np.zeros((dim, dim))
        Uph = -U_ref
        for s in range(2):
            for fr, to in bonds:
                H += -t * c[2 * to + s].T @ c[2 * fr + s]
        self.nop = [[c[2 * i + s].T @ c[2 * i + s] for s in range(2)] for i in range(n_sites)]
        for i in range(n_sites):
            nu, nd = self.nop[i]
            H += Uph * (nu - 0.5 * np.eye(dim)) @ (nd - 0.5 * np.eye(dim))
            H += -mu * (nu + nd)
        self.H = H
        self.E, self.V = np.linalg.eigh(H)
        w = np.exp(-beta * (self.E - self.E.min()))
        self.rho_diag = w / w.sum()

    def expect(self, op):
        """<op> = Tr(rho op)."""
        M = self.V.T @ op @ self.V
        return float(np.sum(self.rho_diag * np.diag(M)))

    def greens(self):
        """G[s][i, j] = <c_{i,s} c^dag_{j,s}>."""
        out = np.zeros((2, self.n, self.n))
        for s in range(2):
            for i in range(self.n):
                for j in range(self.n):
                    out[s, i, j] = self.expect(self.c[2 * i + s] @ self.c[2 * j + s].T)
        return out

    def double_occupancy(self):
        return np.array([self.expect(self.nop[i][0] @ self.nop[i][1]) for i in range(self.n)])

    def sdc_z(self):
        m = [self.nop[i][0] - self.nop[i][1] for i in range(self.n)]
        return np.array([[self.expect(m[i] @ m[j]) for j in range(self.n)] for i in range(self.n)])

    def energy(self):
        return self.expect(self.H)

    def susceptibility_z(self, phases):
        """(1/n) int_0^beta dtau <M(tau) M(0)> with M = sum_i phases_i m_z(i)
        (real phases, e.g. cos(q.r_i) at q = (pi, pi)), from the spectral
        sum over eigenstates: sum_ab rho_a |M_ab|^2 (e^{beta (E_a - E_b)} - 1) / (E_b - E_a)."""
        Mop = sum(phases[i] * (self.nop[i][0] - self.nop[i][1]) for i in range(self.n))
        Mab = self.V.T @ Mop @ self.V
        E = self.E
        d = E[None, :] - E[:, None]          # E_b - E_a
        with np.errstate(over="ignore", invalid="ignore", divide="ignore"):
            f = np.where(np.abs(d) < 1e-12, self.beta, (1.0 - np.exp(-self.beta * d)) / d)
        return float(np.sum(self.rho_diag[:, None] * Mab ** 2 * f)) / self.n

    # ---- time-displaced correlations of the susceptibility measurements ----
    def operators(self, kind, phases):
        """(A, B) with C(tau) = <A(tau) B(0)>: the q-summed charge or spin
        density (phases_i weights) or the on-site pair field."""
        n, c = self.n, self.c
        if kind == "charge":
            O = [self.nop[i][0] + self.nop[i][1] for i in range(n)]
        elif kind == "spin_z":
            O = [self.nop[i][0] - self.nop[i][1] for i in range(n)]
        elif kind == "spin_x":
            O = [c[2 * i].T @ c[2 * i + 1] + c[2 * i + 1].T @ c[2 * i] for i in range(n)]
        elif kind == "spin_y":
            O = [-1j * (c[2 * i].T @ c[2 * i + 1] - c[2 * i + 1].T @ c[2 * i]) for i in range(n)]
        elif kind == "bilinear":   # phases is then the single-particle matrix A
            A = sum(phases[a, b] * c[2 * a + sg].T @ c[2 * b + sg]
                    for a in range(n) for b in range(n) for sg in range(2) if phases[a, b] != 0)
            return A, A.conj().T
        elif kind == "pairing":
            D = sum(c[2 * i] @ c[2 * i + 1] for i in range(n))   # sum_i c_i,up c_i,dn
            return D, D.conj().T
        elif kind == "pair_field":  # phases is then the form factor F[a, b]
            D = sum(phases[a, b] * c[2 * a] @ c[2 * b + 1]
                    for a in range(n) for b in range(n) if phases[a, b] != 0)
            return D, D.conj().T
        else:
            raise ValueError(kind)
        A = sum(phases[i] * O[i] for i in range(n))
        return A, A.conj().T

    def correlation(self, A, B, tau):
        """<A(tau) B(0)> = sum_ab rho_a A_ab B_ba e^{tau (E_a - E_b)}."""
        Aab = self.V.T @ A @ self.V
        Bba = (self.V.T @ B @ self.V).T
        E = self.E
        return complex(np.sum(self.rho_diag[:, None] * Aab * Bba *
                              np.exp(tau * (E[:, None] - E[None, :]))))

    def susceptibility(self, kind, phases):
        """(1/n) int_0^beta <A(tau) B(0)> dtau (pairing: plus the Delta^+ Delta
        term), by the spectral sum with (e^{beta (E_a - E_b)} - 1) / (E_a - E_b)."""
        E = self.E
        d = E[None, :] - E[:, None]          # E_b - E_a
        with np.errstate(over="ignore", invalid="ignore", divide="ignore"):
            f = np.where(np.abs(d) < 1e-12, self.beta, (1.0 - np.exp(-self.beta * d)) / d)
        terms = [self.operators("bilinear" if kind == "current" else kind, phases)]
        if kind in ("pairing", "pair_field"):
            A, B = terms[0]
            terms.append((B, A))
        tot = 0.0
        for A, B in terms:
            Aab = self.V.T @ A @ self.V
            Bba = (self.V.T @ B @ self.V).T
            tot += np.sum(self.rho_diag[:, None] * Aab * Bba * f)
        return float(np.real(tot)) / self.n

    def susceptibility_grid(self, kind, phases, delta_tau):
        """The same time integral on the imaginary-time grid l * delta_tau with
        the trapezoid weights of the reference's TimeIntegral (0.5 dtau at both
        ends), as the reference's ED tests integrate (expectation_value_integrated
        with step = delta_tau): the DQMC estimator's quadrature, exactly."""
        M = int(round(self.beta / delta_tau))
        terms = [self.operators("bilinear" if kind == "current" else kind, phases)]
        if kind in ("pairing", "pair_field"):
            A, B = terms[0]
            terms.append((B, A))
        tot = 0.0
        for l in range(M + 1):
            w = (0.5 if l in (0, M) else 1.0) * delta_tau
            for A, B in terms:
                tot += w * self.correlation(A, B, l * delta_tau)
        return float(np.real(tot)) / self.n
