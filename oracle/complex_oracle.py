"""CPU oracle of the reference's complex (ComplexF64) DQMC path, in numpy.

TEST INFRASTRUCTURE ONLY: imported by tests/; the product never imports it.

A field whose Hubbard-Stratonovich constant alpha is complex -- its kind does
not match the sign of U, e.g. a DensityHirschField for repulsive U in the
reference's sign convention -- turns the interaction exponentials, the Green's
function and the acceptance ratios complex (src/flavors/DQMC/fields.jl:294,
372, 421, 530, 600).  This module restates that path of the reference with
complex128 matrices, one flavour block at a time:

* ``udt_pivot``: udt_AVX_pivot! for CMat64 (linalg/complex.jl:386-696):
  Householder QR with column pivoting, reflector nu = copysign(|x|, re x_1),
  U accumulated backwards, D = |R_ii|, T = D^-1 R (pivot applied or not).
* ``rdivp``: rdivp! for CMat64 (complex.jl:292-380).
* ``calculate_greens_udt``: calculate_greens_AVX! (stack.jl:442-496).
* ``ComplexChain``: the DQMCStack state machine -- reverse_build_stack,
  build_stack, add_slice_sequence_left/right, propagate with the propagation
  error check, wrap_greens! and the slice-matrix products (stack.jl:154-730) --
  and the local sweep (local_updates.jl:7-60) with the complex
  calculate_detratio!, vldiv22! and update_greens! (fields.jl:63-140,
  215-286), drawing from the same Philox4x32-10 stream as the CUDA path.
* ``direct_greens``: the independent check of test/testfunctions.jl:6-118
  (the slice-matrix chain, stabilised with numpy's QR) for complex blocks.

Scalar decisions (R, the determinant ratio, p) use Python complex scalars in
the reference's operation order, so they agree with the CUDA path to the last
bit for identical inputs; matrices agree to rounding.
"""
from __future__ import annotations

import math

import numpy as np

try:
    from . import oracle as _oracle
except ImportError:  # imported as a top-level module (oracle/ on sys.path)
    import oracle as _oracle

DENSITY_HIRSCH, MAGNETIC_HIRSCH, DENSITY_GHQ, MAGNETIC_GHQ = 0, 1, 2, 3


# ---- complex scalars in Julia's Complex{Float64} operation order -------------

def _cexp(z: complex) -> complex:
    """exp(z::Complex): (e^re, im) when im == 0, else e^re (cos im, sin im)."""
    er = math.exp(z.real)
    if z.imag == 0.0:
        return complex(er, z.imag)
    return complex(er * math.cos(z.imag), er * math.sin(z.imag))


def _scale(z: complex, x: float) -> complex:
    """Real * Complex: both parts scaled (no cross terms)."""
    return complex(x * z.real, x * z.imag)


def _inv(w: complex) -> complex:
    """1 / w by Smith's method (R. L. Smith, CACM 5 (1962) 435)."""
    c, d = w.real, w.imag
    if abs(d) <= abs(c):
        r = d / c
        t = 1.0 / (c + d * r)
        return complex(t, -r * t)
    r = c / d
    t = 1.0 / (d + c * r)
    return complex(r * t, -t)


def _mul(a: complex, b: complex) -> complex:
    return complex(a.real * b.real - a.imag * b.imag, a.real * b.imag + a.imag * b.real)


S6 = math.sqrt(6.0)
GAMMA = [1.0 - S6 / 3.0, 1.0 + S6 / 3.0, 1.0 + S6 / 3.0, 1.0 - S6 / 3.0]
ETA = [-math.sqrt(6.0 + 2.0 * S6), -math.sqrt(6.0 - 2.0 * S6), math.sqrt(6.0 - 2.0 * S6),
       math.sqrt(6.0 + 2.0 * S6)]


def tables(kind: int, alpha: complex):
    """Interaction exponentials ev[f][v], evinv[f][v] and per-proposal
    (delta0, delta1, wboson) tables (fields.jl:383, 389-390, 432-443, 553-569,
    621-633; p = exp(-dE_boson) detratio, local_updates.jl:31)."""
    a = complex(alpha)
    ev = [[0j] * 4 for _ in range(2)]
    evinv = [[0j] * 4 for _ in range(2)]
    d0, d1, wb = [0j] * 16, [0j] * 16, [0j] * 16
    if kind in (DENSITY_HIRSCH, MAGNETIC_HIRSCH):
        for v in range(2):
            s = 1.0 if v else -1.0
            ev[0][v] = _cexp(_scale(_scale(a, 1.0), s))
            evinv[0][v] = _cexp(_scale(_scale(a, -1.0), s))
            if kind == MAGNETIC_HIRSCH:
                ev[1][v] = _cexp(_scale(_scale(a, -1.0), s))
                evinv[1][v] = _cexp(_scale(_scale(a, 1.0), s))
            dE = _scale(_scale(a, -2.0), s)
            if kind == DENSITY_HIRSCH:
                d0[v] = _cexp(dE) - 1.0
                wb[v] = _cexp(-dE)
            else:
                d0[v] = _cexp(dE) - 1.0
                d1[v] = _cexp(-dE) - 1.0
                wb[v] = 1 + 0j
    else:
        for v in range(4):
            ev[0][v] = _cexp(_scale(_scale(a, 1.0), ETA[v]))
            evinv[0][v] = _cexp(_scale(_scale(a, -1.0), ETA[v]))
            if kind == MAGNETIC_GHQ:
                ev[1][v] = _cexp(_scale(_scale(a, -1.0), ETA[v]))
                evinv[1][v] = _cexp(_scale(_scale(a, 1.0), ETA[v]))
        for xo in range(4):
            for xn in range(4):
                if xo == xn:
                    continue
                t = xo * 4 + xn
                dE = _scale(a, ETA[xn] - ETA[xo])
                er = _cexp(dE)
                d0[t] = er - 1.0
                if kind == DENSITY_GHQ:
                    wb[t] = _cexp(-dE)
                else:
                    d1[t] = _scale(_inv(er), 1.0) - 1.0
                    wb[t] = 1 + 0j
    return ev, evinv, d0, d1, wb


# ---- linear algebra (linalg/complex.jl) ----------------------------------------

def udt_pivot(A: np.ndarray, apply_pivot: bool = True):
    """udt_AVX_pivot! for a complex matrix: returns U, D, T, pivot with
    A = U Diagonal(D) T (apply_pivot) or A[:, pivot] = U Diagonal(D) triu(T)."""
    X = np.array(A, dtype=np.complex128, copy=True)
    n = X.shape[0]
    piv = np.arange(n)
    tau = np.zeros(n, dtype=np.complex128)
    for j in range(n):
        # indmaxcolumn: squared column norms of the trailing block, first maximum
        norms = np.sum(X.real[j:, j:] ** 2, axis=0) + np.sum(X.imag[j:, j:] ** 2, axis=0)
        jm, sq = j, norms[0]
        for i in range(1, n - j):
            if abs(norms[i]) > sq:
                sq, jm = norms[i], j + i
        if jm != j:
            piv[[j, jm]] = piv[[jm, j]]
            X[:, [j, jm]] = X[:, [jm, j]]
        # reflector!
        x1 = X[j, j]
        if sq == 0.0:
            tau[j] = 0.0
        else:
            nu = math.copysign(math.sqrt(sq), x1.real)
            x1 = x1 + nu
            X[j, j] = complex(-nu, 0.0)
            X[j + 1:, j] = X[j + 1:, j] * (1.0 / x1)
            tau[j] = x1 / nu
        # reflectorApply!: A <- (I - conj(tau) v v^H) A on the trailing columns
        if j + 1 < n:
            v = X[j + 1:, j]
            w = X[j, j + 1:] + np.conj(v) @ X[j + 1:, j + 1:]
            w = np.conj(tau[j]) * w
            X[j, j + 1:] -= w
            X[j + 1:, j + 1:] -= np.outer(v, w)
    # U = H_1 ... H_n, H_k = I - tau_k v_k v_k^H, accumulated backwards
    U = np.eye(n, dtype=np.complex128)
    U[n - 1, n - 1] -= tau[n - 1]
    for k in range(n - 2, -1, -1):
        v = X[k + 1:, k]
        w = U[k, k:] + np.conj(v) @ U[k + 1:, k:]
        w = tau[k] * w
        U[k, k:] -= w
        U[k + 1:, k:] -= np.outer(v, w)
    D = np.abs(X.real.diagonal()).copy()
    R = np.triu(X)
    if apply_pivot:
        T = np.zeros_like(R)
        T[:, piv] = R / D[:, None]
        return U, D, T, piv
    return U, D, R / D[:, None], piv


def rdivp(A: np.ndarray, T: np.ndarray, pivot) -> np.ndarray:
    """rdivp!: A <- A[:, pivot] triu(T)^-1 (column by column)."""
    O = A[:, pivot]
    n = A.shape[0]
    out = np.zeros_like(O)
    for j in range(n):
        x = O[:, j] - out[:, :j] @ T[:j, j]
        out[:, j] = x * (1.0 / T[j, j])
    return out


def calculate_greens_udt(Ul, Dl, Tl, Ur, Dr, Tr):
    """calculate_greens_AVX!: G = [I + Ul Dl Tl Tr^H Dr Ur^H]^-1."""
    G = Tl @ Tr.conj().T
    Tr = G * Dr[None, :]
    G = Dl[:, None] * Tr
    Tr, Dr2, G, piv = udt_pivot(G, apply_pivot=False)
    Tl = Ul @ Tr
    Ur = rdivp(Ur, G, piv)
    Tr = Tl.conj().T @ Ur
    Tr = Tr + np.diag(Dr2)
    Ul, Dr3, Tr, piv = udt_pivot(Tr, apply_pivot=False)
    Ur = rdivp(Ur, Tr, piv)
    Tr = Tl @ Ul
    Dl = 1.0 / Dr3
    Ul = Ur * Dl[None, :]
    return Ul @ Tr.conj().T


def generate_chunks(length, max_chunk):
    """stack.jl:154-158 (1-based inclusive ranges)."""
    n = -(-length // max_chunk)
    step = length / n
    return [(int(round((i - 1) * step)) + 1, int(round(i * step))) for i in range(1, n + 1)]


class ComplexChain:
    """One complex DQMC chain: nf flavour blocks of n x n complex matrices."""

    def __init__(self, n, nf, M, safe_mult, kind, alpha, exps, seed, check_prop=True):
        self.n, self.nf, self.M, self.k, self.kind = n, nf, M, safe_mult, kind
        self.alpha = complex(alpha)
        self.eT2, self.eT2inv, self.eTh, self.eThinv = [np.asarray(e, dtype=np.float64)
                                                        for e in exps]
        self.ev, self.evinv, self.d0, self.d1, self.wb = tables(kind, self.alpha)
        self.key = seed & (2**64 - 1)
        self.ctr = 0
        self.check_prop = check_prop
        self.ranges = generate_chunks(M, safe_mult)
        nr = len(self.ranges)
        I = np.eye(n, dtype=np.complex128)
        self.u = [[I.copy() for _ in range(nf)] for _ in range(nr + 1)]
        self.t = [[I.copy() for _ in range(nf)] for _ in range(nr + 1)]
        self.d = [[np.ones(n) for _ in range(nf)] for _ in range(nr + 1)]
        self.G = np.zeros((nf, n, n), dtype=np.complex128)
        self.conf = np.ones((n, M), dtype=np.int8, order="F")
        self.current_slice, self.current_range, self.direction = 0, 1, 1
        self.prop_err_max = 0.0
        self.n_prop_err = 0
        self.n_neg_p = 0
        self.n_imag_p = 0
        self.max_imag_p = 0.0
        self.accepted = 0
        self.proposals = 0

    # --- random numbers (the CUDA path's Philox4x32-10 stream)
    def _word(self):
        w = _oracle.lib().oc_rng_word(self.key, self.ctr)
        self.ctr += 1
        return w

    def set_rng(self, key, counter):
        self.key, self.ctr = key, counter

    def set_conf(self, conf):
        self.conf = np.asfortranarray(np.array(conf, dtype=np.int8))

    # --- slice matrices (stack.jl:315-367)
    def _evdiag(self, slice_, inverse, b):
        tab = (self.evinv if inverse else self.ev)[b]
        s = self.conf[:, slice_ - 1]
        idx = (s.astype(int) - 1) if self.kind >= 2 else (s > 0).astype(int)
        return np.array([tab[v] for v in idx], dtype=np.complex128)

    def slice_left(self, slice_, M):
        return [self.eT2 @ (self._evdiag(slice_, False, b)[:, None] * M[b])
                for b in range(self.nf)]

    def slice_right(self, slice_, M):
        return [(M[b] @ self.eT2) * self._evdiag(slice_, False, b)[None, :]
                for b in range(self.nf)]

    def slice_inv_right(self, slice_, M):
        return [(M[b] * self._evdiag(slice_, True, b)[None, :]) @ self.eT2inv
                for b in range(self.nf)]

    def slice_inv_left(self, slice_, M):
        return [self._evdiag(slice_, True, b)[:, None] * (self.eT2inv @ M[b])
                for b in range(self.nf)]

    def slice_dagger_left(self, slice_, M):
        return [np.conj(self._evdiag(slice_, False, b))[:, None] * (self.eT2.T @ M[b])
                for b in range(self.nf)]

    def wrap_greens(self, G, curr_slice, direction):
        if direction == -1:
            G = self.slice_inv_left(curr_slice - 1, G)
            return np.array(self.slice_right(curr_slice - 1, G))
        G = self.slice_left(curr_slice, G)
        return np.array(self.slice_inv_right(curr_slice, G))

    # --- stack (stack.jl:257-416)
    def _udt_blocks(self, X):
        out = [udt_pivot(X[b]) for b in range(self.nf)]
        return [o[0] for o in out], [o[1] for o in out], [o[2] for o in out]

    def add_slice_sequence_left(self, idx):
        cur = [u.copy() for u in self.u[idx - 1]]
        a, b = self.ranges[idx - 1]
        for sl in range(a, b + 1):
            cur = self.slice_left(sl, cur)
        tmp = [cur[f] * self.d[idx - 1][f][None, :] for f in range(self.nf)]
        U, D, T = self._udt_blocks(tmp)
        self.u[idx] = U
        self.d[idx] = D
        self.t[idx] = [T[f] @ self.t[idx - 1][f] for f in range(self.nf)]

    def add_slice_sequence_right(self, idx):
        cur = [u.copy() for u in self.u[idx]]
        a, b = self.ranges[idx - 1]
        for sl in range(b, a - 1, -1):
            cur = self.slice_dagger_left(sl, cur)
        tmp = [cur[f] * self.d[idx][f][None, :] for f in range(self.nf)]
        U, D, T = self._udt_blocks(tmp)
        self.u[idx - 1] = U
        self.d[idx - 1] = D
        self.t[idx - 1] = [T[f] @ self.t[idx][f] for f in range(self.nf)]

    def _greens(self, Ul, Dl, Tl, Ur, Dr, Tr):
        return np.array([calculate_greens_udt(Ul[f], Dl[f], Tl[f], Ur[f], Dr[f], Tr[f])
                         for f in range(self.nf)])

    def _eye(self):
        I = np.eye(self.n, dtype=np.complex128)
        return [I.copy() for _ in range(self.nf)], [np.ones(self.n) for _ in range(self.nf)]

    def reverse_build_stack(self):
        nr = len(self.ranges)
        I, one = self._eye()
        self.u[nr], self.d[nr], self.t[nr] = I, one, [x.copy() for x in I]
        for i in range(nr, 0, -1):
            self.add_slice_sequence_right(i)
        self.current_slice, self.current_range, self.direction = 0, 1, 1
        I, one = self._eye()
        self.G = self._greens(I, one, [x.copy() for x in I], self.u[0], self.d[0], self.t[0])

    def build_stack(self):
        nr = len(self.ranges)
        I, one = self._eye()
        self.u[0], self.d[0], self.t[0] = I, one, [x.copy() for x in I]
        for i in range(1, nr + 1):
            self.add_slice_sequence_left(i)
        self.current_slice, self.current_range, self.direction = self.M + 1, nr, -1
        I, one = self._eye()
        self.G = self._greens(self.u[nr], self.d[nr], self.t[nr], I, one, [x.copy() for x in I])

    def _prop_check(self, Gtmp):
        if self.check_prop:
            diff = float(np.max(np.abs(Gtmp - self.G)))
            self.prop_err_max = max(self.prop_err_max, diff)
            if diff > 1e-7:
                self.n_prop_err += 1

    def propagate(self):
        """propagate (stack.jl:605-730)."""
        nr = len(self.ranges)
        self.current_slice += self.direction
        cs = self.current_slice
        if self.direction == 1:
            if cs == 1:
                I, one = self._eye()
                self.u[0], self.d[0], self.t[0] = I, one, [x.copy() for x in I]
            elif cs - 1 == self.ranges[self.current_range - 1][1]:
                idx = self.current_range
                Ur, Dr, Tr = self.u[idx], self.d[idx], self.t[idx]
                self.add_slice_sequence_left(idx)
                Ul, Dl, Tl = self.u[idx], self.d[idx], self.t[idx]
                Gtmp = self.wrap_greens(self.G.copy(), cs - 1, 1)
                self.G = self._greens(Ul, Dl, Tl, Ur, Dr, Tr)
                self._prop_check(Gtmp)
                if self.current_range == nr:
                    self.direction = -1
                    self.propagate()
                else:
                    self.current_range += 1
            else:
                self.G = self.wrap_greens(self.G, cs - 1, 1)
        else:
            if cs == self.M:
                I, one = self._eye()
                self.u[nr], self.d[nr], self.t[nr] = I, one, [x.copy() for x in I]
                self.G = self.wrap_greens(self.G, cs + 1, -1)
            elif cs + 1 == self.ranges[self.current_range - 1][0]:
                idx = self.current_range
                Ul, Dl, Tl = self.u[idx - 1], self.d[idx - 1], self.t[idx - 1]
                self.add_slice_sequence_right(idx)
                Ur, Dr, Tr = self.u[idx - 1], self.d[idx - 1], self.t[idx - 1]
                Gtmp = self.G.copy()
                self.G = self._greens(Ul, Dl, Tl, Ur, Dr, Tr)
                self._prop_check(Gtmp)
                if self.current_range == 1:
                    self.direction = 1
                    self.propagate()
                else:
                    self.G = self.wrap_greens(self.G, cs + 1, -1)
                    self.current_range -= 1
            else:
                self.G = self.wrap_greens(self.G, cs + 1, -1)

    def initialize_run(self):
        self.reverse_build_stack()
        self.propagate()

    # --- local updates (local_updates.jl:23-60, fields.jl:63-140, 215-286)
    def ratio(self, j, t, xnew=0, xold=0):
        """p = exp(-dE_boson) detratio of the move at site j of the current
        slice (table index t), with R and Delta per block."""
        dl = [self.d0[t], self.d1[t]]
        R = [0j, 0j]
        if self.nf == 1:
            g = complex(self.G[0, j, j])
            omg = complex(1.0 - g.real, -g.imag)   # 1.0 - G[i, i]
            pr = _mul(dl[0], omg)
            R[0] = complex(1.0 + pr.real, pr.imag)
            det = _mul(R[0], R[0])
        else:
            for b in range(2):
                g = complex(self.G[b, j, j])
                omg = 1.0 - g.real
                re = (1.0 + dl[b].real * omg) + dl[b].imag * g.imag
                im = dl[b].imag * omg - dl[b].real * g.imag
                R[b] = complex(re, im)
            det = _mul(R[0], R[1])
        if self.kind >= 2:
            gn, go = GAMMA[xnew - 1], GAMMA[xold - 1]
            det = complex((det.real * gn) / go, (det.imag * gn) / go)
        return _mul(self.wb[t], det), R, dl

    def accept(self, j, R, dl, xnew=0):
        """accept_local!: G -= (I - G)[:, j] (Delta/R) G[j, :] per block, flip."""
        for b in range(self.nf):
            f = 1.0 / (R[b].real * R[b].real + R[b].imag * R[b].imag)
            ird = complex(f * (dl[b].real * R[b].real + dl[b].imag * R[b].imag),
                          f * (dl[b].imag * R[b].real - dl[b].real * R[b].imag))
            Gb = self.G[b]
            u = -Gb[:, j].copy()
            u[j] += 1.0
            self.G[b] = Gb - np.outer(u, ird * Gb[j, :])
        sl = self.current_slice
        self.conf[j, sl - 1] = xnew if self.kind >= 2 else -self.conf[j, sl - 1]

    def sweep_spatial(self):
        sl = self.current_slice
        ghq = self.kind >= 2
        acc = 0
        for j in range(self.n):
            xnew = xold = 0
            if ghq:
                xold = int(self.conf[j, sl - 1])
                w = self._word()
                r = (w * 3) >> 64
                xnew = r + (2 if r + 1 >= xold else 1)
                t = (xold - 1) * 4 + (xnew - 1)
            else:
                t = 1 if self.conf[j, sl - 1] > 0 else 0
            p, R, dl = self.ratio(j, t, xnew, xold)
            if abs(p.imag) > 1e-6:
                self.n_imag_p += 1
                self.max_imag_p = max(self.max_imag_p, abs(p.imag))
            if p.real < 0.0:
                self.n_neg_p += 1
            if p.real > 1.0:
                accept = True
            else:
                w = self._word()
                accept = (w >> 11) * 2.0 ** -53 < p.real
            self.proposals += 1
            if accept:
                self.accept(j, R, dl, xnew)
                self.accepted += 1
                acc += 1
        return acc

    def sweeps(self, k):
        for _ in range(k):
            for _ in range(2 * self.M):
                self.sweep_spatial()
                self.propagate()

    # --- calculate_greens(mc, slice) (stack.jl:525-583) and greens! (greens.jl:114-125)
    def calculate_greens_at(self, slice_, safe_mult=0):
        k = safe_mult if safe_mult > 0 else self.k
        I, one = self._eye()
        cur = [x.copy() for x in I]
        Ur, Dr, Tr = [x.copy() for x in I], [o.copy() for o in one], [x.copy() for x in I]
        if slice_ + 1 <= self.M:
            for s in range(self.M, slice_, -1):
                cur = self.slice_dagger_left(s, cur)
                if s % k == 0:
                    tmp = [cur[f] * Dr[f][None, :] for f in range(self.nf)]
                    cur, Dr, T = self._udt_blocks(tmp)
                    Tr = [T[f] @ Tr[f] for f in range(self.nf)]
            tmp = [cur[f] * Dr[f][None, :] for f in range(self.nf)]
            Ur, Dr, T = self._udt_blocks(tmp)
            Tr = [T[f] @ Tr[f] for f in range(self.nf)]
        cur = [x.copy() for x in I]
        Ul, Dl, Tl = [x.copy() for x in I], [o.copy() for o in one], [x.copy() for x in I]
        if slice_ >= 1:
            for s in range(1, slice_ + 1):
                cur = self.slice_left(s, cur)
                if s % k == 0:
                    tmp = [cur[f] * Dl[f][None, :] for f in range(self.nf)]
                    cur, Dl, T = self._udt_blocks(tmp)
                    Tl = [T[f] @ Tl[f] for f in range(self.nf)]
            tmp = [cur[f] * Dl[f][None, :] for f in range(self.nf)]
            Ul, Dl, T = self._udt_blocks(tmp)
            Tl = [T[f] @ Tl[f] for f in range(self.nf)]
        return self._greens(Ul, Dl, Tl, Ur, Dr, Tr)

    def greens_physical(self, G):
        return np.array([self.eThinv @ (G[b] @ self.eTh) for b in range(self.nf)])

    def slice_matrix(self, slice_, b):
        """B_b(l) = eT2 eV_b(l) (stack.jl:319-327)."""
        return self.eT2 * self._evdiag(slice_, False, b)[None, :]


def direct_greens(chain: ComplexChain, slice_: int, safe_mult: int = 4):
    """Independent check (test/testfunctions.jl:6-118): the equal-time G at
    `slice_` from the explicit slice-matrix chain B(slice) ... B(1) B(M) ...
    B(slice+1), stabilised every safe_mult factors with numpy's QR."""
    M = chain.M
    order = list(range(slice_ + 1, M + 1)) + list(range(1, slice_ + 1))
    out = []
    for b in range(chain.nf):
        n = chain.n
        U, D, T = np.eye(n, dtype=complex), np.ones(n), np.eye(n, dtype=complex)
        for i, s in enumerate(order):
            U = chain.slice_matrix(s, b) @ U
            if (i + 1) % safe_mult == 0 or i == len(order) - 1:
                Q, R = np.linalg.qr(U * D[None, :])
                d = np.abs(np.diag(R))
                U, D, T = Q, d, (R / d[:, None]) @ T
        # G = [I + U D T]^-1 = T^-1 [U^H T^-1 + D]^-1 U^H, with a split of D
        Dp = np.maximum(D, 1.0)
        Dm = np.minimum(D, 1.0)
        Ti = np.linalg.inv(T)
        X = (U.conj().T @ Ti) / Dp[:, None] + Dm[:, None] * np.eye(n)
        G = Ti @ np.linalg.solve(X, (U.conj().T / Dp[:, None]))
        out.append(G)
    return np.array(out)


def direct_greens_kl(chain: ComplexChain, k: int, l: int):
    """Unequal-time G(k, l) = <c(k dtau) c^dagger(l dtau)> from the explicit
    chain (the defining products behind unequal_time_stack.jl:400-697):
    k >= l: B(k) ... B(l+1) G(l); k < l: -(I - G(k)) B(k+1)^-1 ... B(l)^-1,
    with G(s) the equal-time G of calculate_greens(mc, s).  Unstabilised:
    for small beta only."""
    out = []
    for b in range(chain.nf):
        n = chain.n
        if k >= l:
            G = chain.calculate_greens_at(l)[b]
            for s in range(l + 1, k + 1):
                G = chain.slice_matrix(s, b) @ G
        else:
            G = -(np.eye(n) - chain.calculate_greens_at(k)[b])
            for s in range(k + 1, l + 1):
                G = G @ np.linalg.inv(chain.slice_matrix(s, b))
        out.append(G)
    return np.array(out)
