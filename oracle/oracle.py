"""ctypes access to the CPU oracle (dqmc_oracle.c) plus numpy restatements of
the reference's test-side helpers.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference arm.  The product never imports it.

* ``OracleChain``: one DQMC chain on the C oracle.
* ``direct_greens``: calculate_greens_and_logdet of test/testfunctions.jl:6-118
  (slice-matrix chain with pivoted-QR UDT via scipy, independent of the stack).
* ``analytic_greens``: test/testfunctions.jl:128-165 (U = 0 equal-time G).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libdqmc_oracle.so")
# Same source built with floating-point contraction allowed (fused multiply-add
# where the target has it): the timed CPU baseline, as the reference's
# LoopVectorization loops also emit FMAs.  The parity build keeps every
# product and sum separately rounded so it gives the same bits on x86_64 and
# aarch64.
FAST_LIB_PATH = os.path.join(HERE, "libdqmc_oracle_fast.so")


def build(force: bool = False) -> str:
    """Compile both oracle builds with gcc (portable flags: x86_64 and aarch64)."""
    src = os.path.join(HERE, "dqmc_oracle.c")
    hdr = os.path.join(HERE, "dqmc_oracle.h")
    for path, contract in ((LIB_PATH, "off"), (FAST_LIB_PATH, "fast")):
        newest = max(os.path.getmtime(src), os.path.getmtime(hdr))
        if force or not os.path.exists(path) or os.path.getmtime(path) < newest:
            tmp = path + f".{os.getpid()}.tmp"
            cmd = ["gcc", "-O3", "-std=gnu11", f"-ffp-contract={contract}", "-fPIC", "-shared",
                   "-o", tmp, src, "-lm", "-lpthread"]
            subprocess.run(cmd, check=True)
            os.replace(tmp, path)
    return LIB_PATH


_lib = None
_fast = False


def use_fast_build(flag: bool = True):
    """Select the contraction-enabled build (CPU-baseline timing only); must be
    called before the first oracle call."""
    global _fast
    if _lib is not None and flag != _fast:
        raise RuntimeError("oracle library already loaded")
    _fast = flag


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(FAST_LIB_PATH if _fast else LIB_PATH)
        P = C.c_void_p
        dp = C.POINTER(C.c_double)
        L.oc_create.restype = P
        L.oc_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                dp, dp, dp, dp, C.c_uint64, C.c_int]
        L.oc_destroy.argtypes = [P]
        for f in ("oc_init_random_conf", "oc_build_stack", "oc_reverse_build_stack",
                  "oc_propagate", "oc_initialize_run"):
            getattr(L, f).argtypes = [P]
        L.oc_set_conf.argtypes = [P, C.c_void_p]
        L.oc_get_conf.argtypes = [P, C.c_void_p]
        L.oc_set_rng.argtypes = [P, C.c_uint64, C.c_uint64]
        L.oc_get_rng_counter.argtypes = [P]
        L.oc_get_rng_counter.restype = C.c_uint64
        L.oc_sweep_spatial.argtypes = [P]
        L.oc_sweep_spatial.restype = C.c_int
        L.oc_local_sweeps.argtypes = [P, C.c_int]
        L.oc_local_sweeps.restype = C.c_long
        L.oc_wrap_greens.argtypes = [P, dp, C.c_int, C.c_int]
        L.oc_calculate_greens_at.argtypes = [P, C.c_int, dp, C.c_int]
        L.oc_greens_physical.argtypes = [P, dp, dp]
        L.oc_get_greens.argtypes = [P, dp]
        L.oc_set_greens.argtypes = [P, dp]
        L.oc_get_state.argtypes = [P, C.POINTER(C.c_int)]
        L.oc_get_stack.argtypes = [P, C.c_int, C.c_int, dp]
        L.oc_get_analysis.argtypes = [P, dp]
        L.oc_udt_pivot.argtypes = [C.c_int, dp, dp, dp, C.POINTER(C.c_int64), dp, C.c_int]
        L.oc_rdivp.argtypes = [C.c_int, dp, dp, dp, C.POINTER(C.c_int64), C.c_int]
        L.oc_calculate_greens_avx.argtypes = [C.c_int, C.c_int, dp, dp, dp, dp, dp, dp, dp]
        L.oc_update_greens.argtypes = [C.c_int, C.c_int, dp, dp, C.c_int]
        L.oc_rng_word.argtypes = [C.c_uint64, C.c_uint64]
        L.oc_rng_word.restype = C.c_uint64
        L.oc_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                       C.POINTER(C.c_uint32)]
        L.oc_generate_chunks.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.oc_generate_chunks.restype = C.c_int
        L.oc_global_update.argtypes = [P, C.c_int]
        L.oc_global_update.restype = C.c_int
        L.oc_global_detratio.argtypes = [P, C.c_void_p, dp]
        L.oc_global_detratio.restype = C.c_double
        L.oc_replica_weight.argtypes = [P, C.c_void_p, dp, dp]
        L.oc_replica_accept.argtypes = [P, C.c_void_p]
        L.oc_local_move_to.argtypes = [P, C.c_int, C.c_int]
        L.oc_local_move_to.restype = C.c_double
        L.oc_get_global_stats.argtypes = [P, C.POINTER(C.c_long), C.POINTER(C.c_long)]
        L.oc_greens_kl.argtypes = [P, C.c_void_p, C.c_void_p, C.c_int, dp]
        L.oc_set_checkerboard.argtypes = [P, C.c_int, dp]
        L.oc_run_chains_threaded.argtypes = [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_int]
        L.oc_run_chains_threaded.restype = C.c_double
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["F_CONTIGUOUS"] or a.ndim == 1
    return a.ctypes.data_as(C.POINTER(C.c_double))


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().oc_philox4x32_10(c, k, o)
    return list(o)


def generate_chunks(length, max_chunk):
    nmax = -(-length // max_chunk)
    f = (C.c_int * nmax)()
    l_ = (C.c_int * nmax)()
    k = lib().oc_generate_chunks(length, max_chunk, f, l_)
    return [(f[i], l_[i]) for i in range(k)]


class OracleChain:
    """A DQMC chain on the CPU oracle.  Matrices come back as (nf, n, n)
    arrays (block b = flavour b), column-major semantics preserved."""

    def __init__(self, n, nf, M, safe_mult, kind, alpha, exps, seed, check_prop=True):
        self.n, self.nf, self.M, self.k, self.kind = n, nf, M, safe_mult, kind
        eT2, eT2inv, eTh, eThinv = [np.asfortranarray(e, dtype=np.float64) for e in exps]
        self._keep = (eT2, eT2inv, eTh, eThinv)
        self.h = lib().oc_create(n, nf, M, safe_mult, kind, float(alpha), _dp(eT2), _dp(eT2inv),
                                 _dp(eTh), _dp(eThinv), C.c_uint64(seed & (2**64 - 1)),
                                 int(bool(check_prop)))

    @classmethod
    def from_model(cls, model, field_cls, beta, delta_tau, safe_mult, seed, check_prop=True):
        sys.path.insert(0, os.path.dirname(HERE))
        from __graft_entry__ import load_package  # noqa
        pkg = load_package()
        param = pkg.DQMCParameters.make(beta=beta, delta_tau=delta_tau, safe_mult=safe_mult)
        field = field_cls(param, model)
        exps = pkg.hopping_exponentials(model.hopping_matrix(), param.delta_tau)
        return cls(len(model.l), field.unique_flavors, param.slices, safe_mult, field.kind,
                   field.alpha, exps, seed, check_prop)

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().oc_destroy(self.h)
                self.h = None
        except Exception:
            pass

    # --- field / rng
    def init_random_conf(self):
        lib().oc_init_random_conf(self.h)

    def set_conf(self, conf):
        c = np.asfortranarray(conf, dtype=np.int8)
        assert c.shape == (self.n, self.M)
        lib().oc_set_conf(self.h, c.ctypes.data)

    def get_conf(self):
        c = np.zeros((self.n, self.M), dtype=np.int8, order="F")
        lib().oc_get_conf(self.h, c.ctypes.data)
        return c

    def set_rng(self, key, counter):
        lib().oc_set_rng(self.h, key, counter)

    def rng_counter(self):
        return lib().oc_get_rng_counter(self.h)

    # --- stack
    def build_stack(self):
        lib().oc_build_stack(self.h)

    def reverse_build_stack(self):
        lib().oc_reverse_build_stack(self.h)

    def propagate(self):
        lib().oc_propagate(self.h)

    def initialize_run(self):
        lib().oc_initialize_run(self.h)

    def sweep_spatial(self):
        return lib().oc_sweep_spatial(self.h)

    def sweeps(self, k):
        return lib().oc_local_sweeps(self.h, int(k))

    def _mat(self):
        return np.zeros((self.nf, self.n, self.n), order="C")

    @staticmethod
    def _blocks_to_buf(G):
        # (nf, n, n) array with [b][i][j] -> column-major buffer per block
        return np.ascontiguousarray(np.transpose(G, (0, 2, 1))).ravel()

    @staticmethod
    def _buf_to_blocks(buf, nf, n):
        return np.transpose(buf.reshape(nf, n, n), (0, 2, 1)).copy()

    def greens(self):
        buf = np.zeros(self.nf * self.n * self.n)
        lib().oc_get_greens(self.h, _dp(buf))
        return self._buf_to_blocks(buf, self.nf, self.n)

    def set_greens(self, G):
        buf = self._blocks_to_buf(np.asarray(G, dtype=np.float64))
        lib().oc_set_greens(self.h, _dp(buf))

    def wrap_greens(self, G, curr_slice, direction):
        buf = self._blocks_to_buf(np.asarray(G, dtype=np.float64))
        lib().oc_wrap_greens(self.h, _dp(buf), curr_slice, direction)
        return self._buf_to_blocks(buf, self.nf, self.n)

    def calculate_greens_at(self, slice_, safe_mult=0):
        buf = np.zeros(self.nf * self.n * self.n)
        lib().oc_calculate_greens_at(self.h, int(slice_), _dp(buf), int(safe_mult))
        return self._buf_to_blocks(buf, self.nf, self.n)

    def greens_physical(self, G):
        src = self._blocks_to_buf(np.asarray(G, dtype=np.float64))
        out = np.zeros_like(src)
        lib().oc_greens_physical(self.h, _dp(src), _dp(out))
        return self._buf_to_blocks(out, self.nf, self.n)

    def state(self):
        s = (C.c_int * 4)()
        lib().oc_get_state(self.h, s)
        return dict(current_slice=s[0], current_range=s[1], direction=s[2], n_ranges=s[3])

    def stack(self, which, idx):
        if which == 2:
            out = np.zeros(self.nf * self.n)
            lib().oc_get_stack(self.h, 2, idx, _dp(out))
            return out.reshape(self.nf, self.n)
        buf = np.zeros(self.nf * self.n * self.n)
        lib().oc_get_stack(self.h, which, idx, _dp(buf))
        return self._buf_to_blocks(buf, self.nf, self.n)

    # --- global updates (global_updates.jl, parallel_updates.jl)
    def global_update(self, kind=0):
        """GlobalFlip (kind 0) or GlobalShuffle (kind 1); True when accepted."""
        return bool(lib().oc_global_update(self.h, int(kind)))

    def global_detratio(self, proposal):
        c = np.asfortranarray(proposal, dtype=np.int8)
        dE = np.zeros(1)
        r = lib().oc_global_detratio(self.h, c.ctypes.data, _dp(dE))
        return r, float(dE[0])

    def replica_weight(self, partner_conf):
        c = np.asfortranarray(partner_conf, dtype=np.int8)
        w, p = np.zeros(1), np.zeros(1)
        lib().oc_replica_weight(self.h, c.ctypes.data, _dp(w), _dp(p))
        return float(w[0]), float(p[0])

    def replica_accept(self, partner_conf):
        c = np.asfortranarray(partner_conf, dtype=np.int8)
        lib().oc_replica_accept(self.h, c.ctypes.data)

    def local_move_to(self, i, x_new):
        return lib().oc_local_move_to(self.h, int(i), int(x_new))

    def set_checkerboard(self, data, n_parts):
        """Checkerboard factors packed as oc_set_checkerboard expects."""
        lib().oc_set_checkerboard(self.h, int(n_parts), _dp(np.ascontiguousarray(data,
                                                                               dtype=np.float64)))

    def greens_kl(self, pairs):
        """Effective unequal-time G(k, l) for a list of (k, l) pairs."""
        k = np.ascontiguousarray([p[0] for p in pairs], dtype=np.int32)
        l = np.ascontiguousarray([p[1] for p in pairs], dtype=np.int32)
        buf = np.zeros(len(pairs) * self.nf * self.n * self.n)
        lib().oc_greens_kl(self.h, k.ctypes.data, l.ctypes.data, len(pairs), _dp(buf))
        per = self.nf * self.n * self.n
        return [self._buf_to_blocks(buf[i * per:(i + 1) * per], self.nf, self.n)
                for i in range(len(pairs))]

    def global_stats(self):
        a, p = C.c_long(), C.c_long()
        lib().oc_get_global_stats(self.h, C.byref(a), C.byref(p))
        return a.value, p.value

    def analysis(self):
        out = np.zeros(7)
        lib().oc_get_analysis(self.h, _dp(out))
        return dict(propagation_error_max=out[0], propagation_error_count=int(out[1]),
                    propagation_error_reported=out[2], negative_probability=int(out[3]),
                    accepted=int(out[4]), near_ties=int(out[5]), min_tie_gap=out[6])


def run_chains_threaded(chains, nsweeps, threads):
    arr = (C.c_void_p * len(chains))(*[c.h for c in chains])
    return lib().oc_run_chains_threaded(arr, len(chains), int(nsweeps), int(threads))


# ----------------------------------------------------------- linalg helpers

def udt_pivot(A, apply_pivot=True):
    """udt_AVX_pivot! on a dense n x n numpy array; returns U, D, T, pivot."""
    n = A.shape[0]
    inp = np.array(A, dtype=np.float64, order="F")
    U = np.zeros((n, n), order="F")
    D = np.zeros(n)
    piv = np.zeros(n, dtype=np.int64)
    tmp = np.zeros(n)
    lib().oc_udt_pivot(n, _dp(U), _dp(D), _dp(inp), piv.ctypes.data_as(C.POINTER(C.c_int64)),
                       _dp(tmp), int(bool(apply_pivot)))
    return U, D, inp, piv


def rdivp(A, T, pivot, block_form=False):
    n = A.shape[0]
    a = np.array(A, dtype=np.float64, order="F")
    t = np.asfortranarray(T, dtype=np.float64)
    o = np.zeros((n, n), order="F")
    p = np.ascontiguousarray(pivot, dtype=np.int64)
    lib().oc_rdivp(n, _dp(a), _dp(t), _dp(o), p.ctypes.data_as(C.POINTER(C.c_int64)), int(block_form))
    return a


def update_greens(G, delta, i):
    """update_greens! on (nf, n, n) G for site i (0-based), returns new G."""
    nf, n, _ = G.shape
    buf = OracleChain._blocks_to_buf(np.asarray(G, dtype=np.float64))
    d = np.ascontiguousarray(delta, dtype=np.float64)
    lib().oc_update_greens(n, nf, _dp(buf), _dp(d), int(i))
    return OracleChain._buf_to_blocks(buf, nf, n)


# ------------------------------------------------ test/testfunctions.jl

def _decompose_udt(A):
    """StableDQMC's pivoted-QR UDT: A = U * Diagonal(D) * T."""
    import scipy.linalg as sla

    Q, R, p = sla.qr(A, pivoting=True)
    D = np.abs(np.diag(R)).copy()
    D[D == 0] = 1.0
    Tp = R / D[:, None]
    T = np.zeros_like(Tp)
    T[:, p] = Tp
    return Q, D, T


def slice_matrix(exps, eV_block):
    """B_l = eT2 * Diagonal(eV) for one flavour block."""
    return exps[0] * eV_block[None, :]


def direct_greens(Bs, slice_, safe_mult):
    """calculate_greens_and_logdet (test/testfunctions.jl:80-118) for one
    flavour block: Bs[l-1] is the dense slice matrix B(l), l = 1..M."""
    M = len(Bs)
    n = Bs[0].shape[0]

    def chain(ks, dagger):
        U = np.eye(n); D = np.ones(n); T = np.eye(n)
        for k in ks:
            B = Bs[k - 1].T if dagger else Bs[k - 1]
            U = B @ U
            if k % safe_mult == 0:
                U, D, Tn = _decompose_udt(U * D[None, :])
                T = Tn @ T
        U, D, Tn = _decompose_udt(U * D[None, :])
        return U, D, Tn @ T

    if slice_ + 1 <= M:
        Ur, Dr, Tr = chain(range(M, slice_, -1), True)
    else:
        Ur, Dr, Tr = np.eye(n), np.ones(n), np.eye(n)
    if slice_ >= 1:
        Ul, Dl, Tl = chain(range(1, slice_ + 1), False)
    else:
        Ul, Dl, Tl = np.eye(n), np.ones(n), np.eye(n)
    tmp = Tl @ Tr.T
    U, D, T = _decompose_udt(Dl[:, None] * tmp * Dr[None, :])
    U = Ul @ U
    T = T @ Ur.T
    u, d, t = _decompose_udt(U.T @ np.linalg.inv(T) + np.diag(D))
    T = np.linalg.inv(t @ T)
    U = (U @ u).T
    return T @ np.diag(1.0 / d) @ U


def analytic_greens(T, beta):
    """Equal-time U = 0 Green's function, test/testfunctions.jl:141-164."""
    vals, U = np.linalg.eigh(T)
    return U @ np.diag(1.0 / (1.0 + np.exp(-beta * vals))) @ np.linalg.inv(U)
