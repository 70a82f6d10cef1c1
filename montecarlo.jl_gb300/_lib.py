"""ctypes binding of libdqmc_gb300.so (include/dqmc_gb300.h).

Loading fails loudly: there is no CPU fallback for the DQMC path.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libdqmc_gb300.so")

DQMC_OK = 0
DQMC_ERR_NUMERICAL = 4
DQMC_ERR_NOT_READY = 5
PREC_FP64 = 0
PREC_MIXED = 1

ERRORS = {1: "invalid argument", 2: "CUDA error", 3: "out of device memory",
          4: "numerical error", 5: "not ready"}


class DQMCError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class ChainConfig(C.Structure):
    _fields_ = [("n_sites", C.c_int32), ("n_flavors", C.c_int32), ("slices", C.c_int32),
                ("safe_mult", C.c_int32), ("field", C.c_int32),
                ("check_propagation_error", C.c_int32), ("alpha", C.c_double),
                ("seed", C.c_uint64), ("alpha_imag", C.c_double)]


class Stats(C.Structure):
    _fields_ = [("accepted", C.c_int64), ("proposals", C.c_int64),
                ("propagation_errors", C.c_int64), ("negative_probability", C.c_int64),
                ("max_propagation_error", C.c_double), ("max_reported_error", C.c_double),
                ("current_slice", C.c_int32), ("current_range", C.c_int32),
                ("direction", C.c_int32), ("status", C.c_int32),
                ("imaginary_probability", C.c_int64),
                ("max_imaginary_probability", C.c_double),
                ("min_reported_error", C.c_double), ("mean_reported_error", C.c_double),
                ("min_negative_probability", C.c_double),
                ("mean_negative_probability", C.c_double),
                ("max_negative_probability", C.c_double),
                ("min_imaginary_probability", C.c_double),
                ("mean_imaginary_probability", C.c_double),
                ("near_ties", C.c_int64), ("min_tie_gap", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class MeasureConfig(C.Structure):
    _fields_ = [("enable", C.c_int32), ("measure_rate", C.c_int32), ("greens_mean", C.c_int32),
                ("reserved", C.c_int32), ("sweep", C.c_int64), ("U", C.c_double),
                ("q_cos", C.POINTER(C.c_double)), ("q_sin", C.POINTER(C.c_double))]


class Observables(C.Structure):
    _fields_ = [("count", C.c_int64), ("mean", C.c_double * 4), ("error", C.c_double * 4),
                ("error_level", C.c_int32 * 4)]


class TdConfig(C.Structure):
    _fields_ = [("enable", C.c_int32), ("measure_rate", C.c_int32), ("n_slots", C.c_int32),
                ("n_form", C.c_int32 * 2), ("n_current", C.c_int32), ("delta_tau", C.c_double),
                ("sweep", C.c_int64), ("pair_slot", C.c_void_p), ("q_cos", C.c_void_p),
                ("q_sin", C.c_void_p), ("form_sites", C.c_void_p), ("form_values", C.c_void_p),
                ("current_sites", C.c_void_p), ("current_values", C.c_void_p)]


class TdObservables(C.Structure):
    _fields_ = [("count", C.c_int64), ("mean", C.c_double * 8), ("error", C.c_double * 8),
                ("error_level", C.c_int32 * 8)]


# susceptibilities of the device time-displaced measurements (dqmc_td_observables
# order) and the correlations of its by-distance arrays
TD_SCALARS = ["charge", "spin_x", "spin_y", "spin_z", "pairing", "pairing_s*", "pairing_d",
              "current"]
TD_KINDS = ["charge", "spin_x", "spin_y", "spin_z", "pairing"]

# scalar observables of the device accumulators, in dqmc_observables order
OBSERVABLES = ["density", "double_occupancy", "interaction_energy", "sz_structure_factor"]

EXPORTS = [
    "dqmc_create", "dqmc_destroy", "dqmc_last_error", "dqmc_abi_version", "dqmc_chain_bytes",
    "dqmc_set_hopping", "dqmc_set_field", "dqmc_get_field", "dqmc_init_random_field",
    "dqmc_set_rng", "dqmc_get_rng", "dqmc_initialize_run", "dqmc_build_stack", "dqmc_propagate",
    "dqmc_sweep_spatial", "dqmc_sweep", "dqmc_sweep_async", "dqmc_query", "dqmc_synchronize",
    "dqmc_get_stats", "dqmc_get_greens", "dqmc_set_greens", "dqmc_calculate_greens",
    "dqmc_get_stack", "dqmc_set_stream", "dqmc_get_timers", "dqmc_calculate_greens_noalloc",
    "dqmc_pool_create", "dqmc_pool_admit", "dqmc_pool_release", "dqmc_pool_set_quota",
    "dqmc_pool_run", "dqmc_pool_slot", "dqmc_pool_free_bytes", "dqmc_pool_set_flavour_split",
    "dqmc_pool_set_split_silence",
    "dqmc_set_measurements", "dqmc_reset_measurements", "dqmc_get_measurements",
    "dqmc_global_update", "dqmc_set_global_schedule", "dqmc_replica_exchange",
    "dqmc_get_global_stats", "dqmc_calculate_greens_kl", "dqmc_set_checkerboard",
    "dqmc_set_small_chain_kernel", "dqmc_get_greens_batch", "dqmc_get_fields_batch",
    "dqmc_set_fields_batch", "dqmc_checkpoint_doubles", "dqmc_get_checkpoint",
    "dqmc_set_checkpoint", "dqmc_set_tensor_products", "dqmc_set_td_measurements",
    "dqmc_td_measure", "dqmc_get_td_measurements",
]

# products on the tensor cores (dqmc_set_tensor_products)
TC_WRAPS, TC_SLICES, TC_GREENS = 1, 2, 4
TC_DEFAULT = TC_WRAPS | TC_SLICES | TC_GREENS

GLOBAL_FLIP = 0
GLOBAL_SHUFFLE = 1

PHASES = ["sweep_spatial", "wrap", "slice_chain", "udt", "greens", "prop_check", "t_update",
          "other"]

_lib = None


def load(path: str = LIB_PATH):
    """Load the CUDA library (build it first with ``build.build()``)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build the CUDA extension (montecarlo.jl_gb300/build.py); "
            "the DQMC path has no CPU fallback")
    L = C.CDLL(path)
    P = C.c_void_p
    dp = C.POINTER(C.c_double)
    i8p = C.POINTER(C.c_int8)
    L.dqmc_create.argtypes = [C.c_int, C.POINTER(ChainConfig), C.c_int, C.c_int, C.POINTER(P)]
    L.dqmc_destroy.argtypes = [P]
    L.dqmc_last_error.restype = C.c_char_p
    L.dqmc_chain_bytes.argtypes = [C.POINTER(ChainConfig), C.c_int]
    L.dqmc_chain_bytes.restype = C.c_int64
    L.dqmc_set_hopping.argtypes = [P, C.c_int, dp, dp, dp, dp]
    L.dqmc_set_field.argtypes = [P, C.c_int, i8p]
    L.dqmc_get_field.argtypes = [P, C.c_int, i8p]
    L.dqmc_init_random_field.argtypes = [P, C.c_int]
    L.dqmc_set_rng.argtypes = [P, C.c_int, C.c_uint64, C.c_uint64]
    L.dqmc_get_rng.argtypes = [P, C.c_int, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
    for f in ("dqmc_initialize_run", "dqmc_build_stack", "dqmc_propagate", "dqmc_sweep_spatial",
              "dqmc_query", "dqmc_synchronize"):
        getattr(L, f).argtypes = [P]
    L.dqmc_sweep.argtypes = [P, C.c_int, C.POINTER(Stats)]
    L.dqmc_sweep_async.argtypes = [P, C.c_int]
    L.dqmc_get_stats.argtypes = [P, C.c_int, C.POINTER(Stats)]
    L.dqmc_get_greens.argtypes = [P, C.c_int, C.c_int, dp]
    L.dqmc_set_greens.argtypes = [P, C.c_int, dp]
    L.dqmc_calculate_greens.argtypes = [P, C.c_int, C.c_int, C.c_int, dp]
    L.dqmc_get_stack.argtypes = [P, C.c_int, C.c_int, C.c_int, dp]
    L.dqmc_set_stream.argtypes = [P, C.c_void_p]
    L.dqmc_set_small_chain_kernel.argtypes = [P, C.c_int]
    L.dqmc_get_greens_batch.argtypes = [P, C.c_int, C.c_int, C.c_int, dp]
    L.dqmc_get_fields_batch.argtypes = [P, C.c_int, C.c_int, i8p]
    L.dqmc_set_fields_batch.argtypes = [P, C.c_int, C.c_int, i8p]
    L.dqmc_get_timers.argtypes = [P, C.c_int, C.POINTER(C.c_uint64)]
    L.dqmc_pool_create.argtypes = [C.c_int, C.c_int, C.c_int64, C.c_int, C.POINTER(P)]
    L.dqmc_pool_admit.argtypes = [P, C.POINTER(ChainConfig), C.POINTER(C.c_int)]
    L.dqmc_pool_release.argtypes = [P, C.c_int]
    L.dqmc_pool_set_quota.argtypes = [P, C.c_int, C.c_int64]
    L.dqmc_pool_run.argtypes = [P, C.c_int, C.c_int]
    L.dqmc_pool_set_flavour_split.argtypes = [P, C.c_int]
    L.dqmc_pool_set_split_silence.argtypes = [P, C.c_int, C.c_int]
    L.dqmc_pool_slot.argtypes = [P, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                 C.POINTER(C.c_int32)]
    L.dqmc_pool_free_bytes.argtypes = [P]
    L.dqmc_set_measurements.argtypes = [P, C.c_int, C.POINTER(MeasureConfig)]
    L.dqmc_reset_measurements.argtypes = [P, C.c_int]
    L.dqmc_global_update.argtypes = [P, C.c_int, C.c_void_p]
    L.dqmc_set_checkerboard.argtypes = [P, C.c_int, C.c_int, dp]
    L.dqmc_calculate_greens_kl.argtypes = [P, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                           dp]
    L.dqmc_set_global_schedule.argtypes = [P, C.c_int, C.c_int]
    L.dqmc_replica_exchange.argtypes = [P, C.c_void_p, C.c_void_p]
    L.dqmc_get_global_stats.argtypes = [P, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    L.dqmc_get_measurements.argtypes = [P, C.c_int, C.POINTER(Observables), C.c_void_p,
                                        C.c_void_p]
    L.dqmc_pool_free_bytes.restype = C.c_int64
    L.dqmc_set_tensor_products.argtypes = [P, C.c_int, C.c_int]
    L.dqmc_set_td_measurements.argtypes = [P, C.c_int, C.POINTER(TdConfig)]
    L.dqmc_td_measure.argtypes = [P]
    L.dqmc_get_td_measurements.argtypes = [P, C.c_int, C.POINTER(TdObservables), C.c_void_p,
                                           C.c_void_p]
    L.dqmc_checkpoint_doubles.argtypes = [P, C.c_int]
    L.dqmc_checkpoint_doubles.restype = C.c_int64
    L.dqmc_get_checkpoint.argtypes = [P, C.c_int, dp]
    L.dqmc_set_checkpoint.argtypes = [P, C.c_int, dp]
    _lib = L
    return L


def check(code: int):
    if code != DQMC_OK:
        raise DQMCError(code, load().dqmc_last_error().decode(errors="replace"))
    return code


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and (a.flags["C_CONTIGUOUS"] or a.flags["F_CONTIGUOUS"])
    return a.ctypes.data_as(C.POINTER(C.c_double))


def i8ptr(a: np.ndarray):
    assert a.dtype == np.int8
    return a.ctypes.data_as(C.POINTER(C.c_int8))


def blocks_to_buf(G: np.ndarray) -> np.ndarray:
    """(nf, n, n) -> flat column-major-per-block buffer."""
    return np.ascontiguousarray(np.transpose(np.asarray(G, dtype=np.float64), (0, 2, 1))).ravel()


def buf_to_blocks(buf: np.ndarray, nf: int, n: int) -> np.ndarray:
    return np.transpose(buf.reshape(nf, n, n), (0, 2, 1)).copy()


def is_complex(cfg) -> bool:
    """A chain with a complex field constant (the reference's ComplexF64 path):
    its matrices cross the ABI as interleaved (re, im) doubles."""
    return cfg.alpha_imag != 0.0


def complex_blocks_to_buf(G: np.ndarray) -> np.ndarray:
    """(nf, n, n) complex -> flat column-major-per-block (re, im) doubles."""
    g = np.ascontiguousarray(np.transpose(np.asarray(G, dtype=np.complex128), (0, 2, 1))).ravel()
    return g.view(np.float64)


class Handle:
    """Owns one dqmc_handle (a batch of chains on one device)."""

    def __init__(self, configs, precision=PREC_FP64, device=0):
        L = load()
        arr = (ChainConfig * len(configs))(*configs)
        self._cfg = list(configs)
        h = C.c_void_p()
        check(L.dqmc_create(device, arr, len(configs), precision, C.byref(h)))
        self.h = h
        self.n_chains = len(configs)

    def close(self):
        if getattr(self, "h", None):
            load().dqmc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def cfg(self, chain):
        if not (0 <= chain < len(self._cfg)) or self._cfg[chain] is None:
            raise DQMCError(1, f"chain index {chain} out of range or slot empty")
        return self._cfg[chain]

    def set_stream(self, stream_ptr):
        """Run on a caller-owned cudaStream_t (an int handle, e.g. torch's
        ``torch.cuda.current_stream().cuda_stream``); 0 restores the own stream."""
        check(load().dqmc_set_stream(self.h, C.c_void_p(stream_ptr or None)))

    def set_small_chain_kernel(self, enable=True):
        """Sweeps of n <= 32 chains one warp per chain (default) or one CTA per chain."""
        check(load().dqmc_set_small_chain_kernel(self.h, int(bool(enable))))

    def set_tensor_products(self, enable=True, chain=-1):
        """Tensor-core split-precision products for mixed chains of
        96 <= n <= 256: True (the library's default set), False (none: the
        double-float FP32-pipe products) or a mask of TC_WRAPS, TC_SLICES,
        TC_GREENS."""
        mask = TC_DEFAULT if enable is True else (0 if enable is False else int(enable))
        check(load().dqmc_set_tensor_products(self.h, int(chain), mask))

    def set_hopping(self, chain, exps):
        e = [np.asfortranarray(x, dtype=np.float64) for x in exps]
        check(load().dqmc_set_hopping(self.h, chain, *[dptr(x) for x in e]))

    def set_field(self, chain, conf):
        c = np.asfortranarray(conf, dtype=np.int8)
        check(load().dqmc_set_field(self.h, chain, i8ptr(c)))

    def get_field(self, chain):
        cfg = self.cfg(chain)
        c = np.zeros((cfg.n_sites, cfg.slices), dtype=np.int8, order="F")
        check(load().dqmc_get_field(self.h, chain, i8ptr(c)))
        return c

    def init_random_field(self, chain=-1):
        check(load().dqmc_init_random_field(self.h, chain))

    def set_rng(self, chain, key, counter):
        check(load().dqmc_set_rng(self.h, chain, key, counter))

    def get_rng(self, chain):
        k, c = C.c_uint64(), C.c_uint64()
        check(load().dqmc_get_rng(self.h, chain, C.byref(k), C.byref(c)))
        return k.value, c.value

    def initialize_run(self):
        check(load().dqmc_initialize_run(self.h))

    def build_stack(self):
        check(load().dqmc_build_stack(self.h))

    def propagate(self):
        check(load().dqmc_propagate(self.h))

    def sweep_spatial(self):
        check(load().dqmc_sweep_spatial(self.h))

    def sweep(self, n_sweeps=1):
        st = (Stats * self.n_chains)()
        check(load().dqmc_sweep(self.h, int(n_sweeps), st))
        return [s.as_dict() for s in st]

    def sweep_async(self, n_sweeps=1):
        check(load().dqmc_sweep_async(self.h, int(n_sweeps)))

    def query(self) -> bool:
        code = load().dqmc_query(self.h)
        if code == DQMC_ERR_NOT_READY:
            return False
        check(code)
        return True

    def synchronize(self):
        check(load().dqmc_synchronize(self.h))

    def stats(self, chain):
        s = Stats()
        check(load().dqmc_get_stats(self.h, chain, C.byref(s)))
        return s.as_dict()

    def timers(self, chain):
        """SM cycles per phase since creation (dict keyed by PHASES)."""
        out = (C.c_uint64 * 8)()
        check(load().dqmc_get_timers(self.h, chain, out))
        return dict(zip(PHASES, list(out)))

    def _mat_buf(self, chain):
        cfg = self.cfg(chain)
        return np.zeros(cfg.n_flavors * cfg.n_sites * cfg.n_sites * (2 if is_complex(cfg) else 1))

    def _blocks(self, chain, buf):
        cfg = self.cfg(chain)
        if is_complex(cfg):
            buf = buf.view(np.complex128)
        return buf_to_blocks(buf, cfg.n_flavors, cfg.n_sites)

    def greens(self, chain, physical=False):
        buf = self._mat_buf(chain)
        check(load().dqmc_get_greens(self.h, chain, int(bool(physical)), dptr(buf)))
        return self._blocks(chain, buf)

    def greens_into(self, chain, buf, physical=False):
        """Download G into a preallocated flat float64 buffer (no reshaping)."""
        check(load().dqmc_get_greens(self.h, chain, int(bool(physical)), dptr(buf)))

    def greens_batch_into(self, first, count, buf, physical=False):
        """Green's functions of chains first .. first+count-1 into one flat buffer."""
        check(load().dqmc_get_greens_batch(self.h, int(first), int(count), int(bool(physical)),
                                           dptr(buf)))

    def fields_batch_into(self, first, count, buf):
        check(load().dqmc_get_fields_batch(self.h, int(first), int(count), i8ptr(buf)))

    def set_fields_batch(self, first, count, buf):
        check(load().dqmc_set_fields_batch(self.h, int(first), int(count), i8ptr(buf)))

    def set_greens(self, chain, G):
        buf = complex_blocks_to_buf(G) if is_complex(self.cfg(chain)) else blocks_to_buf(G)
        check(load().dqmc_set_greens(self.h, chain, dptr(buf)))

    def calculate_greens(self, chain, slice_, safe_mult=0):
        buf = self._mat_buf(chain)
        check(load().dqmc_calculate_greens(self.h, chain, int(slice_), int(safe_mult), dptr(buf)))
        return self._blocks(chain, buf)

    def set_measurements(self, chain=-1, enable=True, rate=1, greens=False, sweep=-1, U=0.0,
                         q=None):
        """Device-side equal-time measurements after every ``rate``-th sweep.
        ``q`` = (cos(q.r_i), sin(q.r_i)) arrays of length n_sites for S^z(q)."""
        qc = qs = None
        if q is not None:
            qc = np.ascontiguousarray(q[0], dtype=np.float64)
            qs = np.ascontiguousarray(q[1], dtype=np.float64)
        m = MeasureConfig(int(bool(enable)), int(rate), int(bool(greens)), 0, int(sweep),
                          float(U),
                          qc.ctypes.data_as(C.POINTER(C.c_double)) if qc is not None else None,
                          qs.ctypes.data_as(C.POINTER(C.c_double)) if qs is not None else None)
        check(load().dqmc_set_measurements(self.h, chain, C.byref(m)))

    def reset_measurements(self, chain=-1):
        check(load().dqmc_reset_measurements(self.h, chain))

    def measurements(self, chain):
        """Means and binning errors of the device accumulators."""
        cfg = self.cfg(chain)
        o = Observables()
        occ = np.zeros(cfg.n_flavors * cfg.n_sites)
        g = self._mat_buf(chain)
        check(load().dqmc_get_measurements(self.h, chain, C.byref(o), occ.ctypes.data,
                                           g.ctypes.data))
        out = {"count": o.count, "occupation": occ.reshape(cfg.n_flavors, cfg.n_sites),
               "greens": buf_to_blocks(g, cfg.n_flavors, cfg.n_sites)}
        for k, name in enumerate(OBSERVABLES):
            out[name] = (o.mean[k], o.error[k])
            out[name + "_level"] = o.error_level[k]
        return out

    def set_td_measurements(self, chain, arrays, delta_tau, enable=True, rate=1, sweep=-1):
        """Device time-displaced measurements (dqmc_set_td_measurements);
        ``arrays`` from measurements.td_arrays (pair slots, q phases, form
        factors, current operator)."""
        a = arrays
        keep = []

        def ptr(x, dt):
            if x is None:
                return None
            v = np.ascontiguousarray(x, dtype=dt)
            keep.append(v)
            return v.ctypes.data

        cfg = TdConfig(int(bool(enable)), int(rate), int(a["n_slots"]),
                       (C.c_int32 * 2)(*a["n_form"]), int(a["n_current"]), float(delta_tau),
                       int(sweep), ptr(a["pair_slot"], np.int32), ptr(a["q_cos"], np.float64),
                       ptr(a["q_sin"], np.float64), ptr(a["form_sites"], np.int32),
                       ptr(a["form_values"], np.float64), ptr(a["current_sites"], np.int32),
                       ptr(a["current_values"], np.float64))
        check(load().dqmc_set_td_measurements(self.h, int(chain), C.byref(cfg)))

    def td_measure(self):
        """One time-displaced measurement of every chain that has them, now."""
        check(load().dqmc_td_measure(self.h))

    def td_measurements(self, chain, n_slots):
        """Means and binning errors of the device time-displaced measurements:
        the susceptibilities and the by-distance arrays (kind, slot)."""
        o = TdObservables()
        mean = np.zeros(len(TD_KINDS) * n_slots)
        err = np.zeros(len(TD_KINDS) * n_slots)
        check(load().dqmc_get_td_measurements(self.h, chain, C.byref(o), mean.ctypes.data,
                                              err.ctypes.data))
        out = {"count": o.count,
               "by_distance": mean.reshape(len(TD_KINDS), n_slots),
               "by_distance_error": err.reshape(len(TD_KINDS), n_slots)}
        for k, name in enumerate(TD_SCALARS):
            out[name] = (o.mean[k], o.error[k])
        return out

    def set_checkerboard(self, chain, data=None, n_parts=-1):
        """Checkerboard factors (model.checkerboard_pack); None: dense."""
        if data is None:
            check(load().dqmc_set_checkerboard(self.h, chain, -1, None))
            return
        buf = np.ascontiguousarray(data, dtype=np.float64)
        check(load().dqmc_set_checkerboard(self.h, chain, int(n_parts), dptr(buf)))

    def greens_kl(self, chain, pairs, physical=False):
        """Unequal-time G(k, l) of the chain's configuration for (k, l) pairs."""
        cfg = self.cfg(chain)
        k = np.ascontiguousarray([p[0] for p in pairs], dtype=np.int32)
        l = np.ascontiguousarray([p[1] for p in pairs], dtype=np.int32)
        per = cfg.n_flavors * cfg.n_sites * cfg.n_sites * (2 if is_complex(cfg) else 1)
        buf = np.zeros(len(pairs) * per)
        check(load().dqmc_calculate_greens_kl(self.h, chain, k.ctypes.data, l.ctypes.data,
                                              len(pairs), int(bool(physical)), dptr(buf)))
        return [self._blocks(chain, buf[i * per:(i + 1) * per]) for i in range(len(pairs))]

    def global_update(self, kind=GLOBAL_FLIP):
        """One global move of every chain; returns the accepted flags."""
        acc = np.zeros(self.n_chains, dtype=np.int32)
        check(load().dqmc_global_update(self.h, int(kind), acc.ctypes.data))
        return acc.astype(bool)

    def set_global_schedule(self, kind, chain=-1):
        """A global move before every sweep but the first (kind None: off)."""
        check(load().dqmc_set_global_schedule(self.h, int(chain), -1 if kind is None else int(kind)))

    def replica_exchange(self, partners):
        """Replica exchange between paired chains (partners[i] = j, -1: none)."""
        p = np.ascontiguousarray(partners, dtype=np.int32)
        assert p.size == self.n_chains
        acc = np.zeros(self.n_chains, dtype=np.int32)
        check(load().dqmc_replica_exchange(self.h, p.ctypes.data, acc.ctypes.data))
        return acc.astype(bool)

    def checkpoint(self, chain):
        """The chain's checkpoint record (counters, schedule, measurement
        accumulators) as a flat float64 array."""
        nd = int(load().dqmc_checkpoint_doubles(self.h, chain))
        if nd < 0:
            check(load().dqmc_get_checkpoint(self.h, chain, None))
        buf = np.zeros(nd)
        check(load().dqmc_get_checkpoint(self.h, chain, dptr(buf)))
        return buf

    def restore_checkpoint(self, chain, record):
        buf = np.ascontiguousarray(record, dtype=np.float64)
        nd = int(load().dqmc_checkpoint_doubles(self.h, chain))
        if buf.size != nd:
            raise DQMCError(1, f"checkpoint record of {buf.size} doubles, chain needs {nd}")
        check(load().dqmc_set_checkpoint(self.h, chain, dptr(buf)))

    def global_stats(self, chain):
        a, p = C.c_int64(), C.c_int64()
        check(load().dqmc_get_global_stats(self.h, chain, C.byref(a), C.byref(p)))
        return a.value, p.value

    def stack(self, chain, which, idx):
        """u/t/d_stack[idx]; a complex chain's are the factors of its real
        2n x 2n representation."""
        cfg = self.cfg(chain)
        n = cfg.n_sites * (2 if is_complex(cfg) else 1)
        if which == 2:
            out = np.zeros(cfg.n_flavors * n)
            check(load().dqmc_get_stack(self.h, chain, 2, idx, dptr(out)))
            return out.reshape(cfg.n_flavors, n)
        buf = np.zeros(cfg.n_flavors * n * n)
        check(load().dqmc_get_stack(self.h, chain, which, idx, dptr(buf)))
        return buf_to_blocks(buf, cfg.n_flavors, n)


DQMC_ERR_OOM = 3


class Pool(Handle):
    """A dqmc pool: slots admitted / released between time-sliced launches."""

    def __init__(self, max_slots, budget_bytes, precision=PREC_FP64, device=0):
        L = load()
        h = C.c_void_p()
        check(L.dqmc_pool_create(device, int(max_slots), int(budget_bytes), precision, C.byref(h)))
        self.h = h
        self.n_chains = int(max_slots)
        self._cfg = [None] * int(max_slots)

    def admit(self, cfg):
        """Slot index, or None when the budget or the slots are exhausted."""
        slot = C.c_int(-1)
        code = load().dqmc_pool_admit(self.h, C.byref(cfg), C.byref(slot))
        if code in (DQMC_ERR_OOM, DQMC_ERR_NOT_READY):
            return None
        check(code)
        self._cfg[slot.value] = cfg
        return slot.value

    def release(self, slot):
        check(load().dqmc_pool_release(self.h, int(slot)))
        self._cfg[slot] = None

    def set_quota(self, slot, n_sweeps):
        check(load().dqmc_pool_set_quota(self.h, int(slot), int(n_sweeps)))

    def run(self, budget_us, use_graph=True):
        check(load().dqmc_pool_run(self.h, int(budget_us), int(bool(use_graph))))

    def set_flavour_split(self, enable=True):
        """Two-flavour chains run their flavour blocks on two CTAs (two SMs)
        of a two-CTA cluster; results are bit-identical."""
        check(load().dqmc_pool_set_flavour_split(self.h, int(bool(enable))))

    def set_split_silence(self, slot, from_epoch):
        """Test hook: the second CTA of the slot's flavour-split chain stops
        announcing itself from rendezvous `from_epoch` on (0: off), so that
        the first one's bounded wait runs out and the chain reports status 9."""
        check(load().dqmc_pool_set_split_silence(self.h, int(slot), int(from_epoch)))

    def slot(self, slot):
        d, l, a = C.c_int64(), C.c_int64(), C.c_int32()
        check(load().dqmc_pool_slot(self.h, int(slot), C.byref(d), C.byref(l), C.byref(a)))
        return d.value, l.value, bool(a.value)

    def free_bytes(self):
        return int(load().dqmc_pool_free_bytes(self.h))


def chain_bytes(cfg, precision=PREC_FP64):
    return int(load().dqmc_chain_bytes(C.byref(cfg), precision))
