"""``DQMC`` simulation object and ``run`` (the reference's ``run!``) on the GPU.

Mirrors src/flavors/DQMC/DQMC.jl:32-394: construction from a model and
keyword parameters, random field initialisation from the seed, the stack
build of ``initialize_run`` and the sweep loop of ``run!`` with measurements
every ``measure_rate`` sweeps after thermalisation.  The sweeps, wraps,
stabilisations and Green's functions run in libdqmc_gb300.so; measurements
are evaluated on the device after every ``measure_rate``-th sweep past
thermalisation (density, double occupancy, interaction energy, S^z(q),
occupations and the mean physical G, log-binned on the device; see
``observables``), and user measurement kernels additionally on the
downloaded physical Green's function.
"""
from __future__ import annotations

import enum
import time

import numpy as np

from . import _lib
from .measurements import LogBinner, MEASUREMENTS
from .model import DQMCParameters, hopping_exponentials


class ExitCode(enum.IntEnum):
    """src/helpers.jl:17-22."""

    SUCCESS = 0
    GENERIC_FAILURE = 1
    CANCELLED_TIME_LIMIT = 2
    CANCELLED_LOW_ACCEPTANCE = 3


class DQMC:
    """``DQMC(model; seed, field, measurements, thermalization, sweeps,
    measure_rate, beta, delta_tau | slices, safe_mult, ...)``.

    Extra keywords of this implementation: ``precision`` ("fp64" or "mixed"),
    ``device``, ``device_measurements`` (default True: the on-device
    equal-time observables), ``structure_factor_q`` (the q of S^z(q),
    default (pi, pi, ...)) and ``global_update`` (None, "flip" or "shuffle":
    the scheduler SimpleScheduler(LocalSweep(), GlobalFlip() / GlobalShuffle()),
    scheduler.jl:258-289).  ``recorder`` (default: a ``ConfigRecorder`` with
    ``recording_rate``, which defaults to ``measure_rate``; ``False``: record
    nothing, the reference's Discarder) receives the field configuration after
    every recorded sweep past thermalisation (DQMC.jl:41, 216).
    ``time_displaced`` (default False) adds the TimeIntegral measurements on
    the device after every ``measure_rate``-th sweep past thermalisation:
    charge, spin x / y / z (at ``structure_factor_q``) and pairing (on site,
    extended s, d) susceptibilities, the current-current susceptibility along
    ``current_direction``, and the by-distance correlation arrays (see
    ``time_displaced_observables``).
    """

    def __init__(self, model, *, seed: int = -1, field=None, measurements=None,
                 thermalization_measurements=None, last_sweep: int = 0, measure_rate: int = 10,
                 precision: str = "fp64", device: int = 0, device_measurements: bool = True,
                 structure_factor_q=None, global_update=None, recorder=None,
                 recording_rate: int = None, time_displaced: bool = False,
                 current_direction=None, **kwargs):
        self.model = model
        self.parameters = DQMCParameters.make(measure_rate=measure_rate, **kwargs)
        fcls = field if field is not None else model.choose_field()
        self.field = fcls(self.parameters, model)
        if seed == -1:
            seed = int(np.random.SeedSequence().generate_state(1, dtype=np.uint64)[0])
        self.seed = int(seed) & (2**64 - 1)
        self.last_sweep = last_sweep
        self.measurements = dict(measurements or {})
        self.thermalization_measurements = dict(thermalization_measurements or {})
        self.precision = precision
        p = self.parameters
        self.n = len(model.l)
        a = complex(self.field.alpha)
        self.config = _lib.ChainConfig(self.n, self.field.unique_flavors, p.slices, p.safe_mult,
                                       self.field.kind, int(p.check_propagation_error),
                                       a.real, self.seed, a.imag)
        if self.field.is_complex:
            # complex Green's functions: measured on the host from the download
            device_measurements = False
        prec = _lib.PREC_MIXED if precision == "mixed" else _lib.PREC_FP64
        self.handle = _lib.Handle([self.config], precision=prec, device=device)
        self.exps = hopping_exponentials(model.hopping_matrix(), p.delta_tau)
        self.handle.set_hopping(0, self.exps)
        if p.checkerboard:  # init_hopping_matrices with checkerboard (stack.jl:240-246)
            from .model import checkerboard_exponentials, checkerboard_pack
            cbf = checkerboard_exponentials(model.hopping_matrix(), model.l, p.delta_tau)
            self.handle.set_checkerboard(0, *checkerboard_pack(cbf))
        self.handle.init_random_field(0)  # rand!(field_data), DQMC.jl:50
        self.field.conf[:] = self.handle.get_field(0)
        self.initialized = False
        self.analysis = {}
        self.max_sweeps_per_launch = 50
        self.device_measurements = device_measurements
        pos = model.l.positions()
        q = np.full(pos.shape[1], np.pi) if structure_factor_q is None else \
            np.asarray(structure_factor_q, dtype=float)
        ph = pos @ q
        self._q_phases = (np.cos(ph), np.sin(ph))
        self._dev_meas_on = None
        if global_update not in (None, "flip", "shuffle"):
            raise ValueError("global_update must be None, 'flip' or 'shuffle'")
        self.global_update = global_update
        if recorder is None:
            recorder = ConfigRecorder(recording_rate or measure_rate)
        # an empty recorder is falsy (len 0): test for the Discarder spelling
        self.recorder = None if recorder is False else recorder
        self._restore_record = None
        self.time_displaced = time_displaced and not self.field.is_complex
        self._td_arrays = None
        if self.time_displaced:
            from .measurements import td_arrays
            self._td_arrays = td_arrays(model, q=structure_factor_q,
                                        current_direction=current_direction)

    # -- stack --------------------------------------------------------------
    def init(self):
        """init! + the stack part of initialize_run (DQMC.jl:144-179)."""
        self.handle.set_field(0, np.asfortranarray(self.field.conf))
        self.handle.initialize_run()
        if self.global_update is not None:
            self.handle.set_global_schedule(
                _lib.GLOBAL_FLIP if self.global_update == "flip" else _lib.GLOBAL_SHUFFLE, 0)
        if self._restore_record is not None:
            # a resumed chain: its counters, scheduler position and measurement
            # accumulators as saved (the rebuild above is not a sweep)
            self.handle.restore_checkpoint(0, self._restore_record)
            self._restore_record = None
        self.initialized = True

    @property
    def current_slice(self):
        return self.handle.stats(0)["current_slice"]

    def greens(self, physical=True):
        """greens(mc) (greens.jl:87): the physical equal-time G by default."""
        return self.handle.greens(0, physical=physical)

    def greens_kl(self, k, l, physical=True):
        """greens(mc, k, l) (unequal_time_stack.jl:309-324): the unequal-time
        G(k dtau, l dtau); physical (the _greens! transform) by default."""
        return self.handle.greens_kl(0, [(k, l)], physical=physical)[0]

    def spin_susceptibility(self, q=None):
        """chi_z(q) of the current configuration (time-displaced spin-density
        correlations integrated over tau, the reference's
        spin_density_susceptibility with a TimeIntegral): the unequal-time
        Green's functions G(0,0), G(l,l), G(0,l), G(l,0) for l = 0..M in one
        device call, contracted on the host.  q defaults to (pi, pi, ...)."""
        from .measurements import spin_susceptibility_z
        M = self.parameters.slices
        pairs = [(0, 0)]
        for l in range(M + 1):
            pairs += [(l, l), (0, l), (l, 0)]
        Gs = self.handle.greens_kl(0, pairs, physical=True)
        G00 = Gs[0]
        by_l = [(G00, Gs[2 + 3 * l], Gs[3 + 3 * l], Gs[1 + 3 * l]) for l in range(M + 1)]
        if q is None:
            phases = self._q_phases
        else:
            ph = self.model.l.positions() @ np.asarray(q, dtype=float)
            phases = (np.cos(ph), np.sin(ph))
        return spin_susceptibility_z(by_l, phases, self.parameters.delta_tau)

    def susceptibilities(self, q=None, current_direction=None):
        """The time-integrated susceptibilities of the current configuration
        (charge, spin x / y / z at q, on-site s-wave pairing, and the uniform
        current-current one along ``current_direction`` (default: the first
        lattice vector); the reference's charge_density_susceptibility,
        spin_density_susceptibility, pairing_susceptibility and
        current_current_susceptibility with TimeIntegral) from one device
        call for the Green's functions G(0,0), G(l,l), G(0,l), G(l,0),
        l = 0..M."""
        from .measurements import current_operator, pair_form_factor, susceptibilities
        M = self.parameters.slices
        pairs = [(0, 0)]
        for l in range(M + 1):
            pairs += [(l, l), (0, l), (l, 0)]
        Gs = self.handle.greens_kl(0, pairs, physical=True)
        by_l = [(Gs[0], Gs[2 + 3 * l], Gs[3 + 3 * l], Gs[1 + 3 * l]) for l in range(M + 1)]
        if q is None:
            phases = self._q_phases
        else:
            ph = self.model.l.positions() @ np.asarray(q, dtype=float)
            phases = (np.cos(ph), np.sin(ph))
        J = current_operator(self.model.hopping_matrix(), self.model.l, current_direction)
        pf = {}
        if len(self.model.l.unitcell.lattice_vectors) >= 2:
            pf = {k: pair_form_factor(self.model.l, k) for k in ("s*", "d")}
        return susceptibilities(by_l, phases, self.parameters.delta_tau, current=J, pair_fields=pf)

    def calculate_greens(self, slice_, safe_mult=0):
        """calculate_greens(mc, slice) (stack.jl:525-583), effective G."""
        return self.handle.calculate_greens(0, slice_, safe_mult)

    def __getitem__(self, key):
        return self.measurements[key]

    def __setitem__(self, key, value):
        self.measurements[key] = value

    # -- run! -----------------------------------------------------------------
    def run(self, *, verbose: bool = False, thermalization: int = None, sweeps: int = None,
            safe_before: float = None, min_acceptance: float = None) -> ExitCode:
        """run! (DQMC.jl:252-394): thermalisation + measurement sweeps."""
        p = self.parameters
        th = p.thermalization if thermalization is None else thermalization
        sw = p.sweeps if sweeps is None else sweeps
        if not self.initialized:
            self.init()
        t0 = time.time()
        total = th + sw
        st = self.handle.stats(0)
        acc0, prop0 = st["accepted"], st["proposals"]
        while self.last_sweep < total:
            # advance in device launches up to the next measurement or
            # recording point (both read the chain after that sweep)
            if self.last_sweep < th:
                k = th - self.last_sweep
            else:
                stops = [total - self.last_sweep]
                if self.measurements:
                    stops.append(p.measure_rate - (self.last_sweep % p.measure_rate))
                if self.recorder is not None:
                    stops.append(self.recorder.rate - (self.last_sweep % self.recorder.rate))
                k = min(stops)
            k = max(1, min(k, total - self.last_sweep, self.max_sweeps_per_launch))
            if self.device_measurements or self.time_displaced:
                self._device_measure(self.last_sweep >= th)
            self.handle.sweep(k)
            self.last_sweep += k
            if self.last_sweep > th:
                if self.recorder is not None:
                    self.recorder.push(self.handle.get_field(0), self.last_sweep,
                                       ghq=self.field.kind >= 2)
                if self.last_sweep % p.measure_rate == 0:
                    self._measure()
            if safe_before is not None and time.time() > safe_before:
                return ExitCode.CANCELLED_TIME_LIMIT
        st = self.handle.stats(0)
        self.analysis = dict(
            acceptance=(st["accepted"] - acc0) / max(1, st["proposals"] - prop0),
            global_moves=self.handle.global_stats(0),
            propagation_errors=st["propagation_errors"],
            max_propagation_error=st["max_propagation_error"],
            negative_probability=st["negative_probability"],
            imaginary_probability=(st["imaginary_probability"],
                                   st["max_imaginary_probability"]),
            # DQMCAnalysis' MagnitudeStats (statistics.jl:9-51), since creation
            magnitude_stats={
                "propagation_error": dict(count=st["propagation_errors"],
                                          min=st["min_reported_error"],
                                          mean=st["mean_reported_error"],
                                          max=st["max_reported_error"]),
                "negative_probability": dict(count=st["negative_probability"],
                                             min=st["min_negative_probability"],
                                             mean=st["mean_negative_probability"],
                                             max=st["max_negative_probability"]),
                "imaginary_probability": dict(count=st["imaginary_probability"],
                                              min=st["min_imaginary_probability"],
                                              mean=st["mean_imaginary_probability"],
                                              max=st["max_imaginary_probability"])},
            runtime=time.time() - t0)
        self.field.conf[:] = self.handle.get_field(0)
        if min_acceptance is not None and self.analysis["acceptance"] < min_acceptance:
            return ExitCode.CANCELLED_LOW_ACCEPTANCE
        if verbose:
            print(f"DQMC run: {total} sweeps, acceptance {self.analysis['acceptance']:.3f}, "
                  f"max propagation error {self.analysis['max_propagation_error']:.2e}")
        return ExitCode.SUCCESS

    def _device_measure(self, on):
        """Switch the device accumulators on (past thermalisation) or off; the
        device counts sweeps from ``last_sweep`` and measures at every
        multiple of ``measure_rate`` while on."""
        if self._dev_meas_on is on:
            return
        if self.device_measurements:
            self.handle.set_measurements(0, enable=on, rate=self.parameters.measure_rate,
                                         greens=True, sweep=self.last_sweep, U=self.model.U,
                                         q=self._q_phases)
        if self.time_displaced:
            self.handle.set_td_measurements(0, self._td_arrays, self.parameters.delta_tau,
                                            enable=on, rate=self.parameters.measure_rate,
                                            sweep=self.last_sweep)
        self._dev_meas_on = on

    def time_displaced_observables(self):
        """The device time-displaced measurements (``time_displaced=True``):
        ``(mean, error)`` per susceptibility, ``by_distance`` (kind, slot)
        means and errors of the charge, spin x / y / z and on-site pairing
        correlations (the reference's EachSitePairByDistance arrays,
        (Ndir, B, B) column-major per kind), and the number of measurements."""
        if not self.time_displaced:
            raise ValueError("time-displaced measurements were not requested (time_displaced=True)")
        return self.handle.td_measurements(0, self._td_arrays["n_slots"])

    def observables(self):
        """The on-device equal-time measurements: ``(mean, error)`` of the
        density, double occupancy, interaction energy and S^z(q), the mean
        occupations and physical G, and the number of measurements."""
        return self.handle.measurements(0)

    def _measure(self):
        G = self.greens(physical=True)
        for name, obs in self.measurements.items():
            obs.measure(G, self)


class ConfigRecorder:
    """Field configurations recorded every `rate` sweeps, compressed
    (ConfigRecorder, src/configurations.jl:24-66; compress / decompress,
    fields.jl:331-334 and 472-491): Hirsch fields as one bit per entry
    (x == 1), Gauss-Hermite fields as two bits (x - 1)."""

    def __init__(self, rate: int = 10):
        self.rate = rate
        self.configs = []
        self.shape = None
        self.ghq = False

    def push(self, conf, sweep, ghq=False):
        if sweep % self.rate != 0:
            return
        self.shape, self.ghq = conf.shape, ghq
        c = np.asarray(conf, dtype=np.int8).ravel(order="F")
        if ghq:
            v = (c - 1).astype(np.uint8)
            bits = np.stack([(v >> 1) & 1, v & 1], axis=1).ravel()
        else:
            bits = (c == 1).astype(np.uint8)
        self.configs.append(np.packbits(bits))

    def __len__(self):
        return len(self.configs)

    def __getitem__(self, i):
        n = int(np.prod(self.shape))
        if self.ghq:
            bits = np.unpackbits(self.configs[i])[: 2 * n].reshape(n, 2)
            c = (1 + 2 * bits[:, 0] + bits[:, 1]).astype(np.int8)
        else:
            bits = np.unpackbits(self.configs[i])[:n]
            c = (2 * bits.astype(np.int8) - 1).astype(np.int8)
        return c.reshape(self.shape, order="F")


def replay(mc, configurations=None, measure_rate: int = 1):
    """replay! (DQMC.jl:418-505): for every recorded configuration from
    ``mc.last_sweep + 1`` on (1-based; every ``measure_rate``-th), recompute G
    from scratch (calculate_greens(mc, 0), the equal-time G at slice 1), run
    the measurements on its physical form and set ``mc.last_sweep`` to the
    configuration's 1-based index, so a replay interrupted (or saved and
    resumed) continues where it stopped.  ``configurations`` defaults to the
    simulation's recorder."""
    if configurations is None:
        configurations = mc.recorder
    for i in range(mc.last_sweep, len(configurations), measure_rate):
        conf = configurations[i]
        mc.handle.set_field(0, np.asfortranarray(conf))
        G_eff = mc.handle.calculate_greens(0, 0)
        mc.handle.set_greens(0, G_eff)
        G = mc.handle.greens(0, physical=True)
        for obs in mc.measurements.values():
            obs.measure(G, mc)
        mc.last_sweep = i + 1


def save(mc, path):
    """Checkpoint of a simulation (FileIO.jl:10-57; flavors/DQMC/FileIO.jl:10-22):
    parameters (including checkerboard and check_propagation_error), model,
    field, RNG state, last sweep, the scheduler's global update, the recorded
    configurations, the DQMCAnalysis counters and the device measurement
    accumulators (one checkpoint record of the chain), and the values pushed
    into every host measurement's binner (by measurement name).  The stack is
    not saved: resume rebuilds it from the field, as the reference does
    (DQMC.jl:178-179)."""
    key, ctr = mc.handle.get_rng(0)
    conf = mc.handle.get_field(0)
    p = mc.parameters
    lat = mc.model.l
    extra = {}
    rec = mc.recorder
    if rec is not None:
        extra["rec_rate"] = np.array([rec.rate])
        extra["rec_ghq"] = np.array([int(rec.ghq)])
        extra["rec_shape"] = np.array(rec.shape if rec.shape is not None else (0, 0))
        extra["rec_configs"] = (np.stack(rec.configs) if rec.configs
                                else np.zeros((0, 0), dtype=np.uint8))
    names = []
    for name, obs in mc.measurements.items():
        binner = getattr(obs, "observable", None)
        if binner is None or not len(binner):
            continue
        names.append(str(name))
        extra[f"meas_{len(names) - 1}"] = np.stack(binner.values)
    extra["meas_names"] = np.array(names, dtype=str)
    np.savez(path, conf=conf, rng=np.array([key, ctr], dtype=np.uint64),
             last_sweep=mc.last_sweep, seed=mc.seed,
             params=np.array([p.beta, p.delta_tau, p.slices, p.safe_mult, p.thermalization,
                              p.sweeps, p.measure_rate, float(p.checkerboard),
                              float(p.check_propagation_error)], dtype=np.float64),
             model=np.array([mc.model.t, mc.model.mu, mc.model.U]),
             lattice=np.array([lat.name] + [str(x) for x in lat.Ls]),
             field=np.array([type(mc.field).__name__]), precision=np.array([mc.precision]),
             global_update=np.array([mc.global_update or ""]),
             device_measurements=np.array([int(mc.device_measurements)]),
             chain_record=mc.handle.checkpoint(0), **extra)


def resume(path, **kwargs):
    """Rebuild a simulation from a checkpoint; the next run continues the
    chain where it stopped (resume!, FileIO.jl:155-171): same field, RNG
    position, parameters, checkerboard hopping, global-update schedule,
    analysis counters, device accumulators and recorded configurations.
    Host measurements passed in ``measurements=`` get back the values saved
    under their names."""
    from . import lattices, model as _model

    d = np.load(path, allow_pickle=False)
    name, *Ls = [str(x) for x in d["lattice"]]
    ctor = {"Square": lattices.SquareLattice, "Honeycomb": lattices.Honeycomb,
            "Chain": lattices.Chain, "Cubic": lattices.CubicLattice,
            "Triangular": lattices.TriangularLattice}[name]
    t, mu, U = [float(x) for x in d["model"]]
    m = _model.HubbardModel(ctor(*[int(x) for x in Ls]), U=U, mu=mu, t=t)
    prm = d["params"]
    beta, dt, slices, k, th, sw, mr = prm[:7]
    cb = bool(prm[7]) if prm.size > 7 else False
    cpe = bool(prm[8]) if prm.size > 8 else True
    gu = str(d["global_update"][0]) if "global_update" in d.files else ""
    kw = dict(kwargs)
    kw.setdefault("global_update", gu or None)
    if "device_measurements" in d.files:
        kw.setdefault("device_measurements", bool(d["device_measurements"][0]))
    if "rec_rate" in d.files:
        kw.setdefault("recorder", ConfigRecorder(int(d["rec_rate"][0])))
    else:
        kw.setdefault("recorder", False)
    mc = DQMC(m, seed=int(d["seed"]), field=getattr(_model, str(d["field"][0])),
              beta=float(beta), delta_tau=float(dt), safe_mult=int(k), thermalization=int(th),
              sweeps=int(sw), measure_rate=int(mr), precision=str(d["precision"][0]),
              checkerboard=cb, check_propagation_error=cpe, **kw)
    mc.field.conf[:] = d["conf"]
    mc.handle.set_field(0, np.asfortranarray(d["conf"]))
    key, ctr = [int(x) for x in d["rng"]]
    mc.handle.set_rng(0, key, ctr)
    mc.last_sweep = int(d["last_sweep"])
    if "chain_record" in d.files:
        mc.handle.restore_checkpoint(0, d["chain_record"])
        mc._restore_record = np.array(d["chain_record"])  # again after the stack rebuild
    if mc.recorder is not None and "rec_configs" in d.files:
        rc = d["rec_configs"]
        mc.recorder.configs = [rc[i].copy() for i in range(rc.shape[0])]
        shp = tuple(int(x) for x in d["rec_shape"])
        mc.recorder.shape = shp if rc.shape[0] else None
        mc.recorder.ghq = bool(d["rec_ghq"][0])
    if "meas_names" in d.files:
        for i, nm in enumerate(d["meas_names"]):
            obs = mc.measurements.get(str(nm))
            if obs is not None and hasattr(obs, "observable"):
                obs.observable.values = [np.array(v) for v in d[f"meas_{i}"]]
    return mc


class Measurement:
    """A DQMC measurement: a kernel over the physical G pushed into a LogBinner
    (DQMCMeasurement, measurements/generic.jl:6-13)."""

    def __init__(self, kernel, post=None):
        self.kernel = MEASUREMENTS.get(kernel, kernel) if isinstance(kernel, str) else kernel
        self.post = post
        self.observable = LogBinner()

    def measure(self, G, mc):
        v = self.kernel(G)
        if self.post is not None:
            v = self.post(v, mc)
        self.observable.push(v)

    def mean(self):
        return self.observable.mean()

    def std_error(self):
        return self.observable.std_error()


def greens_measurement(mc=None, model=None):
    return Measurement("greens")


def occupation(mc=None, model=None):
    return Measurement("occupation")


def double_occupancy(mc=None, model=None):
    return Measurement("double_occupancy", post=lambda v, mc: float(np.mean(v)))


def spin_density_correlation(mc=None, model=None, component="z"):
    if component != "z":
        raise NotImplementedError("only the z component is part of this library")
    return Measurement("spin_density_correlation_z")
