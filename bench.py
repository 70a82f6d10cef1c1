#!/usr/bin/env python
"""DQMC sweep throughput on GB300: sweeps/s of an ensemble of Hubbard-model chains.

Workload (default): the repulsive Hubbard model at half filling on an 8x8
periodic square lattice (N = 64, two spin flavours), t = 1, U = 4 in the
physics convention (U = -4 in the reference's convention), mu = 0,
MagneticHirschField, beta = 8, delta_tau = 0.1 (80 slices), safe_mult = 10,
FP64, run as an ensemble of independent chains (seeds 2 + j), two per SM.
One step = one sweep (2M slice visits x N proposals, with wraps and
stabilisations) of every chain in one launch; ``value`` is aggregate sweeps/s.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--workload c2|c1|c4|l12] [--chains B]

``--impl reference`` times the CPU restatement of the reference's algorithm
(the oracle; the reference itself is Julia, which this machine cannot run) on
all host cores with the same workload and prints the same JSON line.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

# the headline metric; ``value`` is the plain FP64 path on the batched
# ensemble, the mixed / batched / served figures ride along in the same line
METRIC = "DQMC sweeps/s/GPU, batched+served vs plain FP64, at |ΔG|≤1e-6; p50/p99 latency"

WORKLOADS = {
    # name: (lattice L, U (reference convention), beta, safe_mult, field, description)
    "c2": (8, -4.0, 8.0, 10, "MagneticHirschField",
           "8x8 square repulsive Hubbard U=4 (physics), mu=0, MagneticHirschField, beta=8, "
           "dtau=0.1 (M=80), safe_mult=10, FP64"),
    "c1": (4, 4.0, 4.0, 10, "DensityHirschField",
           "4x4 square attractive Hubbard U=-4 (physics), mu=0, DensityHirschField, beta=4, "
           "dtau=0.1 (M=40), safe_mult=10, FP64"),
    "l12": (12, -4.0, 8.0, 10, "MagneticHirschField",
            "12x12 square repulsive Hubbard U=4 (physics), mu=0, MagneticHirschField, beta=8, "
            "dtau=0.1 (M=80), safe_mult=10"),
    "c4": (16, -4.0, 10.0, 10, "MagneticHirschField",
           "16x16 square repulsive Hubbard U=4 (physics), mu=0, MagneticHirschField, beta=10, "
           "dtau=0.1 (M=100), safe_mult=10, FP64"),
    # the field-timing case of the reference's documentation (docs/src/DQMC/fields.md:49-56:
    # 6x6 square, beta = 1, 10 000 sweeps; 6.8 s and 17 s there, hardware not stated)
    "docs6_density": (6, 1.0, 1.0, 10, "DensityHirschField",
                      "6x6 square attractive Hubbard U=-1 (physics; U=+1 reference convention), "
                      "mu=0, DensityHirschField, beta=1, dtau=0.1 (M=10), safe_mult=10, FP64"),
    "docs6_magnetic": (6, -1.0, 1.0, 10, "MagneticHirschField",
                       "6x6 square repulsive Hubbard U=1 (physics; U=-1 reference convention), "
                       "mu=0, MagneticHirschField, beta=1, dtau=0.1 (M=10), safe_mult=10, FP64"),
}
L2_BYTES = 129 * 1000 * 1000  # GB300 L2


def sweep_flops(n, nf, M, nr, acc):
    """Algorithmic FP64 flops of one sweep of one chain (O(n^3) terms only):
    nf * n^3 * (12 M + 48 c + 4 a M) -- wraps 8M, slice chains 4M, UDT + T
    update 2c(10/3 + 2), Green's reconstruction 2c(56/3), rank-1 updates 4aM."""
    return nf * float(n) ** 3 * (12 * M + 48 * nr + 4 * acc * M)


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            if len(r) < 9:
                continue
            for k, nm in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def setup_workload(pkg, name):
    L, U, beta, k, field, desc = WORKLOADS[name]
    model = pkg.HubbardModel(pkg.SquareLattice(L), U=U)
    param = pkg.DQMCParameters.make(beta=beta, delta_tau=0.1, safe_mult=k)
    fld = getattr(pkg, field)(param, model)
    exps = pkg.hopping_exponentials(model.hopping_matrix(), param.delta_tau)
    return model, param, fld, exps, desc


def run_reference(args, pkg, rank):
    """CPU restatement of the reference's sweep (oracle), all host threads."""
    import oracle as O

    O.use_fast_build(True)
    model, param, fld, exps, desc = setup_workload(pkg, args.workload)
    n = len(model.l)
    threads = os.cpu_count() or 1
    chains = []
    for j in range(threads):
        c = O.OracleChain(n, fld.unique_flavors, param.slices, param.safe_mult, fld.kind, fld.alpha,
                          exps, 2 + j)
        c.init_random_conf()
        c.initialize_run()
        chains.append(c)
    # calibrate: one sweep of one chain
    t = time.perf_counter()
    chains[0].sweeps(1)
    t1 = time.perf_counter() - t
    per_step = max(1, int(round(args.cpu_budget / max(args.steps, 1) / t1)))
    for _ in range(min(args.warmup, 1)):
        O.run_chains_threaded(chains, 1, threads)
    wall = 0.0
    for _ in range(args.steps):
        wall += O.run_chains_threaded(chains, per_step, threads)
    value = threads * per_step * args.steps / wall
    cores = threads
    sample = (f"{threads} chains x {per_step * args.steps} sweeps ({per_step} per step) of the "
              f"workload, one chain per host thread")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "sweeps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * wall / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded random HS fields)",
        "config": {"workload": desc, "path": "CPU restatement, FP64", "chains": threads,
                   "ensemble": "independent chains"},
        "cpu_baseline": {"value": value, "unit": "sweeps/s", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "sweeps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": "reference is Julia (not installed on this machine); timed its C restatement "
                "(oracle/dqmc_oracle.c, FMA contraction on)",
    }
    print(json.dumps(line), flush=True)


def cpu_baseline_sample(pkg, workload, budget_s):
    """Bounded oracle run on all host threads (rank 0 only)."""
    import oracle as O

    O.use_fast_build(True)
    model, param, fld, exps, desc = setup_workload(pkg, workload)
    n = len(model.l)
    threads = os.cpu_count() or 1
    chains = []
    for j in range(threads):
        c = O.OracleChain(n, fld.unique_flavors, param.slices, param.safe_mult, fld.kind, fld.alpha,
                          exps, 2 + j)
        c.init_random_conf()
        c.initialize_run()
        chains.append(c)
    t = time.perf_counter()
    chains[0].sweeps(1)
    t1 = time.perf_counter() - t
    nsw = max(1, int(round(budget_s / t1)))
    wall = O.run_chains_threaded(chains, nsw, threads)
    return {"value": threads * nsw / wall, "unit": "sweeps/s", "cores": threads, "kind": "port",
            "sample": f"{threads} chains x {nsw} sweeps, one chain per host thread "
                      f"(C restatement of the reference, FMA contraction on)"}


def nsm_of_device():
    import torch
    return torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count


def ensemble_c3(pkg, _lib, n_chains, seconds, stream, seed=3):
    """Batched ensemble of uneven attractive chains: L in {6,8,10,12}, U_phys in
    [-8,-2] (U_ref = -U_phys), beta in {4,8,12}, dtau = 0.1; safe_mult
    autotuned per chain for a propagation error <= 1e-6 (and lowered for any
    chain that exceeds it over the timed sweeps, after which the timed run is
    repeated); plain FP64 and mixed, both batched, and the unbatched plain FP64
    path (each chain alone in its own launches, one after another)."""
    from montecarlo_gb300 import autotune

    rng = np.random.default_rng(seed)
    specs = []
    for j in range(n_chains):
        L = int(rng.choice([6, 8, 10, 12]))
        U = float(rng.uniform(-8.0, -2.0))
        beta = float(rng.choice([4.0, 8.0, 12.0]))
        model = pkg.HubbardModel(pkg.SquareLattice(L), U=-U)
        specs.append((model, model.choose_field(), beta, 0.1, 1000 + j))
    out = {"workload": f"{n_chains} attractive chains, L in {{6,8,10,12}} square, U in [-8,-2] "
                       "(physics), beta in {4,8,12}, dtau=0.1, safe_mult autotuned per chain "
                       "(propagation error <= 1e-6), started from thermalised configurations",
           "cta_slots": {"chains": n_chains, "slots": 2 * nsm_of_device()}}
    t = time.perf_counter()
    confs = autotune.thermalize(specs)
    therm_s = time.perf_counter() - t
    out["thermalize_s"] = therm_s
    chosen = {}
    for name, prec in (("plain_fp64", _lib.PREC_FP64), ("mixed", _lib.PREC_MIXED)):
        t = time.perf_counter()
        # a 200x margin on the probes: the propagation error's tail over long
        # runs is far above its value on a few probe sweeps
        ks, errs = autotune.tune_safe_mult(specs, tol=1e-6, precision=prec, confs=confs,
                                           safety=0.005)
        tensor, tc_ratio = None, None
        if prec == _lib.PREC_MIXED:  # tensor-core or double-float products, timed per kind
            tensor, tc_ratio = autotune.tune_tensor(specs, ks=ks, confs=confs)
        tune_s = time.perf_counter() - t
        backoffs, attempts = 0, 0
        while True:
            attempts += 1
            ce = []
            for (model, fcls, beta, dt, s), k in zip(specs, ks):
                param = pkg.DQMCParameters.make(beta=beta, delta_tau=dt, safe_mult=k)
                fld = fcls(param, model)
                ce.append((_lib.ChainConfig(len(model.l), 1, param.slices, k, fld.kind, 1,
                                            fld.alpha, s),
                           pkg.hopping_exponentials(model.hopping_matrix(), dt)))
            r = pkg.run_ensemble(ce, seconds=seconds, quantum_us=100000, precision=prec,
                                 confs=confs, tensor=tensor)
            pe = np.array(r["per_chain_propagation_error"])
            if not np.any(pe > 1e-6) or attempts == 3:
                break
            ks, nb = autotune.back_off(specs, ks, pe, tol=1e-6, precision=prec)
            backoffs += nb
            if nb == 0:
                break
        chosen[name] = ks
        # per (L, beta) class: chains and their mean sweeps/s over the timed run
        # (the load balance of the uneven ensemble: a launch ends with its
        # slowest visit, time slices keep every chain's SM busy meanwhile)
        per_class = {}
        for (model, _f, beta, _dt, _s), sw in zip(specs, r["per_chain"]):
            key = f"L={int(round(len(model.l) ** 0.5))},beta={beta:g}"
            per_class.setdefault(key, []).append(sw / r["wall"])
        out[name + "_per_class_sweeps_per_s"] = {
            k: {"chains": len(v), "mean": float(np.mean(v)), "min": float(np.min(v))}
            for k, v in sorted(per_class.items())}
        out[name] = {"sweeps_per_s": r["sweeps_per_s"],
                     "max_propagation_error": r["max_propagation_error"],
                     "median_chain_propagation_error": float(np.median(pe)),
                     "chains_over_1e-6": int(np.sum(pe > 1e-6)),
                     "safe_mult_histogram": {str(k): ks.count(k) for k in sorted(set(ks))},
                     "autotune_s": tune_s, "backoffs": backoffs, "timed_runs": attempts,
                     "timed_s": r["wall"], "launches": r["launches"]}
        if tensor is not None:
            by_n = {}
            for (model, _f, beta, _dt, _s), on, q in zip(specs, tensor, tc_ratio):
                n = len(model.l)
                if 96 <= n <= 256:
                    by_n.setdefault(f"n={n},beta={beta:g}", {"tensor_products": bool(on),
                                             "double_float_over_tensor_cycles":
                                                 None if q != q else round(q, 3)})
            out[name]["product_choice"] = by_n
    out["unbatched_plain_fp64"] = unbatched_plain(pkg, _lib, specs, chosen["plain_fp64"], confs,
                                                  stream)
    out["mixed_vs_plain"] = out["mixed"]["sweeps_per_s"] / out["plain_fp64"]["sweeps_per_s"]
    out["mixed_vs_unbatched_plain"] = (out["mixed"]["sweeps_per_s"] /
                                       out["unbatched_plain_fp64"]["sweeps_per_s"])
    out["plain_vs_unbatched_plain"] = (out["plain_fp64"]["sweeps_per_s"] /
                                       out["unbatched_plain_fp64"]["sweeps_per_s"])
    return out


def unbatched_plain(pkg, _lib, specs, ks, confs, stream, per_class=2):
    """The same ensemble advanced without batching: each chain alone in its own
    sweep launch (the GPU counterpart of update(::LocalSweep) on one
    simulation at a time), one chain after another, FP64 at its autotuned
    safe_mult.  Bounded sample: per (L, beta) class the first `per_class`
    chains each time one sweep (CUDA events on the launch stream, from its
    thermalised configuration after the stack build); the ensemble's serial
    time is the class means weighted by the class sizes."""
    import torch

    classes = {}
    for j, (model, fcls, beta, dt, s) in enumerate(specs):
        classes.setdefault((len(model.l), beta), []).append(j)
    est, sampled, timed = 0.0, 0, 0.0
    for key in sorted(classes):
        js = classes[key]
        ts = []
        for j in js[:per_class]:
            model, fcls, beta, dt, s = specs[j]
            param = pkg.DQMCParameters.make(beta=beta, delta_tau=dt, safe_mult=ks[j])
            fld = fcls(param, model)
            h = _lib.Handle([_lib.ChainConfig(len(model.l), 1, param.slices, ks[j], fld.kind, 1,
                                              fld.alpha, s)], precision=_lib.PREC_FP64)
            h.set_hopping(0, pkg.hopping_exponentials(model.hopping_matrix(), dt))
            h.init_random_field(0)
            h.set_field(0, confs[j])
            h.set_stream(stream.cuda_stream)
            h.initialize_run()
            h.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            h.sweep_async(1)
            e1.record(stream)
            h.synchronize()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1) / 1e3)
            h.close()
        sampled += len(ts)
        timed += sum(ts)
        est += float(np.mean(ts)) * len(js)
    return {"sweeps_per_s": len(specs) / est, "serial_s_per_ensemble_sweep": est,
            "sample": f"{sampled} of {len(specs)} chains (first {per_class} of each (L, beta) "
                      f"class), one sweep each, one chain per launch, launches back to back",
            "timed_s": timed}


def c1_line(pkg, _lib, stream, nsm, seed=1, sweeps=20):
    """4x4 attractive Hubbard (U_ref = +4), DensityHirschField, beta=4, M=40,
    safe_mult=10, FP64: an ensemble of 16 chains per SM on the one-warp-per-
    chain kernel (and 4 per SM on the CTA kernel for comparison), `sweeps`
    timed sweeps after the stack build and one warm-up sweep."""
    import torch

    model = pkg.HubbardModel(pkg.SquareLattice(4), U=4.0)
    param = pkg.DQMCParameters.make(beta=4.0, delta_tau=0.1, safe_mult=10)
    fld = pkg.DensityHirschField(param, model)
    exps = pkg.hopping_exponentials(model.hopping_matrix(), param.delta_tau)
    n, M = len(model.l), param.slices
    out = {"workload": "4x4 square attractive Hubbard U=4 (reference convention), mu=0, "
                       "DensityHirschField, beta=4, dtau=0.1 (M=40), safe_mult=10, FP64"}

    def one(n_chains, warp):
        h = _lib.Handle([_lib.ChainConfig(n, 1, M, 10, fld.kind, 1, fld.alpha, seed + j)
                         for j in range(n_chains)], precision=_lib.PREC_FP64)
        h.set_small_chain_kernel(warp)
        h.set_hopping(-1, exps)
        h.init_random_field(-1)
        h.set_stream(stream.cuda_stream)
        h.initialize_run()
        h.sweep_async(1)
        h.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        h.sweep_async(sweeps)
        e1.record(stream)
        h.synchronize()
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / 1e3
        pe = max(h.stats(i)["max_propagation_error"] for i in range(n_chains))
        h.close()
        return {"chains": n_chains, "sweeps_per_s": n_chains * sweeps / t,
                "max_propagation_error": pe}

    out["warp_kernel"] = one(16 * nsm, True)
    out["cta_kernel"] = one(4 * nsm, False)
    return out


def c4_line(pkg, _lib, stream, n_chains, seed=4):
    """16x16 repulsive Hubbard U=4 (physics), MagneticHirschField, beta=10,
    M=100, safe_mult=10: an ensemble of n_chains chains, one timed sweep each
    on the FP64 and the mixed path after the stack build; the mixed path's
    max|dG| against FP64 for identical configurations at stabilisation slices
    (calculate_greens from scratch)."""
    import torch

    model = pkg.HubbardModel(pkg.SquareLattice(16), U=-4.0)
    param = pkg.DQMCParameters.make(beta=10.0, delta_tau=0.1, safe_mult=10)
    fld = pkg.MagneticHirschField(param, model)
    exps = pkg.hopping_exponentials(model.hopping_matrix(), param.delta_tau)
    n, M = len(model.l), param.slices
    nr = len(pkg.generate_chunks(M, param.safe_mult))
    out = {"workload": "16x16 square repulsive Hubbard U=4 (physics), mu=0, MagneticHirschField, "
                       f"beta=10, dtau=0.1 (M=100), safe_mult=10, {n_chains} chains, one timed "
                       "sweep per path after the stack build; mixed: tensor-core products "
                       "(tcgen05, 7 BF16 digit slices) for the wraps, slice chains and "
                       "reconstruction"}
    def one(prec, k):
        h = _lib.Handle([_lib.ChainConfig(n, 2, M, k, fld.kind, 1, fld.alpha, seed + j)
                         for j in range(n_chains)], precision=prec)
        h.set_hopping(-1, exps)
        h.init_random_field(-1)
        h.set_stream(stream.cuda_stream)
        h.initialize_run()
        h.synchronize()
        s0 = [h.stats(i) for i in range(n_chains)]
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        h.sweep_async(1)
        e1.record(stream)
        h.synchronize()
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / 1e3
        s1 = [h.stats(i) for i in range(n_chains)]
        acc = sum(b["accepted"] - a["accepted"] for a, b in zip(s0, s1)) / max(
            1, sum(b["proposals"] - a["proposals"] for a, b in zip(s0, s1)))
        pe = [x["max_propagation_error"] for x in s1]
        h.close()
        return {"sweeps_per_s": n_chains / t, "launch_s": t, "safe_mult": k,
                "max_propagation_error": max(pe), "chains_over_1e-6": int(sum(v > 1e-6 for v in pe)),
                "acceptance": acc}

    out["fp64"] = one(_lib.PREC_FP64, 10)
    out["fp64"]["tflops"] = n_chains * sweep_flops(n, 2, M, nr, out["fp64"]["acceptance"]) / \
        out["fp64"]["launch_s"] / 1e12
    out["mixed"] = one(_lib.PREC_MIXED, 10)
    out["mixed_vs_fp64"] = out["mixed"]["sweeps_per_s"] / out["fp64"]["sweeps_per_s"]
    # the largest safe_mult at which every mixed chain's propagation error
    # stays <= 1e-6 over the timed sweep
    strict = out["mixed"] if out["mixed"]["max_propagation_error"] <= 1e-6 else None
    for k in (6, 5, 4, 3):
        if strict is not None:
            break
        r = one(_lib.PREC_MIXED, k)
        if r["max_propagation_error"] <= 1e-6:
            strict = r
    out["mixed_strict_1e-6"] = strict
    if strict is not None:
        out["mixed_strict_vs_fp64"] = strict["sweeps_per_s"] / out["fp64"]["sweeps_per_s"]
    hs = [_lib.Handle([_lib.ChainConfig(n, 2, M, 10, fld.kind, 1, fld.alpha, seed)], precision=pr)
          for pr in (_lib.PREC_FP64, _lib.PREC_MIXED)]
    for hc in hs:
        hc.set_hopping(-1, exps)
        hc.init_random_field(0)
    slices = (0, M // 2, M)
    dG = max(float(np.max(np.abs(hs[0].calculate_greens(0, sl) - hs[1].calculate_greens(0, sl))))
             for sl in slices)
    for hc in hs:
        hc.close()
    out["max_dG_mixed_vs_fp64"] = dG
    out["dG_slices"] = list(slices)
    return out


def served_c5(pkg, _lib, n_requests, wall_s, seed=5, full=False):
    """Served request stream: Poisson arrivals, square or honeycomb, HBM-budget
    admission, device-resident chains, time-sliced launches, mixed precision.
    full=True: the stated distribution (L in {4,6,8,12,16}, honeycomb up to
    n = 512, beta in {2,4,8,12}, 200-2000 sweeps), bounded by wall time;
    otherwise a light-load sample (L in {4,6,8}, beta in {2,4,8}, 20-200
    sweeps)."""
    if full:
        kw = dict(Ls=(4, 6, 8, 12, 16), betas=(2.0, 4.0, 8.0, 12.0), sweeps=(200, 2000))
        desc = "L in {4,6,8,12,16}, beta in {2,4,8,12}, 200-2000 sweeps"
    else:
        kw = dict(Ls=(4, 6, 8), betas=(2.0, 4.0, 8.0), sweeps=(20, 200))
        desc = "L in {4,6,8}, beta in {2,4,8}, 20-200 sweeps"
    budget = 64 << 30
    reqs = pkg.poisson_stream(n_requests, rate=20.0, seed=seed, **kw)
    out = {"workload": f"{n_requests} Poisson requests at 20/s, square|honeycomb, {desc}, "
                       f"U in [-8,8] (physics), mixed precision, {budget >> 30} GiB HBM budget, "
                       f"50 ms time slices, stopped after {wall_s:.0f} s"}
    # 50 ms slices: fewer host round trips than 20 ms (p50 0.57 -> 0.51 s,
    # p99 4.08 -> 3.99 s on the light sample), admission still within a slice
    srv = pkg.Server(max_slots=304, budget_bytes=budget, precision=_lib.PREC_MIXED,
                     quantum_us=50000)
    r = srv.serve(reqs, realtime=True, max_wall=wall_s)
    srv.close()
    drawn = {}
    for q in reqs:
        key = f"{q.lattice}{q.L}"
        drawn[key] = drawn.get(key, 0) + 1
    out.update({"sweeps_per_s": r["sweeps_per_s"], "p50_block_s": r["p50_block_s"],
                "p99_block_s": r["p99_block_s"], "blocks_completed": r["blocks"],
                "finished": len(r["results"]), "unfinished": r["unfinished"],
                "launches": r["launches"], "wall_s": r["wall"],
                "sample": {"lattices": drawn,
                           "beta": {str(b): sum(q.beta == b for q in reqs)
                                    for b in sorted({q.beta for q in reqs})},
                           "sweeps_requested": int(sum(q.sweeps for q in reqs))}})
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c2", choices=sorted(WORKLOADS))
    ap.add_argument("--chains", type=int, default=0, help="ensemble size (default 2 per SM)")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"],
                    help="arithmetic of the timed ensemble (mixed: for profiling that path)")
    ap.add_argument("--cpu-budget", type=float, default=15.0, help="seconds of CPU-baseline work")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the mixed / batched-ensemble / served measurements")
    ap.add_argument("--extra-seconds", type=float, default=6.0)
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    import __graft_entry__ as g
    pkg = g.load_package()

    if args.impl == "reference":
        if rank != 0:
            return
        run_reference(args, pkg, rank)
        return

    import torch

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))

    from montecarlo_gb300 import build as B
    B.build()
    from montecarlo_gb300 import _lib

    props = torch.cuda.get_device_properties(local_rank)
    nsm = props.multi_processor_count
    model, param, fld, exps, desc = setup_workload(pkg, args.workload)
    n, nf, M = len(model.l), fld.unique_flavors, param.slices
    nr = len(pkg.generate_chunks(M, param.safe_mult))
    # resident chains: two per SM (one CTA each); for lattices of n <= 32
    # sites, whose sweeps run one warp per chain (eight per CTA), 16 (n <= 16)
    # or 8 per SM
    B_chains = args.chains or (16 if n <= 16 else 8 if n <= 32 else 2) * nsm

    def configs(base_seed):
        return [_lib.ChainConfig(n, nf, M, param.safe_mult, fld.kind, 1, fld.alpha, base_seed + j)
                for j in range(B_chains)]

    # ---- peak of the FP64 pipe, measured in this run (cuBLAS DGEMM 4096^3)
    a = torch.randn(4096, 4096, device="cuda", dtype=torch.float64)
    bm = torch.randn(4096, 4096, device="cuda", dtype=torch.float64)
    for _ in range(2):
        a @ bm
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        a @ bm
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    fp64_peak = 2 * 4096.0 ** 3 / best / 1e12
    del a, bm
    torch.cuda.empty_cache()

    # ---- device-resident throughput (value)
    from montecarlo_gb300 import replicas

    seed0 = replicas.chain_seeds(rank, B_chains)[0]  # disjoint seeds per rank
    prec_main = _lib.PREC_MIXED if args.precision == "mixed" else _lib.PREC_FP64
    h = _lib.Handle(configs(seed0), precision=prec_main)
    h.set_hopping(-1, exps)
    h.init_random_field(-1)
    # a dedicated stream: the library launches on it and the CUDA events below
    # are recorded on it (the legacy default stream has handle 0)
    stream = torch.cuda.Stream()
    assert stream.cuda_stream != 0
    h.set_stream(stream.cuda_stream)
    h.initialize_run()
    for _ in range(args.warmup):
        h.sweep_async(1)
    h.synchronize()
    st0 = [h.stats(i) for i in range(B_chains)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local_rank)
    clocks.start()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    evs[0].record(stream)
    for i in range(args.steps):
        h.sweep_async(1)
        evs[i + 1].record(stream)
    h.synchronize()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    launch_ms = [evs[i].elapsed_time(evs[i + 1]) for i in range(args.steps)]
    elapsed = evs[0].elapsed_time(evs[-1]) / 1e3
    if dist:
        elapsed = replicas.max_over_ranks(elapsed, dist, device="cuda")
    st1 = [h.stats(i) for i in range(B_chains)]
    acc = sum(s1["accepted"] - s0["accepted"] for s0, s1 in zip(st0, st1)) / max(
        1, sum(s1["proposals"] - s0["proposals"] for s0, s1 in zip(st0, st1)))
    max_prop = max(s["max_propagation_error"] for s in st1)
    value = replicas.aggregate_rate(B_chains * args.steps, world, elapsed)
    flops_launch = B_chains * sweep_flops(n, nf, M, nr, acc)
    avg_launch = statistics.mean(launch_ms) / 1e3
    achieved = flops_launch / avg_launch / 1e12
    h.close()

    # ---- end to end through the C ABI with host buffers
    h2 = _lib.Handle(configs(seed0 + 10_000), precision=prec_main)
    pin = torch.empty(4 * n * n, dtype=torch.float64, pin_memory=True)
    pin_np = pin.numpy().reshape(4, n, n)
    for m in range(4):
        pin_np[m] = np.asarray(exps[m])
    conf_pin = torch.empty(B_chains * n * M, dtype=torch.int8, pin_memory=True).numpy()
    rng = np.random.default_rng(seed0)
    conf_pin[:] = rng.choice(np.array([-1, 1], dtype=np.int8), size=conf_pin.size)
    g_pin = torch.empty(B_chains * nf * n * n, dtype=torch.float64, pin_memory=True).numpy()
    f_pin = torch.empty(B_chains * n * M, dtype=torch.int8, pin_memory=True).numpy()
    h2.set_stream(stream.cuda_stream)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    h2.set_hopping(-1, [pin_np[m].T for m in range(4)])  # symmetric: F-order views, no copy
    h2.set_fields_batch(0, B_chains, conf_pin)
    h2.initialize_run()
    for i in range(args.steps):
        h2.sweep(1)
        h2.greens_batch_into(0, B_chains, g_pin)
        h2.fields_batch_into(0, B_chains, f_pin)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    if dist:
        e2e_s = replicas.max_over_ranks(e2e_s, dist, device="cuda")
    h2.close()
    h2d = (4 * n * n * 8 + B_chains * n * M) / args.steps
    d2h = B_chains * (nf * n * n * 8 + n * M + 0)

    # ---- mixed precision on the same ensemble (double-float slice products)
    extras = {}
    if world == 1 and not args.no_extras:
        from montecarlo_gb300 import autotune

        specs2 = [(model, type(fld), param.beta, param.delta_tau, seed0 + j) for j in range(8)]

        def time_mixed(k):
            cfgs_m = [_lib.ChainConfig(n, nf, M, k, fld.kind, 1, fld.alpha, seed0 + j)
                      for j in range(B_chains)]
            hm = _lib.Handle(cfgs_m, precision=_lib.PREC_MIXED)
            hm.set_hopping(-1, exps)
            hm.init_random_field(-1)
            hm.set_stream(stream.cuda_stream)
            hm.initialize_run()
            for _ in range(args.warmup):
                hm.sweep_async(1)
            hm.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for i in range(args.steps):
                hm.sweep_async(1)
            e1.record(stream)
            hm.synchronize()
            torch.cuda.synchronize()
            v = B_chains * args.steps / (e0.elapsed_time(e1) / 1e3)
            mp = max(hm.stats(i)["max_propagation_error"] for i in range(B_chains))
            hm.close()
            return v, mp

        # the plain path's safe_mult (same stabilisation work), and the largest
        # safe_mult at which every chain's propagation error over the timed
        # sweeps stays <= 1e-6 (the double-float wraps drift ~30-70x faster
        # than FP64 ones between stabilisations)
        k_mixed = param.safe_mult
        mixed_v, mp = time_mixed(k_mixed)
        strict = None
        for k_try in (k_mixed, 8, 6, 5, 4):
            v_try, mp_try = (mixed_v, mp) if k_try == k_mixed else time_mixed(k_try)
            if mp_try <= 1e-6:
                strict = {"safe_mult": k_try, "value": v_try, "vs_plain_fp64": v_try / value,
                          "max_propagation_error": mp_try}
                break
        # |dG| of the mixed path against FP64 for the same field configurations:
        # thermalised configurations of 4 chains, G from scratch at every
        # stabilisation slice, mixed (double-float slice chains) vs FP64
        confs = autotune.thermalize(specs2[:4])
        hcmp = [_lib.Handle([_lib.ChainConfig(n, nf, M, k_mixed, fld.kind, 1, fld.alpha, seed0 + j)
                             for j in range(4)], precision=pr)
                for pr in (_lib.PREC_FP64, _lib.PREC_MIXED)]
        for hc in hcmp:
            hc.set_hopping(-1, exps)
            for j in range(4):
                hc.set_field(j, confs[j])
        bounds = sorted({0, M} | {b for _, b in pkg.generate_chunks(M, k_mixed)})
        dG = max(float(np.max(np.abs(hcmp[0].calculate_greens(j, s) - hcmp[1].calculate_greens(j, s))))
                 for j in range(4) for s in bounds)
        for hc in hcmp:
            hc.close()
        extras["mixed"] = {"value": mixed_v, "unit": "sweeps/s", "vs_plain_fp64": mixed_v / value,
                           "max_dG_vs_fp64_at_stabilisations": dG,
                           "max_propagation_error": mp, "safe_mult": k_mixed,
                           "strict_propagation_error_1e-6": strict,
                           "note": "wraps and slice chains as double-float products on the FP32 "
                                   "pipe, and so are the reconstruction's products; UDT, "
                                   "triangular solves, ratios, rank-1 updates FP64"}
        # the reference's checkerboard = true on the same ensemble: the
        # hopping exponentials as bond-factor products (O(n^2) per factor)
        from montecarlo_gb300 import model as _M
        cbd, cbn = _M.checkerboard_pack(
            _M.checkerboard_exponentials(model.hopping_matrix(), model.l, param.delta_tau))
        hcb = _lib.Handle(configs(seed0), precision=_lib.PREC_FP64)
        hcb.set_hopping(-1, exps)
        hcb.set_checkerboard(-1, cbd, cbn)
        hcb.init_random_field(-1)
        hcb.set_stream(stream.cuda_stream)
        hcb.initialize_run()
        for _ in range(args.warmup):
            hcb.sweep_async(1)
        hcb.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(args.steps):
            hcb.sweep_async(1)
        e1.record(stream)
        hcb.synchronize()
        torch.cuda.synchronize()
        cb_v = B_chains * args.steps / (e0.elapsed_time(e1) / 1e3)
        cb_mp = max(hcb.stats(i)["max_propagation_error"] for i in range(B_chains))
        hcb.close()
        extras["checkerboard"] = {"value": cb_v, "unit": "sweeps/s", "vs_plain_fp64": cb_v / value,
                                  "parts_per_factor": cbn, "max_propagation_error": cb_mp,
                                  "note": "checkerboard = true (FP64): exp(-dtau T) as products of "
                                          "site-disjoint bond factors; Trotter-split physics as in "
                                          "the reference's checkerboard path"}
        # complex chains (the reference's ComplexF64 path): the same lattice,
        # U and chains with the density-channel field, whose alpha is then
        # imaginary; FP64 on the real 2n x 2n representation of G
        cfld = pkg.DensityHirschField(param, model)
        ca = complex(cfld.alpha)
        hcx = _lib.Handle([_lib.ChainConfig(n, 1, M, param.safe_mult, cfld.kind, 1, ca.real,
                                            seed0 + j, ca.imag) for j in range(B_chains)],
                          precision=_lib.PREC_FP64)
        hcx.set_hopping(-1, exps)
        hcx.init_random_field(-1)
        hcx.set_stream(stream.cuda_stream)
        hcx.initialize_run()
        for _ in range(args.warmup):
            hcx.sweep_async(1)
        hcx.synchronize()
        cs0 = [hcx.stats(i) for i in range(B_chains)]
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(args.steps):
            hcx.sweep_async(1)
        e1.record(stream)
        hcx.synchronize()
        torch.cuda.synchronize()
        cx_t = e0.elapsed_time(e1) / 1e3
        cs1 = [hcx.stats(i) for i in range(B_chains)]
        hcx.close()
        props = sum(b["proposals"] - a["proposals"] for a, b in zip(cs0, cs1))
        cx_acc = sum(b["accepted"] - a["accepted"] for a, b in zip(cs0, cs1)) / max(1, props)
        cx_tf = B_chains * args.steps * sweep_flops(2 * n, 1, M, nr, cx_acc) / cx_t / 1e12
        extras["complex"] = {
            "value": B_chains * args.steps / cx_t, "unit": "sweeps/s",
            "vs_plain_fp64": B_chains * args.steps / cx_t / value,
            "representation_tflops": cx_tf, "frac_of_measured_dgemm": cx_tf / fp64_peak,
            "acceptance": cx_acc,
            "imaginary_probability_fraction": sum(
                b["imaginary_probability"] - a["imaginary_probability"]
                for a, b in zip(cs0, cs1)) / max(1, props),
            "max_propagation_error": max(s["max_propagation_error"] for s in cs1),
            "note": "DensityHirschField at repulsive U (complex alpha, the reference's "
                    "ComplexF64 path), same 8x8 lattice, chains and safe_mult; one flavour "
                    "block of the real 2n x 2n representation (n = 128): 4x the plain "
                    "chain's flops per sweep"}
        extras["batched"] = ensemble_c3(pkg, _lib, 256, args.extra_seconds, stream)
        extras["served"] = served_c5(pkg, _lib, 48, 5 * args.extra_seconds)
        extras["served_full"] = served_c5(pkg, _lib, 48, 10 * args.extra_seconds, full=True)
        extras["c4"] = c4_line(pkg, _lib, stream, 2 * nsm)
        extras["c1"] = c1_line(pkg, _lib, stream, nsm)
        # the headline ratios of the metric, lifted to the top level
        b = extras["batched"]
        extras["c3_mixed_sweeps_per_s"] = b["mixed"]["sweeps_per_s"]
        extras["c3_plain_fp64_sweeps_per_s"] = b["plain_fp64"]["sweeps_per_s"]
        extras["c3_unbatched_plain_fp64_sweeps_per_s"] = b["unbatched_plain_fp64"]["sweeps_per_s"]
        extras["mixed_vs_plain"] = b["mixed_vs_plain"]
        extras["mixed_vs_unbatched_plain"] = b["mixed_vs_unbatched_plain"]
        extras["c3_chains_over_1e-6"] = {"plain_fp64": b["plain_fp64"]["chains_over_1e-6"],
                                         "mixed": b["mixed"]["chains_over_1e-6"]}
        extras["served_p50_p99_block_s"] = [extras["served"]["p50_block_s"],
                                            extras["served"]["p99_block_s"]]

    # DRAM traffic of the chain kernel from the committed ncu capture, scaled
    # by chains (independent per-chain workspaces)
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "chain_kernel_traffic.json")
    if os.path.exists(tpath):
        tr = json.load(open(tpath))
        if tr.get("workload") == args.workload:
            traffic = tr["dram_bytes_per_launch"] * B_chains / tr["chains_captured"]

    chain_bytes = int(_lib.load().dqmc_chain_bytes(_lib.ChainConfig(
        n, nf, M, param.safe_mult, fld.kind, 1, fld.alpha, 0), 0))
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline_sample(pkg, args.workload, args.cpu_budget)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "sweeps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision == "fp64" else "f64+df32",
            "data": "synthetic (seeded random Hubbard-Stratonovich fields)",
            "config": {"workload": desc,
                       "path": ("plain FP64" if args.precision == "fp64" else "mixed") +
                               " (value); mixed, batched, served below",
                       "chains_per_gpu": B_chains, "parallelism": f"replicas{world}",
                       "l2": ("working set larger than L2 (no flush needed)"
                              if B_chains * chain_bytes > L2_BYTES else
                              "working set fits in L2 (not flushed: every sweep re-reads each "
                              "chain's state many times within the launch)"),
                       "chain_bytes": chain_bytes},
            "e2e": {"value": world * B_chains * args.steps / e2e_s, "unit": "sweeps/s",
                    "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "includes": "hopping + field upload, stack build, sweeps, per-sweep download "
                                "of every chain's G and field"},
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": fp64_peak,
                         "unit": "TFLOP/s", "frac": achieved / fp64_peak, "traffic": traffic,
                         "traffic_unit": "bytes per launch (ncu dram read+write)",
                         "peak_source": "cuBLAS DGEMM 4096^3 measured in this run (FP64 pipe; "
                                        "MEASURED_PEAKS.json has no FP64 figure)",
                         "kernel": "dqmc::chain_kernel",
                         "flops_per_launch": flops_launch,
                         "avg_launch_ms": 1e3 * avg_launch},
            "gpu_launches": args.steps,
            "acceptance": acc, "max_propagation_error": max_prop,
            "clocks": clk,
        }
        line.update(extras)
        if cpu is not None:
            line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
