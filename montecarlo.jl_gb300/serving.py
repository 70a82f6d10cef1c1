"""Continuous batching of DQMC simulations on one GPU (serving and ensembles).

A stream of simulation requests -- lattice, L, U, beta, number of sweeps,
seed -- is served from one device pool (``_lib.Pool``): requests are admitted
as slots and HBM budget free up, every admitted chain keeps its G, UDT stack
and field on the device, and each launch is a time slice in which every chain
advances by as many slice visits as fit (``dqmc_pool_run``).  Requests that
arrive while others run join at the next slice; finished ones leave.  Each
request's trajectory is independent of its neighbours: a request gives the
same field configuration and Green's function alone and in the mix.

Latency is reported per 10-sweep block of a request: the time from the end
of its previous block (or its admission) to the end of the block.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import _lib
from .lattices import Honeycomb, SquareLattice
from .model import DQMCParameters, HubbardModel, hopping_exponentials

BLOCK = 10  # sweeps per latency block


@dataclass
class Request:
    """A simulation request.  ``U`` is in the physics convention (U > 0
    repulsive); the reference's convention is U_ref = -U."""

    rid: int
    lattice: str
    L: int
    U: float
    beta: float
    sweeps: int
    seed: int
    arrival: float = 0.0
    delta_tau: float = 0.1
    safe_mult: int = 10

    def model(self):
        lat = SquareLattice(self.L) if self.lattice == "square" else Honeycomb(self.L)
        U_ref = -self.U
        mu = 0.0
        return HubbardModel(lat, U=U_ref, mu=mu)


@dataclass
class Result:
    rid: int
    conf: np.ndarray
    greens: np.ndarray
    stats: dict
    admitted: float
    finished: float
    block_latencies: List[float] = field(default_factory=list)
    # a chain that reported a nonzero status (non-finite G, a partner CTA
    # that stopped answering, ...): the error text; its conf / greens are
    # the state it stopped in
    error: Optional[str] = None


def request_config(req: Request, precision=None, tol=None):
    """Chain configuration and hopping exponentials of a request.  With a
    propagation-error bound ``tol``, a safe_mult the autotuner already chose
    for this kind of chain (same sites, slices, |U|, mu, field, precision and
    bound) replaces the request's own."""
    model = req.model()
    k = req.safe_mult
    if tol is not None and precision is not None:
        from . import autotune
        hit = autotune.cached(model, model.choose_field(), req.beta, req.delta_tau,
                              precision=precision, tol=tol)
        if hit is not None:
            k = hit
    param = DQMCParameters.make(beta=req.beta, delta_tau=req.delta_tau, safe_mult=k)
    fld = model.choose_field()(param, model)
    cfg = _lib.ChainConfig(len(model.l), fld.unique_flavors, param.slices, param.safe_mult,
                           fld.kind, 1, fld.alpha, req.seed)
    exps = hopping_exponentials(model.hopping_matrix(), param.delta_tau)
    return cfg, exps


def poisson_stream(n, rate, seed, lattices=("square", "honeycomb"), Ls=(4, 6, 8, 12, 16),
                   betas=(2.0, 4.0, 8.0, 12.0), sweeps=(200, 2000), U=(-8.0, 8.0)):
    """Seeded Poisson arrivals at `rate` requests/s with uniformly drawn
    lattice, L, U, beta and sweep count."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=n))
    out = []
    for i in range(n):
        out.append(Request(i, str(rng.choice(lattices)), int(rng.choice(Ls)),
                           float(rng.uniform(*U)), float(rng.choice(betas)),
                           int(rng.integers(sweeps[0], sweeps[1] + 1)), int(seed * 100003 + i),
                           float(t[i])))
    return out


class Server:
    """Serves requests from one pool with time-sliced launches.  ``tol``: a
    propagation-error bound under which requests of kinds the autotuner has
    seen run at its safe_mult; ``flavour_split``: two-flavour requests of 48
    sites or more run their flavour blocks on two SMs (bit-identical
    results)."""

    def __init__(self, max_slots=304, budget_bytes=8 << 30, precision=_lib.PREC_FP64,
                 quantum_us=50000, use_graph=True, device=0, tol=None, flavour_split=True):
        self.pool = _lib.Pool(max_slots, budget_bytes, precision=precision, device=device)
        # two-flavour requests run their flavour blocks on two SMs (same results)
        self.pool.set_flavour_split(flavour_split)
        self.quantum_us = quantum_us
        self.use_graph = use_graph
        self.precision = precision
        # propagation-error bound: requests of kinds the autotuner has seen
        # run at its safe_mult (autotune's cache)
        self.tol = tol

    def close(self):
        self.pool.close()

    def serve(self, requests: List[Request], realtime: bool = True, max_wall: float = None):
        pending = sorted(requests, key=lambda r: r.arrival)
        queue: List[Request] = []
        active = {}  # slot -> (req, admitted_time, last_block_time, blocks_done, latencies)
        results = {}
        configs = {}  # rid -> (chain config, hopping exponentials), built once per request
        t0 = time.perf_counter()
        launches = 0
        total_sweeps = 0
        failed = 0
        while pending or queue or active:
            now = time.perf_counter() - t0
            if max_wall is not None and now > max_wall:
                break
            while pending and (not realtime or pending[0].arrival <= now):
                queue.append(pending.pop(0))
            # admission: every queued request that fits the slots and budget
            still = []
            for req in queue:
                if req.rid not in configs:
                    configs[req.rid] = request_config(req, self.precision, self.tol)
                cfg, exps = configs[req.rid]
                slot = self.pool.admit(cfg)
                if slot is None:
                    still.append(req)
                    continue
                self.pool.set_hopping(slot, exps)
                self.pool.init_random_field(slot)
                self.pool.set_quota(slot, req.sweeps)
                del configs[req.rid]
                t_adm = time.perf_counter() - t0
                active[slot] = [req, t_adm, t_adm, 0, []]
            queue = still
            if not active:
                if pending and realtime:
                    time.sleep(max(0.0, pending[0].arrival - (time.perf_counter() - t0)))
                continue
            try:
                self.pool.run(self.quantum_us, self.use_graph)
            except _lib.DQMCError as err:
                # a chain that reported a nonzero status fails its request
                # alone: release it and keep serving the others (the slice's
                # work of every other chain is kept); anything else is raised
                if err.code != _lib.DQMC_ERR_NUMERICAL:
                    raise
                bad = [sl for sl in active if self.pool.stats(sl)["status"] != 0]
                if not bad:
                    raise
                tnow = time.perf_counter() - t0
                for sl in bad:
                    req, t_adm, _tl, _nb, lats = active.pop(sl)
                    results[req.rid] = Result(req.rid, self.pool.get_field(sl),
                                              self.pool.greens(sl), self.pool.stats(sl),
                                              t_adm, tnow, lats, error=str(err))
                    failed += 1
                    self.pool.release(sl)
            launches += 1
            tnow = time.perf_counter() - t0
            for slot in list(active):
                req, t_adm, t_last, blocks, lats = active[slot]
                done, left, _ = self.pool.slot(slot)
                nb = min(done, req.sweeps) // BLOCK
                if nb > blocks:
                    # blocks completed in this slice share its end time
                    per = (tnow - t_last) / (nb - blocks)
                    lats.extend([per] * (nb - blocks))
                    active[slot][2] = tnow
                    active[slot][3] = nb
                if left == 0:
                    total_sweeps += req.sweeps
                    results[req.rid] = Result(req.rid, self.pool.get_field(slot),
                                              self.pool.greens(slot), self.pool.stats(slot),
                                              t_adm, tnow, lats)
                    self.pool.release(slot)
                    del active[slot]
        wall = time.perf_counter() - t0
        # sweeps of requests still running at a wall-clock stop count too
        for slot, (req, *_rest) in active.items():
            total_sweeps += self.pool.slot(slot)[0]
        # block latencies of finished requests and of the blocks that requests
        # still running at a wall-clock stop completed
        lat = [x for r in results.values() for x in r.block_latencies]
        lat += [x for (_req, _ta, _tl, _nb, lats) in active.values() for x in lats]
        return dict(results=results, wall=wall, launches=launches, sweeps=total_sweeps,
                    blocks=len(lat),
                    sweeps_per_s=total_sweeps / wall if wall > 0 else math.nan,
                    p50_block_s=float(np.percentile(lat, 50)) if lat else None,
                    p99_block_s=float(np.percentile(lat, 99)) if lat else None,
                    unfinished=len(active) + len(queue) + len(pending), failed=failed)


def run_ensemble(configs_and_exps, seconds: float, quantum_us=50000, precision=_lib.PREC_FP64,
                 use_graph=True, device=0, budget_bytes=None, confs=None, tensor=None):
    """Advance an uneven ensemble of chains for about `seconds` of device time
    in time-sliced launches; returns aggregate sweeps/s and per-chain sweeps.
    ``confs`` (optional): starting field configurations (e.g. thermalised
    ones) in place of the seeded random ones; the streams stay seeded.
    ``tensor`` (optional, mixed precision): per chain, tensor-core products
    on or off (``autotune.tune_tensor``)."""
    nbytes = sum(_lib.chain_bytes(c, precision) + 4096 for c, _ in configs_and_exps)
    pool = _lib.Pool(len(configs_and_exps), budget_bytes or nbytes, precision=precision,
                     device=device)
    slots = []
    for j, (cfg, exps) in enumerate(configs_and_exps):
        s = pool.admit(cfg)
        if s is None:
            raise RuntimeError("ensemble does not fit the pool budget")
        pool.set_hopping(s, exps)
        pool.init_random_field(s)
        if confs is not None:
            pool.set_field(s, confs[j])
        if tensor is not None:
            pool.set_tensor_products(bool(tensor[j]), chain=s)
        pool.set_quota(s, 1 << 40)
        slots.append(s)
    pool.run(quantum_us, use_graph)  # stack builds + warm-up slice
    visits0 = [pool.stats(s) for s in slots]
    t0 = time.perf_counter()
    launches = 0
    while time.perf_counter() - t0 < seconds:
        pool.run(quantum_us, use_graph)
        launches += 1
    wall = time.perf_counter() - t0
    sweeps = []
    for s, (cfg, _), st0 in zip(slots, configs_and_exps, visits0):
        st1 = pool.stats(s)
        props = st1["proposals"] - st0["proposals"]
        sweeps.append(props / (2.0 * cfg.slices * cfg.n_sites))
    per_err = [pool.stats(s)["max_propagation_error"] for s in slots]
    maxprop = max(per_err)
    pool.close()
    return dict(wall=wall, launches=launches, sweeps=float(sum(sweeps)),
                sweeps_per_s=float(sum(sweeps)) / wall, per_chain=sweeps,
                max_propagation_error=maxprop, per_chain_propagation_error=per_err)
