"""Replica exchange (parallel tempering) between chains on one GPU.

The reference exchanges configurations between simulations running on
separate Distributed.jl workers (ReplicaExchange, src/flavors/DQMC/updates/
parallel_updates.jl:116-150: wait for the partner, pull its configuration,
swap weights and one uniform, accept with the lower worker id's uniform).
Here every replica is a chain of one handle: an exchange is two launches of
``dqmc_replica_exchange`` and no process or message is involved.  Replicas
are exchanged with their neighbours in the given order, alternating the
even pairs (0,1), (2,3), ... and the odd pairs (1,2), (3,4), ...
"""
from __future__ import annotations

import numpy as np

from . import _lib
from .model import DQMCParameters, hopping_exponentials


def neighbour_partners(n: int, odd: bool) -> np.ndarray:
    """partner[i] for one round of neighbour exchanges (-1: sits out)."""
    p = np.full(n, -1, dtype=np.int32)
    for a in range(1 if odd else 0, n - 1, 2):
        p[a], p[a + 1] = a + 1, a
    return p


def run_tempering(replicas, rounds: int, sweeps_per_round: int = 1, thermalization: int = 0,
                  precision: int = _lib.PREC_FP64, measure_rate: int = 1, device: int = 0):
    """Run ``replicas`` = [(model, beta, delta_tau, safe_mult, seed), ...]
    (equal lattice size, slice count and field kind; U, mu, t may differ) for
    ``rounds`` rounds of ``sweeps_per_round`` sweeps followed by one exchange
    round.  Returns exchange acceptance per neighbour pair, the final
    configurations and the on-device observables of every replica."""
    cfgs, exps, models = [], [], []
    for model, beta, dt, k, seed in replicas:
        p = DQMCParameters.make(beta=beta, delta_tau=dt, safe_mult=k)
        fld = model.choose_field()(p, model)
        cfgs.append(_lib.ChainConfig(len(model.l), fld.unique_flavors, p.slices, k, fld.kind, 1,
                                     fld.alpha, seed))
        exps.append(hopping_exponentials(model.hopping_matrix(), dt))
        models.append(model)
    if len({(c.n_sites, c.n_flavors, c.slices, c.field) for c in cfgs}) != 1:
        raise ValueError("replicas need the same lattice size, slice count and field kind")
    h = _lib.Handle(cfgs, precision=precision, device=device)
    try:
        for j, e in enumerate(exps):
            h.set_hopping(j, e)
        h.init_random_field(-1)
        h.initialize_run()
        if thermalization:
            h.sweep(thermalization)
        for j, m in enumerate(models):
            pos = m.l.positions()
            ph = pos @ np.full(pos.shape[1], np.pi)
            h.set_measurements(j, enable=True, rate=measure_rate, sweep=0, U=m.U,
                               q=(np.cos(ph), np.sin(ph)))
        n = len(cfgs)
        tried = np.zeros(max(n - 1, 0), dtype=np.int64)
        accepted = np.zeros(max(n - 1, 0), dtype=np.int64)
        for r in range(rounds):
            h.sweep(sweeps_per_round)
            partners = neighbour_partners(n, odd=bool(r % 2))
            acc = h.replica_exchange(partners)
            for a in range(n - 1):
                if partners[a] == a + 1:
                    tried[a] += 1
                    accepted[a] += int(acc[a])
        return {"exchange_acceptance": (accepted / np.maximum(tried, 1)).tolist(),
                "exchanges_tried": tried.tolist(),
                "confs": [h.get_field(j) for j in range(n)],
                "observables": [h.measurements(j) for j in range(n)],
                "global_stats": [h.global_stats(j) for j in range(n)]}
    finally:
        h.close()
