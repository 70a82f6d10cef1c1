"""Autotuner of safe_mult (the stabilisation interval) per chain.

The reference takes safe_mult from the user (parameters.jl:90) and reports a
propagation error above 1e-7 as an instability (stack.jl:644-653).  For an
ensemble of uneven chains (different L, U, beta) one safe_mult is either
wasteful (weak coupling, short beta) or unstable (strong coupling, long
beta).  The tuner picks per chain the largest safe_mult whose propagation
error stays below ``safety * tol`` on *thermalised* configurations (random
initial fields are far better conditioned than equilibrium ones, so probes
from them overestimate the stable interval):

1. thermalise every chain for a few sweeps at a conservative interval (FP64);
2. restart probe chains from those configurations at every candidate interval
   -- all chains x candidates in one batched launch -- and measure the largest
   propagation error over a few sweeps;
3. keep the largest candidate under the bound (the smallest one if none is).

Choices are cached per process by (sites, flavours, slices, |U|, mu, field,
precision, bound), so a server that admits a chain of an already tuned kind
reuses the choice without probing, and ``back_off`` lowers the interval of
chains whose propagation error exceeded the bound over a longer run (the
error's tail over many sweeps lies above its value on a few probe sweeps) and
records the lowered choice.

``tune_tensor`` chooses, per kind of mixed-precision chain with
96 <= n <= 256, between the tensor-core split-precision products and the
double-float FP32-pipe products by timing both on the device (the per-chain
phase timers of one probe launch, both variants side by side), cached by
(sites, flavours, slices, field).
"""
from __future__ import annotations

import numpy as np

from . import _lib
from .model import DQMCParameters, hopping_exponentials

CANDIDATES = (2, 3, 4, 5, 6, 8, 10, 12, 15)

# (n, nf, slices, |U|, mu, field kind, precision, bound) -> safe_mult
_CACHE = {}


def cache_key(model, field_cls, beta, delta_tau, precision, tol):
    param = DQMCParameters.make(beta=beta, delta_tau=delta_tau)
    fld = field_cls(param, model)
    return (len(model.l), fld.unique_flavors, param.slices, round(abs(float(model.U)), 9),
            round(float(model.mu), 9), fld.kind, int(precision), float(tol))


def cached(model, field_cls, beta, delta_tau, precision=_lib.PREC_FP64, tol=1e-6):
    """The cached safe_mult of this kind of chain, or None."""
    return _CACHE.get(cache_key(model, field_cls, beta, delta_tau, precision, tol))


def lower(k):
    """The next smaller candidate interval (2 stays 2)."""
    smaller = [c for c in CANDIDATES if c < k]
    return max(smaller) if smaller else min(CANDIDATES)


def back_off(specs, ks, errors, tol=1e-6, precision=_lib.PREC_FP64):
    """Lower the interval of every chain whose measured propagation error
    exceeds `tol`; returns the new choices and the number lowered."""
    out, n = list(ks), 0
    for j, (m, f, b, dt, s) in enumerate(specs):
        if errors[j] > tol and out[j] > min(CANDIDATES):
            out[j] = lower(out[j])
            _CACHE[cache_key(m, f, b, dt, precision, tol)] = out[j]
            n += 1
    return out, n


def _cfg(model, field_cls, beta, delta_tau, k, seed):
    param = DQMCParameters.make(beta=beta, delta_tau=delta_tau, safe_mult=k)
    fld = field_cls(param, model)
    k = min(k, param.slices)
    return _lib.ChainConfig(len(model.l), fld.unique_flavors, param.slices, k, fld.kind, 1,
                            fld.alpha, seed)


def thermalize(specs, sweeps=6, safe_mult=4, device=0):
    """Field configurations of `specs` ((model, field_cls, beta, delta_tau,
    seed) tuples) after `sweeps` FP64 sweeps at `safe_mult`."""
    cfgs = [_cfg(m, f, b, dt, safe_mult, s) for m, f, b, dt, s in specs]
    h = _lib.Handle(cfgs, precision=_lib.PREC_FP64, device=device)
    for j, (m, f, b, dt, s) in enumerate(specs):
        h.set_hopping(j, hopping_exponentials(m.hopping_matrix(), dt))
    h.init_random_field(-1)
    h.initialize_run()
    h.sweep(sweeps)
    confs = [h.get_field(j) for j in range(len(specs))]
    h.close()
    return confs


def tune_safe_mult(specs, tol=1e-6, precision=_lib.PREC_FP64, candidates=CANDIDATES,
                   confs=None, therm_sweeps=6, probe_sweeps=3, safety=0.1, device=0,
                   use_cache=True):
    """Chosen safe_mult per spec and the propagation error measured with it
    (NaN for a choice taken from the cache)."""
    keys = [cache_key(m, f, b, dt, precision, tol) for m, f, b, dt, s in specs]
    todo = [j for j, k in enumerate(keys) if not (use_cache and k in _CACHE)]
    if not todo:
        return [_CACHE[k] for k in keys], [float("nan")] * len(specs)
    if confs is None:
        confs = thermalize(specs, sweeps=therm_sweeps, device=device)
    cfgs, owner, ks = [], [], []
    for j in todo:
        m, f, b, dt, s = specs[j]
        M = DQMCParameters.make(beta=b, delta_tau=dt).slices
        for k in sorted({min(k, M) for k in candidates}):
            cfgs.append(_cfg(m, f, b, dt, k, s))
            owner.append(j)
            ks.append(k)
    h = _lib.Handle(cfgs, precision=precision, device=device)
    for r, j in enumerate(owner):
        m, f, b, dt, s = specs[j]
        h.set_hopping(r, hopping_exponentials(m.hopping_matrix(), dt))
        h.init_random_field(r)  # seeds the stream; the field is replaced next
        h.set_field(r, confs[j])
    h.initialize_run()
    st = h.sweep(probe_sweeps)
    h.close()
    errs = {j: dict() for j in todo}
    for r, j in enumerate(owner):
        errs[j][ks[r]] = st[r]["max_propagation_error"]
    chosen, err_at = [], []
    bound = safety * tol
    for j, key in enumerate(keys):
        if j not in errs:
            chosen.append(_CACHE[key])
            err_at.append(float("nan"))
            continue
        e = errs[j]
        ok = [k for k, v in e.items() if v <= bound]
        k = max(ok) if ok else min(e)
        _CACHE[key] = k
        chosen.append(k)
        err_at.append(e[k])
    return chosen, err_at


# (n, nf, slices, field kind) -> tensor products faster (True / False)
_TC_CACHE = {}


def tensor_key(model, field_cls, beta, delta_tau):
    param = DQMCParameters.make(beta=beta, delta_tau=delta_tau)
    fld = field_cls(param, model)
    return (len(model.l), fld.unique_flavors, param.slices, fld.kind)


def tune_tensor(specs, ks=None, confs=None, sweeps=1, device=0, use_cache=True):
    """Per spec: True when its chain sweeps faster with the tensor-core
    products than with the double-float products (mixed precision; always
    False outside 96 <= n <= 256), and the probe's cycle ratio (NaN for a
    cached or ineligible kind).  `ks`: the specs' safe_mult (default 10)."""
    keys = [tensor_key(m, f, b, dt) for m, f, b, dt, s in specs]
    ratio = [float("nan")] * len(specs)
    todo = {}
    for j, (m, f, b, dt, s) in enumerate(specs):
        n = len(m.l)
        if not (96 <= n <= 256) or (use_cache and keys[j] in _TC_CACHE):
            continue
        todo.setdefault(keys[j], j)
    if todo:
        cfgs, owner = [], []
        for key, j in todo.items():
            m, f, b, dt, s = specs[j]
            k = 10 if ks is None else ks[j]
            for tc in (True, False):
                cfgs.append(_cfg(m, f, b, dt, k, s))
                owner.append((key, j, tc))
        h = _lib.Handle(cfgs, precision=_lib.PREC_MIXED, device=device)
        for r, (key, j, tc) in enumerate(owner):
            m, f, b, dt, s = specs[j]
            h.set_hopping(r, hopping_exponentials(m.hopping_matrix(), dt))
            h.init_random_field(r)
            if confs is not None:
                h.set_field(r, confs[j])
            h.set_tensor_products(tc, chain=r)
        h.initialize_run()
        t0 = [sum(h.timers(r).values()) for r in range(len(cfgs))]
        h.sweep(sweeps)
        cyc = [sum(h.timers(r).values()) - t0[r] for r in range(len(cfgs))]
        h.close()
        per = {}
        for r, (key, j, tc) in enumerate(owner):
            per.setdefault(key, {})[tc] = cyc[r]
        for key, d in per.items():
            _TC_CACHE[key] = d[True] < d[False]
            for jj, kk in enumerate(keys):
                if kk == key:
                    ratio[jj] = d[False] / d[True] if d[True] > 0 else float("nan")
    choice = []
    for j, (m, f, b, dt, s) in enumerate(specs):
        n = len(m.l)
        choice.append(bool(96 <= n <= 256 and _TC_CACHE.get(keys[j], True)))
    return choice, ratio
