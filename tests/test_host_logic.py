"""Host-side logic without a GPU: the autotuner's cache, back-off and
safe_mult choice (on a fake device), the serving path's reuse of cached
choices and its bookkeeping (on a fake pool), run!'s measurement and
recording schedule (on a fake handle), the replica-exchange pairing, and the
by-distance slots of the time-displaced measurements (the reference's
EachSitePairByDistance)."""
import numpy as np
import pytest


def test_autotune_back_off_and_cache(pkg):
    from montecarlo_gb300 import autotune, _lib
    m = pkg.HubbardModel(pkg.SquareLattice(6), U=5.5)
    spec = [(m, m.choose_field(), 8.0, 0.1, 1)]
    key = autotune.cache_key(m, m.choose_field(), 8.0, 0.1, _lib.PREC_MIXED, 1e-6)
    autotune._CACHE.pop(key, None)
    assert autotune.cached(m, m.choose_field(), 8.0, 0.1, _lib.PREC_MIXED, 1e-6) is None
    ks, nb = autotune.back_off(spec, [10], [2e-6], tol=1e-6, precision=_lib.PREC_MIXED)
    assert ks == [8] and nb == 1
    assert autotune.cached(m, m.choose_field(), 8.0, 0.1, _lib.PREC_MIXED, 1e-6) == 8
    # under the bound: unchanged
    assert autotune.back_off(spec, [8], [5e-7], tol=1e-6, precision=_lib.PREC_MIXED) == ([8], 0)
    assert autotune.lower(2) == 2 and autotune.lower(15) == 12
    # a cached kind skips the probes entirely (no device needed)
    ks, errs = autotune.tune_safe_mult(spec, tol=1e-6, precision=_lib.PREC_MIXED)
    assert ks == [8] and np.isnan(errs[0])
    autotune._CACHE.pop(key, None)


def test_serving_reuses_cached_safe_mult(pkg):
    from montecarlo_gb300 import autotune, serving, _lib
    req = serving.Request(0, "square", 6, -4.0, 4.0, 100, 7)  # physics U = -4: U_ref = 4
    m = req.model()
    key = autotune.cache_key(m, m.choose_field(), 4.0, 0.1, _lib.PREC_MIXED, 1e-6)
    autotune._CACHE[key] = 5
    cfg, _ = serving.request_config(req, _lib.PREC_MIXED, 1e-6)
    assert cfg.safe_mult == 5
    cfg, _ = serving.request_config(req)  # no bound: the request's own
    assert cfg.safe_mult == req.safe_mult
    autotune._CACHE.pop(key, None)


def _brute_slots(lat):
    """Slot of (src, trg): Bravais shift of trg's cell from src's, per
    dimension mod L, flattened like _sub2ind, plus the basis pair."""
    nb, B = lat.n_bravais(), len(lat.unitcell.sites)
    n = nb * B
    out = np.zeros((n, n), dtype=int)
    for src in range(n):
        for trg in range(n):
            b1, i1 = divmod(src, nb)
            b2, i2 = divmod(trg, nb)
            shift, stride, r1, r2 = 0, 1, i1, i2
            for L in lat.Ls:
                shift += ((r2 % L - r1 % L) % L) * stride
                stride *= L
                r1 //= L
                r2 //= L
            out[src, trg] = shift + nb * (b1 + B * b2)
    return out


def test_pair_distance_index(pkg):
    for lat in (pkg.SquareLattice(4), pkg.Honeycomb(3), pkg.Chain(5), pkg.CubicLattice(2)):
        P = lat.pair_distance_index()
        assert np.array_equal(P, _brute_slots(lat))
        # every slot of a Bravais shift and basis pair holds one pair per cell
        counts = np.bincount(P.ravel())
        assert np.all(counts == lat.n_bravais())


def test_by_distance_sums_translation_invariant_correlation(pkg):
    lat = pkg.SquareLattice(4)
    P = lat.pair_distance_index()
    rng = np.random.default_rng(3)
    f = rng.normal(size=P.max() + 1)
    C = f[P]  # a correlation that depends on the displacement only
    bd = pkg.by_distance(C, P, P.max() + 1)
    assert np.allclose(bd, f)  # sum over n pairs / n sites


def test_td_arrays_square(pkg):
    m = pkg.HubbardModel(pkg.SquareLattice(4), U=-4.0)
    a = pkg.td_arrays(m)
    n = len(m.l)
    assert a["n_slots"] == 16 and a["pair_slot"].shape == (n * n,)
    assert a["n_form"] == [64, 64]  # directed nearest-neighbour bonds
    assert a["n_current"] == 32     # bonds along +x, two entries each
    assert np.allclose(a["q_cos"] ** 2 + a["q_sin"] ** 2, 1.0)


def test_tensor_choice_cache_and_range(pkg):
    """tune_tensor: kinds outside 96 <= n <= 256 never use the tensor-core
    products; a cached kind is answered without a device probe."""
    from montecarlo_gb300 import autotune
    small = pkg.HubbardModel(pkg.SquareLattice(8), U=4.0)    # n = 64
    big = pkg.HubbardModel(pkg.SquareLattice(10), U=4.0)     # n = 100
    specs = [(small, small.choose_field(), 4.0, 0.1, 1), (big, big.choose_field(), 4.0, 0.1, 2)]
    key = autotune.tensor_key(big, big.choose_field(), 4.0, 0.1)
    autotune._TC_CACHE[key] = False
    choice, ratio = autotune.tune_tensor(specs)
    assert choice == [False, False] and all(r != r for r in ratio)
    autotune._TC_CACHE[key] = True
    assert autotune.tune_tensor(specs)[0] == [False, True]
    autotune._TC_CACHE.pop(key, None)


def _uniform_bits(w):
    """numpy mirror of the device's uniform_bits: the IEEE bits of
    (w >> 11) * 2^-53 assembled with integer operations."""
    m = (w >> np.uint64(11)).astype(np.uint64)
    out = np.zeros_like(m)
    nz = m != 0
    mm = m[nz]
    # leading zeros of a 64-bit value (m < 2^53: at least 11)
    lz = np.full(mm.shape, 64, dtype=np.int64)
    for b in range(63, -1, -1):
        hit = ((mm >> np.uint64(b)) & np.uint64(1)).astype(bool) & (lz == 64)
        lz[hit] = 63 - b
    sh = (lz - 11).astype(np.uint64)
    mant = (mm << sh) & np.uint64((1 << 52) - 1)
    out[nz] = ((np.uint64(1022) - sh) << np.uint64(52)) | mant
    return out


def test_uniform_bits_equal_the_double_formula():
    """The decision loop builds the uniform (w >> 11) 2^-53 on the integer
    pipe; the bits equal those of the floating-point formula for random words
    and for the extremes (m = 0, 1, 2^52, 2^53 - 1)."""
    rng = np.random.default_rng(11)
    w = rng.integers(0, 2 ** 63, size=20000, dtype=np.int64).astype(np.uint64) * np.uint64(2)
    w = np.concatenate([w, np.array([0, 1 << 11, 1 << 63, 0xFFFFFFFFFFFFFFFF, (1 << 52) << 11],
                                    dtype=np.uint64)])
    ref = ((w >> np.uint64(11)).astype(np.float64) * 2.0 ** -53).view(np.uint64)
    assert np.array_equal(_uniform_bits(w), ref)
    # ordering of non-negative doubles by their bits: the comparisons u < p
    p = rng.random(5000)
    u = rng.random(5000)
    assert np.array_equal(u.view(np.int64) < p.view(np.int64), u < p)


class _FakePool:
    """Host-side stand-in for _lib.Pool: `slots` slots, every admitted chain
    advances `per_run` sweeps per time slice."""

    def __init__(self, slots, per_run):
        self.slots, self.per_run = slots, per_run
        self.quota, self.done, self.runs, self.split = {}, {}, 0, None

    def set_flavour_split(self, on):
        self.split = on

    def admit(self, cfg):
        free = [s for s in range(self.slots) if s not in self.quota]
        if not free:
            return None
        self.quota[free[0]], self.done[free[0]] = 0, 0
        return free[0]

    def set_hopping(self, slot, exps):
        assert slot in self.quota

    def init_random_field(self, slot):
        assert slot in self.quota

    def set_quota(self, slot, n):
        self.quota[slot] = n

    def run(self, quantum_us, use_graph):
        self.runs += 1
        for s in self.quota:
            self.done[s] = min(self.quota[s], self.done[s] + self.per_run)

    def slot(self, slot):
        return self.done[slot], self.quota[slot] - self.done[slot], True

    def get_field(self, slot):
        return np.zeros(1, dtype=np.int8)

    def greens(self, slot):
        return np.zeros(1)

    def stats(self, slot):
        return {"status": 0}

    def release(self, slot):
        del self.quota[slot], self.done[slot]

    def close(self):
        pass


def test_server_admission_blocks_and_percentiles(pkg, monkeypatch):
    """The server's bookkeeping on a fake pool: requests beyond the free
    slots wait and are admitted as others finish, each request's chain
    configuration is built once however long it waits, every request
    reports one latency per 10-sweep block, and the throughput counts every
    requested sweep."""
    from montecarlo_gb300 import serving
    pool = _FakePool(slots=2, per_run=7)
    monkeypatch.setattr(serving._lib, "Pool", lambda *a, **k: pool)
    built = []
    real = serving.request_config

    def counting(req, precision=None, tol=None):
        built.append(req.rid)
        return real(req, precision, tol)

    monkeypatch.setattr(serving, "request_config", counting)
    reqs = [serving.Request(i, "square", 4, 4.0, 1.0, sw, 10 + i)
            for i, sw in enumerate((30, 25, 40, 12, 20))]
    srv = serving.Server(max_slots=2, quantum_us=1000)
    out = srv.serve(reqs, realtime=False)
    srv.close()
    assert pool.split is True
    assert sorted(built) == [0, 1, 2, 3, 4]  # once per request, not once per slice waited
    assert set(out["results"]) == {0, 1, 2, 3, 4} and out["unfinished"] == 0
    for r in reqs:
        res = out["results"][r.rid]
        assert len(res.block_latencies) == r.sweeps // serving.BLOCK
        assert all(x >= 0.0 for x in res.block_latencies)
        assert res.finished >= res.admitted
    assert out["sweeps"] == sum(r.sweeps for r in reqs)
    assert out["blocks"] == sum(r.sweeps // serving.BLOCK for r in reqs)
    # two slots at 7 sweeps a slice each: at least total / 14 slices, and at
    # least the longest request's sweeps / 7
    total = sum(r.sweeps for r in reqs)
    assert out["launches"] >= max(-(-total // 14), -(-40 // 7))
    lat = [x for res in out["results"].values() for x in res.block_latencies]
    assert out["p50_block_s"] == float(np.percentile(lat, 50))
    assert out["p99_block_s"] == float(np.percentile(lat, 99))


class _FakeHandle:
    """Host-side stand-in for a one-chain _lib.Handle: counts sweeps and
    returns a field whose first sites spell the sweep count in binary."""

    def __init__(self, configs, precision=None, device=0):
        c = configs[0]
        self.n, self.M, self.swept, self.calls = c.n_sites, c.slices, 0, []

    def set_hopping(self, chain, exps):
        pass

    def init_random_field(self, chain):
        pass

    def set_field(self, chain, conf):
        pass

    def initialize_run(self):
        pass

    def sweep(self, k):
        self.calls.append(k)
        self.swept += k

    def get_field(self, chain):
        conf = -np.ones((self.n, self.M), dtype=np.int8, order="F")
        for b in range(self.n):
            if (self.swept >> b) & 1:
                conf[b, 0] = 1
        return conf

    def greens(self, chain, physical=False):
        return np.zeros((1, self.n, self.n))

    def stats(self, chain):
        return {k: 0 for k in (
            "accepted", "proposals", "propagation_errors", "max_propagation_error",
            "negative_probability", "imaginary_probability", "max_imaginary_probability",
            "min_reported_error", "mean_reported_error", "max_reported_error",
            "min_negative_probability", "mean_negative_probability",
            "max_negative_probability", "min_imaginary_probability",
            "mean_imaginary_probability", "current_slice")}

    def global_stats(self, chain):
        return (0, 0)


def test_run_measures_and_records_like_sweep_once(pkg, monkeypatch):
    """run! (DQMC.jl:252-394 with sweep_once!, :200-225) on a fake handle: the
    sweeps run in launches of at most max_sweeps_per_launch, measurements
    happen after exactly the sweeps i > thermalization with i % measure_rate
    == 0, and the recorder holds the configurations after exactly the sweeps
    i > thermalization with i % recording_rate == 0, whatever the launch
    boundaries."""
    from montecarlo_gb300 import dqmc
    monkeypatch.setattr(dqmc._lib, "Handle", _FakeHandle)

    class Obs:
        def __init__(self):
            self.at = []

        def measure(self, G, mc):
            self.at.append(mc.last_sweep)

    model = pkg.HubbardModel(pkg.SquareLattice(4), U=4.0)
    for th, sw, rate, rec, cap in ((7, 30, 4, 6, 5), (10, 25, 10, 3, 50), (0, 13, 1, 2, 4),
                                   (5, 12, 7, 7, 1)):
        obs = Obs()
        mc = dqmc.DQMC(model, beta=1.0, thermalization=th, sweeps=sw, measure_rate=rate,
                       recording_rate=rec, device_measurements=False, measurements={"m": obs},
                       seed=1)
        mc.max_sweeps_per_launch = cap
        assert mc.run() == dqmc.ExitCode.SUCCESS
        total = th + sw
        assert mc.last_sweep == total and mc.handle.swept == total
        assert max(mc.handle.calls) <= cap
        assert obs.at == [i for i in range(th + 1, total + 1) if i % rate == 0]
        want = [i for i in range(th + 1, total + 1) if i % rec == 0]
        assert len(mc.recorder) == len(want)
        for j, i in enumerate(want):
            conf = mc.recorder[j]
            assert sum(1 << b for b in range(16) if conf[b, 0] == 1) == i


def test_tune_safe_mult_picks_largest_stable_interval(pkg, monkeypatch):
    """tune_safe_mult on a fake device whose propagation error grows with the
    stabilisation interval k as err(k) = c * 10^k (c per chain): each chain gets the
    largest candidate (capped at its slice count) with err <= safety * tol,
    the smallest candidate when none is, one probe launch covers every
    uncached chain x candidate, and cached kinds are not probed again."""
    from montecarlo_gb300 import autotune

    launches = []
    BASE = {1: 1e-18, 2: 1e-16, 3: 1e-18, 4: 1.0}  # by seed: c of err(k) = c * 10^k

    class Probe:
        def __init__(self, cfgs, precision=None, device=0):
            self.cfgs = cfgs
            launches.append(len(cfgs))

        def set_hopping(self, r, exps):
            pass

        def init_random_field(self, r):
            pass

        def set_field(self, r, conf):
            assert conf.shape == (self.cfgs[r].n_sites, self.cfgs[r].slices)

        def initialize_run(self):
            pass

        def sweep(self, n):
            return [{"max_propagation_error": BASE[c.seed] * 10.0 ** c.safe_mult}
                    for c in self.cfgs]

        def close(self):
            pass

    monkeypatch.setattr(autotune._lib, "Handle", Probe)
    weak = pkg.HubbardModel(pkg.SquareLattice(4), U=2.0)
    strong = pkg.HubbardModel(pkg.SquareLattice(4), U=8.0)
    short = pkg.HubbardModel(pkg.SquareLattice(6), U=2.0)
    wild = pkg.HubbardModel(pkg.SquareLattice(6), U=7.0)
    specs = [(weak, weak.choose_field(), 4.0, 0.1, 1), (strong, strong.choose_field(), 4.0, 0.1, 2),
             (short, short.choose_field(), 0.5, 0.1, 3), (wild, wild.choose_field(), 2.0, 0.1, 4)]
    for m, f, b, dt, s in specs:
        autotune._CACHE.pop(autotune.cache_key(m, f, b, dt, autotune._lib.PREC_FP64, 1e-6), None)
    confs = []
    for m, f, b, dt, s in specs:
        M = pkg.DQMCParameters.make(beta=b, delta_tau=dt).slices
        confs.append(np.ones((len(m.l), M), dtype=np.int8))
    ks, errs = autotune.tune_safe_mult(specs, tol=1e-6, confs=confs, safety=0.1)
    bound = 0.1 * 1e-6
    for (m, f, b, dt, s), k, e in zip(specs, ks, errs):
        M = pkg.DQMCParameters.make(beta=b, delta_tau=dt).slices
        err = {c: BASE[s] * 10.0 ** c for c in {min(c, M) for c in autotune.CANDIDATES}}
        ok = [c for c, v in err.items() if v <= bound]
        assert k == (max(ok) if ok else min(err)) and e == err[k]
        assert k <= M
    assert ks == [10, 8, 5, 2]  # largest under 1e-7; five slices; none stable: the smallest
    assert len(launches) == 1
    # all cached now: no probe launch, NaN errors
    ks2, errs2 = autotune.tune_safe_mult(specs, tol=1e-6, confs=confs)
    assert ks2 == ks and all(np.isnan(errs2)) and len(launches) == 1
    for m, f, b, dt, s in specs:
        autotune._CACHE.pop(autotune.cache_key(m, f, b, dt, autotune._lib.PREC_FP64, 1e-6), None)


def test_neighbour_partners_alternate_even_and_odd_pairs(pkg):
    """Replica exchange rounds pair neighbours (0,1), (2,3), ... and then
    (1,2), (3,4), ...; partners are mutual, a replica without a partner
    sits the round out (-1), and two rounds give every neighbour pair one
    attempt."""
    from montecarlo_gb300.tempering import neighbour_partners
    for n in range(1, 9):
        seen = set()
        for odd in (False, True):
            p = neighbour_partners(n, odd)
            assert p.dtype == np.int32 and p.shape == (n,)
            for a in range(n):
                if p[a] >= 0:
                    assert p[p[a]] == a and abs(p[a] - a) == 1
                    assert (min(a, p[a]) % 2 == 1) == odd
                    seen.add(min(a, p[a]))
        assert seen == set(range(n - 1))
    assert neighbour_partners(5, False).tolist() == [1, 0, 3, 2, -1]
    assert neighbour_partners(5, True).tolist() == [-1, 2, 1, 4, 3]


def test_server_fails_one_request_and_serves_the_rest(pkg, monkeypatch):
    """A chain that reports a nonzero status during a time slice (the pool run
    returns DQMC_ERR_NUMERICAL) fails its own request only: the server
    records it with the error, releases its slot, admits the next request
    into it and finishes every other request; any other error is raised."""
    from montecarlo_gb300 import serving, _lib

    class Failing(_FakePool):
        def __init__(self):
            super().__init__(slots=2, per_run=7)
            self.status = {}

        def admit(self, cfg):
            s = super().admit(cfg)
            if s is not None:
                self.status[s] = 0
                self.seed = getattr(self, "seed", {})
                self.seed[s] = cfg.seed
            return s

        def run(self, quantum_us, use_graph):
            super().run(quantum_us, use_graph)
            for s in self.quota:
                if self.seed[s] == 11 and self.done[s] >= 21:  # request 1 breaks
                    self.status[s] = 9
                    raise _lib.DQMCError(_lib.DQMC_ERR_NUMERICAL, f"slot {s} reported status 9")

        def stats(self, slot):
            return {"status": self.status[slot]}

        def release(self, slot):
            super().release(slot)
            del self.status[slot], self.seed[slot]

    pool = Failing()
    monkeypatch.setattr(serving._lib, "Pool", lambda *a, **k: pool)
    reqs = [serving.Request(i, "square", 4, 4.0, 1.0, sw, 10 + i)
            for i, sw in enumerate((30, 40, 25, 12))]
    srv = serving.Server(max_slots=2, quantum_us=1000)
    out = srv.serve(reqs, realtime=False)
    assert out["failed"] == 1 and out["unfinished"] == 0
    bad = out["results"][1]
    assert bad.error and "status 9" in bad.error and bad.stats["status"] == 9
    assert len(bad.block_latencies) == 1  # the block finished in an earlier slice counts
    for rid in (0, 2, 3):
        r = out["results"][rid]
        assert r.error is None and len(r.block_latencies) == reqs[rid].sweeps // serving.BLOCK

    class Broken(_FakePool):
        def run(self, quantum_us, use_graph):
            raise _lib.DQMCError(2, "CUDA error")

    monkeypatch.setattr(serving._lib, "Pool", lambda *a, **k: Broken(2, 7))
    srv = serving.Server(max_slots=2, quantum_us=1000)
    with pytest.raises(_lib.DQMCError):
        srv.serve(reqs[:1], realtime=False)
