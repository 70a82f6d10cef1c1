"""Checkpoint / resume and replay through the DQMC API (FileIO.jl:155-171,
flavors/DQMC/FileIO.jl:10-22, DQMC.jl:418-505): a resumed chain continues
exactly where it stopped -- field, RNG, Green's function, recorded
configurations, acceptance counters and the accumulated observables (device
and host) -- and replaying recorded configurations reproduces the run's
measurements, also when the replay itself is split in two."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _model(pkg):
    return pkg.HubbardModel(pkg.SquareLattice(4), U=-4.0)


def _sim(pkg, m, **kw):
    mc = pkg.DQMC(m, beta=2.0, delta_tau=0.1, safe_mult=5, seed=9, thermalization=2, sweeps=8,
                  measure_rate=2, **kw)
    mc["docc"] = pkg.double_occupancy(mc, m)
    return mc


@pytest.mark.parametrize("checkerboard", [False, True])
def test_resume_continues_chain(pkg, lib, tmp_path, checkerboard):
    from montecarlo_gb300 import dqmc
    m = _model(pkg)
    a = _sim(pkg, m, checkerboard=checkerboard)
    a.run()
    b = _sim(pkg, m, checkerboard=checkerboard)
    b.run(sweeps=4)
    path = str(tmp_path / "chk.npz")
    dqmc.save(b, path)
    c = dqmc.resume(path, measurements={"docc": pkg.double_occupancy(None, m)})
    assert c.parameters.checkerboard == checkerboard
    assert c.last_sweep == 6
    c.run()
    assert c.last_sweep == 10
    assert np.array_equal(c.handle.get_field(0), a.handle.get_field(0))
    assert np.array_equal(c.handle.get_rng(0), a.handle.get_rng(0))
    assert np.abs(c.greens() - a.greens()).max() < 1e-10
    # analysis counters carried over
    sa, sc = a.handle.stats(0), c.handle.stats(0)
    for key in ("accepted", "proposals", "propagation_errors", "negative_probability"):
        assert sa[key] == sc[key], key
    # accumulated observables: device binners and the host measurement
    oa, oc = a.observables(), c.observables()
    assert oa["count"] == oc["count"] == 4
    for k in ("density", "double_occupancy", "interaction_energy", "sz_structure_factor"):
        assert abs(oa[k][0] - oc[k][0]) < 1e-12, k
        assert abs(oa[k][1] - oc[k][1]) < 1e-10 or (np.isinf(oa[k][1]) and np.isinf(oc[k][1]))
    assert len(c["docc"].observable) == len(a["docc"].observable) == 4
    assert abs(float(c["docc"].mean()) - float(a["docc"].mean())) < 1e-12
    # recorded configurations: the uninterrupted run's
    assert len(c.recorder) == len(a.recorder) == 4
    for i in range(4):
        assert np.array_equal(c.recorder[i], a.recorder[i])


def test_resume_keeps_global_schedule(pkg, lib, tmp_path):
    """SimpleScheduler(LocalSweep(), GlobalFlip()) continues in step."""
    from montecarlo_gb300 import dqmc
    m = _model(pkg)
    a = _sim(pkg, m, global_update="flip")
    a.run()
    b = _sim(pkg, m, global_update="flip")
    b.run(sweeps=4)
    path = str(tmp_path / "chk.npz")
    dqmc.save(b, path)
    c = dqmc.resume(path)
    assert c.global_update == "flip"
    c.run()
    assert np.array_equal(c.handle.get_field(0), a.handle.get_field(0))
    assert np.array_equal(c.handle.get_rng(0), a.handle.get_rng(0))
    assert c.handle.global_stats(0) == a.handle.global_stats(0)


def test_replay_reproduces_measurements(pkg, lib):
    from montecarlo_gb300 import dqmc
    m = _model(pkg)
    mc = pkg.DQMC(m, beta=2.0, delta_tau=0.1, safe_mult=5, seed=4, thermalization=2, sweeps=20,
                  measure_rate=1)
    mc["docc"] = pkg.double_occupancy(mc, m)
    mc.run()
    assert len(mc.recorder) == 20
    run_mean = float(mc["docc"].mean())
    rp = pkg.DQMC(m, beta=2.0, delta_tau=0.1, safe_mult=5, seed=4, measure_rate=1)
    rp["docc"] = pkg.double_occupancy(rp, m)
    dqmc.replay(rp, mc.recorder)
    assert rp.last_sweep == 20
    assert len(rp["docc"].observable) == 20
    assert abs(float(rp["docc"].mean()) - run_mean) < 1e-10


def test_replay_in_two_parts_equals_one(pkg, lib):
    """replay! continues from last_sweep (DQMC.jl:455): two partial replays
    measure every configuration exactly once."""
    from montecarlo_gb300 import dqmc
    m = _model(pkg)
    mc = pkg.DQMC(m, beta=2.0, delta_tau=0.1, safe_mult=5, seed=5, thermalization=1, sweeps=12,
                  measure_rate=1)
    mc.run()
    confs = mc.recorder
    whole = pkg.DQMC(m, beta=2.0, delta_tau=0.1, safe_mult=5, seed=5, measure_rate=1)
    whole["docc"] = pkg.double_occupancy(whole, m)
    dqmc.replay(whole, confs)
    parts = pkg.DQMC(m, beta=2.0, delta_tau=0.1, safe_mult=5, seed=5, measure_rate=1)
    parts["docc"] = pkg.double_occupancy(parts, m)
    first = dqmc.ConfigRecorder(rate=1)
    for i in range(5):
        first.push(confs[i], i + 1)
    dqmc.replay(parts, first)
    assert parts.last_sweep == 5
    dqmc.replay(parts, confs)
    assert parts.last_sweep == 12
    a, b = whole["docc"].observable.values, parts["docc"].observable.values
    assert len(a) == len(b) == 12
    for x, y in zip(a, b):
        assert abs(float(x) - float(y)) < 1e-12
