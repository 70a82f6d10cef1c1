"""Checkpoint / resume and replay through the DQMC API (FileIO.jl:155-171,
DQMC.jl:418-505): a resumed chain continues exactly where it stopped, and
replaying recorded configurations reproduces the run's measurements."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _model(pkg):
    return pkg.HubbardModel(pkg.SquareLattice(4), U=-4.0)


def test_resume_continues_chain(pkg, lib, tmp_path):
    from montecarlo_gb300 import dqmc
    m = _model(pkg)
    a = pkg.DQMC(m, beta=2.0, delta_tau=0.1, safe_mult=5, seed=9, thermalization=0, sweeps=8)
    a.run()
    b = pkg.DQMC(m, beta=2.0, delta_tau=0.1, safe_mult=5, seed=9, thermalization=0, sweeps=8)
    b.run(sweeps=4)
    path = str(tmp_path / "chk.npz")
    dqmc.save(b, path)
    c = dqmc.resume(path)
    assert c.last_sweep == 4
    c.run()
    assert c.last_sweep == 8
    assert np.array_equal(c.handle.get_field(0), a.handle.get_field(0))
    assert np.array_equal(c.handle.get_rng(0), a.handle.get_rng(0))
    assert np.abs(c.greens() - a.greens()).max() < 1e-10


def test_replay_reproduces_measurements(pkg, lib):
    from montecarlo_gb300 import dqmc
    m = _model(pkg)
    mc = pkg.DQMC(m, beta=2.0, delta_tau=0.1, safe_mult=5, seed=4, thermalization=2, sweeps=20,
                  measure_rate=1)
    mc["docc"] = pkg.double_occupancy(mc, m)
    rec = dqmc.ConfigRecorder(rate=1)
    mc.run(sweeps=0)  # thermalisation only
    for s in range(20):
        mc.run(sweeps=s + 1)
        rec.push(mc.handle.get_field(0), s + 1)
    run_mean = float(mc["docc"].mean())
    rp = pkg.DQMC(m, beta=2.0, delta_tau=0.1, safe_mult=5, seed=4, measure_rate=1)
    rp["docc"] = pkg.double_occupancy(rp, m)
    dqmc.replay(rp, rec)
    assert len(rp["docc"].observable) == 20
    assert abs(float(rp["docc"].mean()) - run_mean) < 1e-10
