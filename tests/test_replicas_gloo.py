"""The N > 1 path (independent replicas) on CPU with the gloo backend,
world size 2: disjoint seeds per rank, max-over-ranks timing, aggregate
throughput, and per-rank oracle chains that are independent of each other."""
import os

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _worker(rank, world, port, out):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    sys.path.insert(0, os.path.join(root, "oracle"))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import __graft_entry__ as g
    pkg = g.load_package()
    from montecarlo_gb300 import replicas
    import oracle as O

    seeds = replicas.chain_seeds(rank, 3)
    model = pkg.HubbardModel(pkg.SquareLattice(2), U=2.0)
    param = pkg.DQMCParameters.make(beta=1.0, delta_tau=0.1, safe_mult=5)
    fld = model.choose_field()(param, model)
    exps = pkg.hopping_exponentials(model.hopping_matrix(), 0.1)
    confs = []
    for s in seeds:
        c = O.OracleChain(4, 1, param.slices, 5, fld.kind, fld.alpha, exps, s)
        c.init_random_conf()
        c.initialize_run()
        c.sweeps(2)
        confs.append(c.get_conf().tobytes())
    elapsed = 1.0 + rank  # rank 1 is the slow one
    tmax = replicas.max_over_ranks(elapsed, dist)
    gathered = [None] * world
    dist.all_gather_object(gathered, (seeds, confs))
    dist.barrier()
    out[rank] = (tmax, gathered, replicas.aggregate_rate(3, world, tmax))
    dist.destroy_process_group()


def test_two_rank_replicas():
    port = 29500 + (os.getpid() % 2000)
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    for rank in (0, 1):
        tmax, gathered, rate = res[rank]
        assert tmax == 2.0
        assert rate == pytest.approx(3.0)
        s0, c0 = gathered[0]
        s1, c1 = gathered[1]
        assert not set(s0) & set(s1)
        assert all(a != b for a in c0 for b in c1)
