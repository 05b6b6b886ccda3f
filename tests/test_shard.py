"""Multi-rank path on the CPU: two gloo processes split a batch by state
ranges (no collective on the data path), evaluate their ranges with the CPU
oracle, and the gathered result equals the single-process evaluation; the
timing reduction takes the slowest rank."""
import os
import socket

import numpy as np
import pytest

from conftest import pkg


def test_state_ranges_cover_and_balance():
    sh = pkg("shard")
    for n in (0, 1, 127, 128, 129, 1000, 1 << 20):
        for world in (1, 2, 3, 8):
            rs = [sh.state_range(n, r, world) for r in range(world)]
            assert rs[0][0] == 0 and rs[-1][1] == n
            assert all(rs[i][1] == rs[i + 1][0] for i in range(world - 1))
            sizes = [b - a for a, b in rs]
            assert max(sizes) - min(sizes) <= 128 or n < 128 * world
            assert all(a % 128 == 0 for a, _ in rs)
    with pytest.raises(ValueError):
        sh.state_range(10, 2, 2)


def _worker(rank, world, port, out):
    import sys
    import torch.distributed as dist
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, here)
    from conftest import load_mech, oracle_mod, pkg as p
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank,
                            world_size=world)
    mech = load_mech("h2o2")
    n = 1000
    P, phi = p("states").draw_states(mech.n_species, n, seed=4)
    a, b = p("shard").state_range(n, rank, world)
    dphi = oracle_mod().Oracle(mech).species_rates(P[a:b], phi[a:b], nthreads=1)
    parts = [None] * world
    dist.all_gather_object(parts, (a, b, dphi))
    slowest = p("shard").max_over_ranks(1.0 + rank)
    if rank == 0:
        np.save(out, np.concatenate([x[2] for x in sorted(parts, key=lambda t: t[0])]))
        with open(out + ".max", "w") as fh:
            fh.write(repr(slowest))
    dist.destroy_process_group()


def test_two_gloo_ranks_match_one_process(tmp_path):
    import torch.multiprocessing as mp
    from conftest import load_mech, oracle_mod
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = str(tmp_path / "gathered.npy")
    mp.start_processes(_worker, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
    mech = load_mech("h2o2")
    P, phi = pkg("states").draw_states(mech.n_species, 1000, seed=4)
    whole = oracle_mod().Oracle(mech).species_rates(P, phi, nthreads=1)
    assert np.array_equal(np.load(out), whole)
    with open(out + ".max") as fh:
        assert float(fh.read()) == 2.0
