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


def _bench_rank(out):
    """One rank of the benchmark's multi-GPU flow with the CPU oracle in place
    of the GPU kernels: join the group from the environment spawn() set,
    evaluate this rank's own states (weak scaling: every rank the same number),
    take the slowest rank's time, gather to rank 0, which writes the line."""
    import json
    import sys
    import time
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, here)
    import torch.distributed as dist
    from conftest import load_mech, oracle_mod, pkg as p
    sh = p("shard")
    sh.init_process_group("gloo")
    rank, world = int(os.environ["RANK"]), int(os.environ["WORLD_SIZE"])
    assert dist.get_rank() == rank and dist.get_world_size() == world
    mech = load_mech("h2o2")
    n = 512
    P, phi = p("states").draw_states(mech.n_species, world * n, seed=9)
    a, b = sh.state_range(world * n, rank, world)
    sh.barrier()
    t0 = time.perf_counter()
    dphi = oracle_mod().Oracle(mech).species_rates(P[a:b], phi[a:b], nthreads=1)
    sec = sh.max_over_ranks(time.perf_counter() - t0)
    parts = [None] * world
    dist.all_gather_object(parts, (a, dphi))
    if rank == 0:
        np.save(out, np.concatenate([x[1] for x in sorted(parts, key=lambda t: t[0])]))
        with open(out + ".json", "w") as fh:
            json.dump({"n_gpus": world, "value": world * n / sec, "scaling": "weak",
                       "ranks": sorted(x[0] for x in parts)}, fh)
    sh.barrier()
    sh.destroy_process_group()
    return 0


def test_spawned_ranks_match_one_process(tmp_path):
    """shard.spawn, the path bench.py --gpus N takes when no launcher started
    it: two ranks on gloo, each with torchrun's environment; the gathered
    result equals one process's, and the line reports both ranks."""
    import json
    from conftest import load_mech, oracle_mod
    out = str(tmp_path / "spawned.npy")
    assert pkg("shard").spawn(_bench_rank, 2, (out,)) == 0
    with open(out + ".json") as fh:
        line = json.load(fh)
    assert line["n_gpus"] == 2 and line["ranks"] == [0, 512]
    mech = load_mech("h2o2")
    P, phi = pkg("states").draw_states(mech.n_species, 1024, seed=9)
    whole = oracle_mod().Oracle(mech).species_rates(P, phi, nthreads=1)
    assert np.array_equal(np.load(out), whole)


def test_bench_spawns_ranks_only_without_a_launcher(monkeypatch):
    """bench.py --gpus 2 hands its ranks to shard.spawn unless WORLD_SIZE is
    set (torchrun started it), where it runs as the given rank."""
    import importlib
    import sys
    from conftest import ROOT
    sys.path.insert(0, ROOT)
    bench = importlib.import_module("bench")
    calls = []
    monkeypatch.setattr(pkg("shard"), "spawn", lambda fn, world, args: calls.append(world) or 0)
    monkeypatch.setattr(bench, "run_gpu", lambda args: calls.append("rank") or 0)
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    assert bench.main(["--gpus", "2"]) == 0 and calls == [2]
    monkeypatch.setenv("WORLD_SIZE", "2")
    assert bench.main(["--gpus", "2"]) == 0 and calls == [2, "rank"]
    calls.clear()
    monkeypatch.delenv("WORLD_SIZE")
    assert bench.main(["--gpus", "1"]) == 0 and calls == ["rank"]
