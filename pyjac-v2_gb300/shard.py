"""Several GPUs, one process each: states are independent, so a batch is split
into contiguous state ranges and every rank evaluates its own range with no
collective on the data path.  The only collectives are for timing (the
slowest rank's time, barriers) and, optionally, gathering results to one
rank.  spawn() starts the ranks of one node when no launcher (torchrun) did.
"""


def state_range(n, rank, world, align=128):
    """[start, stop) of `rank`'s states of n: contiguous, balanced to within
    `align` states (the kernels' block size), together covering [0, n)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank / world size")
    blocks = (n + align - 1) // align
    b0 = rank * blocks // world
    b1 = (rank + 1) * blocks // world
    return min(n, b0 * align), min(n, b1 * align)


def max_over_ranks(value, device=None):
    """The largest `value` over the ranks of the default process group (the
    value itself without one)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def init_process_group(backend="nccl"):
    """Join the default process group of this rank (rank, world size and the
    rendezvous address from the environment, as torchrun or spawn() set
    them)."""
    import torch.distributed as dist
    if not dist.is_initialized():
        dist.init_process_group(backend)


def barrier():
    """Wait for every rank (nothing without a process group)."""
    d = _dist()
    if d is not None and d.get_world_size() > 1:
        d.barrier()


def destroy_process_group():
    d = _dist()
    if d is not None:
        d.destroy_process_group()


def _free_port():
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _spawned(local_rank, world, port, fn, args):
    import os
    os.environ.update({"RANK": str(local_rank), "LOCAL_RANK": str(local_rank),
                       "WORLD_SIZE": str(world), "LOCAL_WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    rc = fn(*args)
    if rc:
        raise SystemExit(rc)


def spawn(fn, world, args=()):
    """Run fn(*args) in `world` fresh processes of one node, one per GPU, with
    the environment torchrun would give them (RANK, LOCAL_RANK, WORLD_SIZE,
    MASTER_ADDR 127.0.0.1, a free MASTER_PORT); return 0 when all exit
    cleanly.  Processes start by 'spawn', so none inherits a CUDA context."""
    import torch.multiprocessing as mp
    mp.start_processes(_spawned, args=(world, _free_port(), fn, tuple(args)), nprocs=world,
                       join=True, start_method="spawn")
    return 0
