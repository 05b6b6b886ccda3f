"""Several GPUs, one process each: states are independent, so a batch is split
into contiguous state ranges and every rank evaluates its own range with no
collective on the data path.  The only collectives are for timing (the
slowest rank's time) and, optionally, gathering results to one rank.
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
