"""Sensor ranges across ranks: the path's only multi-GPU form.

Every sensor's rays and sums are independent of every other sensor's, and the reference already splits a run into
sensor ranges [i0, i0 + nc) whose results are bit-identical to the whole run's (src/run.cpp:642-688, the chunk loop).
So ranks (one process per GPU) take contiguous sensor ranges with the scene and the direction table replicated, trace
and reduce them with no exchange on the data path, and the caller concatenates the row blocks. The one collective is
the timing's: each rank's step time, maxed over ranks, gives the job's time.
"""


def sensor_range(n, rank, world):
    """(i0, count): rank's contiguous share of n sensors; the first n % world ranks take one more."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d of %d" % (rank, world))
    base, extra = divmod(n, world)
    i0 = rank * base + min(rank, extra)
    return i0, base + (1 if rank < extra else 0)


def max_over_ranks(values, device="cpu"):
    """The element-wise maximum of a list of floats over all ranks of the default process group (itself when there is
    none): the job's step time is its slowest rank's."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(v) for v in values]
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()
