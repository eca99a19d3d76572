"""Multi-GPU use of the march: replicas over independent fields.

A z-march is sequential, but fields (illumination angles, wavelengths, requests) are
independent and share only the read-only dn volume. So N GPUs run N replicas, one process
per GPU, each marching its own contiguous share of the fields with no collective on the
data path. The only cross-GPU reduction the hot path has is the gradient of a loss with
respect to a shared dn, which is the sum over angles of every replica's gradient
(`sum_over_ranks`, an all-reduce over torch.distributed: NCCL between GPUs, gloo on CPU).
The reference is single-device (one OpenCL queue) and has neither.
"""
import torch
import torch.distributed as dist

__all__ = ["shard", "max_over_ranks", "sum_over_ranks", "world"]


def world():
    """(rank, world_size) of the initialised process group, or (0, 1)."""
    if dist.is_available() and dist.is_initialized():
        return dist.get_rank(), dist.get_world_size()
    return 0, 1


def shard(batch, rank, world_size):
    """Contiguous share [b0, b1) of `batch` fields for `rank`; shares differ by at most one
    field and together cover every field exactly once."""
    if world_size < 1 or not 0 <= rank < world_size:
        raise ValueError("rank %d outside a world of %d" % (rank, world_size))
    base, extra = divmod(int(batch), int(world_size))
    b0 = rank * base + min(rank, extra)
    return b0, b0 + base + (1 if rank < extra else 0)


def _device_for_backend():
    if dist.get_backend() == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def max_over_ranks(x):
    """Largest value of the float x over all ranks (timing: the slowest replica)."""
    r, w = world()
    if w == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=_device_for_backend())
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(t):
    """In-place sum of tensor t over all ranks (d loss / d dn summed over angle shards)."""
    r, w = world()
    if w > 1:
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t
