"""Rendering one image on several GPUs, one process per GPU.

Path samples are independent and the film is additive (the reference's
SpectrumStorage::add, BasicTypes/spectrum_types.h:725-734), so the samples of
an image split into disjoint index ranges, one per rank, and the partial
films sum to the whole film: there is no exchange until that one sum.  The
random numbers of a sample depend only on (seed, sample index, pixel), so a
sharded render draws the same samples as a single-GPU render of all spp.
On hosts with one GPU per run the ranks are independent replicas."""
from __future__ import annotations


def sample_range(spp: int, world: int, rank: int) -> tuple[int, int]:
    """(first sample, count) of rank `rank` out of `world`: contiguous,
    disjoint, covering [0, spp), sizes differing by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank out of range")
    base, extra = divmod(spp, world)
    first = rank * base + min(rank, extra)
    return first, base + (1 if rank < extra else 0)


def render_shard(scene, width: int, height: int, spp: int, max_depth: int, seed: int = 0, volumetric: bool = False,
                 world: int = 1, rank: int = 0):
    """This rank's partial film (a host array) and its stats; a rank with no
    samples returns a zero film."""
    import numpy as np
    first, count = sample_range(spp, world, rank)
    if count == 0:
        return np.zeros((height, width, 16), np.float32), None
    return scene.render(width, height, count, max_depth, seed=seed, volumetric=volumetric, sample_base=first)


def reduce_films(film, group=None):
    """Sums the partial films of all ranks in place (torch.distributed
    all_reduce; NCCL for CUDA tensors, gloo for host tensors) and returns it."""
    import torch
    import torch.distributed as dist
    t = film if isinstance(film, torch.Tensor) else torch.from_numpy(film)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t


def max_over_ranks(value: float, device=None, group=None) -> float:
    """The largest of the ranks' values (the timing rule: a multi-GPU step
    takes as long as its slowest rank)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
