"""Independent KPM replicas on several GPUs (one process per GPU).

Random vectors and disorder realisations are independent, so N GPUs run N
replicas with no exchange on the data path; what is shared at the end is
one reduction: the per-vector moments of every rank gathered into the
global set (the reference's ``_moments_list`` of a run with all vectors,
kwant/kpm.py:486-490, whose mean gives the DOS, :378-388), and the
wall-clock of the slowest rank.  Works over any ``torch.distributed``
backend (NCCL between GPUs, gloo on host tensors).
"""

import numpy as np

__all__ = ['gather_moments', 'max_over_ranks', 'replica_seed']


def replica_seed(base_seed, rank):
    """Vector stream of a rank: RandomState(base_seed + rank)."""
    return int(base_seed) + int(rank)


def gather_moments(local, group=None, device=None):
    """Per-vector moments of every rank, concatenated in rank order.

    ``local``: (R_rank, M[, W]) complex array of this rank (ranks may hold
    different numbers of vectors).  Returns the (sum R_rank, M[, W]) array
    on every rank; its mean over axis 0 is the DOS moments of the union of
    all ranks' vectors.
    """
    import torch
    import torch.distributed as dist
    local = np.ascontiguousarray(local, dtype=np.complex128)
    world = dist.get_world_size(group)
    dev = device if device is not None else 'cpu'
    n = torch.tensor([local.shape[0]], dtype=torch.int64, device=dev)
    counts = [torch.zeros_like(n) for _ in range(world)]
    dist.all_gather(counts, n, group=group)
    counts = [int(c.item()) for c in counts]
    tail = local.shape[1:]
    width = int(np.prod(tail)) * 2
    rmax = max(counts)
    buf = np.zeros((rmax, width), dtype=np.float64)
    buf[:local.shape[0]] = local.reshape(local.shape[0], -1).view(
        np.float64).reshape(local.shape[0], width)
    t = torch.from_numpy(buf).to(dev)
    parts = [torch.zeros_like(t) for _ in range(world)]
    dist.all_gather(parts, t, group=group)
    out = [p.cpu().numpy()[:c] for p, c in zip(parts, counts)]
    cat = np.concatenate(out, axis=0)
    return cat.view(np.complex128).reshape((cat.shape[0],) + tail)


def max_over_ranks(value, group=None, device=None):
    """The largest ``value`` (e.g. a timed region in ms) over all ranks."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64,
                     device=device if device is not None else 'cpu')
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
