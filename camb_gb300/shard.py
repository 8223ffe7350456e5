"""Multi-GPU replicas: a batch of cosmologies split across ranks with no collective on
the data path (k-modes and cosmologies are independent, cmbmain.f90:205-209); C_l
are gathered on the host afterwards."""
import numpy as np


def shard_range(n, rank, world):
    """Contiguous, balanced [lo, hi) share of n items for `rank` of `world`."""
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def get_results_sharded(params_list, lmax_out, compute=None, group=None):
    """Each rank computes its share of `params_list` (default: the GPU batch call) and
    all ranks receive every cosmology's (lmax_out+1, 4) C_l array, in input order."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group) if dist.is_initialized() else 1
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    lo, hi = shard_range(len(params_list), rank, world)
    if compute is None:
        from .results import get_results_batch

        def compute(ps, lmax):
            return np.stack([r.get_unlensed_scalar_cls(lmax) for r in get_results_batch(ps, lmax)])
    local = compute(params_list[lo:hi], lmax_out) if hi > lo else np.zeros((0, lmax_out + 1, 4))
    if world == 1:
        return local
    out = [None] * world
    dist.all_gather_object(out, (lo, local), group=group)
    full = np.zeros((len(params_list), lmax_out + 1, 4))
    for lo_r, arr in out:
        full[lo_r:lo_r + len(arr)] = arr
    return full
