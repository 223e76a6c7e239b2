"""Multi-GPU use of the force path: independent replicas, one process per GPU.

The path has no exchange step -- configurations are independent and a
configuration is evaluated whole on one GPU -- so several GPUs run disjoint
work with no collective on the data path.  The only communication is host-side
bookkeeping: splitting a list of configurations across ranks and taking the
maximum time over ranks for a job.  Both work on any torch.distributed
backend (gloo on CPU, nccl on GPUs).
"""

from __future__ import annotations

from typing import List, Sequence, Tuple


def shard_bounds(n_items: int, rank: int, world: int) -> Tuple[int, int]:
    """Contiguous, balanced [start, stop) of n_items for `rank` of `world`."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("rank %d outside world of size %d" % (rank, world))
    base, extra = divmod(n_items, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def shard_by_atoms(atom_counts: Sequence[int], rank: int, world: int) -> List[int]:
    """Indices of configurations for `rank`, balancing total atoms greedily
    (largest first onto the least-loaded rank); deterministic for all ranks."""
    order = sorted(range(len(atom_counts)), key=lambda i: (-atom_counts[i], i))
    load = [0] * world
    owner = [0] * len(atom_counts)
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        owner[i] = r
        load[r] += atom_counts[i]
    return [i for i in range(len(atom_counts)) if owner[i] == rank]


def job_time_and_throughput(local_ms: float, local_atoms: float, steps: int, group=None):
    """Max over ranks of the timed region and the whole-job throughput
    (atoms of all ranks / that time).  Without an initialised process group
    it returns the local figures."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return local_ms, local_atoms * steps / (local_ms * 1e-3)
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    t = torch.tensor([local_ms, local_atoms], dtype=torch.float64, device=dev)
    tmax = t[:1].clone()
    dist.all_reduce(tmax, op=dist.ReduceOp.MAX, group=group)
    atoms = t[1:].clone()
    dist.all_reduce(atoms, op=dist.ReduceOp.SUM, group=group)
    ms = float(tmax.item())
    return ms, float(atoms.item()) * steps / (ms * 1e-3)
