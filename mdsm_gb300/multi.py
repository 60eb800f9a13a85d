"""Multi-GPU sharding of the search: host-side logic only.

The path has no exchange step (no collective on the data path):
  * by beam -- each rank dedisperses and searches its own beams (preferred);
  * by DM range -- every rank gets the whole block and a contiguous slice of the DM plan, as
    src/mdsm/dedispersion_manager.cpp:243,246 and src/mdsm/dedispersion_thread.cu:76,229 split
    it across GPUs.
Candidate lists are gathered on the host at the end (torch.distributed object gather; gloo or
NCCL process groups both work, the payload is host data).
"""
import heapq


def assign_beams(costs, world):
    """Longest-processing-time assignment of beams to ranks.  costs[i] is beam i's work (e.g.
    nchans * ndms * nsamp).  Returns a list of beam-index lists, one per rank, each sorted."""
    if world <= 0:
        raise ValueError("world must be positive")
    heap = [(0, r) for r in range(world)]
    out = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda k: (-costs[k], k)):
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + costs[i], r))
    return [sorted(b) for b in out]


def split_dm_range(lowdm, dmstep, tdms, world, rank):
    """This rank's DM segment when a uniform plan is split across ranks as the reference splits
    it across GPUs: startdm = lowdm + dmstep*tdms/ngpu*rank in float
    (src/mdsm/dedispersion_thread.cu:76,229), tdms/ngpu trials each.  The reference drops the
    remainder trials; here the last rank takes them.  Returns (lowdm_r, dmstep, ndms_r)."""
    import numpy as np
    f = np.float32
    share = tdms // world
    start = f(lowdm) + (f(dmstep) * f(tdms)) / f(world) * f(rank)
    n = share + (tdms - share * world if rank == world - 1 else 0)
    return float(start), float(dmstep), int(n)


def gather_candidates(local, group=None):
    """Gather per-rank candidate lists on every rank (a list of the ranks' objects in rank
    order).  `local` is any picklable object (e.g. a numpy structured array)."""
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return [local]
    out = [None] * dist.get_world_size(group)
    dist.all_gather_object(out, local, group=group)
    return out
