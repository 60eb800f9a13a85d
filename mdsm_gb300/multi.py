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


class ShardedServer:
    """The serving form over several GPUs, one process per GPU: every rank builds the same
    ShardedServer over the full beam list; assign_beams places each beam on one rank by its
    cost, and each rank adds, feeds and polls only its own beams on a local server (the native
    mdsm_gb300.serving.Server on the rank's GPU, or anything with its add_beam /
    add_beam_subband / submit / poll methods).  No sample or series crosses ranks; candidate
    lists are gathered on the host at the end.

    beam_costs: per global beam, its work (nchans * ndms * nsamp)."""

    def __init__(self, beam_costs, rank, world, make_server):
        self.rank, self.world = rank, world
        self.placement = assign_beams(list(beam_costs), world)
        self.owner = {b: r for r, bs in enumerate(self.placement) for b in bs}
        self.local = make_server()
        self._to_local, self._to_global = {}, {}

    def owns(self, beam):
        return self.owner[beam] == self.rank

    def add_beam(self, beam, *args, subband=False, **kw):
        """Add global beam `beam` if this rank owns it; returns whether it did."""
        if not self.owns(beam):
            return False
        add = self.local.add_beam_subband if subband else self.local.add_beam
        lid = add(*args, **kw)
        self._to_local[beam] = lid
        self._to_global[lid] = beam
        return True

    def submit(self, beam, block):
        """Submit a block of an own beam (others are no-ops returning None with owned False):
        (owned, ticket or None when admission refused it for now)."""
        if not self.owns(beam):
            return False, None
        return True, self.local.submit(self._to_local[beam], block)

    def poll(self, wait_ms=0):
        """A finished block of an own beam, with its global beam index, or None."""
        r = self.local.poll(wait_ms=wait_ms)
        if r is None:
            return None
        r = dict(r)
        r["beam"] = self._to_global[r["beam"]]
        return r

    def gather(self, results, group=None):
        """All ranks' results (lists of poll() dicts) merged on every rank, ordered by
        (beam, block)."""
        parts = gather_candidates(list(results), group=group)
        merged = [r for part in parts for r in part]
        return sorted(merged, key=lambda r: (r["beam"], r["block"]))
