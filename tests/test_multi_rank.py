"""Multi-rank sharding on CPU with gloo (world size 2): by beam and by DM range, no collective
on the data path, candidates gathered on the host.  Each rank runs the oracle on its share;
the union must equal the single-process result."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_assign_beams_balances_and_covers():
    from mdsm_gb300.multi import assign_beams
    costs = [5, 1, 9, 3, 3, 7, 2, 8]
    parts = assign_beams(costs, 3)
    assert sorted(i for p in parts for i in p) == list(range(8))
    loads = [sum(costs[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(costs)


def test_split_dm_range_matches_reference_start():
    from mdsm_gb300.multi import split_dm_range
    segs = [split_dm_range(0.0, 0.25, 103, 4, r) for r in range(4)]
    assert sum(n for _, _, n in segs) == 103
    assert segs[1][0] == np.float32(np.float32(0.25) * np.float32(103) / np.float32(4))


def _worker(rank, world, port, result_path):
    import torch.distributed as dist
    from mdsm_gb300.multi import assign_beams, gather_candidates, split_dm_range
    from oracle import oracle as orc
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    nchans, nsamp, fch1, foff, tsamp = 64, 1024, 1500.0, -4.0, 64e-6
    beams = [np.random.default_rng(b).standard_normal((nchans, nsamp + 600), dtype=np.float32)
             for b in range(5)]
    segs = [(0.0, 1.0, 40)]
    S = orc.shift_table(nchans, fch1, foff, tsamp, segs)
    # by beam
    mine = assign_beams([1] * len(beams), world)[rank]
    local = {b: orc.dedisperse(beams[b], S, nsamp) for b in mine}
    got = gather_candidates(local)
    # by DM range on beam 0
    lo, st, n = split_dm_range(0.0, 1.0, 40, world, rank)
    Sr = orc.shift_table(nchans, fch1, foff, tsamp, [(lo, st, n)])
    part = gather_candidates(orc.dedisperse(beams[0], Sr, nsamp))
    if rank == 0:
        merged = {}
        for d in got:
            merged.update(d)
        ok = sorted(merged) == list(range(len(beams)))
        for b in range(len(beams)):
            ok &= np.array_equal(merged[b], orc.dedisperse(beams[b], S, nsamp))
        stacked = np.concatenate(part, axis=0)
        ok &= np.array_equal(stacked, orc.dedisperse(beams[0], S, nsamp))
        with open(result_path, "w") as f:
            f.write("ok" if ok else "mismatch")
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gloo_sharding(tmp_path):
    import torch.multiprocessing as mp
    path = str(tmp_path / "res.txt")
    mp.start_processes(_worker, args=(2, _free_port(), path), nprocs=2, start_method="spawn")
    assert open(path).read() == "ok"
