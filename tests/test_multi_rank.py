"""Multi-rank sharding on CPU with gloo (world size 2): by beam and by DM range, no collective
on the data path, candidates gathered on the host.  Each rank runs the oracle on its share;
the union must equal the single-process result.  The serving form's placement and routing
(mdsm_gb300.multi.ShardedServer) run on each rank over a stand-in for the device server that
has its interface and computes with the oracle (OracleServer)."""
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


class OracleServer:
    """The interface of mdsm_gb300.serving.Server (add_beam, submit, poll) computed on the CPU
    with the oracle: per beam, the overlap tail carried between blocks, brute-force
    dedispersion and the boxcar search; results in submission order."""

    def __init__(self):
        self.beams, self.done = [], []

    def add_beam(self, nchans, fch1, foff, tsamp, nsamp, segments):
        from oracle import oracle as orc
        S = orc.shift_table(nchans, fch1, foff, tsamp, segments)
        self.beams.append({"S": S, "nsamp": nsamp, "tail": None, "k": 0})
        return len(self.beams) - 1

    def submit(self, beam, block):
        from oracle import oracle as orc
        b = self.beams[beam]
        ms = int(b["S"].max())
        full = block if b["tail"] is None else np.concatenate([b["tail"], block], axis=1)
        b["tail"] = full[:, b["nsamp"]: b["nsamp"] + ms].copy()
        y = orc.dedisperse(full, b["S"], b["nsamp"])
        dm, sa, wd, sn = orc.boxcar_detect(y, 9, 6.0)
        self.done.append({"beam": beam, "block": b["k"], "ncand": len(dm),
                          "cands": list(zip(dm.tolist(), sa.tolist(), wd.tolist(),
                                            sn.view(np.uint32).tolist()))})
        b["k"] += 1
        return len(self.done)

    def poll(self, wait_ms=0):
        return self.done.pop(0) if self.done else None


SERVE_NCH, SERVE_NSAMP, SERVE_FCH1, SERVE_FOFF, SERVE_TSAMP = 32, 1024, 1500.0, -8.0, 64e-6


def _serve_beams():
    """Five uint8 beams of three blocks each (block 0 with its tail), one pulse in beam 3."""
    from mdsm_gb300 import synth
    from oracle import oracle as orc
    segs = [(0.0, 2.0, 24)]
    ms = int(orc.shift_table(SERVE_NCH, SERVE_FCH1, SERVE_FOFF, SERVE_TSAMP, segs).max())
    out = []
    for b in range(5):
        x = synth.gaussian_u8(SERVE_NCH, 3 * SERVE_NSAMP + ms, 100 + b)
        if b == 3:
            synth.inject(x, SERVE_FCH1, SERVE_FOFF, SERVE_TSAMP, [(1500, 20.0, 4, 60.0)])
        n = SERVE_NSAMP
        blocks = [x[:, : n + ms]] + [x[:, n * k + ms: n * (k + 1) + ms] for k in (1, 2)]
        out.append((segs, blocks))
    return out


def _serve_worker(rank, world, port, result_path):
    import torch.distributed as dist
    from mdsm_gb300.multi import ShardedServer
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    beams = _serve_beams()
    costs = [SERVE_NCH * 24 * SERVE_NSAMP * (1 + (b == 1)) for b in range(len(beams))]
    sv = ShardedServer(costs, rank, world, OracleServer)
    added = [b for b, (segs, _) in enumerate(beams)
             if sv.add_beam(b, SERVE_NCH, SERVE_FCH1, SERVE_FOFF, SERVE_TSAMP, SERVE_NSAMP, segs)]
    for k in range(3):
        for b, (_, blocks) in enumerate(beams):
            sv.submit(b, blocks[k])
    got = []
    while True:
        r = sv.poll()
        if r is None:
            break
        got.append(r)
    merged = sv.gather(got)
    owners = sv.gather([{"beam": b, "block": -1, "rank": rank} for b in added])
    if rank == 0:
        ref = OracleServer()
        for b, (segs, _) in enumerate(beams):
            ref.add_beam(SERVE_NCH, SERVE_FCH1, SERVE_FOFF, SERVE_TSAMP, SERVE_NSAMP, segs)
        for k in range(3):
            for b, (_, blocks) in enumerate(beams):
                ref.submit(b, blocks[k])
        want = sorted(ref.done, key=lambda r: (r["beam"], r["block"]))
        ok = [(r["beam"], r["block"], r["cands"]) for r in merged] == \
             [(r["beam"], r["block"], r["cands"]) for r in want]
        served = sorted(o["beam"] for o in owners)
        ok &= served == list(range(len(beams)))            # every beam on exactly one rank
        ok &= len({o["rank"] for o in owners}) == world     # both ranks serve
        ok &= any(r["ncand"] > 0 for r in merged if r["beam"] == 3)
        with open(result_path, "w") as f:
            f.write("ok" if ok else "mismatch")
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gloo_serving_placement(tmp_path):
    """Each rank serves only the beams ShardedServer places on it; the gathered per-block
    candidate lists equal one server's over all beams."""
    import torch.multiprocessing as mp
    path = str(tmp_path / "serve.txt")
    mp.start_processes(_serve_worker, args=(2, _free_port(), path), nprocs=2,
                       start_method="spawn")
    assert open(path).read() == "ok"
