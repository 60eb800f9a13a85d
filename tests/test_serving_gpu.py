"""The serving form: continuous batching over several beams with device-resident overlap
tails.  Each beam's candidates must be the same alone and in the mix, and equal the oracle's
boxcar search of the oracle's dedispersion of the beam's stream."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BEAMS = [  # nchans, nsamp, segments, seed
    (128, 2048, [(0.0, 1.0, 48)], 1),
    (256, 4096, [(0.0, 0.5, 64)], 2),
    (64, 1024, [(5.0, 2.0, 40)], 3),
]
FCH1, BW, TSAMP = 1500.0, 300.0, 64e-6
NBLOCKS = 3


def _stream(nchans, nsamp, maxshift, seed):
    from mdsm_gb300 import synth
    total = NBLOCKS * nsamp + maxshift
    x = synth.gaussian_u8(nchans, total, seed)
    rng = np.random.default_rng(seed + 100)
    synth.inject(x, FCH1, -BW / nchans, TSAMP,
                 [(int(rng.integers(100, total - 3000)), 40.0, 8, 30.0)], K=4148.741601)
    return x


def _blocks(x, nsamp, maxshift):
    out = [x[:, : nsamp + maxshift]]
    for k in range(1, NBLOCKS):
        out.append(x[:, k * nsamp + maxshift:(k + 1) * nsamp + maxshift])
    return out


def _run(server_beams, order):
    from mdsm_gb300.serving import Server
    srv = Server(max_inflight=3, nwidths=7, threshold=6.0, cand_cap=2048)
    ids, streams = [], []
    for nchans, nsamp, segs, seed in server_beams:
        b = srv.add_beam(nchans, FCH1, -BW / nchans, TSAMP, nsamp, segs)
        info = srv.beam_info(b)
        x = _stream(nchans, nsamp, info.maxshift, seed)
        ids.append(b)
        streams.append(_blocks(x, nsamp, info.maxshift))
    n = 0
    for beam_pos, k in order:
        if beam_pos < len(ids):
            assert srv.submit(ids[beam_pos], streams[beam_pos][k]) is not None
            n += 1
    res = srv.results(n)
    srv.drain()
    stats = srv.stats()
    srv.close()
    assert len(res) == n
    out = {}
    for r in res:
        out[(r["beam"], r["block"])] = r["cands"]
    return out, stats


def test_alone_equals_mixed_and_oracle(lib, orc, cuda):
    mixed_order = [(b, k) for k in range(NBLOCKS) for b in (2, 0, 1)]
    mixed, stats = _run(BEAMS, mixed_order)
    assert stats["completed"] == len(mixed_order)
    assert stats["p99_latency_s"] >= stats["p50_latency_s"] > 0
    for pos, beam in enumerate(BEAMS):
        alone, _ = _run([beam], [(0, k) for k in range(NBLOCKS)])
        nchans, nsamp, segs, seed = beam
        S = orc.shift_table(nchans, FCH1, -BW / nchans, TSAMP, segs)
        x = _stream(nchans, nsamp, int(S.max()), seed)
        for k in range(NBLOCKS):
            a = alone[(0, k)]
            m = mixed[(pos, k)]
            assert np.array_equal(a, m), (pos, k)
            y = orc.dedisperse(x[:, k * nsamp:], S, nsamp)
            dm, samp, wid, snr = orc.boxcar_detect(y, 7, 6.0)
            assert np.array_equal(a["dm_idx"], dm) and np.array_equal(a["sample"], samp)
            assert np.array_equal(a["width"], wid) and np.array_equal(a["snr"], snr)
    # the injected pulses are found
    assert sum(len(v) for v in mixed.values()) > 0


def test_hbm_budget_refuses_beams(lib, cuda):
    from mdsm_gb300 import MdsmError
    from mdsm_gb300.serving import Server
    srv = Server(hbm_budget_bytes=1 << 20, max_inflight=1)
    with pytest.raises(MdsmError) as e:
        srv.add_beam(256, FCH1, -BW / 256, TSAMP, 4096, [(0.0, 0.5, 64)])
    assert e.value.status == 7
    srv.close()


def test_host_staging_budget_defers_blocks(lib, cuda):
    from mdsm_gb300 import synth
    from mdsm_gb300.serving import Server
    nchans, nsamp = 64, 1024
    srv = Server(host_stage_bytes=nchans * (nsamp + 2000), max_inflight=1)
    b = srv.add_beam(nchans, FCH1, -BW / nchans, TSAMP, nsamp, [(0.0, 1.0, 32)])
    ms = srv.beam_info(b).maxshift
    x = synth.gaussian_u8(nchans, 4 * nsamp + ms, 5)
    assert srv.submit(b, x[:, : nsamp + ms]) is not None
    refused = srv.submit(b, x[:, nsamp + ms: 2 * nsamp + ms])
    if refused is None:  # staging still held by block 0
        srv.drain()
        assert len(srv.results(1)) == 1
        assert srv.submit(b, x[:, nsamp + ms: 2 * nsamp + ms]) is not None
    srv.drain()
    st = srv.stats()
    srv.close()
    assert st["completed"] >= 1


def test_acquire_commit_equals_submit(lib, cuda):
    """The zero-copy form (write into the server's pinned staging buffer, then commit) gives the
    same candidates as submit; staging buffers are reused block after block."""
    from mdsm_gb300.serving import Server
    nchans, nsamp, segs, seed = BEAMS[1]

    def run(zero_copy):
        # room for two staging buffers (maxshift is 507 here): the third block must reuse one
        srv = Server(max_inflight=2, nwidths=7, threshold=6.0, cand_cap=2048,
                     host_stage_bytes=nchans * (2 * nsamp + 600))
        b = srv.add_beam(nchans, FCH1, -BW / nchans, TSAMP, nsamp, segs)
        ms = srv.beam_info(b).maxshift
        assert 2 * nsamp + ms <= 2 * nsamp + 600 < 3 * nsamp
        blocks = _blocks(_stream(nchans, nsamp, ms, seed), nsamp, ms)
        out = []
        for k, blk in enumerate(blocks):
            while True:
                if zero_copy:
                    view = srv.acquire(b)
                    if view is not None:
                        assert view.shape == blk.shape and view.dtype == blk.dtype
                        view[...] = blk
                        srv.commit(b)
                        break
                elif srv.submit(b, blk) is not None:
                    break
                out += srv.results(1)  # staging full: take a result, which frees a buffer
        out += srv.results(NBLOCKS - len(out))
        srv.drain()
        srv.close()
        return {r["block"]: r["cands"] for r in out}

    a, z = run(False), run(True)
    assert sorted(a) == sorted(z) == list(range(NBLOCKS))
    for k in a:
        assert np.array_equal(a[k], z[k])
