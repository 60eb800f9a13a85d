"""The batched form: uneven beams in one persistent launch (and as a replayed CUDA graph), each
beam's series equal to the oracle's; with clipping and detection fused into the pass."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BEAMS = [  # nchans, nsamp, segments
    (1024, 1 << 12, [(0.0, 0.5, 96)]),
    (256, 1 << 13, [(0.0, 0.25, 64), (16.0, 0.5, 32)]),
    (1024, 3000, [(10.0, 1.0, 40)]),
    (256, 1 << 11, [(0.0, 2.0, 33)]),
    (512, 5000, [(0.0, 0.3, 70)]),
]
FCH1, BW, TSAMP = 1500.0, 300.0, 64e-6


# Beams whose DM plans all fit the packed kernels' staging (the fused launch's requirement);
# BEAMS[3]'s 2.0 step is too wide for it and runs on the generic kernel.
FUSABLE = BEAMS[:3] + [(256, 1 << 11, [(0.0, 0.5, 33)])] + BEAMS[4:]


def _setup(torch, seed=0, beams=None):
    import mdsm_gb300 as m
    plans, xs, d_in, d_out = [], [], [], []
    for i, (nchans, nsamp, segs) in enumerate(beams or BEAMS):
        p = m.BrutePlan(nchans, FCH1, -BW / nchans, TSAMP, nsamp, segs, in_dtype="u8",
                        out_dtype="i32")
        nch, stride = p.input_shape()
        x = np.random.default_rng(seed + i).integers(0, 256, (nch, stride), dtype=np.uint8)
        t = p.alloc_input()
        t[: x.size].copy_(torch.from_numpy(x.ravel()))
        plans.append(p)
        xs.append(x)
        d_in.append(t)
        d_out.append(p.alloc_output())
    return plans, xs, d_in, d_out


@pytest.mark.parametrize("graph", [False, True])
def test_batch_matches_oracle_for_every_launch_shape(lib, orc, cuda, graph):
    from mdsm_gb300.batch import Batch
    torch = cuda
    plans, xs, d_in, d_out = _setup(torch)
    want = [orc.dedisperse(x, p.shift_table(), p.info.nsamp) for p, x in zip(plans, xs)]
    b = Batch(plans)
    b.set_buffers(d_in, d_out)
    for choice in (0, 1, 2, 0):
        _set_choice(b, choice)
        for t in d_out:
            t.zero_()
        b.run(graph=graph)
        torch.cuda.synchronize()
        for k, t in enumerate(d_out):
            assert np.array_equal(t.cpu().numpy(), want[k]), (choice, k)
    if not graph:
        assert b.last_launches >= 1
    b.close()


def _set_choice(b, choice):
    """Force a launch shape through the autotune cache."""
    import os
    import tempfile
    from mdsm_gb300 import _lib
    import ctypes
    fd, path = tempfile.mkstemp()
    os.close(fd)
    os.environ["MDSM_AUTOTUNE_CACHE"] = path
    # probe the key by tuning once into an empty cache, then overwrite the choice
    c = ctypes.c_int()
    _lib.check(_lib.load().mdsm_batch_autotune(b._h, None, ctypes.byref(c)))
    key = open(path).read().rsplit(" ", 1)[0]
    with open(path, "w") as f:
        f.write("%s %d\n" % (key, choice))
    _lib.check(_lib.load().mdsm_batch_autotune(b._h, None, ctypes.byref(c)))
    assert c.value == choice
    os.unlink(path)
    del os.environ["MDSM_AUTOTUNE_CACHE"]


def test_batch_autotune_and_fused_clip_detect(lib, orc, cuda):
    from mdsm_gb300 import synth
    from mdsm_gb300.batch import Batch
    torch = cuda
    plans, xs, d_in, d_out = _setup(torch, seed=10)
    # Gaussian data with a pulse per beam, so clipping and detection both do something
    for k, (p, t) in enumerate(zip(plans, d_in)):
        nch, stride = p.input_shape()
        x = synth.gaussian_u8(nch, stride, 40 + k)
        synth.inject(x, FCH1, -BW / nch, TSAMP, [(500 + 100 * k, 20.0, 4, 40.0)],
                     K=4148.741601)
        x[:, 200] = 255  # a broadband impulse for the spectrum clip
        xs[k] = x
        t[: x.size].copy_(torch.from_numpy(x.ravel()))
    b = Batch(plans)
    b.set_buffers(d_in, d_out)
    b.enable_clip(4.0, 4.0)
    b.enable_detect(nwidths=6, threshold=6.0, cap=4096)
    choice = b.autotune()
    assert choice in (0, 1, 2)
    # autotune does not clip; restore the inputs and run the fused pass once as a graph
    for x, t in zip(xs, d_in):
        t[: x.size].copy_(torch.from_numpy(x.ravel()))
    b.run(graph=True)      # ordinary launches; the pass is captured for the next call
    torch.cuda.synchronize()
    for x, t in zip(xs, d_in):
        t[: x.size].copy_(torch.from_numpy(x.ravel()))
    for t in d_out:
        t.zero_()
    b.run(graph=True)      # the captured graph
    torch.cuda.synchronize()
    for k, (p, x) in enumerate(zip(plans, xs)):
        info = p.info
        xc = orc.rfi_clip(x.copy(), info.nsamp + info.maxshift, 4.0, 4.0)
        y = orc.dedisperse(xc, p.shift_table(), info.nsamp)
        assert np.array_equal(d_out[k].cpu().numpy(), y), k
        dm, samp, wid, snr = orc.boxcar_detect(y, 6, 6.0)
        c = b.candidates(k)
        assert np.array_equal(c["dm_idx"], dm) and np.array_equal(c["sample"], samp)
        assert np.array_equal(c["width"], wid) and np.array_equal(c["snr"], snr)
    b.close()


def _restore(torch, xs, d_in):
    for x, t in zip(xs, d_in):
        t[: x.size].copy_(torch.from_numpy(x.ravel()))


@pytest.mark.parametrize("graph", [False, True])
def test_fused_launch_every_shape_equals_oracle(lib, orc, cuda, graph):
    """The fused form (every beam uint8 -> int32, widths 1..256): clip, dedispersion and search
    in one persistent launch.  For every tile shape and item order the autotuner can pick, the
    clipped inputs, the series and each beam's candidates equal the oracle's clip, dedispersion
    and boxcar search."""
    from mdsm_gb300 import synth
    from mdsm_gb300.batch import Batch, choice_info
    torch = cuda
    plans, xs, d_in, d_out = _setup(torch, seed=20, beams=FUSABLE)
    for k, p in enumerate(plans):
        nch, stride = p.input_shape()
        x = synth.gaussian_u8(nch, stride, 60 + k)
        synth.inject(x, FCH1, -BW / nch, TSAMP, [(400 + 150 * k, 15.0, 3 + k, 45.0)],
                     K=4148.741601)
        x[:, 100 + 7 * k] = 255   # broadband impulses for the spectrum clip
        x[3 + k, ::50] = 0        # a channel with dropouts for the channel clip
        xs[k] = x
    _restore(torch, xs, d_in)
    want = []
    for p, x in zip(plans, xs):
        info = p.info
        xc = orc.rfi_clip(x.copy(), info.nsamp + info.maxshift, 4.0, 4.0)
        y = orc.dedisperse(xc, p.shift_table(), info.nsamp)
        want.append((xc, y, orc.boxcar_detect(y, 9, 6.0)))
    b = Batch(plans)
    b.set_buffers(d_in, d_out)
    b.enable_clip(4.0, 4.0)
    b.enable_detect(nwidths=9, threshold=6.0, cap=8192)
    ran = 0
    for choice in range(10, 18):
        _set_choice(b, choice)
        assert choice_info(choice)["fused"] == 1
        for rep in range(2):  # (graph: the first run captures, the second replays)
            _restore(torch, xs, d_in)
            for t in d_out:
                t.zero_()
            b.run(graph=graph)
            torch.cuda.synchronize()
        if not graph:
            # one fused launch, plus the own launches of any beam this shape cannot stage
            assert b.last_launches >= 1
            info_k = p.info
            xc, y, (dm, samp, wid, snr) = want[k]
            nch, stride = p.input_shape()
            ncols = info_k.nsamp + info_k.maxshift
            got_in = d_in[k][: nch * stride].view(nch, stride)[:, :ncols]
            assert np.array_equal(got_in.cpu().numpy(), xc[:, :ncols]), (choice, k)
            assert np.array_equal(d_out[k].cpu().numpy(), y), (choice, k)
            c = b.candidates(k)
            assert len(dm) > 0
            assert np.array_equal(c["dm_idx"], dm) and np.array_equal(c["sample"], samp), (choice, k)
            assert np.array_equal(c["width"], wid) and np.array_equal(c["snr"], snr), (choice, k)
        ran += 1
    assert ran == 8
    b.close()


def test_fused_autotune_picks_the_fastest_candidate(lib, cuda):
    """Fusable beams: the autotuner times fused tile shapes and the unfused passes, all with
    the search on, and keeps the fastest."""
    from mdsm_gb300.batch import Batch, choice_info
    torch = cuda
    plans, xs, d_in, d_out = _setup(torch, seed=30, beams=FUSABLE)
    b = Batch(plans)
    b.set_buffers(d_in, d_out)
    b.enable_detect(nwidths=9, threshold=6.0, cap=1024)
    c = b.autotune()
    times = b.tune_times()
    fused = [ch for ch, _ in times if choice_info(ch)["fused"] == 1]
    assert fused and {0, 1, 2} <= {ch for ch, _ in times}
    assert c == min(times, key=lambda t: t[1])[0]
    for ch in fused:
        info = choice_info(ch)
        assert info["dm_block"] in (32, 38) and info["time_tile"] in (256, 512, 768)
    b.run(graph=True)
    torch.cuda.synchronize()
    b.close()


def test_beam_outside_the_fused_staging_runs_beside_it(lib, orc, cuda):
    """A beam whose DM plan is too wide for every fused tile shape (BEAMS[3], on the generic
    kernel) runs on its own clip, dedispersion and search launches after the fused launch of
    the others: every beam's series and candidates still equal the oracle's."""
    from mdsm_gb300 import synth
    from mdsm_gb300.batch import Batch, choice_info
    torch = cuda
    plans, xs, d_in, d_out = _setup(torch, seed=40)
    for k, p in enumerate(plans):
        nch, stride = p.input_shape()
        x = synth.gaussian_u8(nch, stride, 80 + k)
        synth.inject(x, FCH1, -BW / nch, TSAMP, [(300 + 100 * k, 12.0, 2 + k, 45.0)],
                     K=4148.741601)
        xs[k] = x
    _restore(torch, xs, d_in)
    b = Batch(plans)
    b.set_buffers(d_in, d_out)
    b.enable_detect(nwidths=9, threshold=6.0, cap=4096)
    c = b.autotune()
    assert any(choice_info(ch)["fused"] == 1 for ch, _ in b.tune_times())
    for choice in (c, 10):
        _set_choice(b, choice)
        _restore(torch, xs, d_in)
        b.run(graph=False)
        torch.cuda.synchronize()
        if choice_info(choice)["fused"]:
            # the fused launch, then BEAMS[3]'s dedispersion, statistics and search
            assert b.last_launches > 1, b.last_launches
        for k, (p, x) in enumerate(zip(plans, xs)):
            y = orc.dedisperse(x, p.shift_table(), p.info.nsamp)
            assert np.array_equal(d_out[k].cpu().numpy(), y), (choice, k)
            dm, samp, wid, snr = orc.boxcar_detect(y, 9, 6.0)
            got = b.candidates(k)
            assert len(dm) > 0
            assert np.array_equal(got["dm_idx"], dm) and np.array_equal(got["sample"], samp), k
            assert np.array_equal(got["width"], wid) and np.array_equal(got["snr"], snr), k
    b.close()
