"""The reference stage interface end to end: the call sequence of the standalone driver
(src/MDSM.cpp:137-169) over several blocks, with the overlap tail carried by the library."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OBS = """<observation>
    <frequencies top="1500.0" offset="-0.78125" />
    <dm lowDM="0" numDMs="96" dmStep="0.5" useBruteForce="1" useL1Cache="1" />
    <samples number="4096" />
    <channels number="128" subbands="16" />
    <timing tsamp="0.000064" />
    <detection threshold="6" />
    <output filePrefix="cands" baseDirectory="{dir}" secondsPerFile="600"
            usePCTime="0" singleFileMode="1" />
    <gpus ids="0" />
</observation>
"""


def test_standalone_call_sequence(lib, orc, cuda, tmp_path):
    from mdsm_gb300 import compat
    obs = tmp_path / "obs.xml"
    obs.write_text(OBS.format(dir=str(tmp_path)))
    survey = compat.processSurveyParameters(obs)
    s = survey.contents
    assert (s.nchans, s.tdms, s.nsamp, bool(s.useBruteForce)) == (128, 96, 4096, True)
    buf = compat.initialiseMDSM(survey)
    nsamp, ms = s.nsamp, s.maxshift
    nblocks = 3
    rng = np.random.default_rng(0)
    stream = rng.standard_normal((128, nblocks * nsamp + ms), dtype=np.float32)
    S = orc.shift_table(128, 1500.0, -0.78125, 0.000064, [(0.0, 0.5, 96)], mode="l1")
    assert int(S.max()) == ms
    outs = []
    for k in range(nblocks + 2):
        if k < nblocks:
            if k == 0:
                buf[:, : nsamp + ms] = stream[:, : nsamp + ms]
            else:
                buf[:, ms: ms + nsamp] = stream[:, k * nsamp + ms: (k + 1) * nsamp + ms]
            data_read = nsamp
        else:
            data_read = 0
        ptr, samples = compat.next_chunk(data_read, k * nsamp * 0.000064, 0.000064)
        if ptr is not None and samples:
            outs.append(compat.output_view(ptr, survey).copy())
        if not compat.start_processing(data_read):
            break
    compat.tearDownMDSM()
    assert len(outs) == nblocks
    for k, y in enumerate(outs):
        want = orc.dedisperse(stream[:, k * nsamp:], S, nsamp)
        assert np.array_equal(y, want), k
    assert os.path.exists(tmp_path / "cands.dat")


def test_candidate_file_rotation(lib, orc, cuda, tmp_path):
    """singleFileMode 0: a new candidate file, named by the block timestamp, once the samples
    written reach secondsPerFile (dedispersion_output.cpp:233-302); every candidate the
    detector reports lands in exactly one file."""
    from mdsm_gb300 import compat, synth
    obs = tmp_path / "obs.xml"
    obs.write_text(OBS.format(dir=str(tmp_path)).replace('secondsPerFile="600"',
                                                         'secondsPerFile="1"')
                   .replace('singleFileMode="1"', 'singleFileMode="0"'))
    survey = compat.processSurveyParameters(obs)
    s = survey.contents
    buf = compat.initialiseMDSM(survey)
    nsamp, ms, tsamp = s.nsamp, s.maxshift, 0.000064
    nblocks = 6  # 4 blocks of 0.262 s pass 1 s: blocks 0-3 in one file, 4-5 in the next
    x = synth.gaussian_f32(128, nblocks * nsamp + ms, 3)
    synth.inject(x, 1500.0, -0.78125, tsamp,
                 [(k * nsamp + 1000, 20.0, 4, 3.0) for k in range(nblocks)], K=4148.741601)
    t_start = 1.0e9
    block_s = nsamp * tsamp
    counts = []
    for k in range(nblocks + 2):
        if k < nblocks:
            if k == 0:
                buf[:, : nsamp + ms] = x[:, : nsamp + ms]
            else:
                buf[:, ms: ms + nsamp] = x[:, k * nsamp + ms: (k + 1) * nsamp + ms]
            data_read = nsamp
        else:
            data_read = 0
        compat.next_chunk(data_read, t_start + k * block_s, tsamp)
        if not compat.start_processing(data_read):
            break
        if data_read:
            counts.append(len(compat.candidates()))
    compat.tearDownMDSM()
    files = sorted(f for f in os.listdir(tmp_path) if f.startswith("cands_"))
    assert len(files) == 2, files
    assert all(f.endswith("_1.dat") for f in files)
    lines = [[ln for ln in open(tmp_path / f) if ln.strip()] for f in files]
    assert sum(counts) > 0
    assert len(lines[0]) == sum(counts[:4]) and len(lines[1]) == sum(counts[4:])
    for f, blocks in zip(lines, (range(0, 4), range(4, 6))):
        for ln in f:
            t = float(ln.split(",")[0])
            assert t_start + blocks[0] * block_s <= t < t_start + (blocks[-1] + 1) * block_s


def _run_blocks(compat, survey, x, nblocks, ts0, tsamp, stats=None, before_teardown=None):
    s = survey.contents
    buf = compat.initialiseMDSM(survey)
    nsamp, ms = s.nsamp, s.maxshift
    outs = []
    for k in range(nblocks + 2):
        if k < nblocks:
            if k == 0:
                buf[:, : nsamp + ms] = x[:, : nsamp + ms]
            else:
                buf[:, ms: ms + nsamp] = x[:, k * nsamp + ms: (k + 1) * nsamp + ms]
            data_read = nsamp
        else:
            data_read = 0
        st = stats(k) if (stats and k < nblocks) else (None, None)
        ptr, samples = compat.next_chunk(data_read, ts0 + k * nsamp * tsamp, tsamp, *st)
        if ptr is not None and samples:
            outs.append(compat.output_view(ptr, survey).copy())
        if not compat.start_processing(data_read):
            break
    if before_teardown:
        before_teardown()
    compat.tearDownMDSM()
    return outs


def test_caller_noise_statistics_lines(lib, orc, cuda, tmp_path):
    """next_chunk's mean/rms (as the Pelican module passes them) switch process_brute to its
    caller-statistics form: lines "time, DM, snr, mean, rms" equal to the oracle's."""
    from mdsm_gb300 import compat, synth
    obs = tmp_path / "obs.xml"
    obs.write_text(OBS.format(dir=str(tmp_path)))
    survey = compat.processSurveyParameters(obs)
    s = survey.contents
    s.samplesPerChunk = 512
    tsamp, nblocks = 0.000064, 2
    x = synth.gaussian_f32(128, nblocks * 4096 + 600, 5)
    synth.inject(x, 1500.0, -0.78125, tsamp, [(1500, 25.0, 4, 2.0), (5500, 30.0, 4, 2.0)],
                 K=4148.741601)
    rng = np.random.default_rng(6)
    stats = [((rng.standard_normal(8) * 0.2).astype(np.float32),
              rng.uniform(8.0, 12.0, 8).astype(np.float32)) for _ in range(nblocks)]
    outs = _run_blocks(compat, survey, x, nblocks, 100.0, tsamp, lambda k: stats[k])
    assert len(outs) == nblocks
    got = [tuple(float(v) for v in ln.split(",")) for ln in open(tmp_path / "cands.dat")
           if ln.strip()]
    want = []
    for k, y in enumerate(outs):
        dm, t, snr = orc.ref_detect_chunked(y, 0.0, 0.5, 6.0, stats[k][0], stats[k][1], 512)
        for d, tt, sn in zip(dm, t, snr):
            want.append((100.0 + k * 4096 * tsamp + tt * tsamp, 0.5 * d, sn,
                         stats[k][0][tt // 512], stats[k][1][tt // 512]))
    assert len(got) == len(want) > 0
    for a, b in zip(got, want):
        assert all(abs(u - v) <= 1e-6 * max(1.0, abs(v)) for u, v in zip(a, b)), (a, b)


OBS_SUB = """<observation>
    <frequencies top="1500.0" offset="-1.171875" />
    <dm lowDM="0" numDMs="0" dmStep="0" useBruteForce="0" />
    <samples number="4096" />
    <channels number="256" subbands="16" />
    <timing tsamp="0.000064" />
    <detection threshold="5" />
    <output filePrefix="sub" baseDirectory="{dir}" secondsPerFile="600"
            usePCTime="0" singleFileMode="1" />
    <passes>
        <pass><lowDm>0.0</lowDm><highDm>32.0</highDm><deltaDm>0.5</deltaDm>
              <downsample>1</downsample><subDm>4.0</subDm><numDms>64</numDms>
              <dmsPerCall>8</dmsPerCall><ncalls>8</ncalls></pass>
        <pass><lowDm>32.0</lowDm><highDm>96.0</highDm><deltaDm>2.0</deltaDm>
              <downsample>2</downsample><subDm>16.0</subDm><numDms>32</numDms>
              <dmsPerCall>8</dmsPerCall><ncalls>4</ncalls></pass>
    </passes>
</observation>
"""


def test_subband_stage_interface_detects(lib, orc, cuda, tmp_path):
    """Subband mode through the stage interface: process_subband's per-row statistics branch
    on the plan's own DMs, lines "time, DM, snr" with time counted in each pass's downsampled
    samples, equal to the oracle's detections on the returned series."""
    from mdsm_gb300 import compat, synth
    obs = tmp_path / "obs.xml"
    obs.write_text(OBS_SUB.format(dir=str(tmp_path)))
    survey = compat.processSurveyParameters(obs)
    tsamp, nblocks = 0.000064, 2
    x = synth.gaussian_f32(256, nblocks * 4096 + 4000, 9)
    synth.inject(x, 1500.0, -1.171875, tsamp, [(1000, 20.0, 6, 1.5), (6000, 60.0, 8, 1.5)],
                 K=4148.741601)
    outs = _run_blocks(compat, survey, x, nblocks, 50.0, tsamp)
    assert len(outs) == nblocks
    got = [tuple(float(v) for v in ln.split(",")) for ln in open(tmp_path / "sub.dat")
           if ln.strip()]
    import mdsm_gb300 as m
    want = []
    plan = m.SubbandPlan(256, 1500.0, -1.171875, tsamp, 4096, 16,
                         [dict(lowdm=0.0, highdm=32.0, dmstep=0.5, sub_dmstep=4.0, ncalls=8,
                               calldms=8),
                          dict(lowdm=32.0, highdm=96.0, dmstep=2.0, sub_dmstep=16.0, ncalls=4,
                               calldms=8, binsize=2)], in_dtype="f32", out_dtype="f32")
    dm_values = plan.dm_values()
    for k, y in enumerate(outs):
        row0 = 0
        for rows, b in ((64, 1), (32, 2)):
            dm, t, snr = orc.ref_detect_subband(y[row0:row0 + rows], 4096 // b,
                                                dm_values[row0:row0 + rows], 5.0)
            for d, tt, sn in zip(dm, t, snr):
                want.append((50.0 + k * 4096 * tsamp + tt * tsamp * b, dm_values[row0 + d], sn,
                             row0 + d))
            row0 += rows
    # the library writes each block's candidates sorted by (row, sample)
    want_sorted = []
    for k in range(nblocks):
        blk = [w for w in want if 50.0 + k * 4096 * tsamp <= w[0] < 50.0 + (k + 1) * 4096 * tsamp]
        want_sorted += sorted(blk, key=lambda w: (w[3], w[0]))
    assert len(got) == len(want_sorted) > 0
    for a, b in zip(got, want_sorted):
        assert abs(a[0] - b[0]) <= 1e-6 and abs(a[1] - b[1]) <= 1e-5 and abs(a[2] - b[2]) <= 1e-5


def test_integer_blocks_take_8bit_kernels(lib, orc, cuda, tmp_path):
    """Float blocks whose samples are all integers 0..255 (8-bit data handed in as floats, as
    the reference's file reader does) run on the 8-bit kernels with the float path's output
    bit for bit; a block holding one fraction runs on the float kernels."""
    from mdsm_gb300 import compat
    obs = tmp_path / "obs.xml"
    obs.write_text(OBS.format(dir=str(tmp_path)))
    survey = compat.processSurveyParameters(obs)
    nsamp, tsamp, nblocks = 4096, 0.000064, 3
    S = orc.shift_table(128, 1500.0, -0.78125, tsamp, [(0.0, 0.5, 96)], mode="l1")
    ms = int(S.max())
    x = np.random.default_rng(5).integers(0, 256, (128, nblocks * nsamp + ms)).astype(np.float32)
    x[:3, :50] = 255.0
    x[7, nsamp + ms + 10] = 3.5  # among block 1's new samples, not in block 2's tail
    seen = {}
    outs = _run_blocks(compat, survey, x, nblocks, 0.0, tsamp,
                       before_teardown=lambda: seen.setdefault("n", compat.blocks_8bit()))
    assert seen["n"] == nblocks - 1
    assert len(outs) == nblocks
    for k, y in enumerate(outs):
        assert np.array_equal(y, orc.dedisperse(x[:, k * nsamp:], S, nsamp)), k


OBS_SUB1 = OBS_SUB.replace("""        <pass><lowDm>32.0</lowDm><highDm>96.0</highDm><deltaDm>2.0</deltaDm>
              <downsample>2</downsample><subDm>16.0</subDm><numDms>32</numDms>
              <dmsPerCall>8</dmsPerCall><ncalls>4</ncalls></pass>
""", "")


def test_integer_blocks_take_8bit_kernels_subband(lib, orc, cuda, tmp_path):
    """The same for a subband plan without downsampled passes: the 8-bit stages (uint16
    subband series) give the float stages' output bit for bit."""
    import mdsm_gb300 as m
    from mdsm_gb300 import compat
    assert OBS_SUB1 != OBS_SUB
    obs = tmp_path / "obs.xml"
    obs.write_text(OBS_SUB1.format(dir=str(tmp_path)))
    survey = compat.processSurveyParameters(obs)
    nsamp, tsamp, nblocks = 4096, 0.000064, 2
    pas = dict(lowdm=0.0, highdm=32.0, dmstep=0.5, sub_dmstep=4.0, ncalls=8, calldms=8)
    plan = m.SubbandPlan(256, 1500.0, -1.171875, tsamp, nsamp, 16, [pas], in_dtype="f32",
                         out_dtype="f32")
    S1, S2 = plan.stage_tables()
    nch, stride = plan.input_shape()
    x = np.random.default_rng(6).integers(0, 256, (256, nblocks * nsamp + stride)).astype(
        np.float32)
    seen = {}
    outs = _run_blocks(compat, survey, x, nblocks, 0.0, tsamp,
                       before_teardown=lambda: seen.setdefault("n", compat.blocks_8bit()))
    assert seen["n"] == nblocks and len(outs) == nblocks
    n1 = nsamp + int(S2.max())
    for k, y in enumerate(outs):
        _, want = orc.subband_dedisperse(x[:, k * nsamp: k * nsamp + stride], S1, S2, 16, nsamp,
                                         n1, pas["calldms"])
        assert np.array_equal(y, want), k


def test_exit_with_a_block_in_flight(lib, cuda, tmp_path):
    """A caller that exits right after start_processing, without tearDownMDSM, exits cleanly
    (the block's worker is joined at exit)."""
    import subprocess
    import sys
    obs = tmp_path / "obs.xml"
    obs.write_text(OBS.format(dir=str(tmp_path)))
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = (
        "import numpy as np\n"
        "from mdsm_gb300 import compat\n"
        f"s = compat.processSurveyParameters({str(obs)!r})\n"
        "buf = compat.initialiseMDSM(s)\n"
        "buf[:] = 1.0\n"
        "compat.next_chunk(s.contents.nsamp, 0.0, 0.000064)\n"
        "assert compat.start_processing(s.contents.nsamp) == 1\n"
        "print('submitted', flush=True)\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=root, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "submitted" in r.stdout


def test_integer_blocks_with_downsampled_passes_stay_float(lib, cuda, tmp_path):
    """A subband plan with a downsampled pass keeps integer-valued float blocks on the float
    kernels (its binning averages samples into fractions); the output equals the float plan
    run directly."""
    import mdsm_gb300 as m
    from mdsm_gb300 import compat
    torch = cuda
    obs = tmp_path / "obs.xml"
    obs.write_text(OBS_SUB.format(dir=str(tmp_path)))
    survey = compat.processSurveyParameters(obs)
    nsamp, tsamp, nblocks = 4096, 0.000064, 2
    x = np.random.default_rng(8).integers(0, 256, (256, nblocks * nsamp + 8192)).astype(
        np.float32)
    seen = {}
    outs = _run_blocks(compat, survey, x, nblocks, 0.0, tsamp,
                       before_teardown=lambda: seen.setdefault("n", compat.blocks_8bit()))
    assert seen["n"] == 0 and len(outs) == nblocks
    plan = m.SubbandPlan(256, 1500.0, -1.171875, tsamp, nsamp, 16,
                         [dict(lowdm=0.0, highdm=32.0, dmstep=0.5, sub_dmstep=4.0, ncalls=8,
                               calldms=8),
                          dict(lowdm=32.0, highdm=96.0, dmstep=2.0, sub_dmstep=16.0, ncalls=4,
                               calldms=8, binsize=2)], in_dtype="f32", out_dtype="f32")
    nch, stride = plan.input_shape()
    for k, y in enumerate(outs):
        d_in = plan.alloc_input()
        blk = np.zeros((nch, stride), np.float32)
        w = min(nsamp + plan.info.maxshift, x.shape[1] - k * nsamp)
        blk[:, :w] = x[:, k * nsamp: k * nsamp + w]
        d_in[: blk.size].copy_(torch.from_numpy(blk.ravel()))
        d_out = plan.alloc_output()
        plan.dedisperse_device(d_in, d_out)
        torch.cuda.synchronize()
        want = d_out.cpu().numpy().reshape(y.shape)
        # pass 1: 64 rows of nsamp samples; pass 2 (downsample 2): 32 rows of nsamp / 2
        assert np.array_equal(y[:64], want[:64]), k
        assert np.array_equal(y[64:96, : nsamp // 2], want[64:96, : nsamp // 2]), k
