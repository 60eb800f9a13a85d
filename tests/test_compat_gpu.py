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
