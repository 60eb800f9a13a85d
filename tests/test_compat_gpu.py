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
