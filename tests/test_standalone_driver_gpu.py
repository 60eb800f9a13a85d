"""The reference's standalone call sequence as a C++ program (tests/drivers/standalone_driver.cpp)
compiled against include/dedispersion_manager.h and run on an 8-bit sigproc file with one
dispersed pulse: the program sees the reference's block protocol (first next_chunk reports no
output, each later one the previous block, a zero read stops after one more report) and the
candidate file it leaves names the pulse's DM and arrival time."""
import os
import struct
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

NCHANS, NSAMP, TSAMP, FCH1, FOFF = 256, 8192, 64e-6, 1500.0, -1.171875
OBS = """<observation>
    <frequencies top="1500.0" offset="-1.171875" />
    <dm lowDM="0" numDMs="128" dmStep="1.0" useBruteForce="1" useL1Cache="1" />
    <samples number="8192" />
    <channels number="256" subbands="16" />
    <timing tsamp="0.000064" />
    <detection threshold="6" />
    <output filePrefix="cands" baseDirectory="{dir}" secondsPerFile="600"
            usePCTime="0" singleFileMode="1" />
</observation>
"""


def _filterbank(path, x):
    """Writes a sigproc filterbank: keyword header, then time-major 8-bit spectra."""
    def s(text):
        return struct.pack("<i", len(text)) + text.encode()
    b = s("HEADER_START") + s("source_name") + s("synthetic")
    for k, v in (("machine_id", 0), ("telescope_id", 0), ("data_type", 1), ("nchans", NCHANS),
                 ("nbits", 8), ("nifs", 1)):
        b += s(k) + struct.pack("<i", v)
    for k, v in (("fch1", FCH1), ("foff", FOFF), ("tsamp", TSAMP), ("tstart", 60000.0)):
        b += s(k) + struct.pack("<d", v)
    b += s("HEADER_END")
    with open(path, "wb") as f:
        f.write(b + np.ascontiguousarray(x.T).tobytes())


def test_standalone_driver(lib, cuda, tmp_path):
    from mdsm_gb300 import _lib, synth
    nspec = 3 * NSAMP + 3000  # three whole blocks plus a maxshift tail (2075 samples)
    x = synth.gaussian_u8(NCHANS, nspec, 21)
    synth.inject(x, FCH1, FOFF, TSAMP, [(12000, 73.0, 6, 60.0)], K=4148.741601)
    fil = tmp_path / "pulse.fil"
    _filterbank(fil, x)
    obs = tmp_path / "obs.xml"
    obs.write_text(OBS.format(dir=str(tmp_path)))
    exe = tmp_path / "driver"
    libdir = os.path.dirname(_lib.LIB_PATH)
    subprocess.run(["g++", "-O2", "-I", os.path.join(ROOT, "include"), "-o", str(exe),
                    os.path.join(ROOT, "tests", "drivers", "standalone_driver.cpp"),
                    "-L" + libdir, "-lmdsm_gb300", "-Wl,-rpath," + libdir], check=True)
    r = subprocess.run([str(exe), str(fil), str(obs)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "blocks 4 outputs 3 samples %d" % (3 * NSAMP) in r.stdout, r.stdout
    rows = [list(map(float, ln.split(",")[:3])) for ln in open(tmp_path / "cands.dat")
            if ln.strip()]
    assert rows, "no candidates"
    best = max(rows, key=lambda v: v[2])
    assert abs(best[1] - 73.0) <= 2.0
    assert abs(best[0] / TSAMP - 12000) <= 10
