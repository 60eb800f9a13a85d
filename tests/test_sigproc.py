"""Sigproc ingest: header reader against the reference's read_header (compiled from the MDSM
tree into oracle/_ref where present) and known values; series-file writer round trip; device
unpack + corner turn against the oracle's read_block restatement (GPU)."""
import ctypes
import os
import struct

import numpy as np
import pytest


def _s(b, text):
    b += struct.pack("<i", len(text)) + text.encode()
    return b


def make_header(path, nchans=64, nbits=8, with_strings=True, telescope=True):
    b = b""
    b = _s(b, "HEADER_START")
    if with_strings:
        b = _s(b, "source_name")
        b = _s(b, "B0531+21")
        b = _s(b, "rawdatafile")
        b = _s(b, "crab.raw")
    for k, v in (("machine_id", 10), ("telescope_id", 4), ("data_type", 1), ("nchans", nchans),
                 ("nbits", nbits), ("nifs", 1), ("nbeams", 13), ("ibeam", 2)):
        b = _s(b, k) + struct.pack("<i", v)
    for k, v in (("fch1", 1500.0), ("foff", -0.390625), ("tsamp", 64e-6), ("tstart", 58000.25),
                 ("src_raj", 53431.9), ("src_dej", 220052.1), ("refdm", 56.8)):
        b = _s(b, k) + struct.pack("<d", v)
    if telescope:
        b = _s(b, "Telescope")
        b = _s(b, "Lovell")
    b = _s(b, "HEADER_END")
    with open(path, "wb") as f:
        f.write(b)
    return len(b)


def read(path):
    from mdsm_gb300 import _lib
    h = _lib.SigprocHeader()
    _lib.check(_lib.load().mdsm_sigproc_read_header(str(path).encode(), ctypes.byref(h)))
    return h


def test_header_fields(lib, tmp_path):
    p = tmp_path / "a.fil"
    n = make_header(p, telescope=False)
    h = read(p)
    assert (h.nchans, h.nbits, h.nifs, h.machine_id, h.telescope_id, h.nbeams, h.ibeam) == \
        (64, 8, 1, 10, 4, 13, 2)
    assert (h.fch1, h.foff, h.tsamp, h.tstart, h.refdm) == (1500.0, -0.390625, 64e-6, 58000.25,
                                                           56.8)
    assert h.source_name == b"B0531+21" and h.rawdatafile == b"crab.raw"
    assert h.header_bytes == n


def test_header_matches_reference_reader(lib, orc, tmp_path):
    if not orc.ref_host_available():
        pytest.skip("reference host code not built here")
    h_ref = ctypes.CDLL(orc.REF_HOST_SO)
    for telescope in (False, True):
        p = tmp_path / ("b%d.fil" % telescope)
        make_header(p, nchans=512, nbits=2, telescope=telescope)
        ints = (ctypes.c_int * 8)()
        dbls = (ctypes.c_double * 7)()
        tot = ctypes.c_longlong()
        src = ctypes.create_string_buffer(100)
        assert h_ref.ref_read_header(str(p).encode(), ints, dbls, ctypes.byref(tot), src) == 0
        h = read(p)
        assert list(ints) == [h.nchans, h.nbits, h.nifs, h.machine_id, h.telescope_id,
                              h.data_type, h.nbeams, h.ibeam]
        assert list(dbls) == [h.tstart, h.tsamp, h.fch1, h.foff, h.src_raj, h.src_dej, h.refdm]
        assert tot.value == h.header_bytes   # including the reference's Telescope accounting
        assert src.value == h.source_name


def test_unknown_keyword_is_an_error(lib, tmp_path):
    from mdsm_gb300 import MdsmError
    p = tmp_path / "bad.fil"
    b = _s(b"", "HEADER_START")
    b = _s(b, "no_such_key")
    b = _s(b, "HEADER_END")
    p.write_bytes(b)
    with pytest.raises(MdsmError) as e:
        read(p)
    assert e.value.status == 8


def test_series_writer_round_trip(lib, tmp_path):
    from mdsm_gb300 import sigproc
    p = tmp_path / "dm_56.8.fil"
    y = np.arange(1000, dtype=np.float32) * np.float32(0.5)
    sigproc.write_series(p, y, fch1=1500.0, foff=-300.0, tsamp=64e-6)
    h = read(p)
    assert (h.nchans, h.nbits, h.nifs, h.data_type) == (1, 32, 1, 1)
    data = np.fromfile(p, dtype=np.float32, offset=h.header_bytes)
    assert np.array_equal(data, y)


@pytest.mark.gpu
@pytest.mark.parametrize("nbits", [1, 2, 4, 8, 16, 32])
@pytest.mark.parametrize("invert", [0, 1])
def test_device_unpack_corner_turn(lib, orc, cuda, nbits, invert):
    from mdsm_gb300 import sigproc
    torch = cuda
    nchans, nspec = 96, 1000
    nbytes = nchans * nspec * nbits // 8
    raw = np.random.default_rng(nbits).integers(0, 256, nbytes, dtype=np.uint8)
    if nbits == 32:
        raw = np.random.default_rng(1).standard_normal(nchans * nspec).astype(np.float32).view(
            np.uint8)
    want = orc.unpack(raw, nbits).reshape(nspec, nchans).T
    if invert:
        want = want[::-1]
    dtype = {8: "u8", 16: "u16", 32: "f32"}.get(nbits, "u8")
    stride, col0 = 1200, 37
    out = torch.zeros((nchans, stride), dtype={"u8": torch.uint8, "u16": torch.uint16,
                                               "f32": torch.float32}[dtype], device="cuda")
    sigproc.unpack_device(torch.from_numpy(raw).cuda(), nspec, nchans, nbits, out, dtype,
                          stride, col0, invert=bool(invert))
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    assert np.array_equal(got[:, col0:col0 + nspec].astype(np.float32), want)
    assert not got[:, :col0].any() and not got[:, col0 + nspec:].any()


@pytest.mark.gpu
@pytest.mark.parametrize("invert", [0, 1])
def test_device_unpack_signed_int16(lib, cuda, invert):
    """16-bit samples unpacked to int16 read as two's-complement signed (the int16 data form),
    little-endian as the file stores them."""
    from mdsm_gb300 import sigproc
    torch = cuda
    nchans, nspec, stride, col0 = 80, 777, 900, 5
    raw = np.random.default_rng(16).integers(0, 256, nchans * nspec * 2, dtype=np.uint8)
    raw[:4] = [0x00, 0x80, 0xFF, 0x7F]  # -32768 and 32767
    want = raw.view("<i2").reshape(nspec, nchans).T
    if invert:
        want = want[::-1]
    out = torch.zeros((nchans, stride), dtype=torch.int16, device="cuda")
    sigproc.unpack_device(torch.from_numpy(raw).cuda(), nspec, nchans, 16, out, "i16", stride,
                          col0, invert=bool(invert))
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    assert np.array_equal(got[:, col0:col0 + nspec], want)
    assert not got[:, :col0].any() and not got[:, col0 + nspec:].any()
