"""Sigproc filterbank files: header reading, raw block reading, device unpack + corner turn,
and the dedispersed-series writer (the reference's DedispersedDataWriter)."""
import ctypes

import numpy as np

from ._lib import DTYPES, SigprocHeader, check, load
from .api import _stream_ptr


def read_header(path):
    h = SigprocHeader()
    check(load().mdsm_sigproc_read_header(str(path).encode(), ctypes.byref(h)))
    return h


def read_raw(path, header, first_spectrum, nspectra):
    """Raw bytes of nspectra spectra starting at first_spectrum (time-major, nbits packed)."""
    per = header.nchans * header.nifs * header.nbits // 8
    return np.fromfile(path, dtype=np.uint8, count=nspectra * per,
                       offset=header.header_bytes + first_spectrum * per)


def unpack_device(d_raw, nspectra, nchans, nbits, d_out, out_dtype, out_stride, col0=0,
                  invert=False, stream=None):
    """Unpack and corner-turn raw spectra (torch uint8 tensor on the device) into the
    channel-major device buffer d_out at columns [col0, col0 + nspectra)."""
    check(load().mdsm_unpack_device(ctypes.c_void_p(d_raw.data_ptr()), int(nspectra),
                                    int(nchans), int(nbits), int(bool(invert)),
                                    ctypes.c_void_p(d_out.data_ptr()), DTYPES[out_dtype],
                                    int(out_stride), int(col0), _stream_ptr(stream)))


def write_series(path, series, fch1, foff, tsamp, tstart=0.0, append=False):
    """One dedispersed series as a 32-bit, one-channel sigproc file
    (src/pelican-mdsm/modules/DedispersedDataWriter.cpp:49-63,105-135)."""
    if not append:
        check(load().mdsm_sigproc_write_series_header(str(path).encode(), float(fch1),
                                                      float(foff), float(tsamp), float(tstart)))
    with open(path, "ab") as f:
        f.write(np.ascontiguousarray(series, dtype=np.float32).tobytes())
