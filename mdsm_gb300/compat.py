"""The reference's stage interface under its own names (src/mdsm/dedispersion_manager.h:7-12),
over the C ABI's compatibility functions.  One global instance, as in the reference."""
import ctypes

import numpy as np

from ._lib import SURVEY, Candidate, load


def processSurveyParameters(filepath):
    """Parse an observation XML file into a SURVEY (src/mdsm/dedispersion_manager.cpp:40-199).
    Returns a ctypes pointer to the library-allocated struct."""
    s = load().mdsm_processSurveyParameters(str(filepath).encode())
    if not s:
        raise RuntimeError(load().mdsm_last_error().decode())
    return s


def initialiseMDSM(survey):
    """Returns the library-owned input buffer as a numpy view [nchans][nsamp + maxshift]."""
    p = load().mdsm_initialiseMDSM(survey)
    if not p:
        raise RuntimeError(load().mdsm_last_error().decode())
    s = survey.contents
    pitch = _pitch(s)
    return np.ctypeslib.as_array(p, shape=(s.nchans, pitch))


def _pitch(s):
    return s.nsamp + s.maxshift


_KEEP = []  # caller noise statistics stay alive until the block that uses them is processed


def next_chunk(data_read, timestamp=0.0, blockRate=0.0, mean=None, rms=None):
    """Returns (output [ndms][nsamp] view or None, samples).  mean/rms: the block's noise
    statistics, one value per samplesPerChunk samples (float32 arrays), or None."""
    samples = ctypes.c_uint()
    mp = rp = None
    if mean is not None and rms is not None:
        mean = np.ascontiguousarray(mean, np.float32)
        rms = np.ascontiguousarray(rms, np.float32)
        _KEEP[:] = [mean, rms]
        mp = mean.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        rp = rms.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    p = load().mdsm_next_chunk(int(data_read), ctypes.byref(samples), float(timestamp),
                               float(blockRate), mp, rp)
    if not p:
        return None, samples.value
    return p, samples.value


def output_view(ptr, survey):
    s = survey.contents
    return np.ctypeslib.as_array(ptr, shape=(s.tdms, s.nsamp))


def start_processing(data_read):
    return load().mdsm_start_processing(int(data_read))


def tearDownMDSM():
    load().mdsm_tearDownMDSM()


def blocks_8bit():
    """Blocks that ran on the 8-bit kernels (their float input was all integers 0..255)."""
    return load().mdsm_compat_blocks_8bit()


def candidates(cap=1 << 16):
    buf = (Candidate * cap)()
    n = load().mdsm_compat_candidates(buf, cap)
    from .api import CAND_DTYPE
    return np.frombuffer(buf, dtype=CAND_DTYPE, count=min(n, cap)).copy()
