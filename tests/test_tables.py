"""The library's host-side shift tables (the integer shifts the kernels index with) against
the oracle's restatement of the reference arithmetic, entry for entry."""
import ctypes

import numpy as np
import pytest

from mdsm_gb300 import _lib

MODES = ["l1", "l1_muladd", "opt", "opt_muladd", "fp64_trunc", "fp64_round"]
PLANS = [
    # nchans, fch1, foff, tsamp, segments
    (256, 1500.0, -0.390625, 64e-6, [(0.0, 0.2, 500)]),
    (4096, 1500.0, -300.0 / 4096, 64e-6,
     [(0.0, 0.244140625, 2048), (500.0, 0.48828125, 1024), (1000.0, 0.9765625, 1024)]),
    (1024, 1400.0, -400.0 / 1024, 1e-4, [(3.0, 0.37, 700)]),
    (128, 126.0, -6.0 / 128, 5e-6 * 128, [(0.0, 0.065, 128)]),
]


def lib_table(nchans, fch1, foff, tsamp, segs, mode):
    L = _lib.load()
    arr = (_lib.Segment * len(segs))(*[_lib.Segment(a, b, n) for a, b, n in segs])
    d = _lib.BruteDesc(nchans, fch1, foff, tsamp, 1024, arr, len(segs), _lib.SHIFT_MODES[mode],
                       0.0, 0, 1, 0, 0, 0)
    ndms = sum(n for _, _, n in segs)
    S = np.empty((ndms, nchans), np.int32)
    dmv = np.empty(ndms, np.float32)
    ms = ctypes.c_int()
    _lib.check(L.mdsm_brute_shift_table(ctypes.byref(d), S.ctypes.data_as(ctypes.c_void_p),
                                        dmv.ctypes.data_as(ctypes.c_void_p), ctypes.byref(ms)))
    return S, dmv, ms.value


@pytest.mark.parametrize("plan", PLANS)
@pytest.mark.parametrize("mode", MODES)
def test_brute_tables_match_oracle(lib, orc, plan, mode):
    nchans, fch1, foff, tsamp, segs = plan
    S, dmv, ms = lib_table(nchans, fch1, foff, tsamp, segs, mode)
    want = orc.shift_table(nchans, fch1, foff, tsamp, segs, mode=mode)
    assert np.array_equal(S, want)
    assert ms == want.max()


def test_dmshifts_and_dmdelay(lib, orc):
    L = _lib.load()
    out = np.empty(4096, np.float32)
    L.mdsm_dmshifts(4096, 1500.0, -300.0 / 4096, out.ctypes.data_as(ctypes.c_void_p))
    assert np.array_equal(out, orc.dmshifts(4096, 1500.0, -300.0 / 4096))
    assert L.mdsm_dmdelay(1200.0, 1500.0) == orc.lib().orc_dmdelay(1200.0, 1500.0)


def test_reference_maxshift_relation(lib, orc):
    """The reference sizes its rows with float(dmshifts[last]*hiDM)/tsamp
    (src/mdsm/dedispersion_manager.cpp:291-297); the true largest shift of the table can
    exceed it by one.  The library sizes by the table."""
    for nchans, fch1, foff, tsamp, segs in PLANS:
        lo, st, n = segs[-1]
        ref = orc.ref_maxshift(nchans, fch1, foff, lo, st, n, tsamp)
        S, _, ms = lib_table(nchans, fch1, foff, tsamp, segs, "l1")
        assert ms >= ref - 1 and ms <= ref + 1


def test_contraction_changes_some_shifts(orc):
    """The contracted (fma) and uncontracted evaluations of start + i*step differ on real
    plans, so the choice is observable (the GPU test pins it against the reference kernel)."""
    nchans, fch1, foff, tsamp, segs = PLANS[1]
    a = orc.shift_table(nchans, fch1, foff, tsamp, segs, mode="l1")
    b = orc.shift_table(nchans, fch1, foff, tsamp, segs, mode="l1_muladd")
    assert 0 < int((a != b).sum()) < a.size // 1000
    assert int(np.abs(a - b).max()) == 1


@pytest.mark.parametrize("use_fma", [True, False])
def test_subband_tables_match_oracle(lib, orc, use_fma):
    L = _lib.load()
    nchans, nsubs, tsamp, fch1, foff = 1024, 32, 64e-6, 1500.0, -300.0 / 1024
    p = _lib.SUBBAND_PASSES(0.0, 500.0, 0.25, 4.0, 1, 2000, 125, 16, 0, 0)
    arr = (_lib.SUBBAND_PASSES * 1)(p)
    d = _lib.SubbandDesc(nchans, fch1, foff, tsamp, 4096, nsubs, arr, 1, int(use_fma), 0, 1, 0)
    S1 = np.empty((125, nchans), np.int32)
    S2 = np.empty((125 * 16, nsubs), np.int32)
    _lib.check(L.mdsm_subband_shift_tables(ctypes.byref(d), 0,
                                           S1.ctypes.data_as(ctypes.c_void_p),
                                           S2.ctypes.data_as(ctypes.c_void_p)))
    W1, W2 = orc.subband_tables(nchans, fch1, foff, tsamp, nsubs, 0.0, 4.0, 125, 0.25, 16,
                                use_fma=use_fma)
    assert np.array_equal(S1, W1)
    assert np.array_equal(S2, W2)
    assert S1.min() >= 0 and S2.min() >= 0
