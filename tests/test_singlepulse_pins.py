"""The oracle's single-pulse search (template form) pinned to the prototype's own functions.

src/prototypes/singlepulse.cpp does not build here as it stands (FFTW is absent); its template,
convolution and pruning functions were compiled against a stand-in for FFTW's interface and
run on seeded inputs by tests/golden/make_golden.py --singlepulse, giving
tests/golden/ref_singlepulse.npz.  These tests hold the oracle to those outputs, and to a numpy
FFT convolution (the prototype's own method) of the same templates.
"""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_singlepulse.npz")


def template(w, n):
    """The convolution kernel of the oracle's width-w window on a circle of n samples.  The
    window of sample t is [t - w//2, t - w//2 + w), so the kernel K (result[t] = sum_k K[k]
    x[t - k]) is 1/sqrt(w) (rounded to float, as singlepulse.cpp:60-61 divides a float by sqrt)
    at k = w//2 - w + 1 .. w//2."""
    t = np.zeros(n)
    for k in range(w // 2 - w + 1, w // 2 + 1):
        t[k % n] = np.float32(1.0 / np.sqrt(w))
    return t


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def test_templates_equal_reference_kernels(gold):
    """createFFTKernel (:41-67): the inverse transform of the prototype's kernel spectrum is the
    oracle's centred template, for every width of the downfactor ladder."""
    n = int(gold["fftlen"])
    for i, w in enumerate(gold["ladder"]):
        sp = gold["spectra"][i].astype(np.float64)
        t = np.fft.irfft(sp[0::2] + 1j * sp[1::2], n)
        assert np.abs(t - template(int(w), n)).max() < 2e-6, w


def test_reference_convolution_equals_direct_sums(orc, gold):
    """convolve (:69-87) on one chunk equals the oracle's direct template sums, once the bin the
    prototype leaves unset (n/2: its spectra hold n/2 complex values, the real transform
    n/2 + 1) is put back.  Positions whose window wraps around the chunk are excluded."""
    n = int(gold["fftlen"])
    x = gold["chunk"].astype(np.float64)
    alt = (-1.0) ** np.arange(n)
    for i, w in enumerate(gold["ladder"][:8]):
        w = int(w)
        ref = gold["conv"][i].astype(np.float64)
        nyq = (x @ alt) * (template(w, n) @ alt) / n * alt
        direct = orc.sp_values(gold["chunk"], w).astype(np.float64)
        lo, hi = w // 2, n - w
        assert np.abs(ref + nyq - direct)[lo:hi].max() < 2e-6, w


def test_numpy_fft_convolution_equals_direct_sums(orc):
    """The prototype's method, an FFT circular convolution with the centred templates, done by
    numpy in double over a zero-padded 8192-sample chunk, equals the oracle's FP32 direct sums
    to FP32 rounding (no wrap: the padding covers the widest template)."""
    rng = np.random.default_rng(8)
    n = 8192
    for trial in range(3):
        x = rng.standard_normal(n).astype(np.float32) * np.float32(1 + trial)
        x[:96] = 0.0
        x[-96:] = 0.0
        X = np.fft.rfft(x.astype(np.float64))
        for w in orc.sp_widths(150):
            conv = np.fft.irfft(X * np.fft.rfft(template(int(w), n)), n)
            direct = orc.sp_values(x, int(w)).astype(np.float64)
            tol = 4e-7 * np.sqrt(w) * (1 + trial) * 8
            assert np.abs(conv - direct).max() < tol, (trial, w)


def test_prune_related_equals_reference(orc, gold):
    """pruneRelated (:90-120) as written, over 140 lists (4 of them longer than 256 entries)."""
    off = gold["pr_off"]
    for k, f in enumerate(gold["pr_fac"]):
        a, b = int(off[k]), int(off[k + 1])
        keep = orc.sp_prune_related(gold["pr_bins"][a:b], gold["pr_vals"][a:b], int(f))
        want = gold["pr_vals_out"][a:b] != 0
        assert np.array_equal(keep, want), k


def test_prune_downfactors_equals_reference(orc, gold):
    """pruneRelatedDownfactors (:122-146) as written (mask starting at zero), over 120 lists in
    the prototype's order."""
    off = gold["pd_off"]
    ladder = gold["ladder"]
    for k, nf in enumerate(gold["pd_nf"]):
        a, b = int(off[k]), int(off[k + 1])
        mask = orc.sp_prune_downfactors(gold["pd_bins"][a:b], gold["pd_vals"][a:b],
                                        gold["pd_df"][a:b], int(ladder[nf - 1]))
        assert np.array_equal(mask, gold["pd_mask"][a:b] != 0), k


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(os.path.dirname(
    os.path.abspath(__file__))), "oracle", "_ref", "libref_singlepulse.so")),
    reason="single-pulse prototype not built on this machine")
def test_prune_functions_live(orc):
    """Where the prototype's functions are built here, fresh seeded lists through both."""
    import ctypes
    h = orc.ref_singlepulse()
    P = ctypes.c_void_p
    rng = np.random.default_rng(12345)
    for k in range(200):
        n = int(rng.integers(1, 300))
        b = (np.cumsum(rng.choice([1, 1, 2, 4, 8, 16], n))).astype(np.uint32)
        v = (5 + 0.5 * rng.integers(0, 10, n)).astype(np.float32)
        f = int(rng.choice([2, 3, 4, 6, 9, 14, 20, 30]))
        bo, vo = b.copy(), v.copy()
        h.ref_sp_prune_related(bo.ctypes.data_as(P), vo.ctypes.data_as(P), n, f)
        assert np.array_equal(orc.sp_prune_related(b.astype(np.int32), v, f), vo != 0)
        nf = int(rng.integers(1, 13))
        df = rng.choice(np.r_[1, orc.sp_widths(150)[1:nf + 1]], n).astype(np.uint32)
        bb = rng.integers(0, 400, n).astype(np.int64)
        mask = np.zeros(n, np.uint8)
        h.ref_sp_prune_downfactors(bb.ctypes.data_as(P), v.ctypes.data_as(P),
                                   df.ctypes.data_as(P), n, nf, mask.ctypes.data_as(P))
        ladder = orc.sp_widths(150)[1:]
        got = orc.sp_prune_downfactors(bb, v, df.astype(np.int32), int(ladder[nf - 1]))
        assert np.array_equal(got, mask != 0)


def pow2_values(y, w, mu_f, inv):
    """The boxcar mode's width-w response at t (window [t, t + w), pairwise-doubled FP32 sums)."""
    b = y.astype(np.float32)
    k = 1
    while k < w:
        nb = np.full_like(b, np.nan)
        nb[: b.size - k] = b[: b.size - k] + b[k:]
        b = nb
        k *= 2
    return (b - np.float32(w) * mu_f) * inv


def test_template_and_boxcar_modes_agree_where_templates_coincide(orc):
    """At widths 2 and 4 the template (centred) and boxcar (leading) windows hold the same
    samples, shifted by w/2.  On an integer series whose sums are exact in FP32 the two modes'
    responses are then identical with the same statistics."""
    rng = np.random.default_rng(21)
    # one row of integer sums over 4096 uint8 channels (values ~5e5, sums of 4 < 2^24)
    y = (rng.integers(0, 256, (4096, 3000)).sum(axis=0)).astype(np.int32)
    mu, sig = orc_stats_int(orc, y)
    for w in (2, 4):
        inv = np.float32(1.0 / (sig * np.sqrt(w)))
        tm = orc.sp_values(y, w, normalise=True, is_int=True)
        bx = pow2_values(y, w, np.float32(mu), inv)
        n = y.size
        assert np.array_equal(tm[w // 2: n - w + w // 2 + 1], bx[: n - w + 1])


def orc_stats_int(orc, y):
    import ctypes
    yd = np.ascontiguousarray(y, np.float64)
    m, s = ctypes.c_double(), ctypes.c_double()
    orc.lib().orc_series_stats_int(yd.ctypes.data_as(ctypes.c_void_p), ctypes.c_long(yd.size),
                                   ctypes.byref(m), ctypes.byref(s))
    return m.value, s.value


def test_singlepulse_search_finds_injected_pulses(orc):
    """The oracle's search on a normalised series: each injected boxcar is reported once, at a
    width of the ladder near its own, inside its extent."""
    rng = np.random.default_rng(5)
    n = 20000
    y = rng.standard_normal((3, n)).astype(np.float32)
    y[0, 5000:5009] += np.float32(3.0)     # width 9, SNR 9
    y[1, 12345:12365] += np.float32(2.5)   # width 20, SNR 11
    y[2, 7999:8001] += np.float32(8.0)     # width 2 across the chunk boundary, SNR 11
    dm, samp, wid, snr = orc.singlepulse_detect(y, max_downfact=30, threshold=7.0)
    for d, lo, hi in ((0, 5000, 5009), (1, 12345, 12365), (2, 7999, 8001)):
        sel = dm == d
        assert sel.any(), d
        assert ((samp[sel] >= lo - 15) & (samp[sel] < hi + 15)).all(), (d, samp[sel])
        assert snr[sel].max() >= 7.0
