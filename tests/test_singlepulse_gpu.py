"""The device single-pulse search (template form) against the oracle, bit for bit.

Candidates (dm, sample, width, response bits) and their order must equal the oracle's
orc_singlepulse_detect, which tests/test_singlepulse_pins.py pins to the prototype's own
template, convolution and pruning functions (src/prototypes/singlepulse.cpp).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run(m, cuda, y, **kw):
    d = cuda.from_numpy(np.ascontiguousarray(y)).cuda()
    cands, n = m.singlepulse_detect_device(d, **kw)
    cuda.cuda.synchronize()
    return cands, n


def same(c, n, ref):
    dm, sa, wd, sn = ref
    assert n == len(dm), (n, len(dm))
    assert np.array_equal(c["dm_idx"], dm)
    assert np.array_equal(c["sample"], sa)
    assert np.array_equal(c["width"], wd)
    assert np.array_equal(c["snr"].view(np.uint32), sn.view(np.uint32))


def normalised_rows(ndms, n, seed):
    rng = np.random.default_rng(seed)
    y = rng.standard_normal((ndms, n)).astype(np.float32)
    for d in range(ndms):
        for _ in range(3):
            w = int(rng.choice([1, 2, 3, 5, 9, 17, 30, 60]))
            t = int(rng.integers(0, n - w))
            y[d, t:t + w] += np.float32(rng.uniform(1.0, 6.0) * 6 / np.sqrt(w))
    return y


@pytest.mark.parametrize("max_df,chunk,thr", [(30, 8000, 5.0), (150, 8000, 5.0),
                                              (30, 512, 4.0), (9, 1000, 4.5)])
def test_float_series_equal_oracle(lib, orc, cuda, max_df, chunk, thr):
    import mdsm_gb300 as m
    y = normalised_rows(24, 20000, 3 + max_df)
    c, n = run(m, cuda, y, max_downfact=max_df, chunk_len=chunk, threshold=thr)
    ref = orc.singlepulse_detect(y, max_downfact=max_df, chunk_len=chunk, threshold=thr)
    assert n > 0
    same(c, n, ref)


def test_int_series_with_row_statistics(lib, orc, cuda):
    """int32 dedispersed series (sums of uint8 samples) with each row's exact statistics."""
    import mdsm_gb300 as m
    rng = np.random.default_rng(17)
    y = rng.normal(128 * 512, 16 * np.sqrt(512), (16, 9000)).astype(np.int32)
    y[3, 4000:4012] += 3000
    y[9, 100:102] += 5000
    y[12] = 7  # a constant row: sigma 0, skipped
    c, n = run(m, cuda, y, max_downfact=30, chunk_len=8000, threshold=6.0, normalise=True)
    ref = orc.singlepulse_detect(y, max_downfact=30, chunk_len=8000, threshold=6.0,
                                 normalise=True, is_int=True)
    assert n > 0 and not (c["dm_idx"] == 12).any()
    same(c, n, ref)


def test_long_crossing_lists(lib, orc, cuda):
    """Rows that cross the threshold over long stretches: per-width lists of thousands of
    entries, where the prototype's pruneRelated keys on the list index modulo 256."""
    import mdsm_gb300 as m
    rng = np.random.default_rng(23)
    n = 16000
    t = np.arange(n)
    y = rng.standard_normal((6, n)).astype(np.float32) * np.float32(0.3)
    y[0] += np.float32(6.0) * (np.sin(t / 3.0) > -0.2)
    y[1] += np.float32(5.5)
    y[2, ::7] += np.float32(9.0)
    y[3] += (np.float32(7.0) * rng.random(n)).astype(np.float32)
    c, cnt = run(m, cuda, y, max_downfact=30, chunk_len=8000, threshold=5.0)
    ref = orc.singlepulse_detect(y, max_downfact=30, chunk_len=8000, threshold=5.0)
    same(c, cnt, ref)


def test_detrended_pipeline(lib, orc, cuda):
    """The prototype pipeline: a dedispersed float block, detrend and normalise on the device
    (mdsm_detrend_normalise_device), then the search; the oracle searches the device's
    normalised series."""
    import mdsm_gb300 as m
    rng = np.random.default_rng(31)
    n = 16384
    y = (rng.standard_normal((12, n)) * 40 + 1000 + 0.05 * np.arange(n)).astype(np.float32)
    y[4, 9000:9006] += np.float32(400.0)
    d = cuda.from_numpy(y).cuda()
    m.detrend_normalise_device(d, length=1024)
    cands, cnt = m.singlepulse_detect_device(d, max_downfact=30, chunk_len=8000, threshold=6.0)
    yn = d.cpu().numpy()
    ref = orc.singlepulse_detect(yn, max_downfact=30, chunk_len=8000, threshold=6.0)
    same(cands, cnt, ref)
    assert ((cands["dm_idx"] == 4) & (np.abs(cands["sample"] - 9003) < 8)).any()


def test_argument_errors(lib, cuda):
    import mdsm_gb300 as m
    d = cuda.zeros((2, 1000), dtype=cuda.float32, device="cuda")
    for kw in ({"max_downfact": 1}, {"chunk_len": 16}, {"chunk_len": 40000}):
        with pytest.raises(m.MdsmError):
            m.singlepulse_detect_device(d, **kw)
