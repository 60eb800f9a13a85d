"""Detectors on the GPU: candidates identical to the oracle's (and so to the reference's
process_brute, which tests/test_oracle_pins.py pins the oracle to)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_ref_detector_on_golden_block(lib, orc, cuda):
    import mdsm_gb300 as m
    torch = cuda
    import importlib.util
    spec = importlib.util.spec_from_file_location("mk", os.path.join(GOLD, "make_golden.py"))
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    cube = mk.detector_cube()
    g = np.load(os.path.join(GOLD, "ref_host.npz"))
    cands, mean, rms, n = m.ref_detect_device(torch.from_numpy(cube).cuda(), 0.0, 0.5, 4.0)
    rows = g["detect_rows"]
    assert n == len(rows)
    assert np.array_equal(cands["sample"].astype(np.float64), rows[:, 0])
    assert np.allclose(cands["snr"], rows[:, 2], atol=5e-7, rtol=0)
    (dm, samp, snr), om, orms = orc.ref_detect(cube, 0.0, 0.5, 4.0)
    assert mean == om and rms == orms
    assert np.array_equal(cands["dm_idx"], dm) and np.array_equal(cands["snr"], snr)


def test_ref_detector_on_dedispersed_block(lib, orc, cuda):
    """Dedisperse config-1 data on the GPU, detect on the GPU; compare with the oracle's
    detector on the same series (more than 32K values: several statistics chunks)."""
    import mdsm_gb300 as m
    from mdsm_gb300 import synth
    torch = cuda
    x, meta = synth.cfg1(nsamp_total=12000)
    S = orc.shift_table(256, meta["fch1"], meta["foff"], meta["tsamp"], [(0.0, 0.2, 500)])
    nsamp = 12000 - int(S.max())
    plan = m.BrutePlan(256, meta["fch1"], meta["foff"], meta["tsamp"], nsamp, [(0.0, 0.2, 500)],
                       in_dtype="f32")
    y = plan.dedisperse_host(x)
    cands, mean, rms, n = m.ref_detect_device(torch.from_numpy(y).cuda(), 0.0, 0.2, 5.0)
    (dm, samp, snr), om, orms = orc.ref_detect(y, 0.0, 0.2, 5.0)
    assert (mean, rms) == (om, orms)
    assert n == len(dm) > 0
    assert np.array_equal(cands["dm_idx"], dm)
    assert np.array_equal(cands["sample"], samp)
    assert np.array_equal(cands["snr"], snr)


@pytest.mark.parametrize("dtype,nw,n", [("i32", 9, 9000), ("f32", 9, 9000), ("i32", 1, 4097),
                                        ("f32", 2, 2049), ("i32", 5, 301), ("i32", 9, 12289)])
def test_boxcar_matches_oracle(lib, orc, cuda, dtype, nw, n):
    """Interior tiles (no bounds tests) and edge tiles, 1 to 9 widths, odd lengths."""
    import mdsm_gb300 as m
    torch = cuda
    rng = np.random.default_rng(12 + nw + n)
    ndms = 24
    if dtype == "i32":
        y = rng.integers(-3000, 3000, (ndms, n)).astype(np.int32)
        y[3, min(1000, n - 70):min(1064, n - 6)] += 900
        y[10, n // 2:n // 2 + 2] += 20000
        y[20, n - 10:n] += 9000
        y[21, 0:3] += 15000
    else:
        y = rng.standard_normal((ndms, n)).astype(np.float32)
        y[3, min(1000, n - 70):min(1064, n - 6)] += np.float32(0.9)
        y[10, n // 2:n // 2 + 2] += np.float32(8.0)
        y[21, 0:3] += np.float32(6.0)
    cands, cnt = m.boxcar_detect_device(torch.from_numpy(y).cuda(), nwidths=nw, threshold=6.0)
    dm, samp, wid, snr = orc.boxcar_detect(y, nw, 6.0)
    assert cnt == len(dm) > 0
    assert np.array_equal(cands["dm_idx"], dm)
    assert np.array_equal(cands["sample"], samp)
    assert np.array_equal(cands["width"], wid)
    assert np.array_equal(cands["snr"], snr)


def test_detrend_normalise_matches_oracle(lib, orc, cuda):
    """src/prototypes/detrend.cu:12-100 restated; double sums in a different order on the two
    sides, so the bar is 1e-5 relative."""
    import mdsm_gb300 as m
    torch = cuda
    rng = np.random.default_rng(8)
    ndms, n, L = 12, 5000, 1024
    t = np.arange(n, dtype=np.float32)
    y = (rng.standard_normal((ndms, n)) * 3 + 0.01 * t + 50).astype(np.float32)
    d = torch.from_numpy(y.copy()).cuda()
    m.detrend_normalise_device(d, L)
    got = d.cpu().numpy()
    for k in range(ndms):
        want = orc.detrend_normalise(y[k], L)
        full = (n // L) * L
        assert np.allclose(got[k, :full], want[:full], rtol=1e-5, atol=1e-5)
        assert np.array_equal(got[k, full:], y[k, full:])
