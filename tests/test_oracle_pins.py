"""Pins the oracle to the reference: its golden outputs (tests/golden/, made by the reference's
own code) and, where this machine has the reference tree, the reference code itself."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


@pytest.fixture(scope="module")
def host_gold():
    return np.load(os.path.join(GOLD, "ref_host.npz"))


def test_median_of_five_matches_reference(orc, host_gold):
    tup, med = host_gold["median_in"], host_gold["median_out"]
    got = np.array([orc.median_of_five(*map(float, t)) for t in tup], np.float32)
    assert np.array_equal(got, med)
    # and the network is a true median on these inputs
    assert np.array_equal(med, np.sort(tup, axis=1)[:, 2])


def _detector_cube():
    import importlib.util
    spec = importlib.util.spec_from_file_location("mk", os.path.join(GOLD, "make_golden.py"))
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    return mk.detector_cube()


def test_reference_detector_matches_reference(orc, host_gold):
    cube = _detector_cube()
    (dm, samp, snr), mean, rms = orc.ref_detect(cube, float(host_gold["detect_lowdm"]),
                                                float(host_gold["detect_dmstep"]),
                                                float(host_gold["detect_threshold"]))
    rows = host_gold["detect_rows"]
    assert len(rows) == len(dm)
    dmv = np.float32(host_gold["detect_lowdm"]) + dm.astype(np.float32) * np.float32(
        host_gold["detect_dmstep"])
    # the reference prints "%lf, %f, %f": compare at printed precision
    assert np.array_equal(rows[:, 0], samp.astype(np.float64))
    assert np.allclose(rows[:, 1], dmv, atol=5e-7)
    assert np.allclose(rows[:, 2], snr, atol=5e-7, rtol=0)


def test_chunked_detector_matches_reference(orc, host_gold):
    """process_brute with caller noise statistics (one mean/rms per 256 samples): the reference
    prints time, DM, (median - mean)/rms, mean and rms."""
    cube = _detector_cube()
    spc = int(host_gold["chunk_spc"])
    cm, cr = host_gold["chunk_mean"], host_gold["chunk_rms"]
    dm, samp, snr = orc.ref_detect_chunked(cube, 0.0, 0.5, 4.0, cm, cr, spc)
    rows = host_gold["detect_chunked_rows"]
    assert len(rows) == len(dm) > 0
    assert np.array_equal(rows[:, 0], samp.astype(np.float64))
    assert np.allclose(rows[:, 1], dm.astype(np.float32) * np.float32(0.5), atol=5e-7)
    assert np.allclose(rows[:, 2], snr, atol=5e-7, rtol=0)
    assert np.allclose(rows[:, 3], cm[samp // spc], atol=5e-7, rtol=0)
    assert np.allclose(rows[:, 4], cr[samp // spc], atol=5e-7, rtol=0)


@pytest.mark.parametrize("binsize", [1, 2])
def test_subband_detector_matches_reference(orc, host_gold, binsize):
    """process_subband, one pass of 16 rows with caller noise statistics: time is
    t * binsize, DM lowdm + row * dmstep, snr median / rms."""
    cube = _detector_cube()
    n = cube.shape[1] // binsize
    rows_in = np.ascontiguousarray(cube[:, :n])
    dmv = np.float32(0.0) + np.arange(16, dtype=np.float32) * np.float32(0.5)
    spc = int(host_gold["chunk_spc"])
    dm, samp, snr = orc.ref_detect_subband(rows_in, n, dmv, 4.0, host_gold["chunk_mean"],
                                           host_gold["chunk_rms"], spc)
    rows = host_gold["subband_rows_b%d" % binsize]
    assert len(rows) == len(dm) > 0
    assert np.array_equal(rows[:, 0], (samp * binsize).astype(np.float64))
    assert np.allclose(rows[:, 1], dmv[dm], atol=5e-7)
    assert np.allclose(rows[:, 2], snr, atol=5e-7, rtol=0)


def test_subband_row_statistics(orc):
    """The per-row statistics branch of process_subband (mean == NULL), which the reference
    cannot run (it prints mean[0] first): restated, checked against numpy's FP64 sums."""
    rng = np.random.default_rng(8)
    rows = (rng.standard_normal((6, 1000)) * 2.0 + 1.0).astype(np.float32)
    rows[4, 500:503] += np.float32(30.0)
    dmv = np.array([0.5, 1.5, 2.5, 3.5, 4.5, 5.5], np.float32)
    dm, samp, snr = orc.ref_detect_subband(rows, 1000, dmv, 5.0)
    assert len(dm) > 0 and set(dm.tolist()) == {4}
    r = rows[4].astype(np.float64)
    lm = np.float32(r.sum() / 1000)
    lr = np.float32(np.sqrt((r * r).sum() / 1000 - np.float64(lm) ** 2))
    med = np.median(np.lib.stride_tricks.sliding_window_view(rows[4], 5), axis=1)
    want = np.nonzero(med.astype(np.float32) - lm >= lr * np.float32(5.0))[0]
    assert np.array_equal(samp, want)
    assert np.allclose(snr, med[want].astype(np.float32) / lr, rtol=1e-7)


def test_unpack_matches_reference(orc, host_gold):
    raw = host_gold["unpack_raw"]
    for nbits in (1, 2, 4, 8, 16):
        assert np.array_equal(orc.unpack(raw, nbits), host_gold["unpack_%d" % nbits]), nbits


def test_known_answer_channel_index(orc):
    """src/prototypes/brute_dedisp_imp_tex.cu:112-114,168-175: x[c][t] = c sums to
    nchans*(nchans-1)/2 for every output, whatever the shifts."""
    nchans, nsamp = 200, 512
    S = orc.shift_table(nchans, 1400.0, -0.5, 1e-4, [(0.0, 5.0, 30)])
    x = np.repeat(np.arange(nchans, dtype=np.float32)[:, None], nsamp + S.max() + 1, axis=1)
    y = orc.dedisperse(x, S, nsamp)
    assert np.all(y == nchans * (nchans - 1) / 2)


def test_float_sum_order_is_channel_sequential(orc):
    """The oracle's float output equals a plain left-to-right float32 sum over channels."""
    rng = np.random.default_rng(3)
    nchans, nsamp = 37, 64
    S = orc.shift_table(nchans, 1500.0, -2.0, 64e-6, [(0.0, 3.0, 5)])
    x = rng.standard_normal((nchans, nsamp + S.max() + 1), dtype=np.float32) * 1e3
    y = orc.dedisperse(x, S, nsamp)
    for d in range(5):
        acc = np.zeros(nsamp, np.float32)
        for c in range(nchans):
            acc = acc + x[c, S[d, c]:S[d, c] + nsamp]
        assert np.array_equal(y[d], acc)


@pytest.mark.skipif(not os.path.isdir("/root/reference/src"), reason="reference tree absent")
def test_reference_detector_live(orc):
    """Where the reference builds here, run its process_brute on a fresh seeded block."""
    import ctypes
    import tempfile
    orc.build(reference=True)
    h = orc.ref_host()
    rng = np.random.default_rng(99)
    cube = rng.standard_normal((24, 3000), dtype=np.float32)
    cube[7, 1000:1004] += np.float32(9.0)
    fd, path = tempfile.mkstemp()
    os.close(fd)
    h.ref_process_brute(cube.ctypes.data_as(ctypes.c_void_p), 24, 3000, ctypes.c_float(0.5),
                        ctypes.c_float(0.25), ctypes.c_float(3.5), path.encode())
    rows = np.array([[float(v) for v in ln.split(",")[:3]] for ln in open(path) if ln.strip()])
    os.unlink(path)
    (dm, samp, snr), _, _ = orc.ref_detect(cube, 0.5, 0.25, 3.5)
    assert len(rows) == len(dm) > 0
    assert np.array_equal(rows[:, 0], samp)
    assert np.allclose(rows[:, 2], snr, atol=5e-7, rtol=0)


GPU_GOLD = os.path.join(GOLD, "ref_gpu.npz")


@pytest.mark.skipif(not os.path.exists(GPU_GOLD), reason="GPU golden fixtures not generated")
def test_oracle_matches_reference_kernel_outputs(orc):
    """The reference CUDA kernels' outputs (tests/golden/ref_gpu.npz, made on a GB300 by
    make_golden.py --gpu) equal the oracle's float sums with the contracted L1 shifts."""
    g = np.load(GPU_GOLD)
    nchans, nsamp, ms, tdms = [int(v) for v in g["l1_meta"]]
    fch1, foff, tsamp, lowdm, dmstep = [float(v) for v in g["l1_f"]]
    S = orc.shift_table(nchans, fch1, foff, tsamp, [(lowdm, dmstep, tdms)], mode="l1")
    y = orc.dedisperse(g["l1_x"], S, nsamp)
    assert np.array_equal(y, g["l1_y"])
    nchans, nsamp2, ms2, tdms = [int(v) for v in g["opt_meta"]]
    S2 = orc.shift_table(nchans, fch1, foff, tsamp, [(lowdm, dmstep, tdms)], mode="opt")
    y2 = orc.dedisperse(g["opt_x"], S2, nsamp2)
    assert np.array_equal(y2, g["opt_y"])
