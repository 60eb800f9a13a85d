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
    """Tiles inside the rows (16-byte copies) and the last tile of each row (staged with zeros
    past the row), 1 to 9 widths, odd lengths."""
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


@pytest.mark.parametrize("dtype,nw,thr,tail", [("i32", 1, 6.0, 777), ("f32", 3, 6.0, 776),
                                               ("i32", 4, 6.0, 777), ("f32", 6, 6.0, 776),
                                               ("i32", 8, 6.0, 777), ("f32", 9, 3.5, 777),
                                               ("i32", 9, 6.0, 776)])
def test_boxcar_fast_path_and_tile_boundaries(lib, orc, cuda, dtype, nw, thr, tail):
    """Rows long enough for several tiles at every width count, with pulses on both sides of
    the tile boundaries (tiles of 3840 - WMAX + 1 samples, rounded down to a multiple of 4: a
    staged region of 256 threads x 15) and of the exact search's part boundaries inside a tile
    (parts of 1792 - 2 HL - WMAX samples, rounded the same way: 256 x 7); rows of 16-byte
    multiples (tail 776) and not (777, staged in 4-byte copies); at a 3.5 sigma threshold most
    tiles are flagged for the exact search."""
    import mdsm_gb300 as m
    torch = cuda
    wmax = 1 << (nw - 1)
    hl = max(wmax // 2, 1)
    tile = (3840 - wmax + 1) & ~3
    part = (1792 - 2 * hl - wmax) & ~3
    n = 6 * tile + tail
    rng = np.random.default_rng(70 + nw + tail)
    ndms = 16
    if dtype == "i32":
        y = rng.integers(-3000, 3000, (ndms, n)).astype(np.int32)
        amp = [40000, 9000, 3000]
    else:
        y = rng.standard_normal((ndms, n)).astype(np.float32)
        amp = [np.float32(30.0), np.float32(7.0), np.float32(2.5)]
    for k in range(1, 6):
        for j, off in enumerate((-hl - 1, -1, 0, 1, hl)):
            row = (3 * k + j) % ndms
            w = min(1 << ((k + j) % nw), 64)
            for t in (k * tile + off, (k - 1) * tile + part + off, (k - 1) * tile + 2 * part + off):
                if 0 <= t and t + w <= n:
                    y[row, t:t + w] += amp[(k + j) % 3]
    cands, cnt = m.boxcar_detect_device(torch.from_numpy(y).cuda(), nwidths=nw, threshold=thr,
                                        cap=1 << 20)
    dm, samp, wid, snr = orc.boxcar_detect(y, nw, thr)
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


def _golden_cube():
    import importlib.util
    spec = importlib.util.spec_from_file_location("mk", os.path.join(GOLD, "make_golden.py"))
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    return mk.detector_cube()


def test_chunked_detector_on_golden_block(lib, orc, cuda):
    """process_brute with caller noise statistics: the reference's own lines (golden) and the
    oracle's candidates."""
    import mdsm_gb300 as m
    torch = cuda
    cube = _golden_cube()
    g = np.load(os.path.join(GOLD, "ref_host.npz"))
    spc, cm, cr = int(g["chunk_spc"]), g["chunk_mean"], g["chunk_rms"]
    cands, n = m.ref_detect_chunked_device(torch.from_numpy(cube).cuda(), 0.0, 0.5, 4.0, cm, cr,
                                           spc)
    rows = g["detect_chunked_rows"]
    assert n == len(rows) > 0
    assert np.array_equal(cands["sample"].astype(np.float64), rows[:, 0])
    assert np.allclose(cands["snr"], rows[:, 2], atol=5e-7, rtol=0)
    dm, samp, snr = orc.ref_detect_chunked(cube, 0.0, 0.5, 4.0, cm, cr, spc)
    assert np.array_equal(cands["dm_idx"], dm) and np.array_equal(cands["sample"], samp)
    assert np.array_equal(cands["snr"], snr)


def _subband_block(torch):
    import mdsm_gb300 as m
    from mdsm_gb300 import synth
    nchans, nsamp, tsamp = 256, 4096, 64e-6
    passes = [dict(lowdm=0.0, highdm=32.0, dmstep=0.5, sub_dmstep=4.0, ncalls=8, calldms=8),
              dict(lowdm=32.0, highdm=96.0, dmstep=2.0, sub_dmstep=16.0, ncalls=4, calldms=8,
                   binsize=2)]
    plan = m.SubbandPlan(nchans, 1500.0, -300.0 / nchans, tsamp, nsamp, 16, passes,
                         in_dtype="f32", out_dtype="f32")
    nch, stride = plan.input_shape()
    x = synth.gaussian_f32(nch, stride, 17)
    synth.inject(x, 1500.0, -300.0 / nchans, tsamp, [(1200, 20.0, 6, 1.5), (3000, 60.0, 8, 1.5)],
                 K=4148.741601)
    d_in = plan.alloc_input()
    d_in[: x.size].copy_(torch.from_numpy(x.ravel()))
    d_out = plan.alloc_output()
    plan.dedisperse_device(d_in, d_out)
    torch.cuda.synchronize()
    return plan, passes, d_out


@pytest.mark.parametrize("chunked", [False, True])
def test_subband_detector_matches_oracle(lib, orc, cuda, chunked):
    """process_subband per pass (rows of nsamp / binsize samples) with per-row statistics or
    caller chunk statistics, on the plan's own DMs, against the oracle pass by pass."""
    import mdsm_gb300 as m
    torch = cuda
    plan, passes, d_out = _subband_block(torch)
    y = d_out.cpu().numpy()
    dmv = plan.dm_values()
    spc = 512
    rng = np.random.default_rng(4)
    cm = (rng.standard_normal(8) * 0.1).astype(np.float32) if chunked else None
    cr = (rng.uniform(1.0, 3.0, 8)).astype(np.float32) if chunked else None
    cands, n = m.ref_detect_subband_device(plan, d_out, 5.0, cm, cr, spc)
    want_dm, want_t, want_snr, want_w = [], [], [], []
    row0 = 0
    for p in passes:
        rows = p["ncalls"] * p["calldms"]
        b = p.get("binsize", 1)
        nvalid = 4096 // b
        dm, t, snr = orc.ref_detect_subband(y[row0:row0 + rows], nvalid, dmv[row0:row0 + rows],
                                            5.0, cm, cr, spc)
        want_dm += (dm + row0).tolist()
        want_t += t.tolist()
        want_snr += snr.tolist()
        want_w += [b] * len(dm)
        row0 += rows
    order = np.lexsort((np.array(want_t), np.array(want_dm)))
    assert n == len(want_dm) > 0
    assert np.array_equal(cands["dm_idx"], np.array(want_dm)[order])
    assert np.array_equal(cands["sample"], np.array(want_t)[order])
    assert np.array_equal(cands["width"], np.array(want_w)[order])
    assert np.array_equal(cands["snr"], np.array(want_snr, np.float32)[order])


def test_detectors_from_several_threads(lib, cuda):
    """Detector calls from four threads at once (each its own stream and series) return what
    the same calls return one after another."""
    import threading
    import mdsm_gb300 as m
    torch = cuda
    rng = np.random.default_rng(31)
    series = []
    for i in range(4):
        y = rng.integers(-3000, 3000, (16, 6000)).astype(np.int32)
        y[i + 2, 1000 + 100 * i: 1010 + 100 * i] += 20000
        series.append(torch.from_numpy(y).cuda())
    fseries = [s.float() for s in series]
    torch.cuda.synchronize()

    def run(i):
        st = torch.cuda.Stream()
        a = m.boxcar_detect_device(series[i], nwidths=7, threshold=6.0, stream=st)
        b = m.ref_detect_device(fseries[i], 0.0, 0.5, 5.0, stream=st)
        st.synchronize()
        return a, b

    serial = [run(i) for i in range(4)]
    out = [None] * 4

    def worker(i):
        for _ in range(5):
            out[i] = run(i)

    th = [threading.Thread(target=worker, args=(i,)) for i in range(4)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for i in range(4):
        (ca, na), (cb, mb, rb, nb) = out[i]
        (sa, sna), (sb, smb, srb, snb) = serial[i]
        assert na == sna > 0 and np.array_equal(ca, sa)
        assert nb == snb and np.array_equal(cb, sb) and (mb, rb) == (smb, srb)
