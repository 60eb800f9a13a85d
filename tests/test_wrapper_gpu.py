"""The reference's internal C ABI, call_initialise_devices / call_dedisperse
(src/mdsm/dedispersion_wrapper.cu:4-13), driven by a C manager that follows
src/mdsm/dedispersion_manager.cpp's thread set-up and barrier handshake and src/MDSM.cpp's block
loop (tests/drivers/manager_driver.c).  Every block's series, as the manager's output thread
sees it, equals the oracle's dedispersion of that block (brute force, the L1 and the opt shift
arithmetic), or the library's own subband plan on that block (two passes, the second
downsampled, packed as the reference packs them)."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NCH, FCH1, FOFF, TSAMP = 128, 1500.0, -2.34375, 64e-6


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    from mdsm_gb300 import _lib
    d = tmp_path_factory.mktemp("mgr")
    exe = d / "manager_driver"
    libdir = os.path.dirname(_lib.LIB_PATH)
    subprocess.run(["gcc", "-std=gnu11", "-O2", "-I", os.path.join(ROOT, "include"), "-o",
                    str(exe), os.path.join(ROOT, "tests", "drivers", "manager_driver.c"),
                    "-L" + libdir, "-lmdsm_gb300", "-lpthread", "-Wl,-rpath," + libdir],
                   check=True)
    return exe


def run(driver, tmp_path, x, nsamp, *mode, env=None):
    spec = tmp_path / "spectra.f32"
    out = tmp_path / "series.f32"
    np.ascontiguousarray(x.T).astype(np.float32).tofile(spec)
    args = [str(driver), str(spec), str(out), str(NCH), str(nsamp), repr(FCH1), repr(FOFF),
            repr(TSAMP)] + [str(a) for a in mode]
    r = subprocess.run(args, capture_output=True, text=True, timeout=300,
                       env=dict(os.environ, **(env or {})))
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mdsm worker" not in r.stderr, r.stderr  # a block the worker could not process
    f = r.stdout.split()
    info = {f[i]: int(f[i + 1]) for i in range(0, len(f) - 1, 2)}
    return info, np.fromfile(out, np.float32)


def block_input(x, k, nsamp, ms, width):
    """Block k as the reference's worker holds it: stream columns [k nsamp, k nsamp + nsamp +
    maxshift), zero beyond (the plan may shift a sample past the manager's maxshift)."""
    b = np.zeros((NCH, width), np.float32)
    seg = x[:, k * nsamp: k * nsamp + nsamp + ms]
    b[:, : seg.shape[1]] = seg
    return b


@pytest.mark.parametrize("l1", [1, 0])
def test_brute_blocks_equal_oracle(lib, orc, cuda, driver, tmp_path, l1):
    nsamp, tdms, lowdm, dmstep, nblocks = 2048, 96, 2.0, 0.75, 3
    hidm = np.float32(lowdm) + np.float32(dmstep) * np.float32(tdms - 1)
    dms = orc.dmshifts(NCH, FCH1, FOFF)
    ms = int(np.float32(dms[-1]) * hidm / np.float32(TSAMP))
    rng = np.random.default_rng(40 + l1)
    x = rng.standard_normal((NCH, nblocks * nsamp + ms), dtype=np.float32)
    info, got = run(driver, tmp_path, x, nsamp, "brute", lowdm, dmstep, tdms, l1)
    # the loop counts the final empty read too (src/MDSM.cpp:141-166)
    assert info["maxshift"] == ms and info["blocks"] == nblocks + 1, info
    assert info["outputs"] == nblocks, info
    assert info["dedispersed_size"] == tdms * nsamp
    got = got.reshape(nblocks, tdms, nsamp)
    S = orc.shift_table(NCH, FCH1, FOFF, TSAMP, [(lowdm, dmstep, tdms)],
                        mode="l1" if l1 else "opt")
    width = nsamp + max(ms, int(S.max())) + 1
    for k in range(nblocks):
        want = orc.dedisperse(block_input(x, k, nsamp, ms, width), S, nsamp)
        assert np.array_equal(got[k], want), k


def test_subband_blocks_equal_library_plan(lib, cuda, driver, tmp_path):
    import mdsm_gb300 as m
    torch = cuda
    nsamp, nsubs, nblocks = 2048, 16, 3
    passes = [dict(lowdm=0.0, highdm=32.0, dmstep=0.5, sub_dmstep=8.0, ncalls=4, calldms=16,
                   binsize=1),
              dict(lowdm=32.0, highdm=96.0, dmstep=1.0, sub_dmstep=16.0, ncalls=4, calldms=16,
                   binsize=2)]
    spec = ";".join("%r,%r,%r,%r,%d,%d,%d" % (p["lowdm"], p["highdm"], p["dmstep"],
                                               p["sub_dmstep"], p["ncalls"], p["calldms"],
                                               p["binsize"]) for p in passes)
    rng = np.random.default_rng(44)
    from oracle import oracle as orc
    dshift = orc.dmshifts(NCH, FCH1, FOFF)
    ms = int(np.float32(dshift[-1]) * np.float32(96.0) / np.float32(TSAMP))
    x = rng.standard_normal((NCH, nblocks * nsamp + ms), dtype=np.float32)
    info, got = run(driver, tmp_path, x, nsamp, "subband", nsubs, spec)
    per_block = 4 * 16 * nsamp + 4 * 16 * nsamp // 2
    assert info["maxshift"] == ms and info["blocks"] == nblocks + 1, info
    assert info["outputs"] == nblocks, info
    assert info["dedispersed_size"] == per_block
    got = got.reshape(nblocks, per_block)
    plan = m.SubbandPlan(NCH, FCH1, FOFF, TSAMP, nsamp, nsubs, passes, in_dtype="f32",
                         out_dtype="f32")
    i = plan.info
    for k in range(nblocks):
        b = block_input(x, k, nsamp, ms, max(i.in_stride, nsamp + ms))
        d_in = plan.alloc_input()
        rows = d_in[: NCH * i.in_stride].view(NCH, i.in_stride)
        w = min(i.in_stride, b.shape[1])
        rows[:, :w].copy_(torch.from_numpy(np.ascontiguousarray(b[:, :w])))
        d_out = plan.alloc_output()
        plan.dedisperse_device(d_in, d_out)
        torch.cuda.synchronize()
        y = d_out.cpu().numpy().reshape(i.ndms, nsamp)
        want = np.concatenate([y[:64].ravel(), y[64:, : nsamp // 2].ravel()])
        assert np.array_equal(got[k], want), k


def _pulses(x, nsamp, nblocks):
    """Broadband 6-sample bursts (DM 0) at a few times of every block."""
    for k in range(nblocks):
        for off, amp in ((300, 4.0), (1100, 2.5), (1900, 6.0)):
            t = k * nsamp + off
            x[:, t:t + 6] += np.float32(amp)


@pytest.mark.parametrize("threads", [1, 2])
def test_output_thread_brute_candidates(lib, orc, cuda, driver, tmp_path, threads):
    """process_output (the reference's output thread, src/mdsm/dedispersion_output.cpp:216-356)
    beside call_dedisperse workers (two of them sharing the GPU when threads = 2): its
    candidate file holds, block after block, the lines of process_brute over every worker's
    rows (block statistics, the thread's DM of each row, median-of-five) with the block's
    timestamp, here computed from the oracle's series with the library's detector."""
    torch = cuda
    import mdsm_gb300 as m
    nsamp, tdms, lowdm, dmstep, nblocks, thr = 2048, 96, 2.0, 0.75, 3, 5.0
    hidm = np.float32(lowdm) + np.float32(dmstep) * np.float32(tdms - 1)
    dms = orc.dmshifts(NCH, FCH1, FOFF)
    ms = int(np.float32(dms[-1]) * hidm / np.float32(TSAMP))
    rng = np.random.default_rng(60 + threads)
    x = rng.standard_normal((NCH, nblocks * nsamp + ms), dtype=np.float32)
    _pulses(x, nsamp, nblocks)
    odir = tmp_path / "out"
    odir.mkdir()
    info, _ = run(driver, tmp_path, x, nsamp, "brute", lowdm, dmstep, tdms, 1,
                  env={"MDSM_DRIVER_OUTPUT": str(odir), "MDSM_DRIVER_THREADS": str(threads),
                       "MDSM_DRIVER_THRESHOLD": repr(thr)})
    assert info["threads"] == threads and info["blocks"] == nblocks + 1, info
    got = (odir / "cands.dat").read_text().splitlines()
    rpt = tdms // threads
    f32 = np.float32
    tshift = int(f32(f32(tdms) * f32(dmstep)) / f32(threads))
    want = []
    for k in range(nblocks):
        ys = []
        for t in range(threads):
            # the thread's first DM as the reference's launcher forms it, in float
            start = f32(f32(lowdm) + f32(f32(f32(dmstep) * f32(tdms)) / f32(threads)) * f32(t))
            S = orc.shift_table(NCH, FCH1, FOFF, TSAMP, [(float(start), dmstep, rpt)], mode="l1")
            width = nsamp + max(ms, int(S.max())) + 1
            ys.append(orc.dedisperse(block_input(x, k, nsamp, ms, width), S, nsamp))
        y = np.ascontiguousarray(np.concatenate(ys).astype(np.float32))
        # every row passes the detector's DM filter with lowdm 1e6; the thread's DM below
        c = m.ref_detect_device(torch.from_numpy(y).cuda(), 1e6, dmstep, thr)[0]
        ts = 1000.0 + float(k) * float(nsamp) * float(f32(TSAMP))
        for row, samp, snr in zip(c["dm_idx"], c["sample"], c["snr"]):
            t, kk = divmod(int(row), rpt)
            dm = f32(f32(f32(lowdm) + f32(np.uint32(tshift) * np.uint32(t))) + f32(f32(kk) * f32(dmstep)))
            if not float(dm) > 1.0:
                continue
            want.append("%f, %f, %f" % (ts + float(samp) * float(f32(TSAMP)), float(dm), float(snr)))
    assert len(want) > 3 * nblocks
    assert got == want


def test_output_thread_subband_candidates(lib, cuda, driver, tmp_path):
    """process_output on subband blocks (two passes, the second downsampled): its lines equal
    process_subband's on the library's own plan output of each block (per-row statistics,
    the plan's row DMs, times in samples of the pass's downsample factor)."""
    import mdsm_gb300 as m
    from oracle import oracle as orc
    torch = cuda
    nsamp, nsubs, nblocks, thr = 2048, 16, 3, 5.0
    passes = [dict(lowdm=0.0, highdm=32.0, dmstep=0.5, sub_dmstep=8.0, ncalls=4, calldms=16,
                   binsize=1),
              dict(lowdm=32.0, highdm=96.0, dmstep=1.0, sub_dmstep=16.0, ncalls=4, calldms=16,
                   binsize=2)]
    spec = ";".join("%r,%r,%r,%r,%d,%d,%d" % (p["lowdm"], p["highdm"], p["dmstep"],
                                               p["sub_dmstep"], p["ncalls"], p["calldms"],
                                               p["binsize"]) for p in passes)
    dshift = orc.dmshifts(NCH, FCH1, FOFF)
    ms = int(np.float32(dshift[-1]) * np.float32(96.0) / np.float32(TSAMP))
    x = np.random.default_rng(64).standard_normal((NCH, nblocks * nsamp + ms), dtype=np.float32)
    _pulses(x, nsamp, nblocks)
    odir = tmp_path / "out"
    odir.mkdir()
    info, _ = run(driver, tmp_path, x, nsamp, "subband", nsubs, spec,
                  env={"MDSM_DRIVER_OUTPUT": str(odir), "MDSM_DRIVER_THRESHOLD": repr(thr)})
    assert info["blocks"] == nblocks + 1, info
    got = (odir / "cands.dat").read_text().splitlines()
    plan = m.SubbandPlan(NCH, FCH1, FOFF, TSAMP, nsamp, nsubs, passes, in_dtype="f32",
                         out_dtype="f32")
    i = plan.info
    dmv = plan.dm_values()
    rate = float(np.float32(TSAMP))
    want = []
    for k in range(nblocks):
        b = block_input(x, k, nsamp, ms, max(i.in_stride, nsamp + ms))
        d_in = plan.alloc_input()
        rows = d_in[: NCH * i.in_stride].view(NCH, i.in_stride)
        w = min(i.in_stride, b.shape[1])
        rows[:, :w].copy_(torch.from_numpy(np.ascontiguousarray(b[:, :w])))
        d_out = plan.alloc_output()
        plan.dedisperse_device(d_in, d_out)
        torch.cuda.synchronize()
        c, _ = m.ref_detect_subband_device(plan, d_out.view(i.ndms, nsamp), thr)
        ts = 1000.0 + float(k) * float(nsamp) * rate
        for row, samp, wid, snr in zip(c["dm_idx"], c["sample"], c["width"], c["snr"]):
            want.append("%f, %f, %f" % (ts + float(samp) * rate * float(max(1, int(wid))),
                                        float(dmv[row]), float(snr)))
    assert len(want) > 3 * nblocks
    assert got == want
