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


def run(driver, tmp_path, x, nsamp, *mode):
    spec = tmp_path / "spectra.f32"
    out = tmp_path / "series.f32"
    np.ascontiguousarray(x.T).astype(np.float32).tofile(spec)
    args = [str(driver), str(spec), str(out), str(NCH), str(nsamp), repr(FCH1), repr(FOFF),
            repr(TSAMP)] + [str(a) for a in mode]
    r = subprocess.run(args, capture_output=True, text=True, timeout=300)
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
