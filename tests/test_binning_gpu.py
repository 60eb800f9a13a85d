"""Time downsampling of channel-major blocks and subband passes with downsample > 1."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ds(torch, x, dtype_in, nchans, stride, length, b, mode, dtype_out, out_stride):
    from mdsm_gb300 import _lib
    tdt = {"u8": torch.uint8, "u16": torch.uint16, "i16": torch.int16, "f32": torch.float32,
           "i32": torch.int32}
    d_in = torch.from_numpy(x).cuda()
    d_out = torch.zeros((nchans, out_stride), dtype=tdt[dtype_out], device="cuda")
    _lib.check(_lib.load().mdsm_downsample_device(
        ctypes.c_void_p(d_in.data_ptr()), _lib.DTYPES[dtype_in], nchans, stride, length, b, mode,
        ctypes.c_void_p(d_out.data_ptr()), _lib.DTYPES[dtype_out], out_stride,
        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    torch.cuda.synchronize()
    return d_out.cpu().numpy()


@pytest.mark.parametrize("b", [1, 2, 3, 8])
def test_downsample_sum_mean_sqrt(lib, cuda, b):
    torch = cuda
    rng = np.random.default_rng(b)
    nchans, stride, length = 37, 1000, 997
    x = rng.integers(0, 256, (nchans, stride), dtype=np.uint8)
    nout = length // b
    want = x[:, : nout * b].reshape(nchans, nout, b).astype(np.int64).sum(axis=2)
    got = _ds(torch, x, "u8", nchans, stride, length, b, 0, "u16", 1024)
    assert np.array_equal(got[:, :nout], want) and not got[:, nout:].any()
    got = _ds(torch, x, "u8", nchans, stride, length, b, 0, "i32", 1024)
    assert np.array_equal(got[:, :nout], want)
    # mean and 1/sqrt(b) in float32: left-to-right float sums, then one multiply
    acc = np.zeros((nchans, nout), np.float32)
    for k in range(b):
        acc = acc + x[:, k: nout * b: b][:, :nout].astype(np.float32)
    for mode, scale in ((1, np.float32(1.0) / np.float32(b)),
                        (2, np.float32(1.0) / np.sqrt(np.float32(b)))):
        got = _ds(torch, x, "u8", nchans, stride, length, b, mode, "f32", 1024)
        assert np.array_equal(got[:, :nout], acc * scale), mode


def test_subband_downsampled_passes(lib, orc, cuda):
    import mdsm_gb300 as m
    torch = cuda
    nchans, nsubs, tsamp, fch1, foff = 256, 16, 64e-6, 1500.0, -0.390625
    nsamp = 4096
    passes = [dict(lowdm=0.0, highdm=40.0, dmstep=0.25, sub_dmstep=4.0, ncalls=10, calldms=16,
                   binsize=1),
              dict(lowdm=40.0, highdm=120.0, dmstep=0.5, sub_dmstep=8.0, ncalls=10, calldms=16,
                   binsize=2),
              dict(lowdm=120.0, highdm=280.0, dmstep=1.0, sub_dmstep=16.0, ncalls=10, calldms=16,
                   binsize=4)]
    plan = m.SubbandPlan(nchans, fch1, foff, tsamp, nsamp, nsubs, passes, in_dtype="u8",
                         out_dtype="i32")
    nch, stride = plan.input_shape()
    x = np.random.default_rng(3).integers(0, 256, (nch, stride), dtype=np.uint8)
    d_in = plan.alloc_input()
    d_in[: x.size].copy_(torch.from_numpy(x.ravel()))
    d_out = plan.alloc_output()
    d_out.zero_()
    plan.dedisperse_device(d_in, d_out)
    torch.cuda.synchronize()
    got = d_out.cpu().numpy()
    row = 0
    info = plan.info
    for p in passes:
        b = p["binsize"]
        tsb = float(np.float32(tsamp) * np.float32(b))
        S1, S2 = orc.subband_tables(nchans, fch1, foff, tsb, nsubs, p["lowdm"], p["sub_dmstep"],
                                    p["ncalls"], p["dmstep"], p["calldms"])
        nsb = nsamp // b
        length = (nsamp + info.maxshift) // b
        xd = x[:, : length * b].reshape(nch, length, b).astype(np.int64).sum(axis=2)
        n1 = nsb + int(S2.max())
        _, want = orc.subband_dedisperse(xd.astype(np.float32), S1, S2, nsubs, nsb, n1,
                                         p["calldms"])
        k = want.shape[0]
        assert np.array_equal(got[row:row + k, :nsb].astype(np.float32), want), b
        assert not got[row:row + k, nsb:].any()
        row += k
