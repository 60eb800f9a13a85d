"""Precision modes: 8/16-bit samples accumulated exactly in INT32, or in FP32, against the
FP64 oracle.  The FP32 error is measured as |y32 - y64| / sum_c |x| (the summation's own
condition scale)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(plan, x, torch):
    d_in = plan.alloc_input()
    d_in[: x.size].copy_(torch.from_numpy(x.ravel()))
    d_out = plan.alloc_output()
    plan.dedisperse_device(d_in, d_out)
    torch.cuda.synchronize()
    return d_out.cpu().numpy()


@pytest.mark.parametrize("dtype", ["u8", "i16"])
def test_int32_exact_and_fp32_bounded(lib, orc, cuda, dtype):
    import mdsm_gb300 as m
    from mdsm_gb300 import synth
    torch = cuda
    nchans, nsamp, segs = 4096, 2048, [(0.0, 0.5, 64)]
    exact = m.BrutePlan(nchans, 1500.0, -300.0 / nchans, 64e-6, nsamp, segs, in_dtype=dtype,
                        out_dtype="i32", acc="i32")
    fp32 = m.BrutePlan(nchans, 1500.0, -300.0 / nchans, 64e-6, nsamp, segs, in_dtype=dtype,
                       out_dtype="f32", acc="f32")
    nch, stride = exact.input_shape()
    x = synth.gaussian_u8(nch, stride, 1) if dtype == "u8" else synth.gaussian_i16(nch, stride, 1)
    x[:, ::97] = np.iinfo(x.dtype).max  # impulses push partial sums far from zero
    S = exact.shift_table()
    y64 = orc.dedisperse(x, S, nsamp).astype(np.float64)  # exact integer sums
    yi = _run(exact, x, torch)
    assert np.array_equal(yi.astype(np.float64), y64)
    yf = _run(fp32, x, torch).astype(np.float64)
    scale = orc.dedisperse(np.abs(x.astype(np.int32)).astype(np.float32), S, nsamp,
                           out="f64")
    rel = np.abs(yf - y64) / np.maximum(scale, 1.0)
    if dtype == "u8":
        assert rel.max() == 0.0          # sums below 2^24 are exact in FP32
    else:
        # exact INT32 chunk sums, Kahan-compensated FP32 across chunks: within
        # 2 * 2^-24 * sum|x| plus the final rounding; the stated target is 1e-6
        assert rel.max() <= 2.5 * 2.0 ** -24
        assert rel.max() < 1e-6
        assert (yf != y64).any()         # sums above 2^24 did round
