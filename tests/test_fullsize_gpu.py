"""Parity at the full benchmark size: uint8 4096 channels x 2^18 samples, 4096 DM trials
0-2000 (steps doubling at 500 and 1000), exact INT32 sums.  The oracle cannot sum the whole
4.4e12-add cube in a test, so: (1) 6 DM rows spread over the three segments are compared bit
for bit with the oracle's sums of those rows; (2) the whole cube through exact integer
linearity, y(x1 + x2) = y(x1) + y(x2) for inputs whose sum stays within uint8; (3) the
host-buffer path in 16 time segments equals the device path over the whole cube."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NCHANS, NSAMP, FCH1, BW, TSAMP = 4096, 1 << 18, 1500.0, 300.0, 64e-6


@pytest.fixture(scope="module")
def full(cuda):
    import mdsm_gb300 as m
    from mdsm_gb300 import synth
    torch = cuda
    plan = m.BrutePlan(NCHANS, FCH1, -BW / NCHANS, TSAMP, NSAMP, synth.cfg2_segments(),
                       in_dtype="u8", out_dtype="i32")
    info = plan.info
    assert info.kernel == 2 and info.ndms == 4096
    gen = torch.Generator(device="cuda")
    gen.manual_seed(123)
    n = info.nchans * info.in_stride
    x1 = plan.alloc_input()
    x1[:n].copy_(torch.randint(0, 128, (n,), generator=gen, device="cuda", dtype=torch.uint8))
    x2 = plan.alloc_input()
    x2[:n].copy_(torch.randint(0, 128, (n,), generator=gen, device="cuda", dtype=torch.uint8))
    return plan, x1, x2


def _run(plan, d_in, torch):
    d_out = plan.alloc_output()
    plan.dedisperse_device(d_in, d_out)
    torch.cuda.synchronize()
    return d_out


def test_rows_equal_oracle(lib, orc, cuda, full):
    torch = cuda
    plan, x1, _ = full
    info = plan.info
    y = _run(plan, x1, torch)
    rows = np.array([0, 1337, 2047, 2048, 3071, 4095])
    got = y[torch.from_numpy(rows).cuda()].cpu().numpy()
    del y
    x = x1[: info.nchans * info.in_stride].view(info.nchans, info.in_stride).cpu().numpy()
    S = plan.shift_table()[rows]
    want = orc.dedisperse(x, S, NSAMP)
    assert np.array_equal(got, want)


def test_linearity_whole_cube(lib, cuda, full):
    torch = cuda
    plan, x1, x2 = full
    y1 = _run(plan, x1, torch)
    y2 = _run(plan, x2, torch)
    y1 += y2
    del y2
    x3 = x1 + x2  # at most 254: no uint8 overflow
    y3 = _run(plan, x3, torch)
    del x3
    assert torch.equal(y1, y3)


def test_host_path_equals_device_path_whole_cube(lib, cuda, full):
    torch = cuda
    plan, x1, _ = full
    info = plan.info
    y = _run(plan, x1, torch).cpu().numpy()
    h = x1[: info.nchans * info.in_stride].view(info.nchans, info.in_stride)[
        :, : NSAMP + info.maxshift].cpu().numpy()
    got = plan.dedisperse_host(np.ascontiguousarray(h))
    assert np.array_equal(got, y)
