"""Failure detection on the device, in the form this pool allows: a bounded wait that runs out.

The dedispersion kernels' mbarrier waits are bounded (src of the bound: ptx.cuh
mbar_wait_bounded); a wait that runs out records ERR_WAIT_TIMEOUT in the plan's device error
word and the kernel returns.  mdsm_plan_wait_selftest runs that same wait on an mbarrier nothing
arrives at, with a short spin limit, so it runs out without any fault, trap or hang.  The test
checks that the timeout surfaces as MDSM_ETIMEOUT (mdsm_plan_check, and the host-buffer entry
point, which checks by itself), that the record is cleared by reading it, and that the same plan
and context keep producing correct results afterwards."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ETIMEOUT = 4


def test_wait_timeout_reported_and_plan_recovers(lib, orc, cuda):
    import mdsm_gb300 as m
    torch = cuda
    nchans, nsamp, segs = 256, 4096, [(0.0, 1.0, 64)]
    plan = m.BrutePlan(nchans, 1500.0, -1.0, 64e-6, nsamp, segs, in_dtype="u8",
                       out_dtype="i32")
    rng = np.random.default_rng(9)
    nch, stride = plan.input_shape()
    x = rng.integers(0, 256, (nch, stride), dtype=np.uint8)
    d_in = plan.alloc_input()
    d_in[: x.size].copy_(torch.from_numpy(x.ravel()))
    d_out = plan.alloc_output()
    want = orc.dedisperse(x, plan.shift_table(), nsamp)
    st = torch.cuda.Stream()
    for limit in (1, 4096):
        # the bounded wait runs out: reported once, then cleared
        plan.wait_selftest(limit, stream=st)
        with pytest.raises(m.MdsmError) as e:
            plan.check(stream=st)
        assert e.value.status == ETIMEOUT
        plan.check(stream=st)
        # the plan and the context still work
        d_out.zero_()
        plan.dedisperse_device(d_in, d_out, stream=st)
        plan.check(stream=st)
        assert np.array_equal(d_out.cpu().numpy(), want)
    # the host-buffer entry point reports a timeout recorded before it, then recovers
    plan.wait_selftest(64, stream=st)
    h = x[:, : nsamp + plan.info.maxshift].copy()
    with pytest.raises(m.MdsmError) as e:
        plan.dedisperse_host(h, stream=st)
    assert e.value.status == ETIMEOUT
    assert np.array_equal(plan.dedisperse_host(h, stream=st), want)


def test_selftest_argument_errors(lib, cuda):
    import mdsm_gb300 as m
    plan = m.BrutePlan(64, 1500.0, -1.0, 64e-6, 1024, [(0.0, 1.0, 8)], in_dtype="u8")
    for bad in (0, 1 << 17):
        with pytest.raises(m.MdsmError):
            plan.wait_selftest(bad)
