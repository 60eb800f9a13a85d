"""Parity with the reference's own CUDA kernels.

src/mdsm/dedispersion_kernel.cu is compiled unmodified for sm_103a into
oracle/_ref/ref_kernels.cubin (oracle/Makefile) and launched by oracle/ref_gpu_harness.c with
the grids of src/mdsm/dedispersion_thread.cu.  Our kernels must reproduce its float outputs
bit for bit on the region it computes.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def refgpu(orc, cuda):
    if not os.path.exists(orc.REF_CUBIN):
        pytest.skip("reference cubin not built (needs the reference tree when building)")
    if not os.path.exists(orc.HARNESS_SO):
        pytest.skip("reference launcher not built")
    return orc.RefGPU()


def _ours(plan, x, torch):
    d_in = plan.alloc_input()
    nchans, stride = plan.input_shape()
    buf = np.zeros((nchans, stride), x.dtype)
    w = min(stride, x.shape[1])
    buf[:, :w] = x[:, :w]
    d_in[: buf.size].copy_(torch.from_numpy(buf.ravel()))
    d_out = plan.alloc_output()
    plan.dedisperse_device(d_in, d_out)
    torch.cuda.synchronize()
    return d_out.cpu().numpy()


@pytest.mark.parametrize("mode,kind", [("l1", 0), ("opt", 1)])
def test_reference_brute_kernels_bitexact(lib, orc, cuda, refgpu, mode, kind):
    import mdsm_gb300 as m
    from mdsm_gb300 import synth
    torch = cuda
    nchans, tsamp = 256, 64e-6
    fch1, foff = 1500.0, -0.390625
    lowdm, dmstep, tdms = 0.0, 0.2, 480
    nsamp = 210 * 64 if kind == 0 else 128 * 100
    plan = m.BrutePlan(nchans, fch1, foff, tsamp, nsamp, [(lowdm, dmstep, tdms)],
                       shift_mode=mode, in_dtype="f32")
    ms = plan.maxshift + 2
    x, _ = synth.cfg1(nsamp_total=nsamp + ms)
    ref, _ = refgpu.brute(kind, x, nsamp, ms, lowdm, dmstep, tsamp, tdms, plan.dmshifts())
    got = _ours(plan, x, torch)
    assert np.array_equal(got, ref), "%d of %d differ" % (int((got != ref).sum()), ref.size)


def test_shift_contraction_variant(lib, orc, cuda, refgpu):
    """Which evaluation of start + i*step the compiled reference kernel uses: the default
    (contracted) table must match, and we record whether the uncontracted one would too."""
    import mdsm_gb300 as m
    torch = cuda
    nchans, nsamp, tsamp = 1024, 210 * 8, 64e-6
    fch1, foff = 1500.0, -300.0 / 1024
    segs = [(0.0, 0.9765625 / 3.0, 4096)]
    plan = m.BrutePlan(nchans, fch1, foff, tsamp, nsamp, segs, shift_mode="l1", in_dtype="f32")
    ms = plan.maxshift + 2
    # probe input: x[c][t] = t for one channel at a time would isolate shifts; a ramp per
    # channel with distinct slopes shows any shift difference in the sum.
    rng = np.random.default_rng(3)
    x = rng.standard_normal((nchans, nsamp + ms), dtype=np.float32)
    ref, _ = refgpu.brute(0, x, nsamp, ms, 0.0, segs[0][1], tsamp, segs[0][2], plan.dmshifts())
    got = _ours(plan, x, torch)
    assert np.array_equal(got, ref)


def test_reference_subband_bitexact(lib, orc, cuda, refgpu):
    import mdsm_gb300 as m
    torch = cuda
    nchans, nsubs, tsamp = 256, 16, 64e-6
    fch1, foff = 1500.0, -0.390625
    nsamp = 128 * 40
    p = dict(lowdm=0.0, highdm=100.0, dmstep=0.2, sub_dmstep=3.2, ncalls=32, calldms=16, ndms=512)
    plan = m.SubbandPlan(nchans, fch1, foff, tsamp, nsamp, nsubs, [p], in_dtype="f32")
    dms = plan.dmshifts()
    tempval = orc.lib().orc_subband_tempval(dms.ctypes.data_as(orc.ctypes.c_void_p), nchans, nsubs,
                                            orc.ctypes.c_float(p["highdm"]),
                                            orc.ctypes.c_float(tsamp))
    S1, S2 = plan.stage_tables()
    # The reference's stage-1 rows hold nsamp + tempval samples, but its fine DMs run past
    # highdm (dm0 = subDM - calldms*dmstep/2 + k*dmstep), so some stage-2 shifts exceed tempval
    # and the reference then reads the next subband's row.  Ours sizes rows by max(S2).
    assert S2.max() >= tempval
    ms = max(plan.maxshift, tempval + int(S1.max())) + 2
    rng = np.random.default_rng(11)
    x = rng.standard_normal((nchans, nsamp + ms), dtype=np.float32)
    z, ref, _ = refgpu.subband(x, nsamp, ms, nsubs, tempval, p["lowdm"], p["sub_dmstep"],
                               p["ncalls"], p["dmstep"], p["calldms"], tsamp, dms)
    got = _ours(plan, x, torch)
    # compare where the reference stage 2 stays inside its stage-1 rows
    ok_rows = (S2 <= tempval).all(axis=1)
    assert ok_rows.sum() > 0.9 * len(ok_rows)
    assert np.array_equal(got[ok_rows], ref[ok_rows])


def test_reference_kernels_timing_data_point(lib, orc, cuda, refgpu):
    """The reference's two brute-force kernels and ours on the same GB300, the same float
    input and the same plan (2048 channels x 65520 samples x 512 DM trials 0-255.5): kernel-only
    DM-trial-samples/s of each, printed as one JSON line (run with -s).  Ours must be faster
    than both, and equal to the L1 kernel's output on the region it computes."""
    import json
    import mdsm_gb300 as m
    torch = cuda
    nchans, nsamp, tsamp = 2048, 210 * 312, 64e-6
    fch1, foff = 1500.0, -300.0 / 2048
    lowdm, dmstep, tdms = 0.0, 0.5, 512
    plan = m.BrutePlan(nchans, fch1, foff, tsamp, nsamp, [(lowdm, dmstep, tdms)],
                       shift_mode="l1", in_dtype="f32")
    ms = plan.maxshift + 2
    rng = np.random.default_rng(9)
    x = rng.standard_normal((nchans, nsamp + ms), dtype=np.float32)
    rates = {}
    ref = None
    for kind, name in ((0, "reference global_for_time_dedisperse_loop"),
                       (1, "reference opt_dedisperse_loop")):
        t = []
        for _ in range(2):
            y, ms_k = refgpu.brute(kind, x, nsamp, ms, lowdm, dmstep, tsamp, tdms,
                                   plan.dmshifts())
            t.append(ms_k)
        covered = (tdms // 32 * 32) * (nsamp // 210 * 210) if kind == 0 else \
            tdms * (nsamp // 128 * 128)
        rates[name] = covered / (min(t) / 1e3)
        if kind == 0:
            ref = y
    d_in = plan.alloc_input()
    nch, stride = plan.input_shape()
    buf = np.zeros((nch, stride), np.float32)
    w = min(stride, x.shape[1])
    buf[:, :w] = x[:, :w]
    d_in[: buf.size].copy_(torch.from_numpy(buf.ravel()))
    d_out = plan.alloc_output()
    st = torch.cuda.current_stream()
    t = []
    for _ in range(4):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        plan.dedisperse_device(d_in, d_out, stream=st)
        e1.record(st)
        torch.cuda.synchronize()
        t.append(e0.elapsed_time(e1))
    rates["mdsm_gb300 k_shift_sum (float in, same plan)"] = tdms * nsamp / (min(t[1:]) / 1e3)
    got = d_out.cpu().numpy()
    assert np.array_equal(got, ref)
    print(json.dumps({"case": "float32 2048 ch x 65520 samples x 512 DM trials, kernel only",
                      "dm_trial_samples_per_s": rates}))
    ours = rates["mdsm_gb300 k_shift_sum (float in, same plan)"]
    assert ours > rates["reference global_for_time_dedisperse_loop"]
    assert ours > rates["reference opt_dedisperse_loop"]
