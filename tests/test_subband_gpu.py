"""Two-stage subband dedispersion on the GPU against the oracle (the reference's stage order:
channels within a subband, then subbands, each summed in increasing index)."""
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


@pytest.mark.parametrize("dtype", ["f32", "u8"])
def test_subband_matches_oracle(lib, orc, cuda, dtype):
    import mdsm_gb300 as m
    torch = cuda
    nchans, nsubs, tsamp, fch1, foff = 512, 32, 64e-6, 1500.0, -300.0 / 512
    nsamp = 3000
    p = dict(lowdm=0.0, highdm=300.0, dmstep=0.5, sub_dmstep=8.0, ncalls=37, calldms=16)
    plan = m.SubbandPlan(nchans, fch1, foff, tsamp, nsamp, nsubs, [p], in_dtype=dtype,
                         out_dtype="f32" if dtype == "f32" else "i32")
    nch, stride = plan.input_shape()
    rng = np.random.default_rng(4)
    if dtype == "f32":
        x = rng.standard_normal((nch, stride), dtype=np.float32)
    else:
        x = rng.integers(0, 256, (nch, stride), dtype=np.uint8)
    got = _run(plan, x, torch)
    S1, S2 = plan.stage_tables()
    W1, W2 = orc.subband_tables(nchans, fch1, foff, tsamp, nsubs, p["lowdm"], p["sub_dmstep"],
                                p["ncalls"], p["dmstep"], p["calldms"])
    assert np.array_equal(S1, W1) and np.array_equal(S2, W2)
    n1 = nsamp + int(S2.max())
    _, want = orc.subband_dedisperse(x.astype(np.float32), S1, S2, nsubs, nsamp, n1, p["calldms"])
    assert np.array_equal(got.astype(np.float32), want)


def test_subband_multi_pass(lib, orc, cuda):
    import mdsm_gb300 as m
    torch = cuda
    nchans, nsubs, tsamp, fch1, foff = 256, 16, 64e-6, 1500.0, -0.390625
    nsamp = 2048
    passes = [dict(lowdm=0.0, highdm=50.0, dmstep=0.25, sub_dmstep=4.0, ncalls=13, calldms=16),
              dict(lowdm=50.0, highdm=150.0, dmstep=0.5, sub_dmstep=8.0, ncalls=13, calldms=16)]
    plan = m.SubbandPlan(nchans, fch1, foff, tsamp, nsamp, nsubs, passes, in_dtype="u8",
                         out_dtype="i32")
    nch, stride = plan.input_shape()
    x = np.random.default_rng(8).integers(0, 256, (nch, stride), dtype=np.uint8)
    got = _run(plan, x, torch)
    assert got.shape[0] == 13 * 16 * 2
    row = 0
    for p in passes:
        S1, S2 = orc.subband_tables(nchans, fch1, foff, tsamp, nsubs, p["lowdm"], p["sub_dmstep"],
                                    p["ncalls"], p["dmstep"], p["calldms"])
        n1 = nsamp + int(S2.max())
        _, want = orc.subband_dedisperse(x.astype(np.float32), S1, S2, nsubs, nsamp, n1,
                                         p["calldms"])
        k = want.shape[0]
        assert np.array_equal(got[row:row + k].astype(np.float32), want)
        row += k


def test_subband_recovers_injected_pulse(lib, orc, cuda):
    """A dispersed pulse peaks at the right DM in both brute force and subband series."""
    import mdsm_gb300 as m
    from mdsm_gb300 import synth
    torch = cuda
    nchans, nsubs, tsamp, fch1, foff = 1024, 32, 64e-6, 1500.0, -300.0 / 1024
    nsamp = 8192
    p = dict(lowdm=0.0, highdm=256.0, dmstep=0.5, sub_dmstep=8.0, ncalls=32, calldms=16)
    plan = m.SubbandPlan(nchans, fch1, foff, tsamp, nsamp, nsubs, [p], in_dtype="u8",
                         out_dtype="i32")
    nch, stride = plan.input_shape()
    x = synth.gaussian_u8(nch, stride, seed=3)
    synth.inject(x, fch1, foff, tsamp, [(3000, 150.0, 8, 8.0)], K=4148.741601)
    y = _run(plan, x, torch).astype(np.float64)
    dms = plan.dm_values()
    z = (y - y.mean(axis=1, keepdims=True)) / y.std(axis=1, keepdims=True)
    d, t = np.unravel_index(np.argmax(z), z.shape)
    assert abs(dms[d] - 150.0) < 2.0 and abs(t - 3000) < 10


def test_subband_first_stage_tile_widths(lib, orc, cuda):
    """The uint16 first stage takes 1024-, 768- or 512-sample tiles as its staging fits shared
    memory (wider sub-DM steps widen the shift span); every width, and the int32 fallback past
    them, against the oracle."""
    import mdsm_gb300 as m
    torch = cuda
    nchans, nsubs, tsamp, fch1, foff = 1024, 16, 64e-6, 1500.0, -300.0 / 1024
    nsamp = 3000
    seen = set()
    for sub_dmstep in (2.0, 6.0, 12.0, 40.0):
        p = dict(lowdm=0.0, highdm=32 * sub_dmstep, dmstep=sub_dmstep / 16, sub_dmstep=sub_dmstep,
                 ncalls=32, calldms=16)
        plan = m.SubbandPlan(nchans, fch1, foff, tsamp, nsamp, nsubs, [p], in_dtype="u8",
                             out_dtype="i32")
        s1 = plan.stage_info(0)
        seen.add(s1.time_tile if s1.out_u16 else 0)
        nch, stride = plan.input_shape()
        x = np.random.default_rng(int(sub_dmstep)).integers(0, 256, (nch, stride), dtype=np.uint8)
        got = _run(plan, x, torch)
        S1, S2 = plan.stage_tables()
        n1 = nsamp + int(S2.max())
        _, want = orc.subband_dedisperse(x.astype(np.float32), S1, S2, nsubs, nsamp, n1,
                                         p["calldms"])
        assert np.array_equal(got.astype(np.float32), want), sub_dmstep
    assert {1024, 768, 512} <= seen, seen
