"""Brute-force dedispersion on the GPU through the C ABI, against the oracle.

Float input: bit-identical to the oracle's sequential float sum (the reference kernels' order).
Integer input: exact INT32 sums, equal to the oracle's integer sums.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(plan, x, torch):
    d_in = plan.alloc_input()
    flat = x.ravel()
    d_in[: flat.size].copy_(torch.from_numpy(flat))
    d_out = plan.alloc_output()
    plan.dedisperse_device(d_in, d_out)
    torch.cuda.synchronize()
    return d_out.cpu().numpy()


def _input(plan, dtype, rng):
    nchans, stride = plan.input_shape()
    if dtype == "f32":
        return rng.standard_normal((nchans, stride), dtype=np.float32)
    if dtype == "u8":
        return rng.integers(0, 256, (nchans, stride), dtype=np.uint8)
    if dtype == "u16":
        return rng.integers(0, 65536, (nchans, stride), dtype=np.uint16)
    return rng.integers(-32768, 32768, (nchans, stride), dtype=np.int16)


CASES = [
    # nchans, nsamp, segments, dtype, mode
    (64, 3000, [(0.0, 1.5, 40)], "f32", "l1"),
    (256, 4096, [(0.0, 0.2, 500)], "f32", "l1"),
    (100, 1000, [(3.0, 0.7, 33)], "u8", "opt"),
    (48, 777, [(0.0, 2.0, 17), (34.0, 4.0, 9)], "u16", "l1"),
    (48, 300, [(0.0, 3.0, 70)], "i16", "l1_muladd"),
    (16, 5, [(0.0, 1.0, 1)], "f32", "fp64_trunc"),
    (1, 257, [(0.0, 1.0, 8)], "u8", "l1"),
    (513, 1025, [(0.0, 0.5, 65)], "u8", "fp64_round"),
]


@pytest.mark.parametrize("nchans,nsamp,segs,dtype,mode", CASES)
def test_brute_matches_oracle(lib, orc, cuda, nchans, nsamp, segs, dtype, mode):
    import mdsm_gb300 as m
    torch = cuda
    out = "f32" if dtype == "f32" else "i32"
    plan = m.BrutePlan(nchans, 1500.0, -300.0 / max(nchans, 1) if nchans > 1 else -1.0, 64e-6,
                       nsamp, segs, shift_mode=mode, in_dtype=dtype, out_dtype=out)
    rng = np.random.default_rng(nchans * 7 + nsamp)
    x = _input(plan, dtype, rng)
    got = _run(plan, x, torch)
    S = plan.shift_table()
    want = orc.dedisperse(x, S, nsamp)
    assert got.dtype == want.dtype
    assert np.array_equal(got, want), "%d mismatches" % int((got != want).sum())
    assert plan.last_launches == 1


def test_known_answer_channel_index(lib, orc, cuda):
    """x[c][t] = c gives sum_c c for every DM and sample, for any shift table
    (src/prototypes/brute_dedisp_imp_tex.cu:112-114,168-175)."""
    import mdsm_gb300 as m
    torch = cuda
    nchans, nsamp = 300, 2048
    plan = m.BrutePlan(nchans, 1400.0, -0.5, 1e-4, nsamp, [(0.0, 5.0, 96)], in_dtype="f32")
    _, stride = plan.input_shape()
    x = np.repeat(np.arange(nchans, dtype=np.float32)[:, None], stride, axis=1)
    got = _run(plan, x, torch)
    assert np.all(got == nchans * (nchans - 1) / 2)


def test_host_path_equals_device_path(lib, orc, cuda):
    import mdsm_gb300 as m
    torch = cuda
    nchans, nsamp = 128, 5000
    plan = m.BrutePlan(nchans, 1500.0, -1.0, 64e-6, nsamp, [(0.0, 1.0, 64)], in_dtype="u8",
                       out_dtype="i32")
    info = plan.info
    rng = np.random.default_rng(5)
    # reference host layout: pitch exactly nsamp + maxshift
    h = rng.integers(0, 256, (nchans, nsamp + info.maxshift), dtype=np.uint8)
    got = plan.dedisperse_host(h)
    want = orc.dedisperse(h, plan.shift_table(), nsamp)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("dtype,nsamp", [("u8", 40000), ("f32", 33001), ("u8", 16384 * 9 + 7)])
def test_pipelined_host_path(lib, orc, cuda, dtype, nsamp):
    """Blocks of >= 32768 samples go through the host path in time segments (copy in,
    compute and copy out overlapped); the result equals the oracle's whole-block sum, including
    a ragged last segment and the most segments."""
    import mdsm_gb300 as m
    nchans = 64
    plan = m.BrutePlan(nchans, 1500.0, -4.0, 64e-6, nsamp, [(0.0, 2.0, 40)], in_dtype=dtype,
                       out_dtype="i32" if dtype == "u8" else "f32")
    info = plan.info
    rng = np.random.default_rng(nsamp)
    h = rng.integers(0, 256, (nchans, nsamp + info.maxshift + 3)).astype(
        np.uint8 if dtype == "u8" else np.float32)
    want = orc.dedisperse(h, plan.shift_table(), nsamp)
    for _ in range(2):  # a second call reuses the plan's streams and events
        got = plan.dedisperse_host(h)
        assert np.array_equal(got, want)


def test_cfg1_full_size_bitexact_and_fp64_error(lib, orc, cuda):
    """Config 1 at full size: 256 ch x 32768 float samples, 500 DMs 0-99.8.  Bit-identical to
    the reference kernels' float arithmetic (the oracle), and against FP64:
    * normwise error max |y32 - y64| / sum_c |x| (the error relative to the summation's own
      scale, which bounds sequential FP32 summation), required below 1e-6;
    * elementwise relative error max |y32 - y64| / |y64| over outputs with |y64| > 1e-3 sum_c
      |x|, printed: the reference's sequential FP32 order makes it ~1e-4 on sums of N(0,1)
      samples that cancel to 1e-3 of their scale, so no 1e-6 bound holds elementwise for this
      input type (integer samples take the exact INT32 or compensated FP32 sums instead)."""
    import mdsm_gb300 as m
    from mdsm_gb300 import synth
    torch = cuda
    x, meta = synth.cfg1()
    S = orc.shift_table(256, meta["fch1"], meta["foff"], meta["tsamp"], synth.cfg1_segments())
    nsamp = 32768 - int(S.max())
    plan = m.BrutePlan(256, meta["fch1"], meta["foff"], meta["tsamp"], nsamp,
                       synth.cfg1_segments(), in_dtype="f32")
    assert np.array_equal(plan.shift_table(), S)
    got = plan.dedisperse_host(x)
    want = orc.dedisperse(x, S, nsamp)
    assert np.array_equal(got, want)
    y64 = orc.dedisperse(x, S, nsamp, out="f64")
    scale = orc.dedisperse(np.abs(x), S, nsamp, out="f64")
    err = np.abs(got.astype(np.float64) - y64)
    rel = err / scale
    big = np.abs(y64) > 1e-3 * scale
    elem = (err[big] / np.abs(y64[big])).max()
    print("cfg1 FP32: normwise %.3g, elementwise %.3g" % (rel.max(), elem))
    assert rel.max() < 1e-6


@pytest.mark.parametrize("nchans,nsamp,ndms", [(4096, 2000, 40), (257, 511, 33), (9, 4, 1),
                                               (600, 3333, 100)])
def test_packed_u8_matches_generic_and_oracle(lib, orc, cuda, nchans, nsamp, ndms):
    """The packed 8-bit kernel (default for uint8) against the generic kernel and the oracle,
    including all-255 input where every partial-sum stage is filled to its limit."""
    import mdsm_gb300 as m
    torch = cuda
    segs = [(0.0, 0.5, ndms)]
    packed = m.BrutePlan(nchans, 1500.0, -300.0 / nchans, 64e-6, nsamp, segs, in_dtype="u8",
                         out_dtype="i32")
    generic = m.BrutePlan(nchans, 1500.0, -300.0 / nchans, 64e-6, nsamp, segs, in_dtype="u8",
                          out_dtype="i32", kernel=1)
    assert packed.info.kernel == 2 and generic.info.kernel == 1
    for fill in ("random", "max"):
        nch, stride = packed.input_shape()
        if fill == "max":
            x = np.full((nch, stride), 255, np.uint8)
        else:
            x = np.random.default_rng(nchans).integers(0, 256, (nch, stride), dtype=np.uint8)
        got = _run(packed, x, torch)
        want = orc.dedisperse(x, packed.shift_table(), nsamp)
        assert np.array_equal(got, want), fill
        xg = np.zeros(generic.input_shape(), np.uint8)
        w = min(xg.shape[1], x.shape[1])
        xg[:, :w] = x[:, :w]
        assert np.array_equal(_run(generic, xg, torch), want), fill


@pytest.mark.parametrize("nchans,nsamp,ndms", [(1024, 2000, 40), (257, 511, 17), (9, 4, 1),
                                               (600, 3333, 100), (32767, 600, 3)])
def test_packed_u16_matches_generic_and_oracle(lib, orc, cuda, nchans, nsamp, ndms):
    """The packed 16-bit kernel (default for uint16) against the generic kernel and the
    oracle, including all-65535 input (lane sums up to 2^31 - 1 over 32767 channels)."""
    import mdsm_gb300 as m
    torch = cuda
    segs = [(0.0, 0.5 if nchans < 10000 else 0.02, ndms)]
    packed = m.BrutePlan(nchans, 1500.0, -300.0 / nchans, 64e-6, nsamp, segs, in_dtype="u16",
                         out_dtype="i32")
    generic = m.BrutePlan(nchans, 1500.0, -300.0 / nchans, 64e-6, nsamp, segs,
                          in_dtype="u16", out_dtype="i32", kernel=1)
    assert packed.info.kernel == 3 and generic.info.kernel == 1
    for fill in ("random", "max"):
        nch, stride = packed.input_shape()
        if fill == "max":
            x = np.full((nch, stride), 65535, np.uint16)
        else:
            x = np.random.default_rng(nchans).integers(0, 65536, (nch, stride), dtype=np.uint16)
        got = _run(packed, x, torch)
        want = orc.dedisperse(x, packed.shift_table(), nsamp)
        assert np.array_equal(got, want), fill
        xg = np.zeros(generic.input_shape(), np.uint16)
        w = min(xg.shape[1], x.shape[1])
        xg[:, :w] = x[:, :w]
        assert np.array_equal(_run(generic, xg, torch), want), fill


def test_int32_accumulation_refused_when_sums_may_overflow(lib):
    import mdsm_gb300 as m
    from mdsm_gb300 import MdsmError
    with pytest.raises(MdsmError) as e:
        m.BrutePlan(32769, 1500.0, -300.0 / 32769, 64e-6, 100, [(0.0, 0.01, 2)], in_dtype="u16",
                    out_dtype="i32", acc="i32")
    assert e.value.status == 6  # MDSM_ERANGE
    auto = m.BrutePlan(32769, 1500.0, -300.0 / 32769, 64e-6, 100, [(0.0, 0.01, 2)],
                       in_dtype="u16", out_dtype="f32")
    assert auto.info.acc == 2  # automatic: FP32 (MDSM_ACC_F32) for sums that may not fit


def test_packed_falls_back_for_wide_plans(lib, orc, cuda):
    """A DM block whose shift span does not fit the packed kernel's staging runs on the
    generic kernel, with the same exact result."""
    import mdsm_gb300 as m
    torch = cuda
    plan = m.BrutePlan(1024, 1500.0, -300.0 / 1024, 64e-6, 1000, [(0.0, 20.0, 40)],
                       in_dtype="u8", out_dtype="i32")
    assert plan.info.kernel == 1
    nch, stride = plan.input_shape()
    x = np.random.default_rng(9).integers(0, 256, (nch, stride), dtype=np.uint8)
    assert np.array_equal(_run(plan, x, torch), orc.dedisperse(x, plan.shift_table(), 1000))


def test_packed_u8_float_output(lib, orc, cuda):
    import mdsm_gb300 as m
    torch = cuda
    plan = m.BrutePlan(512, 1500.0, -0.5, 64e-6, 1500, [(0.0, 1.0, 64)], in_dtype="u8",
                       out_dtype="f32")
    nch, stride = plan.input_shape()
    x = np.random.default_rng(2).integers(0, 256, (nch, stride), dtype=np.uint8)
    got = _run(plan, x, torch)
    assert got.dtype == np.float32
    assert np.array_equal(got, orc.dedisperse(x, plan.shift_table(), 1500).astype(np.float32))


def test_packed_u16_tile_widths(lib, orc, cuda):
    """The packed 16-bit kernel takes 768- or 512-sample tiles as its staging fits shared memory
    (larger DM steps widen the staged rows); each width exact against the oracle, with
    all-65535 rows included."""
    import mdsm_gb300 as m
    torch = cuda
    nchans, nsamp = 512, 2500
    seen = set()
    for dmstep in (0.25, 0.5, 1.0, 1.5, 4.0):
        plan = m.BrutePlan(nchans, 1500.0, -300.0 / nchans, 64e-6, nsamp, [(0.0, dmstep, 40)],
                           in_dtype="u16", out_dtype="i32")
        st = plan.stage_info(0)
        if st.kernel != 3:
            continue
        seen.add(st.time_tile)
        nch, stride = plan.input_shape()
        x = np.random.default_rng(int(dmstep * 10)).integers(0, 65536, (nch, stride),
                                                              dtype=np.uint16)
        x[::7] = 65535
        got = _run(plan, x, torch)
        assert np.array_equal(got, orc.dedisperse(x, plan.shift_table(), nsamp)), dmstep
    assert {768, 512} <= seen, seen


@pytest.mark.parametrize("nchans,nsamp,ndms", [(48, 3000, 70), (600, 2222, 40), (32767, 600, 3)])
def test_packed_i16_matches_oracle(lib, orc, cuda, nchans, nsamp, ndms):
    """int16 samples on the packed 16-bit kernel (offset binary in shared memory, 32768 per
    channel taken off at the store): exact against the oracle, with rows of -32768 and of
    32767 throughout (sums down to -32768 * 32767)."""
    import mdsm_gb300 as m
    torch = cuda
    segs = [(0.0, 0.5 if nchans < 10000 else 0.02, ndms)]
    plan = m.BrutePlan(nchans, 1500.0, -300.0 / nchans, 64e-6, nsamp, segs, in_dtype="i16",
                       out_dtype="i32")
    assert plan.info.kernel == 3
    nch, stride = plan.input_shape()
    for fill in ("random", "min", "max"):
        if fill == "random":
            x = np.random.default_rng(nchans).integers(-32768, 32768, (nch, stride),
                                                       dtype=np.int16)
        else:
            x = np.full((nch, stride), -32768 if fill == "min" else 32767, np.int16)
        got = _run(plan, x, torch)
        assert np.array_equal(got, orc.dedisperse(x, plan.shift_table(), nsamp)), fill
