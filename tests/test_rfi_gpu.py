"""RFI clipping on the GPU against the oracle, bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _with_rfi(dtype, nchans, length, stride, seed):
    from mdsm_gb300 import synth
    rng = np.random.default_rng(seed)
    if dtype == "u8":
        x = synth.gaussian_u8(nchans, stride, seed)
        sig = 16
    elif dtype == "i16":
        x = synth.gaussian_i16(nchans, stride, seed)
        sig = 1000
    else:
        x = synth.gaussian_f32(nchans, stride, seed)
        sig = 1
    # 1% broadband impulses at 50 sigma, 5 narrowband 10-sigma sinusoids
    cols = rng.choice(length, length // 100, replace=False)
    if dtype == "f32":
        x[:, cols] += np.float32(50 * sig)
    else:
        info = np.iinfo(x.dtype)
        x[:, cols] = np.clip(x[:, cols].astype(np.int64) + 50 * sig, info.min, info.max)
    for c in rng.choice(nchans, 5, replace=False):
        s = 10 * sig * np.sin(np.arange(stride) * 0.05)
        if dtype == "f32":
            x[c] += s.astype(np.float32)
        else:
            info = np.iinfo(x.dtype)
            x[c] = np.clip(x[c].astype(np.int64) + np.rint(s).astype(np.int64), info.min, info.max)
    return x


@pytest.mark.parametrize("dtype", ["u8", "i16", "f32"])
def test_rfi_clip_matches_oracle(lib, orc, cuda, dtype):
    import mdsm_gb300 as m
    torch = cuda
    nchans, length, stride = 96, 5000, 5008
    x = _with_rfi(dtype, nchans, length, stride, 17)
    want = orc.rfi_clip(x.copy(), length, 4.0, 4.0)
    tdt = {"u8": torch.uint8, "i16": torch.int16, "f32": torch.float32}[dtype]
    d = torch.from_numpy(x.copy()).to(device="cuda", dtype=tdt)
    m.rfi_clip_device(d, nchans, stride, length, 4.0, 4.0, dtype=dtype)
    got = d.cpu().numpy()
    assert np.array_equal(got, want)
    assert not np.array_equal(got, x)   # something was clipped
    assert np.array_equal(got[:, length:], x[:, length:])  # beyond len untouched


def test_rfi_clip_single_pass(lib, orc, cuda):
    import mdsm_gb300 as m
    torch = cuda
    nchans, length = 64, 4096
    x = _with_rfi("u8", nchans, length, length, 5)
    for kc, ks in ((4.0, 0.0), (0.0, 3.0)):
        want = orc.rfi_clip(x.copy(), length, kc, ks)
        d = torch.from_numpy(x.copy()).cuda()
        m.rfi_clip_device(d, nchans, length, length, kc, ks, dtype="u8")
        assert np.array_equal(d.cpu().numpy(), want)
