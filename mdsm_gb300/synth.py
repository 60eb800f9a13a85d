"""Seeded synthetic filterbanks with the shapes of the benchmark configurations.

No observation data ships with the reference (its example files point at absent paths), so
tests and the benchmark use Gaussian noise with injected dispersed boxcar pulses, as the
reference's own fake-signal generator does (src/prototypes/genrateFakeBroadbandSignal.py:6-18).
Pulse delays use K = 4148.808 s MHz^2 cm^3/pc and are rounded to whole samples.
"""
import numpy as np

K_INJECT = 4148.808


def band_offsets(nchans, bw_mhz):
    """Channel width for a band of bw_mhz split into nchans (descending frequency)."""
    return -float(bw_mhz) / nchans


def cfg2_segments():
    """4096 DM trials 0-2000 with the step doubling at 500 and 1000."""
    return [(0.0, 0.244140625, 2048), (500.0, 0.48828125, 1024), (1000.0, 0.9765625, 1024)]


def cfg1_segments():
    return [(0.0, 0.2, 500)]


def pulse_delays(nchans, fch1, foff, tsamp, dm, K=K_INJECT):
    f = fch1 + foff * np.arange(nchans, dtype=np.float64)
    return np.floor(K * dm * (f ** -2 - fch1 ** -2) / tsamp + 0.5).astype(np.int64)


def inject(x, fch1, foff, tsamp, pulses, K=K_INJECT):
    """Add boxcar pulses in place.  pulses: iterable of (t0 at the top channel, dm, width,
    amplitude per channel).  Integer arrays are saturated to their range."""
    nchans, ncols = x.shape
    is_int = np.issubdtype(x.dtype, np.integer)
    for t0, dm, w, amp in pulses:
        d = pulse_delays(nchans, fch1, foff, tsamp, dm, K)
        for c in range(nchans):
            a = int(t0 + d[c])
            b = min(a + int(w), ncols)
            if a >= ncols or b <= 0:
                continue
            a = max(a, 0)
            if is_int:
                info = np.iinfo(x.dtype)
                seg = x[c, a:b].astype(np.int64) + int(round(amp))
                x[c, a:b] = np.clip(seg, info.min, info.max).astype(x.dtype)
            else:
                x[c, a:b] += np.float32(amp)
    return x


def gaussian_f32(nchans, ncols, seed=0):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((nchans, ncols), dtype=np.float32)


def gaussian_u8(nchans, ncols, seed=0, mean=128.0, sigma=16.0):
    rng = np.random.default_rng(seed)
    out = np.empty((nchans, ncols), np.uint8)
    for c in range(nchans):
        v = rng.standard_normal(ncols, dtype=np.float32) * np.float32(sigma) + np.float32(mean)
        out[c] = np.clip(np.rint(v), 0, 255).astype(np.uint8)
    return out


def gaussian_i16(nchans, ncols, seed=0, sigma=1000.0):
    rng = np.random.default_rng(seed)
    out = np.empty((nchans, ncols), np.int16)
    for c in range(nchans):
        v = rng.standard_normal(ncols, dtype=np.float32) * np.float32(sigma)
        out[c] = np.clip(np.rint(v), -32768, 32767).astype(np.int16)
    return out


def cfg1(nsamp_total=32768, nchans=256, seed=0):
    """Config 1: float32 256 x 32768, 1500 MHz top, 0.390625 MHz channels, 64 us, three pulses
    (DM 12.5/57.3/88.0, width 4, per-channel amplitude 20/sqrt(4*256))."""
    fch1, foff, tsamp = 1500.0, -0.390625, 64e-6
    x = gaussian_f32(nchans, nsamp_total, seed)
    amp = 20.0 / np.sqrt(4 * nchans)
    pulses = [(6000, 12.5, 4, amp), (14000, 57.3, 4, amp), (22000, 88.0, 4, amp)]
    inject(x, fch1, foff, tsamp, pulses)
    return x, dict(fch1=fch1, foff=foff, tsamp=tsamp, pulses=pulses)


def random_pulses(rng, n, nsamp, dm_max, sigma, nchans, widths=(1, 64), snr=(8, 30)):
    out = []
    for _ in range(n):
        dm = float(rng.uniform(0, dm_max))
        w = int(rng.integers(widths[0], widths[1] + 1))
        s = float(rng.uniform(*snr))
        amp = s * sigma / np.sqrt(nchans * w)
        t0 = int(rng.integers(0, max(1, nsamp - w)))
        out.append((t0, dm, w, amp))
    return out


def cfg3(dtype, nchans, ncols, seed=0, fch1=1500.0, bw=300.0, tsamp=64e-6, pulses=(),
         impulse_frac=0.01, impulse_sigma=50.0, nb_channels=20, nb_sigma=10.0):
    """Config 3's block: Gaussian samples (uint8: mean 128, sigma 16; int16: mean 0, sigma
    1000), broadband impulses of impulse_sigma on impulse_frac of the time samples (all
    channels), sinusoids of amplitude nb_sigma in nb_channels random channels, and dispersed
    boxcar pulses (t0, dm, width, amplitude per channel).  Integer samples saturate.  Returns
    (x, meta) with the impulse columns and narrowband channels in meta."""
    rng = np.random.default_rng(seed)
    if dtype == "u8":
        x = gaussian_u8(nchans, ncols, seed)
        mean, sigma, lo, hi = 128.0, 16.0, 0, 255
    elif dtype == "i16":
        x = gaussian_i16(nchans, ncols, seed)
        mean, sigma, lo, hi = 0.0, 1000.0, -32768, 32767
    else:
        raise ValueError(dtype)
    foff = -float(bw) / nchans
    inject(x, fch1, foff, tsamp, pulses)
    cols = np.sort(rng.choice(ncols, max(1, int(round(impulse_frac * ncols))), replace=False))
    imp = int(round(impulse_sigma * sigma))
    x[:, cols] = np.clip(x[:, cols].astype(np.int64) + imp, lo, hi).astype(x.dtype)
    chans = np.sort(rng.choice(nchans, nb_channels, replace=False))
    t = np.arange(ncols, dtype=np.float64)
    for c in chans:
        period = float(rng.uniform(8.0, 200.0))
        ph = float(rng.uniform(0, 2 * np.pi))
        s = np.rint(nb_sigma * sigma * np.sin(2 * np.pi * t / period + ph)).astype(np.int64)
        x[c] = np.clip(x[c].astype(np.int64) + s, lo, hi).astype(x.dtype)
    return x, dict(fch1=fch1, foff=foff, tsamp=tsamp, impulse_cols=cols, nb_channels=chans,
                   mean=mean, sigma=sigma)
