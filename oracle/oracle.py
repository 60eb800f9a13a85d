"""ctypes wrapper of the CPU oracle (oracle/mdsm_oracle.c) and of the reference builds.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline / reference arm.  The product package never imports this module.
"""
import ctypes
import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", platform.machine(), "libmdsm_oracle.so")
HARNESS_SO = os.path.join(HERE, "_build", platform.machine(), "libref_gpu_harness.so")
REF_HOST_SO = os.path.join(HERE, "_ref", "libref_host.so")
REF_CUBIN = os.path.join(HERE, "_ref", "ref_kernels.cubin")
REF_DETREND_CUBIN = os.path.join(HERE, "_ref", "ref_detrend.cubin")
REF_RFI_CUBIN = os.path.join(HERE, "_ref", "ref_rfi.cubin")
REF_SP_SO = os.path.join(HERE, "_ref", "libref_singlepulse.so")
# the reference tree (MDSM's src/ directory): where it is present, build() compiles the
# reference's own code into oracle/_ref/
REF_TREE = os.environ.get("MDSM_REFERENCE_SRC", "")

SHIFT = {"l1": 0, "l1_muladd": 1, "opt": 2, "opt_muladd": 3, "fp64_trunc": 4, "fp64_round": 5}


def build(reference=True):
    """Build the oracle (always) and, when the reference tree is present here, its builds."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    if reference and REF_TREE and os.path.isdir(REF_TREE):
        subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + REF_TREE], check=True)
    cuda_lib = any(os.path.exists(os.path.join(d, "libcuda.so")) for d in
                   ("/usr/local/cuda/lib64/stubs", "/usr/lib/x86_64-linux-gnu",
                    "/usr/lib/aarch64-linux-gnu", "/usr/local/cuda/lib64"))
    if cuda_lib:
        subprocess.run(["make", "-s", "-C", HERE, "harness"], check=True)


class Seg(ctypes.Structure):
    _fields_ = [("lowdm", ctypes.c_float), ("dmstep", ctypes.c_float), ("ndms", ctypes.c_int)]


_O = None


def lib():
    global _O
    if _O is None:
        if not os.path.exists(ORACLE_SO):
            build(reference=False)
        _O = ctypes.CDLL(ORACLE_SO)
        _O.orc_dmdelay.restype = ctypes.c_float
        _O.orc_dmdelay.argtypes = [ctypes.c_float, ctypes.c_float]
        _O.orc_median_of_five.restype = ctypes.c_float
        _O.orc_median_of_five.argtypes = [ctypes.c_float] * 5
        _O.orc_ref_maxshift.restype = ctypes.c_uint
        _O.orc_ref_maxshift.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_float,
                                        ctypes.c_float, ctypes.c_int, ctypes.c_float]
        _O.orc_subband_tempval.restype = ctypes.c_int
        _O.orc_subband_tempval.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_float, ctypes.c_float]
        _O.orc_ref_detect.restype = ctypes.c_long
        _O.orc_ref_detect_chunked.restype = ctypes.c_long
        _O.orc_ref_detect_subband.restype = ctypes.c_long
        _O.orc_boxcar_detect.restype = ctypes.c_long
        _O.orc_unpack.restype = ctypes.c_long
        _O.orc_singlepulse_detect.restype = ctypes.c_long
        _O.orc_sp_widths.restype = ctypes.c_int
    return _O


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def dmshifts(nchans, fch1, foff):
    out = np.empty(nchans, np.float32)
    lib().orc_dmshifts(nchans, ctypes.c_float(fch1), ctypes.c_float(foff), _p(out))
    return out


def shift_table(nchans, fch1, foff, tsamp, segments, mode="l1", K=4148.741601):
    dms = dmshifts(nchans, fch1, foff)
    segs = (Seg * len(segments))(*[Seg(a, b, n) for a, b, n in segments])
    ndms = sum(n for _, _, n in segments)
    out = np.empty((ndms, nchans), np.int32)
    lib().orc_shift_table(_p(dms), nchans, ctypes.c_double(fch1), ctypes.c_double(foff),
                          ctypes.c_double(K), segs, len(segments), ctypes.c_float(tsamp),
                          SHIFT[mode], _p(out))
    return out


def ref_maxshift(nchans, fch1, foff, lowdm, dmstep, tdms, tsamp):
    dms = dmshifts(nchans, fch1, foff)
    return lib().orc_ref_maxshift(_p(dms), nchans, lowdm, dmstep, tdms, tsamp)


def dedisperse(x, S, nsamp, out="auto"):
    """x [nchans][stride] (f32/u8/u16/i16), S [ndms][nchans] -> [ndms][nsamp]."""
    S = np.ascontiguousarray(S, np.int32)
    ndms, nchans = S.shape
    stride = x.shape[1]
    x = np.ascontiguousarray(x)
    if out == "f64":
        y = np.empty((ndms, nsamp), np.float64)
        lib().orc_dedisperse_f64(_p(x), nchans, ctypes.c_long(stride), nsamp, _p(S), ndms, _p(y))
        return y
    if x.dtype == np.float32:
        y = np.empty((ndms, nsamp), np.float32)
        lib().orc_dedisperse_f32(_p(x), nchans, ctypes.c_long(stride), nsamp, _p(S), ndms, _p(y))
        return y
    fn = {np.dtype(np.uint8): lib().orc_dedisperse_u8_i32,
          np.dtype(np.uint16): lib().orc_dedisperse_u16_i32,
          np.dtype(np.int16): lib().orc_dedisperse_i16_i32}[x.dtype]
    y = np.empty((ndms, nsamp), np.int32)
    fn(_p(x), nchans, ctypes.c_long(stride), nsamp, _p(S), ndms, _p(y))
    return y


def subband_tables(nchans, fch1, foff, tsamp, nsubs, lowdm, sub_dmstep, ncalls, dmstep, calldms,
                   use_fma=True):
    dms = dmshifts(nchans, fch1, foff)
    S1 = np.empty((ncalls, nchans), np.int32)
    S2 = np.empty((ncalls * calldms, nsubs), np.int32)
    lib().orc_subband_shifts(_p(dms), nchans, nsubs, ctypes.c_float(lowdm),
                             ctypes.c_float(sub_dmstep), ncalls, ctypes.c_float(dmstep), calldms,
                             ctypes.c_float(tsamp), int(use_fma), _p(S1), _p(S2))
    return S1, S2


def subband_dedisperse(x, S1, S2, nsubs, nsamp, nsamp1, calldms):
    """Reference two-stage order: stage 1 to z [ncalls][nsubs][nsamp1], stage 2 to y."""
    x = np.ascontiguousarray(x, np.float32)
    ncalls, nchans = S1.shape
    z = np.empty((ncalls, nsubs, nsamp1), np.float32)
    lib().orc_subband_stage1_f32(_p(x), nchans, ctypes.c_long(x.shape[1]), nsubs, nsamp1,
                                 _p(np.ascontiguousarray(S1)), ncalls, _p(z))
    y = np.empty((ncalls * calldms, nsamp), np.float32)
    lib().orc_subband_stage2_f32(_p(z), nsubs, nsamp1, nsamp, _p(np.ascontiguousarray(S2)),
                                 ncalls, calldms, _p(y))
    return z, y


def median_of_five(a, b, c, d, e):
    return lib().orc_median_of_five(a, b, c, d, e)


def ref_stats(buf):
    buf = np.ascontiguousarray(buf, np.float32)
    m, r = ctypes.c_float(), ctypes.c_float()
    lib().orc_ref_stats(_p(buf), ctypes.c_uint(buf.size), ctypes.byref(m), ctypes.byref(r))
    return m.value, r.value


def ref_detect(buf, lowdm, dmstep, threshold, cap=1 << 22):
    buf = np.ascontiguousarray(buf, np.float32)
    ndms, nsamp = buf.shape
    mean, rms = ref_stats(buf)
    dm = np.empty(cap, np.int32)
    sa = np.empty(cap, np.int32)
    sn = np.empty(cap, np.float32)
    n = lib().orc_ref_detect(_p(buf), ndms, nsamp, ctypes.c_float(lowdm), ctypes.c_float(dmstep),
                             ctypes.c_float(threshold), ctypes.c_float(mean), ctypes.c_float(rms),
                             _p(dm), _p(sa), _p(sn), ctypes.c_long(cap))
    k = min(n, cap)
    return (dm[:k].copy(), sa[:k].copy(), sn[:k].copy()), mean, rms


def ref_detect_chunked(buf, lowdm, dmstep, threshold, mean, rms, spc, cap=1 << 22):
    """process_brute with caller noise statistics: (dm, sample, snr)."""
    buf = np.ascontiguousarray(buf, np.float32)
    ndms, nsamp = buf.shape
    mean = np.ascontiguousarray(mean, np.float32)
    rms = np.ascontiguousarray(rms, np.float32)
    dm = np.empty(cap, np.int32)
    sa = np.empty(cap, np.int32)
    sn = np.empty(cap, np.float32)
    n = lib().orc_ref_detect_chunked(_p(buf), ndms, nsamp, ctypes.c_float(lowdm),
                                     ctypes.c_float(dmstep), ctypes.c_float(threshold),
                                     _p(mean), _p(rms), int(spc), _p(dm), _p(sa), _p(sn),
                                     ctypes.c_long(cap))
    k = min(n, cap)
    return dm[:k].copy(), sa[:k].copy(), sn[:k].copy()


def ref_detect_subband(rows, nvalid, dm_values, threshold, mean=None, rms=None, spc=1,
                       cap=1 << 22):
    """process_subband over rows [nrows][>= nvalid] with DMs dm_values: (row, sample, snr)."""
    rows = np.ascontiguousarray(rows, np.float32)
    nrows, stride = rows.shape
    dmv = np.ascontiguousarray(dm_values, np.float32)
    mp = rp = None
    if mean is not None:
        mean = np.ascontiguousarray(mean, np.float32)
        rms = np.ascontiguousarray(rms, np.float32)
        mp, rp = _p(mean), _p(rms)
    dm = np.empty(cap, np.int32)
    sa = np.empty(cap, np.int32)
    sn = np.empty(cap, np.float32)
    n = lib().orc_ref_detect_subband(_p(rows), ctypes.c_long(stride), nrows, int(nvalid),
                                     _p(dmv), ctypes.c_float(threshold), mp, rp, int(spc),
                                     _p(dm), _p(sa), _p(sn), ctypes.c_long(cap))
    k = min(n, cap)
    return dm[:k].copy(), sa[:k].copy(), sn[:k].copy()


KIND = {np.dtype(np.uint8): 0, np.dtype(np.uint16): 1, np.dtype(np.int16): 2,
        np.dtype(np.float32): 3}


def rfi_clip(x, length, k_chan=4.0, k_spec=4.0):
    """In place on a channel-major array [nchans][stride]."""
    assert x.flags.c_contiguous
    lib().orc_rfi_clip(_p(x), KIND[x.dtype], x.shape[0], ctypes.c_long(x.shape[1]),
                       ctypes.c_long(length), ctypes.c_double(k_chan), ctypes.c_double(k_spec))
    return x


def boxcar_detect(y, nw=9, threshold=6.0, cap=1 << 22, is_int=None):
    """is_int: exact integer statistics (default: y has an integer dtype, or every value of a
    float array is integral)."""
    if is_int is None:
        is_int = np.issubdtype(np.asarray(y).dtype, np.integer)
    yd = np.ascontiguousarray(y, np.float64)
    ndms, n = yd.shape
    dm = np.empty(cap, np.int32)
    sa = np.empty(cap, np.int32)
    wd = np.empty(cap, np.int32)
    sn = np.empty(cap, np.float32)
    cnt = lib().orc_boxcar_detect(_p(yd), ndms, ctypes.c_long(n), nw, ctypes.c_double(threshold),
                                  _p(dm), _p(sa), _p(wd), _p(sn), ctypes.c_long(cap),
                                  int(bool(is_int)))
    k = min(cnt, cap)
    return dm[:k].copy(), sa[:k].copy(), wd[:k].copy(), sn[:k].copy()


def unpack(raw, nbits):
    raw = np.ascontiguousarray(raw, np.uint8)
    out = np.empty(raw.size * 8, np.float32)
    n = lib().orc_unpack(_p(raw), ctypes.c_long(raw.size), nbits, _p(out))
    return out[:n].copy()


def sp_widths(max_downfact=30):
    w = np.zeros(13, np.int32)
    n = lib().orc_sp_widths(int(max_downfact), _p(w))
    return w[:n].copy()


def sp_prune_related(bins, values, factor):
    """keep flags of singlepulse.cpp's pruneRelated (as written) over one sorted list."""
    bins = np.ascontiguousarray(bins, np.int32)
    values = np.ascontiguousarray(values, np.float32)
    keep = np.zeros(bins.size, np.uint8)
    lib().orc_sp_prune_related(_p(bins), _p(values), ctypes.c_long(bins.size), int(factor),
                               _p(keep))
    return keep.astype(bool)


def sp_prune_downfactors(bins, values, downfacts, maxdf):
    """mask of singlepulse.cpp's pruneRelatedDownfactors (as written, mask starting at 0)."""
    bins = np.ascontiguousarray(bins, np.int64)
    values = np.ascontiguousarray(values, np.float32)
    df = np.ascontiguousarray(downfacts, np.int32)
    mask = np.zeros(bins.size, np.uint8)
    lib().orc_sp_prune_downfactors(_p(bins), _p(values), _p(df), ctypes.c_long(bins.size),
                                   int(maxdf), _p(mask))
    return mask.astype(bool)


def sp_values(y, w, normalise=False, is_int=False):
    """Width-w template response of a 1-D series at every sample."""
    yd = np.ascontiguousarray(y, np.float64)
    out = np.empty(yd.size, np.float32)
    lib().orc_sp_values(_p(yd), ctypes.c_long(yd.size), int(w), int(bool(normalise)),
                        int(bool(is_int)), _p(out))
    return out


def singlepulse_detect(y, max_downfact=30, chunk_len=8000, threshold=6.0, normalise=False,
                       is_int=None, cap=1 << 22):
    """The prototype's search (template form): (dm, sample, width, snr) in list order."""
    if is_int is None:
        is_int = np.issubdtype(np.asarray(y).dtype, np.integer)
    yd = np.ascontiguousarray(y, np.float64)
    ndms, n = yd.shape
    dm = np.empty(cap, np.int32)
    sa = np.empty(cap, np.int32)
    wd = np.empty(cap, np.int32)
    sn = np.empty(cap, np.float32)
    cnt = lib().orc_singlepulse_detect(_p(yd), ndms, ctypes.c_long(n), int(max_downfact),
                                       ctypes.c_long(chunk_len), int(bool(normalise)),
                                       int(bool(is_int)), ctypes.c_double(threshold), _p(dm),
                                       _p(sa), _p(wd), _p(sn), ctypes.c_long(cap))
    k = min(cnt, cap)
    return dm[:k].copy(), sa[:k].copy(), wd[:k].copy(), sn[:k].copy()


def detrend_ref_f32(y, length, contract):
    """detrend.cu's kernel arithmetic on y [ndms][nsamp] (a copy is returned)."""
    y = np.array(y, np.float32, copy=True, order="C")
    lib().orc_detrend_ref_f32(_p(y), y.shape[0], y.shape[1], int(length), int(contract))
    return y


def rfi_clip_ref_f32(x, blockdim, contract):
    """rfi_clipper.cu's kernel arithmetic on x [nrows][nsamp]: (clipped copy, row means)."""
    x = np.array(x, np.float32, copy=True, order="C")
    means = np.empty(x.shape[0], np.float32)
    lib().orc_rfi_clip_ref_f32(_p(x), x.shape[0], x.shape[1], int(blockdim), int(contract),
                               _p(means))
    return x, means


def detrend_normalise(y, length=1024):
    y = np.array(y, np.float32, copy=True)
    lib().orc_detrend_normalise(_p(y), ctypes.c_long(y.size), length)
    return y


# ------------------------------------------------------------------------------------------
# the reference's own code (oracle/_ref), where it was built
# ------------------------------------------------------------------------------------------

def ref_host_available():
    return os.path.exists(REF_HOST_SO)


def ref_singlepulse_available():
    return os.path.exists(REF_SP_SO)


def ref_singlepulse():
    """src/prototypes/singlepulse.cpp's own functions (built here against the FFTW stand-in)."""
    h = ctypes.CDLL(REF_SP_SO)
    return h


def ref_host():
    h = ctypes.CDLL(REF_HOST_SO)
    h.ref_median_of_five.restype = ctypes.c_float
    h.ref_median_of_five.argtypes = [ctypes.c_float] * 5
    h.ref_read_block.restype = ctypes.c_long
    return h


class RefGPU:
    """The reference kernels from oracle/_ref/ref_kernels.cubin (and, where built, the
    prototype kernels of detrend.cu and rfi_clipper.cu), launched on device 0."""

    def __init__(self, cubin=REF_CUBIN, proto=False):
        self.h = ctypes.CDLL(HARNESS_SO)
        self.h.rg_error.restype = ctypes.c_char_p
        rc = self.h.rg_init(cubin.encode())
        if rc:
            raise RuntimeError("rg_init: %d %s" % (rc, self.h.rg_error().decode()))
        if proto:
            rc = self.h.rg_init_proto(REF_DETREND_CUBIN.encode(), REF_RFI_CUBIN.encode())
            if rc:
                raise RuntimeError("rg_init_proto: %d %s" % (rc, self.h.rg_error().decode()))

    def detrend(self, y, length):
        """detrend_normalise on y [ndms][nsamp] (copy returned) and the kernel time in ms."""
        y = np.array(y, np.float32, copy=True, order="C")
        ms = ctypes.c_float()
        rc = self.h.rg_detrend(_p(y), y.shape[0], y.shape[1], int(length), ctypes.byref(ms))
        if rc:
            raise RuntimeError("rg_detrend: %d %s" % (rc, self.h.rg_error().decode()))
        return y, ms.value

    def rfi_clip(self, x, blockdim):
        """rfi_clipping on x [nrows][nsamp]: (clipped copy, row means, kernel ms)."""
        x = np.array(x, np.float32, copy=True, order="C")
        means = np.zeros(x.shape[0], np.float32)
        ms = ctypes.c_float()
        rc = self.h.rg_rfi_clip(_p(x), x.shape[0], x.shape[1], int(blockdim), _p(means),
                                ctypes.byref(ms))
        if rc:
            raise RuntimeError("rg_rfi_clip: %d %s" % (rc, self.h.rg_error().decode()))
        return x, means, ms.value

    def brute(self, kind, x, nsamp, maxshift, lowdm, dmstep, tsamp, tdms, dms):
        x = np.ascontiguousarray(x, np.float32)
        nchans = x.shape[0]
        assert x.shape[1] == nsamp + maxshift
        out = np.zeros((tdms, nsamp), np.float32)
        ms = ctypes.c_float()
        rc = self.h.rg_brute(kind, _p(x), nsamp, nchans, maxshift, ctypes.c_float(lowdm),
                             ctypes.c_float(dmstep), ctypes.c_float(tsamp), tdms,
                             _p(np.ascontiguousarray(dms, np.float32)), _p(out), ctypes.byref(ms))
        if rc:
            raise RuntimeError("rg_brute: %d %s" % (rc, self.h.rg_error().decode()))
        return out, ms.value

    def subband(self, x, nsamp, maxshift, nsubs, tempval, lowdm, sub_dmstep, ncalls, dmstep,
                calldms, tsamp, dms):
        x = np.ascontiguousarray(x, np.float32)
        nchans = x.shape[0]
        z = np.zeros((ncalls, nsubs, nsamp + tempval), np.float32)
        out = np.zeros((ncalls * calldms, nsamp), np.float32)
        ms = ctypes.c_float()
        rc = self.h.rg_subband(_p(x), nsamp, nchans, maxshift, nsubs, tempval,
                               ctypes.c_float(lowdm), ctypes.c_float(sub_dmstep), ncalls,
                               ctypes.c_float(dmstep), calldms, ctypes.c_float(tsamp),
                               _p(np.ascontiguousarray(dms, np.float32)), _p(z), _p(out),
                               ctypes.byref(ms))
        if rc:
            raise RuntimeError("rg_subband: %d %s" % (rc, self.h.rg_error().decode()))
        return z, out, ms.value
