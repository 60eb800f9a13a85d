"""Python host API over the C ABI: DM plans, dedispersion, RFI clipping, detection.

Device buffers are torch CUDA tensors (plumbing only: their data pointers and the current
stream are handed to the library).  Host buffers are numpy arrays.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import (ACC, DTYPES, OUT_DTYPES, SHIFT_MODES, BruteDesc, Candidate, PlanInfo,
                   Segment, StageInfo, SubbandDesc, SUBBAND_PASSES, check, load)

_NP_OF = {"u8": np.uint8, "u16": np.uint16, "i16": np.int16, "f32": np.float32,
          "i32": np.int32}


def _stream_ptr(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def dmdelay(f1, f2):
    """src/mdsm/dedispersion_manager.cpp:262-265."""
    return load().mdsm_dmdelay(f1, f2)


class _PlanBase:
    _h = None

    def __del__(self):
        if self._h:
            try:
                load().mdsm_plan_destroy(self._h)
            except Exception:
                pass
            self._h = None

    @property
    def info(self):
        i = PlanInfo()
        check(load().mdsm_plan_get_info(self._h, ctypes.byref(i)))
        return i

    def stage_info(self, stage):
        """Launch stage `stage` (brute force: 0; subband pass i: 2i, 2i+1)."""
        i = StageInfo()
        check(load().mdsm_plan_stage_info(self._h, int(stage), ctypes.byref(i)))
        return i

    @property
    def ndms(self):
        return self.info.ndms

    @property
    def maxshift(self):
        return self.info.maxshift

    def dm_values(self):
        out = np.empty(self.info.ndms, np.float32)
        check(load().mdsm_plan_dm_values(self._h, out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def dmshifts(self):
        out = np.empty(self.info.nchans, np.float32)
        check(load().mdsm_plan_dmshifts(self._h, out.ctypes.data_as(ctypes.c_void_p)))
        return out

    @property
    def last_launches(self):
        return load().mdsm_plan_last_launches(self._h)

    def check(self, stream=None):
        """Synchronise and raise if a device-side wait of an earlier call ran out."""
        check(load().mdsm_plan_check(self._h, _stream_ptr(stream)))

    def wait_selftest(self, spin_limit=4096, stream=None):
        """Run the bounded-wait self-test kernel (its wait runs out on purpose)."""
        check(load().mdsm_plan_wait_selftest(self._h, int(spin_limit), _stream_ptr(stream)))

    def set_stage_timing(self, on=True):
        """Record CUDA events around every stage of each dedisperse_device call."""
        check(load().mdsm_plan_set_stage_timing(self._h, int(bool(on))))

    def stage_times(self):
        """Milliseconds of each stage of the last timed dedisperse_device call."""
        cap = 64
        ms = (ctypes.c_float * cap)()
        n = ctypes.c_int()
        check(load().mdsm_plan_stage_times(self._h, ms, cap, ctypes.byref(n)))
        return [float(ms[i]) for i in range(n.value)]

    def input_shape(self):
        """(nchans, row pitch) of the device input the plan reads."""
        i = self.info
        return i.nchans, i.in_stride

    def alloc_input(self, device="cuda"):
        """A zeroed device buffer laid out as the plan expects: [nchans][in_stride] plus the
        readable tail the tile overrun needs."""
        import torch
        i = self.info
        elem = np.dtype(_NP_OF[self.in_dtype]).itemsize
        total = max(i.in_bytes, i.nchans * i.in_stride * elem)
        n = (total + elem - 1) // elem + 64
        tdt = {"u8": torch.uint8, "u16": torch.uint16, "i16": torch.int16,
               "f32": torch.float32}[self.in_dtype]
        flat = torch.zeros(n, dtype=tdt, device=device)
        return flat

    def alloc_output(self, device="cuda"):
        import torch
        i = self.info
        dt = torch.int32 if self.out_dtype == "i32" else torch.float32
        return torch.empty((i.ndms, i.nsamp), dtype=dt, device=device)

    def dedisperse_device(self, d_in, d_out, in_stride=None, stream=None):
        """Dedisperse a device input (flat tensor from alloc_input, or any tensor whose memory
        holds [nchans][in_stride]) into d_out [ndms][nsamp] (or with a row pitch)."""
        i = self.info
        stride = in_stride if in_stride is not None else i.in_stride
        in_bytes = d_in.numel() * d_in.element_size()
        out_stride = d_out.stride(0) if d_out.dim() == 2 else i.nsamp
        check(load().mdsm_dedisperse_device(self._h, ctypes.c_void_p(d_in.data_ptr()), stride,
                                            in_bytes, ctypes.c_void_p(d_out.data_ptr()),
                                            out_stride, _stream_ptr(stream)))
        return d_out

    def dedisperse_host(self, h_in, h_out=None, stream=None):
        """Host filterbank [nchans][>= nsamp+maxshift] -> host series [ndms][nsamp]."""
        i = self.info
        h_in = np.ascontiguousarray(h_in) if not h_in.flags.c_contiguous else h_in
        if h_in.dtype != _NP_OF[self.in_dtype]:
            raise TypeError("input dtype %s, plan expects %s" % (h_in.dtype, self.in_dtype))
        if h_out is None:
            h_out = np.empty((i.ndms, i.nsamp),
                             np.int32 if self.out_dtype == "i32" else np.float32)
        check(load().mdsm_dedisperse_host(self._h, h_in.ctypes.data_as(ctypes.c_void_p),
                                          h_in.shape[1], h_out.ctypes.data_as(ctypes.c_void_p),
                                          _stream_ptr(stream)))
        return h_out


class BrutePlan(_PlanBase):
    """Brute-force DM plan (one or more uniform DM segments)."""

    def __init__(self, nchans, fch1, foff, tsamp, nsamp, segments, shift_mode="l1",
                 in_dtype="u8", out_dtype="f32", acc="auto", K=0.0, dm_block=0, kernel=0):
        segs = (Segment * len(segments))(*[Segment(float(a), float(b), int(n))
                                           for a, b, n in segments])
        d = BruteDesc(int(nchans), float(fch1), float(foff), float(tsamp), int(nsamp), segs,
                      len(segments), SHIFT_MODES[shift_mode], float(K), DTYPES[in_dtype],
                      OUT_DTYPES[out_dtype], ACC[acc], int(dm_block), int(kernel))
        h = ctypes.c_void_p()
        check(load().mdsm_brute_plan_create(ctypes.byref(d), ctypes.byref(h)))
        self._h = h
        self.in_dtype, self.out_dtype, self.acc = in_dtype, out_dtype, acc
        self.segments = list(segments)

    def shift_table(self):
        i = self.info
        out = np.empty((i.ndms, i.nchans), np.int32)
        check(load().mdsm_plan_shift_table(self._h, 0, out.ctypes.data_as(ctypes.c_void_p)))
        return out


class SubbandPlan(_PlanBase):
    """Two-stage subband plan; passes are dicts/tuples of the reference's pass fields."""

    def __init__(self, nchans, fch1, foff, tsamp, nsamp, nsubs, passes, use_fma=True,
                 in_dtype="u8", out_dtype="f32", acc="auto"):
        arr = (SUBBAND_PASSES * len(passes))()
        for k, p in enumerate(passes):
            for f in ("lowdm", "highdm", "dmstep", "sub_dmstep", "ncalls", "calldms", "ndms"):
                if f in p:
                    setattr(arr[k], f, p[f])
            arr[k].binsize = int(p.get("binsize", 1))
        d = SubbandDesc(int(nchans), float(fch1), float(foff), float(tsamp), int(nsamp),
                        int(nsubs), arr, len(passes), int(bool(use_fma)), DTYPES[in_dtype],
                        OUT_DTYPES[out_dtype], ACC[acc])
        h = ctypes.c_void_p()
        check(load().mdsm_subband_plan_create(ctypes.byref(d), ctypes.byref(h)))
        self._h = h
        self._passes = arr
        self.in_dtype, self.out_dtype, self.acc = in_dtype, out_dtype, acc
        self.nsubs = nsubs
        self.passes = [dict(p) for p in passes]

    def stage_tables(self):
        """(S1 [ncalls][nchans], S2 [ncalls*calldms][nsubs]) of the first pass."""
        p = self.passes[0]
        i = self.info
        s1 = np.empty((p["ncalls"], i.nchans), np.int32)
        s2 = np.empty((p["ncalls"] * p["calldms"], self.nsubs), np.int32)
        check(load().mdsm_plan_shift_table(self._h, 1, s1.ctypes.data_as(ctypes.c_void_p)))
        check(load().mdsm_plan_shift_table(self._h, 2, s2.ctypes.data_as(ctypes.c_void_p)))
        return s1, s2


def rfi_clip_device(x, nchans, stride, length, k_chan=4.0, k_spec=4.0, dtype="u8", stream=None):
    """In-place RFI clip of a channel-major device buffer (torch tensor)."""
    check(load().mdsm_rfi_clip_device(ctypes.c_void_p(x.data_ptr()), DTYPES[dtype], int(nchans),
                                      int(stride), int(length), float(k_chan), float(k_spec),
                                      _stream_ptr(stream)))
    return x


CAND_DTYPE = np.dtype([("dm_idx", np.int32), ("sample", np.int32), ("snr", np.float32),
                       ("width", np.int32)])


def _cands_to_array(buf, n):
    return np.frombuffer(buf, dtype=CAND_DTYPE, count=n).copy()


def ref_detect_device(series, lowdm, dmstep, threshold, cap=1 << 20, stream=None):
    """Reference detector on a device float series [ndms][nsamp].  Returns (cands, mean, rms)
    with cands a structured array sorted by (dm_idx, sample)."""
    ndms, nsamp = series.shape
    buf = (Candidate * cap)()
    n = ctypes.c_longlong()
    mean, rms = ctypes.c_float(), ctypes.c_float()
    check(load().mdsm_ref_detect_device(ctypes.c_void_p(series.data_ptr()), ndms, nsamp,
                                        float(lowdm), float(dmstep), float(threshold), buf, cap,
                                        ctypes.byref(n), ctypes.byref(mean), ctypes.byref(rms),
                                        _stream_ptr(stream)))
    return _cands_to_array(buf, min(n.value, cap)), mean.value, rms.value, n.value


def ref_detect_chunked_device(series, lowdm, dmstep, threshold, mean, rms, spc, cap=1 << 20,
                              stream=None):
    """Reference detector with caller noise statistics (one mean/rms per spc samples) on a
    device float series [ndms][nsamp]: (cands, total)."""
    ndms, nsamp = series.shape
    mean = np.ascontiguousarray(mean, np.float32)
    rms = np.ascontiguousarray(rms, np.float32)
    buf = (Candidate * cap)()
    n = ctypes.c_longlong()
    check(load().mdsm_ref_detect_chunked_device(
        ctypes.c_void_p(series.data_ptr()), ndms, nsamp, float(lowdm), float(dmstep),
        float(threshold), mean.ctypes.data_as(ctypes.c_void_p),
        rms.ctypes.data_as(ctypes.c_void_p), mean.size, int(spc), buf, cap, ctypes.byref(n),
        _stream_ptr(stream)))
    return _cands_to_array(buf, min(n.value, cap)), n.value


def ref_detect_subband_device(plan, series, threshold, mean=None, rms=None, spc=0,
                              cap=1 << 20, stream=None):
    """process_subband on a subband plan's device float output [ndms][>= nsamp]: per-row
    statistics, or the caller's chunk statistics.  (cands, total); width holds the pass's
    downsample factor."""
    out_stride = series.stride(0) if series.dim() == 2 else plan.info.nsamp
    mp = rp = None
    nch = 0
    if mean is not None:
        mean = np.ascontiguousarray(mean, np.float32)
        rms = np.ascontiguousarray(rms, np.float32)
        mp = mean.ctypes.data_as(ctypes.c_void_p)
        rp = rms.ctypes.data_as(ctypes.c_void_p)
        nch = mean.size
    buf = (Candidate * cap)()
    n = ctypes.c_longlong()
    check(load().mdsm_ref_detect_subband_device(
        plan._h, ctypes.c_void_p(series.data_ptr()), out_stride, float(threshold), mp, rp, nch,
        int(spc), buf, cap, ctypes.byref(n), _stream_ptr(stream)))
    return _cands_to_array(buf, min(n.value, cap)), n.value


def boxcar_detect_device(series, nwidths=9, threshold=6.0, cap=1 << 20, stream=None):
    """Boxcar search on a device series [ndms][nsamp] (float32 or int32)."""
    import torch
    ndms, nsamp = series.shape
    dt = 1 if series.dtype == torch.int32 else 0
    buf = (Candidate * cap)()
    n = ctypes.c_longlong()
    check(load().mdsm_boxcar_detect_device(ctypes.c_void_p(series.data_ptr()), dt, ndms, nsamp,
                                           int(nwidths), float(threshold), buf, cap,
                                           ctypes.byref(n), _stream_ptr(stream)))
    return _cands_to_array(buf, min(n.value, cap)), n.value


def singlepulse_detect_device(series, max_downfact=30, chunk_len=8000, threshold=6.0,
                              normalise=False, cap=1 << 20, stream=None):
    """The single-pulse prototype's search (template form) on a device series [ndms][nsamp]
    (float32 or int32): candidates in the prototype's list order (dm, chunk, width, sample)."""
    import torch
    ndms, nsamp = series.shape
    dt = 1 if series.dtype == torch.int32 else 0
    buf = (Candidate * max(cap, 1))()
    n = ctypes.c_longlong()
    check(load().mdsm_singlepulse_detect_device(ctypes.c_void_p(series.data_ptr()), dt, ndms,
                                                nsamp, int(max_downfact), int(chunk_len),
                                                int(bool(normalise)), float(threshold), buf, cap,
                                                ctypes.byref(n), _stream_ptr(stream)))
    return _cands_to_array(buf, min(n.value, cap)), n.value


def detrend_normalise_device(series, length=1024, stream=None):
    """In-place detrend and normalise of a float32 device series [ndms][nsamp]."""
    ndms, nsamp = series.shape
    check(load().mdsm_detrend_normalise_device(ctypes.c_void_p(series.data_ptr()), ndms, nsamp,
                                               int(length), _stream_ptr(stream)))
    return series
