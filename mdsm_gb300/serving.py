"""Python host API of the serving form: a continuous-batching search server over many beams
(native code in mdsm_gb300/csrc/serve.cpp; C ABI mdsm_server_* in include/mdsm_gb300.h)."""
import ctypes
import time

import numpy as np

from . import _lib
from .api import _NP_OF
from ._lib import (ACC, DTYPES, OUT_DTYPES, SHIFT_MODES, BruteDesc, Candidate, PlanInfo,
                   Segment, SubbandDesc, SUBBAND_PASSES, check, load)


class ServerDesc(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_longlong), ("host_stage_bytes", ctypes.c_longlong),
                ("max_inflight", ctypes.c_int), ("detector", ctypes.c_int),
                ("nwidths", ctypes.c_int), ("threshold", ctypes.c_double),
                ("cand_cap", ctypes.c_longlong)]


class BlockResult(ctypes.Structure):
    _fields_ = [("beam", ctypes.c_int), ("block", ctypes.c_longlong),
                ("ticket", ctypes.c_longlong), ("submit_time", ctypes.c_double),
                ("done_time", ctypes.c_double), ("ncand", ctypes.c_longlong),
                ("status", ctypes.c_int)]


class ServerStats(ctypes.Structure):
    _fields_ = [("admitted", ctypes.c_longlong), ("refused", ctypes.c_longlong),
                ("completed", ctypes.c_longlong), ("held_bytes", ctypes.c_longlong),
                ("dm_trial_samples", ctypes.c_longlong), ("wall_s", ctypes.c_double),
                ("p50_latency_s", ctypes.c_double), ("p99_latency_s", ctypes.c_double),
                ("max_latency_s", ctypes.c_double)]


_vp = ctypes.c_void_p
SIGNATURES = {
    "mdsm_server_create": (ctypes.c_int, [ctypes.POINTER(ServerDesc), ctypes.POINTER(_vp)]),
    "mdsm_server_add_beam_brute": (ctypes.c_int, [_vp, ctypes.POINTER(BruteDesc),
                                                  ctypes.POINTER(ctypes.c_int)]),
    "mdsm_server_add_beam_subband": (ctypes.c_int, [_vp, ctypes.POINTER(SubbandDesc),
                                                    ctypes.POINTER(ctypes.c_int)]),
    "mdsm_server_beam_info": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(PlanInfo)]),
    "mdsm_server_submit": (ctypes.c_int, [_vp, ctypes.c_int, _vp, ctypes.c_longlong,
                                          ctypes.POINTER(ctypes.c_longlong)]),
    "mdsm_server_poll": (ctypes.c_int, [_vp, ctypes.POINTER(BlockResult),
                                        ctypes.POINTER(Candidate), ctypes.c_longlong,
                                        ctypes.c_int]),
    "mdsm_server_acquire": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(_vp),
                                           ctypes.POINTER(ctypes.c_longlong)]),
    "mdsm_server_commit": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_longlong)]),
    "mdsm_server_drain": (ctypes.c_int, [_vp]),
    "mdsm_server_get_stats": (ctypes.c_int, [_vp, ctypes.POINTER(ServerStats)]),
    "mdsm_server_destroy": (None, [_vp]),
}

_BOUND = False


def lib():
    global _BOUND
    L = load()
    if not _BOUND:
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _BOUND = True
    return L


class Server:
    """Continuous-batching server.  Add every beam first, then submit blocks as they arrive
    (block 0 of a beam carries nsamp + maxshift samples, later blocks nsamp new samples) and
    poll for per-block candidate lists."""

    def __init__(self, hbm_budget_bytes=64 << 30, host_stage_bytes=16 << 30, max_inflight=4,
                 nwidths=9, threshold=6.0, cand_cap=4096, detector="boxcar"):
        d = ServerDesc(int(hbm_budget_bytes), int(host_stage_bytes), int(max_inflight),
                       1 if detector == "boxcar" else 0, int(nwidths), float(threshold),
                       int(cand_cap))
        h = ctypes.c_void_p()
        check(lib().mdsm_server_create(ctypes.byref(d), ctypes.byref(h)))
        self._h = h
        self.cand_cap = cand_cap
        self.beams = []
        self._beam_shape = {}

    def close(self):
        if self._h:
            lib().mdsm_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_beam(self, nchans, fch1, foff, tsamp, nsamp, segments, in_dtype="u8",
                 shift_mode="l1", dm_block=0, kernel=0):
        segs = (Segment * len(segments))(*[Segment(float(a), float(b), int(n))
                                           for a, b, n in segments])
        d = BruteDesc(int(nchans), float(fch1), float(foff), float(tsamp), int(nsamp), segs,
                      len(segments), SHIFT_MODES[shift_mode], 0.0, DTYPES[in_dtype],
                      OUT_DTYPES["i32" if in_dtype != "f32" else "f32"], ACC["auto"],
                      int(dm_block), int(kernel))
        b = ctypes.c_int()
        check(lib().mdsm_server_add_beam_brute(self._h, ctypes.byref(d), ctypes.byref(b)))
        self.beams.append(segs)
        self._beam_shape[b.value] = (int(nchans), _NP_OF[in_dtype])
        return b.value

    def add_beam_subband(self, nchans, fch1, foff, tsamp, nsamp, nsubs, passes, in_dtype="u8"):
        arr = (SUBBAND_PASSES * len(passes))()
        for k, p in enumerate(passes):
            for f in ("lowdm", "highdm", "dmstep", "sub_dmstep", "ncalls", "calldms", "ndms"):
                if f in p:
                    setattr(arr[k], f, p[f])
            arr[k].binsize = int(p.get("binsize", 1))
        d = SubbandDesc(int(nchans), float(fch1), float(foff), float(tsamp), int(nsamp),
                        int(nsubs), arr, len(passes), 1, DTYPES[in_dtype],
                        OUT_DTYPES["i32" if in_dtype != "f32" else "f32"], ACC["auto"])
        b = ctypes.c_int()
        check(lib().mdsm_server_add_beam_subband(self._h, ctypes.byref(d), ctypes.byref(b)))
        self.beams.append(arr)
        self._beam_shape[b.value] = (int(nchans), _NP_OF[in_dtype])
        return b.value

    def beam_info(self, beam):
        i = PlanInfo()
        check(lib().mdsm_server_beam_info(self._h, beam, ctypes.byref(i)))
        return i

    def submit(self, beam, block):
        """Returns the ticket, or None when admission refuses the block for now."""
        block = np.ascontiguousarray(block)
        t = ctypes.c_longlong()
        st = lib().mdsm_server_submit(self._h, beam, block.ctypes.data_as(ctypes.c_void_p),
                                      block.shape[1], ctypes.byref(t))
        if st == 7:  # MDSM_EBUDGET
            return None
        check(st)
        return t.value

    def acquire(self, beam):
        """A pinned staging buffer for the beam's next block as a writable numpy view
        [nchans][cols], or None when admission refuses for now.  Fill it, then commit(beam)."""
        ptr = _vp()
        cols = ctypes.c_longlong()
        st = lib().mdsm_server_acquire(self._h, beam, ctypes.byref(ptr), ctypes.byref(cols))
        if st == 7:  # MDSM_EBUDGET
            return None
        check(st)
        nchans, dtype = self._beam_shape[beam]
        n = nchans * cols.value * np.dtype(dtype).itemsize
        buf = (ctypes.c_char * n).from_address(ptr.value)
        return np.frombuffer(buf, dtype=dtype).reshape(nchans, cols.value)

    def commit(self, beam):
        t = ctypes.c_longlong()
        check(lib().mdsm_server_commit(self._h, beam, ctypes.byref(t)))
        return t.value

    def poll(self, wait_ms=0):
        r = BlockResult()
        buf = (Candidate * self.cand_cap)()
        st = lib().mdsm_server_poll(self._h, ctypes.byref(r), buf, self.cand_cap, int(wait_ms))
        if st == 10:  # MDSM_EAGAIN
            return None
        check(st)
        from .api import CAND_DTYPE
        n = min(r.ncand, self.cand_cap)
        cands = np.frombuffer(buf, dtype=CAND_DTYPE, count=n).copy()
        return {"beam": r.beam, "block": r.block, "ticket": r.ticket,
                "latency_s": r.done_time - r.submit_time, "ncand": r.ncand, "cands": cands}

    def drain(self):
        check(lib().mdsm_server_drain(self._h))

    def stats(self):
        s = ServerStats()
        check(lib().mdsm_server_get_stats(self._h, ctypes.byref(s)))
        return {f: getattr(s, f) for f, _ in ServerStats._fields_}

    def results(self, expected, timeout_s=120.0):
        """Poll until `expected` results arrived."""
        out = []
        t0 = time.time()
        while len(out) < expected and time.time() - t0 < timeout_s:
            r = self.poll(wait_ms=20)
            if r is not None:
                out.append(r)
        return out
