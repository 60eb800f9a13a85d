"""Python host API of the batched form (native code in mdsm_gb300/csrc/batch.cpp)."""
import ctypes

import numpy as np

from ._lib import Candidate, check, load
from .api import CAND_DTYPE, _stream_ptr


class Batch:
    """Several BrutePlans dedispersed together by one persistent launch (optionally clipped
    before and searched after), replayable as one CUDA graph."""

    def __init__(self, plans):
        self.plans = list(plans)  # the plans must outlive the batch
        arr = (ctypes.c_void_p * len(plans))(*[p._h.value for p in plans])
        h = ctypes.c_void_p()
        check(load().mdsm_batch_create(arr, len(plans), ctypes.byref(h)))
        self._h = h
        self.cap = 0

    def close(self):
        if self._h:
            load().mdsm_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_buffers(self, d_in, d_out):
        n = len(self.plans)
        ins = (ctypes.c_void_p * n)(*[t.data_ptr() for t in d_in])
        outs = (ctypes.c_void_p * n)(*[t.data_ptr() for t in d_out])
        ist = (ctypes.c_longlong * n)(*[p.info.in_stride for p in self.plans])
        ost = (ctypes.c_longlong * n)(*[t.stride(0) for t in d_out])
        self._keep = (d_in, d_out)
        check(load().mdsm_batch_set_buffers(self._h, ins, ist, outs, ost))

    def enable_clip(self, k_chan=4.0, k_spec=4.0):
        check(load().mdsm_batch_enable_clip(self._h, float(k_chan), float(k_spec)))

    def enable_detect(self, nwidths=9, threshold=6.0, cap=4096):
        check(load().mdsm_batch_enable_detect(self._h, int(nwidths), float(threshold), int(cap)))
        self.cap = cap

    def autotune(self, stream=None):
        c = ctypes.c_int()
        check(load().mdsm_batch_autotune(self._h, _stream_ptr(stream), ctypes.byref(c)))
        return c.value

    def tune_times(self):
        """[(choice, ms per pass)] of the candidates the last autotune timed."""
        n = ctypes.c_int()
        check(load().mdsm_batch_autotune_times(self._h, None, None, 0, ctypes.byref(n)))
        ch = (ctypes.c_int * max(n.value, 1))()
        ms = (ctypes.c_float * max(n.value, 1))()
        check(load().mdsm_batch_autotune_times(self._h, ch, ms, n.value, ctypes.byref(n)))
        return [(ch[i], ms[i]) for i in range(n.value)]

    def run(self, graph=True, stream=None):
        check(load().mdsm_batch_run(self._h, int(bool(graph)), _stream_ptr(stream)))

    @property
    def last_launches(self):
        return load().mdsm_batch_last_launches(self._h)

    def candidates(self, beam, stream=None):
        buf = (Candidate * max(self.cap, 1))()
        n = ctypes.c_longlong()
        check(load().mdsm_batch_candidates(self._h, beam, buf, self.cap, ctypes.byref(n),
                                           _stream_ptr(stream)))
        return np.frombuffer(buf, dtype=CAND_DTYPE, count=min(n.value, self.cap)).copy()


def choice_info(choice):
    """What an autotuner choice means: a dict with fused, dm_block, time_tile, warps, order."""
    v = [ctypes.c_int() for _ in range(5)]
    check(load().mdsm_batch_choice_info(int(choice), *[ctypes.byref(x) for x in v]))
    return dict(zip(("fused", "dm_block", "time_tile", "warps", "order"), [x.value for x in v]))
