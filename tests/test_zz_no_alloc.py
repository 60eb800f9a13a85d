"""The reference detector's no-allocation entry point, for callers that cannot allocate device
memory (a real-time stage that must not stall on the allocator between blocks, a host that
hands out all device memory at start-up, a plugin where allocation is not permitted).

Called through the C ABI twice in a row on different blocks; each result must equal the
allocating entry point's (mdsm_ref_detect_device) on the same block: the same candidates and
the same statistics, bit for bit.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _block(seed, ndms, nsamp):
    rng = np.random.default_rng(seed)
    y = rng.standard_normal((ndms, nsamp), dtype=np.float32) * np.float32(4.0)
    y[ndms // 2, 1000:1006] += np.float32(40.0)
    y[ndms - 3, 5000:5003] += np.float32(35.0)
    return y


def _detect(fn, d, ndms, nsamp, cap, stream):
    from mdsm_gb300 import _lib
    buf = (_lib.Candidate * cap)()
    n = ctypes.c_longlong(-1)
    mean, rms = ctypes.c_float(), ctypes.c_float()
    st = fn(ctypes.c_void_p(d.data_ptr()), ndms, nsamp, ctypes.c_float(2.0),
            ctypes.c_float(0.25), ctypes.c_float(5.0), buf, cap, ctypes.byref(n),
            ctypes.byref(mean), ctypes.byref(rms), stream)
    from mdsm_gb300.api import CAND_DTYPE
    return st, np.frombuffer(buf, dtype=CAND_DTYPE, count=min(n.value, cap)).copy(), n.value, \
        mean.value, rms.value


def test_noalloc_detector_matches_allocating_one(lib, cuda):
    torch = cuda
    L = lib
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    # two calls in a row, different block sizes (the second smaller, so stale contents of the
    # shared array from the first call would show)
    for seed, ndms, nsamp in ((1, 64, 40000), (2, 24, 9000)):
        y = _block(seed, ndms, nsamp)
        d = torch.from_numpy(y).cuda()
        st1, c1, n1, m1, r1 = _detect(L.mdsm_ref_detect_device_noalloc, d, ndms, nsamp, 4096,
                                      stream)
        st2, c2, n2, m2, r2 = _detect(L.mdsm_ref_detect_device, d, ndms, nsamp, 4096, stream)
        assert st1 == 0 and st2 == 0
        assert n1 == n2 > 0
        assert (m1, r1) == (m2, r2)
        assert np.array_equal(c1, c2)


def test_noalloc_detector_rejects_oversize_requests(lib, cuda):
    torch = cuda
    from mdsm_gb300 import _lib
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    d = torch.zeros((4, 1000), dtype=torch.float32, device="cuda")
    st, _, _, _, _ = _detect(lib.mdsm_ref_detect_device_noalloc, d, 4, 1000, 70000, stream)
    assert st == 6  # MDSM_ERANGE: cap beyond the fixed array
    assert b"exceeds" in lib.mdsm_last_error()
