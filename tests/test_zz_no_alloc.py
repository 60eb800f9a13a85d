"""The reference detector's no-allocation entry point, for callers that cannot allocate device
memory (a real-time stage that must not stall on the allocator between blocks, a host that
hands out all device memory at start-up, a plugin where allocation is not permitted).

Called through the C ABI twice in a row on different blocks; each result must equal the
allocating entry point's (mdsm_ref_detect_device) on the same block: the same candidates and
the same statistics, bit for bit.  A fresh process checks that the calls allocate no device
memory (a process where earlier tests already made the library's scratch buffer could not
show an allocation that came back).
"""
import ctypes
import os
import subprocess
import sys

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


_ALLOC_PROBE = r"""
import ctypes, sys
import numpy as np, torch
sys.path.insert(0, sys.argv[1])
from mdsm_gb300 import _lib
lib = _lib.load()
torch.cuda.init()
ys = [torch.from_numpy(np.random.default_rng(s).standard_normal((n, 20000), dtype=np.float32)).cuda()
      for s, n in ((1, 16), (2, 96))]
buf = (_lib.Candidate * 1024)()
n = ctypes.c_longlong(); m = ctypes.c_float(); r = ctypes.c_float()
def call(fn, y):
    st = fn(ctypes.c_void_p(y.data_ptr()), y.shape[0], y.shape[1], ctypes.c_float(0.0),
            ctypes.c_float(1.0), ctypes.c_float(5.0), buf, 1024, ctypes.byref(n), ctypes.byref(m),
            ctypes.byref(r), None)
    assert st == 0, lib.mdsm_last_error()
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]
call(lib.mdsm_ref_detect_device_noalloc, ys[0])  # (the first use loads the kernels' code)
free0 = torch.cuda.mem_get_info()[0]
free1 = call(lib.mdsm_ref_detect_device_noalloc, ys[1])
free2 = call(lib.mdsm_ref_detect_device_noalloc, ys[0])
free3 = call(lib.mdsm_ref_detect_device, ys[1])  # the allocating detector: its scratch buffer
print(free0, free1, free2, free3)
"""


def test_noalloc_detector_allocates_nothing(lib, cuda, tmp_path):
    """Free device memory is unchanged across no-allocation calls on a larger and a smaller
    block, and drops when the allocating detector then makes its scratch buffer (the
    measurement sees an allocation of this size)."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    probe = tmp_path / "probe.py"
    probe.write_text(_ALLOC_PROBE)
    r = subprocess.run([sys.executable, str(probe), root], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    free0, free1, free2, free3 = map(int, r.stdout.split()[-4:])
    assert free1 == free0 and free2 == free0, (free0, free1, free2)
    assert free3 < free0, (free0, free3)


def test_noalloc_detector_rejects_oversize_requests(lib, cuda):
    torch = cuda
    from mdsm_gb300 import _lib
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    d = torch.zeros((4, 1000), dtype=torch.float32, device="cuda")
    st, _, _, _, _ = _detect(lib.mdsm_ref_detect_device_noalloc, d, 4, 1000, 70000, stream)
    assert st == 6  # MDSM_ERANGE: cap beyond the fixed array
    assert b"exceeds" in lib.mdsm_last_error()
    # more than 2^31 values: refused before the series is touched, as by the allocating
    # detector (the pointer's buffer is far smaller than the sizes passed)
    for fn in (lib.mdsm_ref_detect_device_noalloc, lib.mdsm_ref_detect_device):
        st, _, _, _, _ = _detect(fn, d, 65536, 32769, 16, stream)
        assert st == 1, lib.mdsm_last_error()  # MDSM_EINVAL
        assert b"32 bits" in lib.mdsm_last_error()
