"""Generate the golden fixtures in tests/golden/ from the reference's own code.

Host fixtures (this script, run where the MDSM source tree is present): the reference's
detector and helpers (src/mdsm/dedispersion_output.cpp, src/mdsm/file_handler.cpp) are built
unmodified into oracle/_ref/libref_host.so by oracle/Makefile and run on seeded inputs.

GPU fixtures (--gpu, run on a machine with a GPU and oracle/_ref/ref_kernels.cubin): the
reference's CUDA kernels (src/mdsm/dedispersion_kernel.cu) launched as
src/mdsm/dedispersion_thread.cu launches them.

Usage:  python tests/golden/make_golden.py [--gpu]
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as orc  # noqa: E402


def detector_cube():
    """A small dedispersed block with three strong rows of excess, seed 42."""
    rng = np.random.default_rng(42)
    cube = rng.standard_normal((16, 2048), dtype=np.float32) * np.float32(3.0)
    cube[5, 700:706] += np.float32(30.0)
    cube[9, 1500:1503] += np.float32(25.0)
    cube[12, 100:140] += np.float32(12.0)
    return cube


def host_fixtures():
    orc.build(reference=True)
    if not orc.ref_host_available():
        raise SystemExit("reference host code not built (MDSM source tree absent)")
    h = orc.ref_host()
    import ctypes
    # median of five over random tuples with ties
    rng = np.random.default_rng(5)
    tup = rng.integers(0, 4, (3000, 5)).astype(np.float32)
    tup[1000:] = rng.standard_normal((2000, 5)).astype(np.float32)
    med = np.array([h.ref_median_of_five(*map(float, t)) for t in tup], np.float32)
    # process_brute on a small block: lowdm 0, dmstep 0.5 (rows 0-2 have DM <= 1.0)
    cube = detector_cube()
    fd, path = tempfile.mkstemp(suffix=".dat")
    os.close(fd)
    buf = np.ascontiguousarray(cube)
    rc = h.ref_process_brute(buf.ctypes.data_as(ctypes.c_void_p), cube.shape[0], cube.shape[1],
                             ctypes.c_float(0.0), ctypes.c_float(0.5), ctypes.c_float(4.0),
                             path.encode())
    assert rc == 0
    rows = []
    with open(path) as f:
        for line in f:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 3:
                rows.append((float(parts[0]), float(parts[1]), float(parts[2])))
    os.unlink(path)
    det = np.array(rows, np.float64).reshape(-1, 3)
    # process_brute with caller noise statistics (one mean/rms per 256 samples)
    spc = 256
    nchunk = (cube.shape[1] - 4 + spc - 1) // spc
    crng = np.random.default_rng(77)
    cmean = (crng.standard_normal(nchunk) * 0.5).astype(np.float32)
    crms = (3.0 + crng.uniform(0.0, 1.0, nchunk)).astype(np.float32)

    def lines(path, nf):
        out = []
        with open(path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= nf:
                    out.append(tuple(float(v) for v in parts[:nf]))
        os.unlink(path)
        return np.array(out, np.float64).reshape(-1, nf)

    fd, path = tempfile.mkstemp(suffix=".dat")
    os.close(fd)
    rc = h.ref_process_brute_chunked(buf.ctypes.data_as(ctypes.c_void_p), cube.shape[0],
                                     cube.shape[1], ctypes.c_float(0.0), ctypes.c_float(0.5),
                                     ctypes.c_float(4.0), spc,
                                     cmean.ctypes.data_as(ctypes.c_void_p),
                                     crms.ctypes.data_as(ctypes.c_void_p), path.encode())
    assert rc == 0
    det_chunked = lines(path, 5)
    # process_subband, one pass of 4 calls x 4 fine DMs, caller noise statistics; binsize 1
    # and 2 (rows of nsamp / binsize samples)
    sub = {}
    for b in (1, 2):
        rows = np.ascontiguousarray(cube[:, : cube.shape[1] // b])
        fd, path = tempfile.mkstemp(suffix=".dat")
        os.close(fd)
        rc = h.ref_process_subband_chunked(rows.ctypes.data_as(ctypes.c_void_p), cube.shape[1],
                                           ctypes.c_float(0.0), ctypes.c_float(0.5),
                                           ctypes.c_float(2.0), 4, 4, b, ctypes.c_float(4.0),
                                           spc, cmean.ctypes.data_as(ctypes.c_void_p),
                                           crms.ctypes.data_as(ctypes.c_void_p), path.encode())
        assert rc == 0
        sub[b] = lines(path, 3)
    # read_block unpack for every bit width
    raw = rng.integers(0, 256, 256, dtype=np.uint8)
    fd, rpath = tempfile.mkstemp(suffix=".raw")
    os.close(fd)
    raw.tofile(rpath)
    unpacked = {}
    for nbits in (1, 2, 4, 8, 16):
        nsamp = raw.size * 8 // nbits
        out = np.zeros(nsamp, np.float32)
        n = h.ref_read_block(rpath.encode(), nbits, out.ctypes.data_as(ctypes.c_void_p),
                             ctypes.c_ulong(nsamp))
        unpacked[nbits] = out[:n].copy()
    os.unlink(rpath)
    np.savez_compressed(os.path.join(HERE, "ref_host.npz"), median_in=tup, median_out=med,
                        detect_rows=det, detect_threshold=np.float32(4.0),
                        detect_lowdm=np.float32(0.0), detect_dmstep=np.float32(0.5),
                        chunk_spc=np.int32(spc), chunk_mean=cmean, chunk_rms=crms,
                        detect_chunked_rows=det_chunked, subband_rows_b1=sub[1],
                        subband_rows_b2=sub[2],
                        unpack_raw=raw, **{"unpack_%d" % k: v for k, v in unpacked.items()})
    print("wrote ref_host.npz: %d detections, %d with chunk statistics, %d / %d subband"
          % (len(det), len(det_chunked), len(sub[1]), len(sub[2])))


def gpu_fixtures(out_dir=HERE):
    orc.build(reference=False)
    g = orc.RefGPU()
    out = {}
    # L1 kernel (the default path) on a small float block; contraction-sensitive plan
    nchans, nsamp, tsamp, fch1, foff = 64, 420, 64e-6, 1500.0, -300.0 / 64
    lowdm, dmstep, tdms = 0.0, 0.9765625 / 3.0, 64
    dms = orc.dmshifts(nchans, fch1, foff)
    S = orc.shift_table(nchans, fch1, foff, tsamp, [(lowdm, dmstep, tdms)], mode="l1")
    ms = int(S.max()) + 2
    rng = np.random.default_rng(21)
    x = rng.standard_normal((nchans, nsamp + ms), dtype=np.float32)
    y, _ = g.brute(0, x, nsamp, ms, lowdm, dmstep, tsamp, tdms, dms)
    out.update(l1_x=x, l1_y=y, l1_meta=np.array([nchans, nsamp, ms, tdms], np.int64),
               l1_f=np.array([fch1, foff, tsamp, lowdm, dmstep], np.float64))
    # opt kernel
    nsamp2 = 384
    S2 = orc.shift_table(nchans, fch1, foff, tsamp, [(lowdm, dmstep, tdms)], mode="opt")
    ms2 = int(S2.max()) + 2
    x2 = rng.standard_normal((nchans, nsamp2 + ms2), dtype=np.float32)
    y2, _ = g.brute(1, x2, nsamp2, ms2, lowdm, dmstep, tsamp, tdms, dms)
    out.update(opt_x=x2, opt_y=y2, opt_meta=np.array([nchans, nsamp2, ms2, tdms], np.int64))
    np.savez_compressed(os.path.join(out_dir, "ref_gpu.npz"), **out)
    print("wrote ref_gpu.npz")


if __name__ == "__main__":
    if "--gpu" in sys.argv:
        od = sys.argv[sys.argv.index("--out") + 1] if "--out" in sys.argv else HERE
        gpu_fixtures(od)
    else:
        host_fixtures()
