"""Generate the golden fixtures in tests/golden/ from the reference's own code.

Host fixtures (this script, run where the MDSM source tree is present): the reference's
detector and helpers (src/mdsm/dedispersion_output.cpp, src/mdsm/file_handler.cpp) are built
unmodified into oracle/_ref/libref_host.so by oracle/Makefile and run on seeded inputs.

Single-pulse fixtures (--singlepulse, here): the prototype's own template, convolution and
pruning functions (src/prototypes/singlepulse.cpp), built by oracle/Makefile against our
stand-in for FFTW into oracle/_ref/libref_singlepulse.so, on seeded inputs.

GPU fixtures (--gpu, run on a machine with a GPU and oracle/_ref/ref_kernels.cubin): the
reference's CUDA kernels (src/mdsm/dedispersion_kernel.cu) launched as
src/mdsm/dedispersion_thread.cu launches them; with --proto, the prototype kernels of
src/prototypes/detrend.cu and src/prototypes/rfi_clipper.cu (oracle/_ref/ref_detrend.cubin,
ref_rfi.cubin) launched as their own main() launches them, into ref_gpu_proto.npz.

Usage:  python tests/golden/make_golden.py [--singlepulse] [--gpu [--proto] [--out DIR]]
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


def singlepulse_fixtures(out_dir=HERE):
    """Outputs of singlepulse.cpp's createFFTKernel, convolve, pruneRelated and
    pruneRelatedDownfactors on seeded inputs (fftlen 512: the functions take any power of two)."""
    import ctypes
    orc.build(reference=True)
    if not orc.ref_singlepulse_available():
        raise SystemExit("single-pulse prototype not built (MDSM source tree absent)")
    h = orc.ref_singlepulse()
    P = ctypes.c_void_p
    ladder = np.array([2, 3, 4, 6, 9, 14, 20, 30, 45, 70, 100, 150], np.int32)
    N = 512
    spectra = np.zeros((ladder.size, 2 * (N // 2 + 1)), np.float32)
    for i, w in enumerate(ladder):
        h.ref_sp_kernel(int(w), N, spectra[i].ctypes.data_as(P))
    rng = np.random.default_rng(314)
    chunk = rng.standard_normal(N).astype(np.float32)
    chunk[:48] = 0.0  # the first chunk's zero padding (:226-230, 96 samples at fftlen 8192)
    chunk[200:206] += np.float32(4.0)
    chunk[330:333] += np.float32(6.0)
    conv = np.zeros((8, N), np.float32)
    for i, w in enumerate(ladder[:8]):
        h.ref_sp_convolve(chunk.ctypes.data_as(P), int(w), N, conv[i].ctypes.data_as(P))
    # pruneRelated on sorted lists: clusters of nearby bins, quantised values (ties), a few
    # lists longer than 256 entries (the prototype's char mask takes the list index mod 256)
    pr_bins, pr_vals, pr_off, pr_fac, pr_bins_out, pr_vals_out = [], [], [0], [], [], []
    for k in range(140):
        n = int(rng.integers(1, 40)) if k < 136 else int(rng.integers(280, 700))
        gaps = rng.choice([1, 1, 1, 2, 3, 5, 9, 20, 60], size=n)
        b = (int(rng.integers(0, 50)) + np.cumsum(gaps)).astype(np.uint32)
        v = (5.0 + 0.25 * rng.integers(0, 24, n)).astype(np.float32)
        f = int(rng.choice(ladder[:8]))
        bo, vo = b.copy(), v.copy()
        h.ref_sp_prune_related(bo.ctypes.data_as(P), vo.ctypes.data_as(P), n, f)
        pr_bins.append(b)
        pr_vals.append(v)
        pr_bins_out.append(bo)
        pr_vals_out.append(vo)
        pr_off.append(pr_off[-1] + n)
        pr_fac.append(f)
    # pruneRelatedDownfactors on lists in the prototype's order: per chunk, width 1 then each
    # downfactor, bins ascending within a width
    pd_bins, pd_vals, pd_df, pd_off, pd_nf, pd_mask = [], [], [], [0], [], []
    for k in range(120):
        nf = int(rng.integers(1, 9))
        widths = [1] + list(ladder[:nf])
        bins, vals, dfs = [], [], []
        for c in range(int(rng.integers(1, 4))):
            for w in widths:
                m = int(rng.integers(0, 6))
                bb = np.sort(rng.choice(np.arange(c * 400, c * 400 + 400), m, replace=False))
                bins += list(bb)
                vals += list(5.0 + 0.5 * rng.integers(0, 12, m))
                dfs += [w] * m
        n = len(bins)
        bins = np.array(bins, np.int64)
        vals = np.array(vals, np.float32)
        dfs = np.array(dfs, np.uint32)
        mask = np.zeros(max(n, 1), np.uint8)
        if n:
            h.ref_sp_prune_downfactors(bins.ctypes.data_as(P), vals.ctypes.data_as(P),
                                       dfs.ctypes.data_as(P), n, nf, mask.ctypes.data_as(P))
        pd_bins.append(bins)
        pd_vals.append(vals)
        pd_df.append(dfs.astype(np.int32))
        pd_mask.append(mask[:n])
        pd_off.append(pd_off[-1] + n)
        pd_nf.append(nf)
    cat = np.concatenate
    np.savez_compressed(os.path.join(out_dir, "ref_singlepulse.npz"), ladder=ladder,
                        fftlen=np.int32(N), spectra=spectra, chunk=chunk, conv=conv,
                        pr_bins=cat(pr_bins).astype(np.int32), pr_vals=cat(pr_vals),
                        pr_off=np.array(pr_off, np.int64), pr_fac=np.array(pr_fac, np.int32),
                        pr_bins_out=cat(pr_bins_out).astype(np.int32),
                        pr_vals_out=cat(pr_vals_out), pd_bins=cat(pd_bins),
                        pd_vals=cat(pd_vals), pd_df=cat(pd_df),
                        pd_off=np.array(pd_off, np.int64), pd_nf=np.array(pd_nf, np.int32),
                        pd_mask=cat(pd_mask))
    print("wrote ref_singlepulse.npz: %d prune lists, %d downfactor lists"
          % (len(pr_fac), len(pd_nf)))


def proto_gpu_fixtures(out_dir=HERE):
    """detrend_normalise and rfi_clipping, the prototype kernels, on seeded float blocks."""
    orc.build(reference=False)
    g = orc.RefGPU(proto=True)
    rng = np.random.default_rng(2718)
    out = {}
    # detrend: 4 rows x 4096 samples, blocks of 1024: noise on a per-row line and offset
    t = np.arange(4096, dtype=np.float64)
    dt_in = (rng.standard_normal((4, 4096)) * 3.0 + 100.0 + 0.01 * t[None, :] *
             np.arange(1, 5)[:, None]).astype(np.float32)
    dt_in[2, 1500:1510] += np.float32(40.0)
    dt_out, _ = g.detrend(dt_in, 1024)
    out.update(detrend_in=dt_in, detrend_out=dt_out, detrend_len=np.int32(1024))
    # the same input again: the kernel's unsynchronised second reduction, if it raced,
    # would show here as a difference between runs
    dt_out2, _ = g.detrend(dt_in, 1024)
    out.update(detrend_out_repeat=dt_out2)
    # rfi: 8 rows x 1024 samples, 512 threads (the prototype's default block): Gaussian
    # float rows and integer-valued rows, each with impulsive outliers
    rf_f = (rng.standard_normal((8, 1024)) * 2.0 + 10.0).astype(np.float32)
    rf_f[:, rng.choice(1024, 12, replace=False)] += np.float32(30.0)
    rf_u = np.clip(np.round(rng.standard_normal((8, 1024)) * 16 + 128), 0, 255).astype(np.float32)
    rf_u[:, rng.choice(1024, 12, replace=False)] = np.float32(255.0)
    for name, x in (("rfi_f", rf_f), ("rfi_u", rf_u)):
        y, means, _ = g.rfi_clip(x, 512)
        out.update({name + "_in": x, name + "_out": y, name + "_means": means})
    out.update(rfi_blockdim=np.int32(512))
    np.savez_compressed(os.path.join(out_dir, "ref_gpu_proto.npz"), **out)
    print("wrote ref_gpu_proto.npz; detrend repeat identical: %s"
          % bool(np.array_equal(dt_out, dt_out2)))


if __name__ == "__main__":
    if "--gpu" in sys.argv:
        od = sys.argv[sys.argv.index("--out") + 1] if "--out" in sys.argv else HERE
        if "--proto" in sys.argv:
            proto_gpu_fixtures(od)
        else:
            gpu_fixtures(od)
    elif "--singlepulse" in sys.argv:
        singlepulse_fixtures()
    else:
        host_fixtures()
