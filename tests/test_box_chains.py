"""The boxcar search's tile geometry and chain index arithmetic (mdsm_gb300/csrc/box.cuh),
restated on the host for the thread counts and chain lengths the two search kernels are built
with (read from detect.cu and dedisp.cu): every chain access inside its shared-memory buffer,
every position stored once per step, each warp's chain accesses in 32 distinct banks, the
largest sum of every width over a region equal to the pairwise-doubled sums formed directly
(so the fast path's threshold test sees exactly the sums the exact path forms), and the
standalone kernel's shared memory within four CTAs per SM."""
import os
import re

import numpy as np
import pytest

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "mdsm_gb300",
                    "csrc")
SMEM_PER_SM = 228 * 1024  # bytes of shared memory per SM (sm_100 family)
SMEM_PER_CTA_RESERVED = 1024


def _const(fname, name):
    src = open(os.path.join(CSRC, fname)).read()
    m = re.search(r"constexpr int %s = (\d+);" % name, src)
    assert m, (fname, name)
    return int(m.group(1))


def _shapes():
    return [(_const("detect.cu", "kBoxThreads"), _const("detect.cu", "kBoxK"),
             _const("detect.cu", "kBoxKE")),
            (_const("dedisp.cu", "kFusedBoxThreads"), _const("dedisp.cu", "kFusedBoxK"),
             _const("dedisp.cu", "kFusedBoxK"))]


def geom(nw, threads, k, ke):
    """BoxGeom<NW, THREADS, K, KE>."""
    wmax = 1 << (nw - 1)
    hl = max(wmax // 2, 1)
    n, ne = threads * k, threads * ke
    g = dict(wmax=wmax, hl=hl, n=n, tile=(n - wmax + 1) & ~3, etile=(ne - 2 * hl - wmax) & ~3)
    g["nbest"] = g["etile"] + 2 * hl
    g["steps"] = (nw + 1) // 3
    g["nd"] = lambda s: min(3, nw - 1 - 3 * (s - 1))
    g["la"] = lambda s: (1 << g["nd"](s)) - 1
    g["umax"] = 1 << (3 * (g["steps"] - 1)) if g["steps"] else 1
    pad = max([(1 << (3 * (s - 1))) * g["la"](s) for s in range(2, g["steps"] + 1)], default=0)
    pairs = (ne + 2 * threads - 1) // (2 * threads)
    buf0 = pairs * 2 * threads + max(wmax, 2)
    g["buf"] = (max(buf0, n + pad) + 3) // 4 * 4
    g["nbf"] = n + 8
    g["smem"] = g["nbf"] * 4 + g["buf"] * 8 + g["nbest"] * 4 + 80
    return g


@pytest.mark.parametrize("nw", range(1, 10))
@pytest.mark.parametrize("shape", _shapes(), ids=["k_boxcar", "fused"])
def test_chain_steps_cover_the_region_and_form_the_pairwise_sums(shape, nw):
    threads, k, ke = shape
    g = geom(nw, threads, k, ke)
    n = g["n"]
    assert k % 2 == 1 and g["umax"] <= threads
    assert g["etile"] >= threads and g["tile"] >= g["etile"]
    assert g["tile"] + g["wmax"] - 1 <= n  # every boxcar starting in the tile is staged
    assert g["tile"] % 4 == 0 and g["nbf"] % 4 == 0 and g["nbest"] % 2 == 0
    rng = np.random.default_rng(nw)
    x = rng.standard_normal(n).astype(np.float32)
    nb = np.zeros(g["nbf"], np.float32)
    nb[:n] = x
    bufs = [np.zeros(g["buf"], np.float32), np.zeros(g["buf"], np.float32)]  # A, Bf
    m = np.full((threads, nw), -np.inf, np.float32)
    if g["steps"] == 0:
        for tid in range(threads):
            m[tid, 0] = nb[k * tid + np.arange(k)].max()
    for s in range(1, g["steps"] + 1):
        u, nd, la = 1 << (3 * (s - 1)), g["nd"](s), g["la"](s)
        src = nb if s == 1 else bufs[0 if s % 2 == 0 else 1]
        nxt = bufs[0 if s % 2 == 1 else 1]
        stored = np.zeros(n, np.int64)
        out = []
        for tid in range(threads):
            p0 = (tid & (u - 1)) + u * k * (tid // u)
            idx = p0 + (np.arange(k + la) if s == 1 else u * np.arange(k + la))
            assert idx.max() < (g["nbf"] if s == 1 else g["buf"])
            c = src[idx].copy()
            if s == 1:
                m[tid, 0] = max(m[tid, 0], c[:k].max())
            for e in range(1, nd + 1):
                h = 1 << (e - 1)
                for j in range(k + la + 1 - 2 * h):
                    c[j] = np.float32(c[j] + c[j + h])
                m[tid, 3 * (s - 1) + e] = max(m[tid, 3 * (s - 1) + e], c[:k].max())
            if s < g["steps"]:
                st = p0 + u * np.arange(k)
                assert st.max() < n
                stored[st] += 1
                out.append((st, c[:k].copy()))
        if s < g["steps"]:
            assert (stored == 1).all()
            for st, v in out:
                nxt[st] = v
        for w0 in range(0, threads, 32):  # one warp's accesses of chain element j
            for j in range(k):
                banks = {((t & (u - 1)) + u * k * (t // u) + u * j) % 32 for t in range(w0, w0 + 32)}
                assert len(banks) == 32
    # direct: B_2w[i] = B_w[i] + B_w[i + w], zeros past the region
    cur = np.concatenate([x, np.zeros(2 * g["wmax"], np.float32)])
    want = [cur[:n].max()]
    for l in range(1, nw):
        w = 1 << (l - 1)
        cur = (cur[:-w] + cur[w:]).astype(np.float32)
        want.append(cur[:n].max())
    assert np.array_equal(m.max(axis=0), np.array(want, np.float32))


@pytest.mark.parametrize("nw", range(1, 10))
def test_standalone_search_fits_four_ctas_per_sm(nw):
    threads, k, ke = _shapes()[0]
    g = geom(nw, threads, k, ke)
    assert 4 * (g["smem"] + SMEM_PER_CTA_RESERVED) <= SMEM_PER_SM


@pytest.mark.parametrize("nw", range(1, 10))
@pytest.mark.parametrize("shape", _shapes(), ids=["k_boxcar", "fused"])
def test_exact_path_reads_stay_in_its_buffers(shape, nw):
    """box_tile_exact: position pairs i = 2 tid + 2 THREADS q (q < PAIRS) of its own region;
    step s (u = 4^(s-1)) reads the float2 partners at i + u and, when it forms two widths, at
    i + 2u and i + 3u (i + 2 .. i + 4 for u = 1); the candidate pass reads best[q + HL +- h]
    for h <= max(w/2, 1) <= HL and q < ETILE."""
    threads, k, ke = shape
    g = geom(nw, threads, k, ke)
    pairs = (threads * ke + 2 * threads - 1) // (2 * threads)
    imax = 2 * (threads - 1) + 2 * threads * (pairs - 1)
    top = imax + 1  # the pair's own values
    s = 1
    while 2 * s - 1 < nw:
        u = 1 << (2 * s - 2)
        two = 2 * s < nw
        if u == 1:
            top = max(top, imax + (4 if two else 3))
        else:
            top = max(top, imax + (3 * u if two else u) + 1)
        s += 1
    assert top < g["buf"]
    assert pairs * 2 * threads >= g["nbest"]  # every position with a best SNR is formed
    h = max(g["wmax"] // 2, 1)
    assert h <= g["hl"] and (g["etile"] - 1) + g["hl"] + h < g["nbest"]
