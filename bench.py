"""Benchmark: DM-trial-samples/s of brute-force incoherent dedispersion on one GB300.

Workload (default): the full-band plain path -- uint8 filterbank, 4096 channels
(1500 MHz top, 300 MHz band), tsamp 64 us, blocks of 2^18 samples, 4096 DM trials 0-2000 with
the step doubling at 500 and 1000, exact INT32 accumulation, int32 series out.  One step is
one block.  Synthetic Gaussian data (mean 128, sigma 16) generated on the device from a seed;
each block's input (1.2 GB) is larger than L2, so no flush is needed between steps.

value : DM-trial-samples/s with the input resident in HBM (device-pointer C-ABI call).
e2e   : the same metric through the host-buffer C-ABI call (pinned host input copied in,
        full dedispersed block copied out, every step).
serving: the serving form on 64 beams x 2^16-sample blocks x 4096 DM trials (every tenth beam
        at 1024 channels), subband and brute force: saturating throughput, p50/p99 block
        latency, real-time factor, and the ratio to the plain per-block path on the same blocks
        (same algorithm; detections compared block by block); a run at Poisson arrivals of
        1.0-1.5x real time; the first subband stage's add rate; clocks sampled meanwhile.
batched: the batched form on 32 uneven beams (RFI clip, dedispersion and boxcar search as one
        fused persistent launch in a CUDA graph, launch shape autotuned) against the plain
        per-beam path on the same blocks, detections compared beam by beam; clocks sampled.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
       python bench.py --case serve   (the serving object alone)
       python bench.py --case batch   (the batched object alone)
For N > 1 run under torch.distributed.run; each rank processes its own beam (weak scaling).
"""
import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NCHANS, NSAMP, FCH1, BW, TSAMP = 4096, 1 << 18, 1500.0, 300.0, 64e-6
SEGMENTS = [(0.0, 0.244140625, 2048), (500.0, 0.48828125, 1024), (1000.0, 0.9765625, 1024)]
METRIC = "DM-trial-samples/s"
WORKLOAD = ("full-band plain path, brute force: uint8 4096 ch x 2^18 samples per block, "
            "4096 DM trials 0-2000 (steps 0.244/0.488/0.977 pc cm^-3 with doubling at 500 and "
            "1000), INT32 accumulation, int32 output")


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d, "measured"
    return {"hbm_gbs": 6800.0, "sm_max_mhz": 2070.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during a region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        import tempfile
        self.idx = gpu_index
        self.p = None
        # the raw samples (MDSM_CLOCKS_DIR keeps them; by default a temporary directory)
        d = os.environ.get("MDSM_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = os.path.join(d, "clocks_bench_%d_%d.csv" % (os.getpid(), id(self)))

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p is not None:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()
            self.f.close()

    def summary(self):
        if self.p is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    mx.append(float(parts[2]))
                except ValueError:
                    continue
                for k, n in enumerate(names):
                    if parts[5 + k].lower().startswith("active"):
                        reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


_CPU_CACHE = {}


def cpu_sample(orc, ndms, nsamp, nchans, seed=7):
    """Time the oracle's brute force (the reference algorithm, OpenMP over DMs) on a sample."""
    key = ("S", nchans)
    if key not in _CPU_CACHE:
        _CPU_CACHE[key] = orc.shift_table(nchans, FCH1, -BW / nchans, TSAMP, SEGMENTS, mode="l1")
    S_full = _CPU_CACHE[key]
    pick = np.linspace(0, S_full.shape[0] - 1, ndms).astype(int)
    S = np.ascontiguousarray(S_full[pick])
    ncols = nsamp + int(S_full.max()) + 1
    xkey = ("x", nchans, ncols)
    if xkey not in _CPU_CACHE:
        rng = np.random.default_rng(seed)
        _CPU_CACHE[xkey] = rng.integers(96, 160, (nchans, ncols), dtype=np.uint8)
    x = _CPU_CACHE[xkey]
    t0 = time.perf_counter()
    orc.dedisperse(x, S, nsamp)
    return time.perf_counter() - t0


def calibrate(orc, budget_s, nchans=NCHANS):
    """(ndms, nsamp) of a sample that takes about budget_s on this host."""
    nsamp = 16384
    t_small = cpu_sample(orc, 8, nsamp, nchans)
    scale = budget_s / max(t_small, 1e-3)
    ndms = int(max(8, min(4096, 8 * scale)))
    if ndms == 4096:
        nsamp = int(min(NSAMP, nsamp * scale * 8 / 4096))
        nsamp = max(16384, nsamp // 1024 * 1024)
    return ndms, nsamp


def cpu_baseline(orc, budget_s=10.0, nchans=NCHANS):
    cores = os.cpu_count() or 1
    ndms, nsamp = calibrate(orc, budget_s, nchans)
    t = cpu_sample(orc, ndms, nsamp, nchans)
    if t < 0.6 * budget_s and nsamp < NSAMP:
        # the small calibration sample overstates the cost per unit: widen to the budget
        nsamp = max(16384, int(min(NSAMP, nsamp * budget_s / max(t, 1e-3))) // 1024 * 1024)
        t = cpu_sample(orc, ndms, nsamp, nchans)
    return {"value": ndms * nsamp / t, "unit": METRIC, "cores": cores, "kind": "port",
            "sample": "oracle brute force (reference index math, OpenMP over DM trials) on "
                      "uint8 %d ch x %d samples x %d of the 4096 DM trials, %.1f s" %
                      (nchans, nsamp, ndms, t)}


def run_reference(args, rank, world):
    """The reference algorithm on the host cores (oracle port; the reference's own host code is
    not built on this machine), one bounded sample per step."""
    if rank != 0:
        return
    from oracle import oracle as orc
    orc.build(reference=False)
    ndms, nsamp = calibrate(orc, 6.0)
    for _ in range(args.warmup):
        cpu_sample(orc, ndms, nsamp, NCHANS)
    ts = [cpu_sample(orc, ndms, nsamp, NCHANS) for _ in range(args.steps)]
    t = max(float(np.mean(ts)), 1e-9)
    val = ndms * nsamp / t
    line = {"metric": METRIC, "value": val, "unit": METRIC, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD, "nchans": NCHANS, "nsamp": NSAMP, "ndms": 4096},
            "cpu_baseline": {"value": val, "unit": METRIC, "cores": os.cpu_count() or 1,
                             "kind": "port",
                             "sample": "uint8 %d ch x %d samples x %d DM trials per step" %
                                       (NCHANS, nsamp, ndms)},
            "e2e": {"value": val, "unit": METRIC, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def serve_passes(nchans):
    """Subband passes over the 4096-trial plan: 16 fine DM trials per sub-DM call."""
    out = []
    for lo, st, n in SEGMENTS:
        out.append(dict(lowdm=lo, highdm=lo + n * st, dmstep=st, sub_dmstep=16 * st,
                        ncalls=n // 16, calldms=16))
    return out


def block_adds(algo, nchans, nsamp):
    """Algorithmic adds of one block: brute force nchans per DM-trial-sample; subband, per
    output sample, ncalls * nchans for stage 1 plus ndms * nsubs for stage 2 per pass."""
    if algo != "subband":
        return sum(n for _, _, n in SEGMENTS) * nchans * nsamp
    nsubs = 64 if nchans == 4096 else 32
    return sum(p["ncalls"] * nchans + p["ncalls"] * p["calldms"] * nsubs
               for p in serve_passes(nchans)) * nsamp


SERVE_NSAMP = 1 << 16


def serve_nchans(b):
    """Channel count of serving beam b: every tenth beam has 1024 channels, the rest 4096."""
    return 1024 if b % 10 == 9 else 4096


def serve_plan_args(algo, nch):
    if algo == "subband":
        return dict(nsubs=64 if nch == 4096 else 32, passes=serve_passes(nch))
    return dict(segments=SEGMENTS)


def serve_workload(algo, seed=11):
    """The blocks of the serving workload, per channel count: seeded Gaussian uint8 (mean 128,
    sigma 16, generated on the device) with dispersed boxcar pulses.  A beam's stream is
    init (nsamp + maxshift samples) then regs[k % 2] for block k >= 1, so block k's full
    input (what the plain path copies in) is init for k = 0, init's tail + regs[1] for k = 1
    and regs[(k - 1) % 2]'s tail + regs[k % 2] after."""
    import torch

    import mdsm_gb300 as m
    from mdsm_gb300 import synth
    rng = np.random.default_rng(seed)
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    out = {}
    for nch in (4096, 1024):
        if algo == "subband":
            p = m.SubbandPlan(nch, FCH1, -BW / nch, TSAMP, SERVE_NSAMP, **serve_plan_args(algo, nch),
                              in_dtype="u8", out_dtype="i32")
        else:
            p = m.BrutePlan(nch, FCH1, -BW / nch, TSAMP, SERVE_NSAMP, SEGMENTS, in_dtype="u8",
                            out_dtype="i32")
        ms = p.info.maxshift

        def gauss(cols):
            v = torch.empty((nch, cols), device="cuda")
            v.normal_(128.0, 16.0, generator=g)
            a = torch.clamp(torch.round(v), 0, 255).to(torch.uint8).cpu().numpy()
            del v
            return a

        init = gauss(SERVE_NSAMP + ms)
        regs = [gauss(SERVE_NSAMP) for _ in range(2)]
        for a in [init] + regs:  # two pulses of SNR 10-40 per block, DM 50-1900
            pul = synth.random_pulses(rng, 2, SERVE_NSAMP - 256, 1900.0, 16.0, nch,
                                      widths=(1, 32), snr=(10, 40))
            synth.inject(a, FCH1, -BW / nch, TSAMP, [(t0, max(dm, 50.0), w, amp)
                                                     for t0, dm, w, amp in pul])
        full = [init,
                np.ascontiguousarray(np.concatenate([init[:, SERVE_NSAMP:], regs[1]], axis=1)),
                np.ascontiguousarray(np.concatenate([regs[1][:, SERVE_NSAMP - ms:], regs[0]],
                                                    axis=1)),
                np.ascontiguousarray(np.concatenate([regs[0][:, SERVE_NSAMP - ms:], regs[1]],
                                                    axis=1))]
        out[nch] = {"plan": p, "maxshift": ms, "init": init, "regs": regs, "full": full}
    return out


def serve_run(args, algo, wl, speed, blocks_per_beam, seed=12):
    """The serving form on the workload: 64 beams, blocks arriving per beam as Poisson streams
    at speed x (1.0-1.5x) real time (speed inf: all at once), continuous batching on one GPU.
    Returns throughput, latency percentiles and each block's candidates."""
    import threading

    from mdsm_gb300.serving import Server
    nbeams = args.serve_beams
    block_s = SERVE_NSAMP * TSAMP
    srv = Server(hbm_budget_bytes=200 << 30, host_stage_bytes=24 << 30,
                 max_inflight=args.serve_slots, nwidths=9, threshold=6.0, cand_cap=4096)
    beams = []
    for b in range(nbeams):
        nch = serve_nchans(b)
        if algo == "subband":
            bid = srv.add_beam_subband(nch, FCH1, -BW / nch, TSAMP, SERVE_NSAMP,
                                       **serve_plan_args(algo, nch))
        else:
            bid = srv.add_beam(nch, FCH1, -BW / nch, TSAMP, SERVE_NSAMP, SEGMENTS)
        beams.append((bid, nch, srv.beam_info(bid)))
    rng = np.random.default_rng(seed)
    rate = rng.uniform(1.0, 1.5, nbeams) * speed
    order = []
    for b in range(nbeams):
        t = rng.exponential(block_s / rate[b]) * 0.1 if np.isfinite(rate[b]) else 0.0
        for k in range(blocks_per_beam):
            order.append((t, b, k))
            t += rng.exponential(block_s / rate[b]) if np.isfinite(rate[b]) else 0.0
    order.sort()
    got = []

    def consumer():
        while len(got) < len(order):
            r = srv.poll(wait_ms=50)
            if r is not None:
                got.append(r)

    th = threading.Thread(target=consumer)
    th.start()
    t0 = time.perf_counter()
    deferred = 0
    for t, b, k in order:
        now = time.perf_counter() - t0
        if np.isfinite(t) and t > now:
            time.sleep(t - now)
        bid, nch, info = beams[b]
        blk = wl[nch]["init"] if k == 0 else wl[nch]["regs"][k % 2]
        while srv.submit(bid, blk) is None:
            deferred += 1
            time.sleep(0.002)
    th.join()
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    beam_of = {beams[b][0]: b for b in range(nbeams)}
    units = sum(beams[b][2].ndms * SERVE_NSAMP for _, b, _ in order)
    adds = sum(block_adds(algo, beams[b][1], SERVE_NSAMP) for _, b, _ in order)
    offered_rtf = float(np.sum(rate)) if np.all(np.isfinite(rate)) else None
    return {"value": units / wall, "unit": METRIC, "blocks": len(order), "wall_s": wall,
            "real_time_factor": len(order) * block_s / wall,
            "offered_real_time_factor": offered_rtf,
            "p50_s": st["p50_latency_s"], "p99_s": st["p99_latency_s"],
            "max_s": st["max_latency_s"], "deferred_submits": deferred,
            "add_rate_tadd_s": adds / wall / 1e12,
            "cands": {(beam_of[r["beam"]], r["block"]): r["cands"] for r in got}}


def serve_plain(args, algo, wl, blocks_per_beam, series_out=True):
    """The plain per-block path on the same blocks and detector: one block at a time on one
    stream, as the reference's worker processes a block (src/mdsm/dedispersion_thread.cu:
    284-355): the whole block (tail included) copied in from pinned host memory, dedispersed,
    boxcar-searched on the device, and (series_out) the dedispersed series copied out to
    pinned host memory, as the reference hands its output buffer to its detector thread; then
    the candidates read back before the next block starts."""
    import torch

    import mdsm_gb300 as m
    nbeams = args.serve_beams
    block_s = SERVE_NSAMP * TSAMP
    st = torch.cuda.Stream()
    bufs = {}
    for nch, w in wl.items():
        p = w["plan"]
        i = p.info
        hs = [torch.from_numpy(a).pin_memory() for a in w["full"]]
        h_out = torch.empty((i.ndms, SERVE_NSAMP), dtype=torch.int32, pin_memory=True)
        bufs[nch] = (hs, p.alloc_input(), p.alloc_output(), h_out)

    def one(nch, k):
        p = wl[nch]["plan"]
        hs, d_in, d_out, h_out = bufs[nch]
        i = p.info
        h = hs[k] if k < 2 else hs[2 + (k % 2)]  # the block layouts of serve_workload
        with torch.cuda.stream(st):
            d_in[: nch * i.in_stride].view(nch, i.in_stride)[:, : SERVE_NSAMP + i.maxshift].copy_(
                h, non_blocking=True)
        p.dedisperse_device(d_in, d_out, stream=st)
        if series_out:
            with torch.cuda.stream(st):
                h_out.copy_(d_out.view(i.ndms, SERVE_NSAMP), non_blocking=True)
        return m.boxcar_detect_device(d_out.view(i.ndms, SERVE_NSAMP), nwidths=9, threshold=6.0,
                                      cap=4096, stream=st)

    for k in range(3):
        one(4096, k)
    torch.cuda.synchronize()
    order = [(b, k) for k in range(blocks_per_beam) for b in range(nbeams)]
    t0 = time.perf_counter()
    cands = {}
    units = 0
    for b, k in order:
        nch = serve_nchans(b)
        c, _ = one(nch, k)
        cands[(b, k)] = c
        units += wl[nch]["plan"].info.ndms * SERVE_NSAMP
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    return {"value": units / wall, "unit": METRIC, "blocks": len(order), "wall_s": wall,
            "real_time_factor": len(order) * block_s / wall,
            "ms_per_block": wall * 1e3 / len(order), "series_out": series_out, "cands": cands}


def serve_roofline(wl, pk, pk_kind, sm_count):
    """Per-stage launch times of one 4096-channel block through the subband plan (CUDA events
    on the launching stream) and the add rate of the dominant stage, the first subband stage."""
    import torch
    p = wl[4096]["plan"]
    i = p.info
    d_in, d_out = p.alloc_input(), p.alloc_output()
    st = torch.cuda.Stream()
    p.set_stage_timing(True)
    for _ in range(3):
        p.dedisperse_device(d_in, d_out, stream=st)
    ms = p.stage_times()
    p.set_stage_timing(False)
    passes = serve_passes(4096)
    nsubs = 64
    s1 = sum(pp["ncalls"] * 4096 * SERVE_NSAMP for pp in passes)
    s2 = sum(pp["ncalls"] * pp["calldms"] * nsubs * SERVE_NSAMP for pp in passes)
    t1, t2 = sum(ms[0::2]), sum(ms[1::2])
    peak = sm_count * 128 * pk.get("sm_max_mhz", 2070.0) * 1e6
    return {"bound": "alu", "kernel": "k_shift_sum_packed<uint8> (first subband stage)",
            "achieved": s1 / (t1 / 1e3) / 1e12, "peak": peak / 1e12, "unit": "Tadd/s",
            "frac": s1 / (t1 / 1e3) / peak, "traffic": None,
            "peak_source": "%d SMs x 128 lanes x sm_max_mhz (%s)" % (sm_count, pk_kind),
            "per_launch_ms": ms, "stage1_ms": t1, "stage2_ms": t2,
            "stage2_tadd_s": s2 / (t2 / 1e3) / 1e12,
            "algorithmic_adds_per_block": {"stage1": s1, "stage2": s2}}


def same_cands(a, b):
    if a.shape != b.shape:
        return False
    return all(np.array_equal(a[f], b[f]) for f in ("dm_idx", "sample", "width")) and \
        np.array_equal(a["snr"].view(np.uint32), b["snr"].view(np.uint32))


def serving_object(args, local=0):
    """The serving form on the 64-beam workload: saturating throughput and latency for the
    subband and brute-force algorithms, each against the plain per-block path on the same
    blocks (same algorithm, same detector: detections compared block by block), plus a run at
    Poisson arrivals of 1.0-1.5x real time for the latency a keeping-up server gives."""
    import torch
    pk, pk_kind = peaks()
    sm_count = torch.cuda.get_device_properties(local).multi_processor_count
    out = {"workload": "serving: %d beams (every tenth at 1024 ch, the rest 4096) x 2^16-sample "
                       "uint8 blocks x 4096 DM trials 0-2000, boxcar search over widths 1..256 "
                       "at 6 sigma" % args.serve_beams,
           "data": "seeded Gaussian uint8 (mean 128, sigma 16) with two dispersed pulses per "
                   "block (SNR 10-40), generated on the device",
           "slots": args.serve_slots}
    with ClockSampler(local) as clk:
        for algo, nblk in (("subband", args.serve_blocks), ("brute", args.serve_blocks_brute)):
            if nblk <= 0:
                continue
            wl = serve_workload(algo)
            # the plain runs first: their untimed first blocks load every kernel of the path
            plain = serve_plain(args, algo, wl, nblk, series_out=True)
            plain_c = serve_plain(args, algo, wl, nblk, series_out=False)
            sat = serve_run(args, algo, wl, float("inf"), nblk)
            ident = all(same_cands(sat["cands"][key], plain["cands"][key])
                        for key in plain["cands"])
            res = {k: v for k, v in sat.items() if k != "cands"}
            res["plain"] = {k: v for k, v in plain.items() if k != "cands"}
            res["plain_candidates_only"] = {k: v for k, v in plain_c.items() if k != "cands"}
            res["vs_plain"] = sat["value"] / plain["value"]
            res["vs_plain_candidates_only"] = sat["value"] / plain_c["value"]
            res["detections_identical_to_plain"] = bool(ident)
            res["candidates"] = int(sum(len(c) for c in sat["cands"].values()))
            if algo == "subband":
                out["roofline"] = serve_roofline(wl, pk, pk_kind, sm_count)
                if args.serve_paced:
                    paced = serve_run(args, algo, wl, 1.0, nblk, seed=13)
                    res["paced"] = {k: v for k, v in paced.items() if k != "cands"}
                    # keeping up: every block done well inside one block's duration (4.19 s)
                    res["paced"]["kept_up"] = bool(paced["p99_s"] < SERVE_NSAMP * TSAMP)
            out[algo] = res
            del wl
            torch.cuda.empty_cache()
    out["clocks"] = clk.summary()
    return out


def batch_workload(nbeams, seed=4):
    """Config 4's beams: 2^14..2^18 samples, 1024 or 4096 channels, 1024-4096 DM trials (in
    32s) to 500-2000, Gaussian uint8 (mean 128, sigma 16) with two dispersed pulses each,
    generated on the device.  Returns [(plan, host copy of the block)]."""
    import torch

    import mdsm_gb300 as m
    from mdsm_gb300 import synth
    rng = np.random.default_rng(seed)
    g = torch.Generator(device="cuda")
    g.manual_seed(seed + 3)
    out = []
    for b in range(nbeams):
        nsamp = 1 << int(rng.integers(14, 19))
        nch = int(rng.choice([1024, 4096]))
        ndms = int(rng.integers(32, 129)) * 32
        maxdm = float(rng.uniform(500, 2000))
        p = m.BrutePlan(nch, FCH1, -BW / nch, TSAMP, nsamp, [(0.0, maxdm / ndms, ndms)],
                        in_dtype="u8", out_dtype="i32")
        i = p.info
        ncols = nsamp + i.maxshift
        v = torch.empty((nch, i.in_stride), device="cuda")
        v.normal_(128.0, 16.0, generator=g)
        for t0, dm, w, amp in synth.random_pulses(rng, 2, nsamp - 64, 0.9 * maxdm, 16.0, nch,
                                                  widths=(1, 32), snr=(15, 40)):
            dl = synth.pulse_delays(nch, FCH1, -BW / nch, TSAMP, dm)
            idx = torch.from_numpy((t0 + dl)[:, None] + np.arange(w)[None, :]).cuda()
            v.scatter_add_(1, idx.clamp(max=ncols - 1),
                           torch.full(idx.shape, float(amp), device="cuda"))
        x = torch.clamp(torch.round(v), 0, 255).to(torch.uint8).cpu().numpy()
        del v
        out.append((p, x))
    return out


def tune_label(choice):
    """A readable name for an autotuner choice of the batched form."""
    from mdsm_gb300.batch import choice_info
    i = choice_info(choice)
    if i["fused"]:
        return "fused %dx%d %s" % (i["dm_block"], i["time_tile"],
                                   ("tile-major", "block-major")[i["order"]])
    return ("unfused persistent tile-major", "unfused persistent block-major",
            "unfused per beam")[i["order"]]


def batch_object(args, local=0):
    """The batched form on config 4: the beams' clip, dedispersion and boxcar search as one
    pass (the fused persistent launch where the beams allow it) replayed as a CUDA graph, with
    the launch shape the autotuner picks; against the plain per-beam path on the same blocks
    (clip, dedispersion, search and candidates back, one beam after another), detections
    compared beam by beam."""
    import torch

    import mdsm_gb300 as m
    from mdsm_gb300.batch import Batch, choice_info
    beams = batch_workload(args.batch_beams)
    plans = [p for p, _ in beams]
    d_in = [p.alloc_input() for p in plans]
    d_out = [p.alloc_output() for p in plans]

    def load_inputs():
        for (p, x), t in zip(beams, d_in):
            t[: x.size].copy_(torch.from_numpy(x.ravel()))

    batch = Batch(plans)
    batch.set_buffers(d_in, d_out)
    batch.enable_clip(4.0, 4.0)
    batch.enable_detect(nwidths=9, threshold=6.0, cap=4096)
    load_inputs()
    choice = batch.autotune()
    stream = torch.cuda.current_stream()
    # detections of one pass on fresh inputs
    load_inputs()
    batch.run(graph=True)  # (runs and captures)
    torch.cuda.synchronize()
    bc = [batch.candidates(k) for k in range(len(plans))]
    units = sum(p.info.ndms * p.info.nsamp for p in plans)
    data_s = sum(p.info.nsamp * TSAMP for p in plans)

    def plain_pass():
        cands = []
        for p, t, o in zip(plans, d_in, d_out):
            i = p.info
            m.rfi_clip_device(t, i.nchans, i.in_stride, i.nsamp + i.maxshift, 4.0, 4.0,
                              dtype="u8", stream=stream)
            p.dedisperse_device(t, o, stream=stream)
            cands.append(m.boxcar_detect_device(o, nwidths=9, threshold=6.0, cap=4096,
                                                stream=stream)[0])
        return cands

    load_inputs()
    pc = plain_pass()
    ident = all(same_cands(a, b) for a, b in zip(bc, pc))
    res = {"workload": "batched: %d beams, 2^14-2^18 samples, 1024/4096 ch, 1024-4096 DM trials "
                       "to 500-2000, uint8, RFI clip 4 sigma + dedispersion + boxcar widths "
                       "1..256 at 6 sigma" % len(plans),
           "data": "seeded Gaussian uint8 (mean 128, sigma 16) with two dispersed pulses per "
                   "beam, generated on the device",
           "autotune_choice": choice_info(choice),
           # every candidate the autotuner timed (search on, clip off): ms per pass
           "autotune_ms": {tune_label(c): round(t, 2) for c, t in batch.tune_times()},
           "detections_identical_to_plain": bool(ident),
           "candidates": int(sum(len(c) for c in bc))}
    with ClockSampler(local) as clk:
        for _ in range(args.warmup):
            batch.run(graph=True)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            batch.run(graph=True)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        plain_pass()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(max(1, args.steps // 2)):
            plain_pass()
        torch.cuda.synchronize()
        plain_ms = (time.perf_counter() - t0) * 1e3 / max(1, args.steps // 2)
    res.update({"value": units / (ms / 1e3), "unit": METRIC, "ms_per_pass": ms,
                "real_time_factor": data_s / (ms / 1e3), "launches_per_pass": batch.last_launches,
                "plain": {"value": units / (plain_ms / 1e3), "ms_per_pass": plain_ms,
                          # per beam: two clips, the dedispersion, statistics and search
                          "launches_per_pass": 5 * len(plans)},
                "vs_plain": plain_ms / ms, "clocks": clk.summary()})
    batch.close()
    return res


def run_batch(args):
    """The batched form alone (config 4), as its own JSON line."""
    import torch
    torch.cuda.set_device(0)
    print(json.dumps({"batched": batch_object(args)}), flush=True)


def run_boxcar(args):
    """The boxcar search alone (mdsm_boxcar_detect_device: exact row statistics, then the
    search over widths 1..256 at 6 sigma) on an int32 series of 4096 DM trials x 2^16 samples
    (1.07 GB > L2): Gaussian sums (mean 128 x 4096, sigma 16 x 64) with two injected pulses,
    generated on the device.  Per call the series is read twice (statistics, search)."""
    import torch

    import mdsm_gb300 as m
    torch.cuda.set_device(0)
    ndms, n = 4096, 1 << 16
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    y = torch.empty((ndms, n), device="cuda").normal_(128.0 * 4096, 16.0 * 64, generator=g)
    y = y.round_().to(torch.int32)
    y[100, 5000:5008] += 40000
    y[3000, 60000:60100] += 9000
    st = torch.cuda.current_stream()
    for _ in range(args.warmup):
        cands, k = m.boxcar_detect_device(y, nwidths=9, threshold=6.0, cap=4096, stream=st)
    torch.cuda.synchronize()
    with ClockSampler(0) as clk:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(args.steps):
            cands, k = m.boxcar_detect_device(y, nwidths=9, threshold=6.0, cap=4096, stream=st)
        e1.record(st)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    pk, src = peaks()
    gbs = 2 * 4.0 * ndms * n / (ms / 1e3) / 1e9
    print(json.dumps({
        "metric": METRIC, "value": ndms * n / (ms / 1e3), "unit": METRIC, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "dtype": "f32 (int32 series)", "data": "synthetic",
        "config": {"workload": "boxcar search: int32 series 4096 DM trials x 2^16 samples, "
                               "widths 1..256, threshold 6 sigma, statistics included",
                   "l2": "inputs larger than L2"},
        "candidates": int(k),
        "roofline_hbm": {"bound": "hbm", "achieved": gbs, "peak": pk.get("hbm_gbs"),
                         "unit": "GB/s", "frac": gbs / pk.get("hbm_gbs", 6800.0),
                         "algorithmic_bytes_per_call": 2 * 4 * ndms * n, "peak_source": src},
        "clocks": clk.summary()}), flush=True)


def run_stage(args):
    """The reference's stage interface (processSurveyParameters, initialiseMDSM, next_chunk,
    start_processing, tearDownMDSM) driven as src/MDSM.cpp drives it: float blocks of 8-bit
    samples (as its file reader fills them; they take the 8-bit kernels) and, for comparison,
    the same blocks with fractional values (the float kernels).  Wall time per block with the
    caller's buffer fill inside the loop; brute force, 4096 ch x 2^16 samples x 1024 DM trials
    0-250, process_brute detection."""
    import tempfile

    from mdsm_gb300 import compat
    nch, nsamp, ndms, step = 4096, 1 << 16, 1024, 0.244140625
    xml = ("<observation><frequencies top=\"%.1f\" offset=\"%.10f\" />"
           "<dm lowDM=\"0\" numDMs=\"%d\" dmStep=\"%.9f\" useBruteForce=\"1\" useL1Cache=\"1\" />"
           "<samples number=\"%d\" /><channels number=\"%d\" subbands=\"64\" />"
           "<timing tsamp=\"%g\" /><detection threshold=\"6\" />"
           "<output filePrefix=\"stage\" baseDirectory=\"%s\" secondsPerFile=\"600\" "
           "usePCTime=\"0\" singleFileMode=\"1\" /><gpus ids=\"0\" /></observation>")
    out = {}
    with tempfile.TemporaryDirectory() as d:
        obs = os.path.join(d, "obs.xml")
        with open(obs, "w") as f:
            f.write(xml % (FCH1, -BW / nch, ndms, step, nsamp, nch, TSAMP, d))
        for kind in ("8bit", "float"):
            survey = compat.processSurveyParameters(obs)
            buf = compat.initialiseMDSM(survey)
            ms = survey.contents.maxshift
            rng = np.random.default_rng(5)
            src = rng.integers(96, 160, buf.shape).astype(np.float32)
            if kind == "float":
                src += 0.25
            buf[:] = src
            times = []
            nblocks = args.warmup + args.steps
            for k in range(nblocks):
                t0 = time.perf_counter()
                if k:
                    buf[:, ms:] = src[:, ms:]  # the caller's read of the next block
                compat.next_chunk(nsamp, k * nsamp * TSAMP, TSAMP)
                compat.start_processing(nsamp)
                times.append(time.perf_counter() - t0)
            compat.next_chunk(0, nblocks * nsamp * TSAMP, TSAMP)
            n8 = compat.blocks_8bit()
            compat.tearDownMDSM()
            per = float(np.mean(times[args.warmup:]))
            out[kind] = {"value": ndms * nsamp / per, "ms_per_block": per * 1e3,
                         "blocks_on_8bit_kernels": int(n8)}
    line = {"metric": METRIC, "value": out["8bit"]["value"], "unit": METRIC, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": out["8bit"]["ms_per_block"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "float32 in, int32 sums",
            "data": "synthetic 8-bit samples (uniform 96-159) handed in as float32",
            "config": {"workload": "stage interface (next_chunk / start_processing), brute force "
                                   "4096 ch x 2^16 samples x 1024 DM trials 0-250, "
                                   "process_brute detection, caller fill in the loop"},
            "real_time_factor": nsamp * TSAMP / (out["8bit"]["ms_per_block"] / 1e3),
            "blocks_on_8bit_kernels": out["8bit"]["blocks_on_8bit_kernels"],
            "fractional_floats": out["float"]}
    print(json.dumps(line), flush=True)


def run_precision(args):
    """Precision report: INT32 and FP32 accumulation against the FP64 oracle, per sample type
    (uint8 mean 128 sigma 16, int16 sigma 1000, float32 N(0,1)), 4096 channels, 64 DM trials;
    and uint16 over 40000 channels, where INT32 sums could overflow and the automatic mode
    takes FP32."""
    import torch

    import mdsm_gb300 as m
    from mdsm_gb300 import synth
    from oracle import oracle as orc
    orc.build(reference=False)
    out = {}
    nchans, nsamp, segs = 4096, 4096, [(0.0, 0.5, 64)]
    for dtype in ("u8", "i16", "f32"):
        accs = ("i32", "f32") if dtype != "f32" else ("f32",)
        res = {}
        for acc in accs:
            plan = m.BrutePlan(nchans, FCH1, -BW / nchans, TSAMP, nsamp, segs, in_dtype=dtype,
                               out_dtype="i32" if acc == "i32" else "f32", acc=acc)
            nch, stride = plan.input_shape()
            if dtype == "u8":
                x = synth.gaussian_u8(nch, stride, 1)
            elif dtype == "i16":
                x = synth.gaussian_i16(nch, stride, 1)
            else:
                x = synth.gaussian_f32(nch, stride, 1)
            d_in = plan.alloc_input()
            d_in[: x.size].copy_(torch.from_numpy(x.ravel()))
            d_out = plan.alloc_output()
            plan.dedisperse_device(d_in, d_out)
            torch.cuda.synchronize()
            y = d_out.cpu().numpy().astype(np.float64)
            S = plan.shift_table()
            xf = x.astype(np.float32)
            y64 = orc.dedisperse(xf, S, nsamp, out="f64")
            scale = orc.dedisperse(np.abs(xf), S, nsamp, out="f64")
            err = np.abs(y - y64)
            res[acc] = {"max_abs": float(err.max()),
                        "max_rel_sum_abs": float((err / np.maximum(scale, 1e-30)).max()),
                        "max_rel_value": float((err / np.maximum(np.abs(y64), 1.0)).max()),
                        "exact": bool(err.max() == 0.0)}
        out[dtype] = res
    # uint16 samples over 40000 channels: sums reach 2.6e9 > 2^31, so the automatic mode
    # accumulates in FP32 (exact INT32 sums per 16 channels, Kahan-compensated across them)
    nch16, ns16, segs16 = 40000, 1024, [(0.0, 0.01, 8)]
    plan = m.BrutePlan(nch16, FCH1, -BW / nch16, TSAMP, ns16, segs16, in_dtype="u16",
                       out_dtype="f32")
    nch, stride = plan.input_shape()
    x = np.random.default_rng(3).integers(0, 65536, (nch, stride), dtype=np.uint16)
    d_in = plan.alloc_input()
    d_in[: x.size].copy_(torch.from_numpy(x.ravel()))
    d_out = plan.alloc_output()
    plan.dedisperse_device(d_in, d_out)
    torch.cuda.synchronize()
    y = d_out.cpu().numpy().astype(np.float64)
    xf = x.astype(np.float32)
    y64 = orc.dedisperse(xf, plan.shift_table(), ns16, out="f64")
    err = np.abs(y - y64)
    out["u16_40000ch_auto"] = {"acc": "f32" if plan.info.acc == 2 else "i32",
                               "max_abs": float(err.max()),
                               "max_rel_value": float((err / np.maximum(np.abs(y64), 1.0)).max()),
                               "max_sum": float(y64.max())}
    print(json.dumps({"precision": out, "config": {"nchans": nchans, "nsamp": nsamp,
                                                   "ndms": 64}}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--case", default="full",
                    choices=["full", "small", "serve", "batch", "precision", "stage", "boxcar"],
                    help="small: 2048 ch x 2^16 samples x 512 DM trials (profiling case); "
                         "serve: the multi-beam serving form")
    ap.add_argument("--algo", default="subband", choices=["subband", "brute"])
    ap.add_argument("--serve-beams", type=int, default=64)
    ap.add_argument("--serve-blocks", type=int, default=3,
                    help="blocks per beam of the subband serving runs")
    ap.add_argument("--serve-blocks-brute", type=int, default=2,
                    help="blocks per beam of the brute-force serving runs (0: skip)")
    ap.add_argument("--serve-paced", type=int, default=1,
                    help="1: also a run at Poisson arrivals of 1.0-1.5x real time")
    ap.add_argument("--no-serving", action="store_true",
                    help="leave the serving object out of the default line")
    ap.add_argument("--serve-slots", type=int, default=4)
    ap.add_argument("--batch-beams", type=int, default=32)
    ap.add_argument("--kernel", default="auto", choices=["auto", "generic"],
                    help="plain path: the plan's own kernel choice, or the generic kernel "
                         "(profiling comparisons)")
    ap.add_argument("--no-batched", action="store_true",
                    help="leave the batched object out of the default line")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.case == "serve":
        import torch
        torch.cuda.set_device(0)
        print(json.dumps({"serving": serving_object(args)}), flush=True)
        return
    if args.case == "batch":
        return run_batch(args)
    if args.case == "precision":
        return run_precision(args)
    if args.case == "stage":
        return run_stage(args)
    if args.case == "boxcar":
        return run_boxcar(args)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch
    import torch.distributed as dist

    import mdsm_gb300 as m

    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if world > 1:
            dist.barrier()

    global NCHANS, NSAMP, SEGMENTS, WORKLOAD
    if args.case == "small":
        NCHANS, NSAMP = 2048, 1 << 16
        SEGMENTS = [(0.0, 0.9765625, 512)]
        WORKLOAD = ("profiling case: uint8 2048 ch x 2^16 samples, 512 DM trials 0-500, INT32 "
                    "accumulation (input 168 MB > L2)")
    plan = m.BrutePlan(NCHANS, FCH1, -BW / NCHANS, TSAMP, NSAMP, SEGMENTS, shift_mode="l1",
                       in_dtype="u8", out_dtype="i32",
                       kernel=1 if args.kernel == "generic" else 0)
    info = plan.info
    stream = torch.cuda.Stream()
    gen = torch.Generator(device="cuda")
    gen.manual_seed(1234 + rank)
    d_in = plan.alloc_input()
    nrow = info.nchans * info.in_stride
    with torch.cuda.stream(stream):
        v = torch.randn(nrow, generator=gen, device="cuda", dtype=torch.float32)
        d_in[:nrow].copy_(torch.clamp(torch.round(v * 16 + 128), 0, 255).to(torch.uint8))
        del v
    d_out = plan.alloc_output()
    stream.synchronize()

    # ---- device-resident timing ----
    for _ in range(args.warmup):
        plan.dedisperse_device(d_in, d_out, stream=stream)
    stream.synchronize()
    barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    launches = 0
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        barrier()
        t_start = torch.cuda.Event(enable_timing=True)
        t_end = torch.cuda.Event(enable_timing=True)
        t_start.record(stream)
        for k in range(args.steps):
            ev[k][0].record(stream)
            plan.dedisperse_device(d_in, d_out, stream=stream)
            ev[k][1].record(stream)
            launches += plan.last_launches
        t_end.record(stream)
        torch.cuda.synchronize()
        barrier()
    total_ms = t_start.elapsed_time(t_end)
    if world > 1:
        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    per_launch_ms = float(np.mean([a.elapsed_time(b) for a, b in ev]))
    ms_step = total_ms / args.steps
    units = info.ndms * info.nsamp
    value = units * world / (ms_step / 1e3)

    # ---- end to end through the host-buffer C-ABI call ----
    h_in = torch.empty((info.nchans, info.nsamp + info.maxshift), dtype=torch.uint8,
                       pin_memory=True)
    h_in.copy_(d_in[: info.nchans * info.in_stride].view(info.nchans, info.in_stride)
               [:, : info.nsamp + info.maxshift].cpu())
    h_out = torch.empty((info.ndms, info.nsamp), dtype=torch.int32, pin_memory=True)
    hin_np, hout_np = h_in.numpy(), h_out.numpy()
    plan.dedisperse_host(hin_np, hout_np, stream=stream)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        plan.dedisperse_host(hin_np, hout_np, stream=stream)
    e2e_s = (time.perf_counter() - t0) / args.e2e_steps
    if world > 1:
        t = torch.tensor([e2e_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_val = units * world / e2e_s

    pk, pk_kind = peaks()
    sm_count = torch.cuda.get_device_properties(local).multi_processor_count
    add_peak = sm_count * 128 * pk.get("sm_max_mhz", 2070.0) * 1e6
    ops = float(info.ndms) * info.nsamp * info.nchans
    achieved_ops = ops / (per_launch_ms / 1e3)
    alg_bytes = info.nchans * (info.nsamp + info.maxshift) * 1 + info.ndms * info.nsamp * 4
    hbm_achieved = alg_bytes / (per_launch_ms / 1e3) / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic.txt")
    key = "packed" if info.kernel == 2 else "generic"
    if os.path.exists(tp):
        for ln in open(tp):
            parts = ln.split()
            if len(parts) == 2 and parts[0] == key + "_traffic_over_algorithmic":
                traffic = float(parts[1]) * alg_bytes
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded Gaussian uint8 on the device; block input 1.2 GB > L2)",
        "config": {"workload": WORKLOAD, "nchans": NCHANS, "nsamp": info.nsamp,
                   "ndms": info.ndms, "maxshift": info.maxshift, "in": "u8", "out": "i32",
                   "dm_block": info.dm_block, "time_tile": info.time_tile,
                   "l2": "inputs larger than L2", "parallelism": "beam-per-rank" if world > 1
                   else "single GPU"},
        "real_time_factor": (info.nsamp * TSAMP) * world / (ms_step / 1e3),
        "e2e": {"value": e2e_val, "unit": METRIC,
                "h2d_bytes_per_step": int(info.nchans * (info.nsamp + info.maxshift)),
                "d2h_bytes_per_step": int(info.ndms * info.nsamp * 4),
                "ms_per_step": e2e_s * 1e3},
        "roofline": {"bound": "alu", "achieved": achieved_ops / 1e12,
                     "peak": add_peak / 1e12, "unit": "Tadd/s",
                     "frac": achieved_ops / add_peak, "traffic": traffic,
                     "peak_source": "%d SMs x 128 lanes x sm_max_mhz (%s)" % (sm_count, pk_kind),
                     "kernel": {2: "k_shift_sum_packed<uint8>", 3: "k_shift_sum_packed<uint16>"}
                     .get(info.kernel, "k_shift_sum"),
                     "per_launch_ms": per_launch_ms,
                     "algorithmic_adds_per_launch": ops},
        "roofline_hbm": {"bound": "hbm", "achieved": hbm_achieved, "peak": pk.get("hbm_gbs"),
                         "unit": "GB/s", "frac": hbm_achieved / pk.get("hbm_gbs", 6800.0),
                         "algorithmic_bytes_per_launch": alg_bytes, "peak_source": pk_kind},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import oracle as orc
        orc.build(reference=False)
        line["cpu_baseline"] = cpu_baseline(orc)
    if world == 1 and args.case == "full" and not args.no_serving:
        del d_in, d_out, h_in, h_out, hin_np, hout_np
        plan = None
        torch.cuda.empty_cache()
        line["serving"] = serving_object(args, local)
        torch.cuda.empty_cache()
    if world == 1 and args.case == "full" and not args.no_batched:
        line["batched"] = batch_object(args, local)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
