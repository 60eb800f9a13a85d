"""DM plan generator: the smearing-balanced dedispersion plan of the reference's planner
(python/ddplan.py:6-312), restated, emitting the observation file's <passes> section in the
schema src/mdsm/dedispersion_manager.cpp:150-185 reads, and converting a plan into the
library's brute-force segments or subband passes.

All arithmetic is Python double, in the reference's order, so plans are identical.
"""
import math

# ddplan.py:178-179: allowed DM steps
ALLOWED_DM_STEPS = [0.0001, 0.0002, 0.0005, 0.001, 0.002, 0.005, 0.01, 0.02, 0.03, 0.05, 0.1,
                    0.2, 0.3, 0.5, 1.0, 2.0, 3.0, 5.0, 10.0, 20.0, 30.0, 50.0, 100.0, 200.0,
                    300.0, 500.0, 1000.0]
# ddplan.py:181: allowed downsampling factors
ALLOWED_DOWNSAMPS = [math.pow(2, i) for i in range(0, 20)]


def dm_smear(dm, bw, f_ctr):
    """Smearing (ms) of a DM over bw MHz centred at f_ctr MHz (ddplan.py:118-124)."""
    return 1000.0 * dm * bw / (0.0001205 * f_ctr ** 3.0)


def bw_smear(dmstep, bw, f_ctr):
    """Smearing (ms) from the worst DM error of a step (ddplan.py:126-133)."""
    return dm_smear(0.5 * dmstep, bw, f_ctr)


def guess_dmstep(dt, bw, f_ctr):
    """DM step whose smearing across the band equals dt (ddplan.py:135-141)."""
    return dt * 0.0001205 * f_ctr ** 3.0 / (0.5 * bw)


def subband_smear(sub_dmstep, numsub, bw, f_ctr):
    """ddplan.py:143-153."""
    if numsub == 0:
        return 0.0
    return dm_smear(0.5 * sub_dmstep, bw / numsub, f_ctr)


def total_smear(dm, dmstep, dt, f_ctr, bw, numchan, sub_dmstep, numsub=0):
    """ddplan.py:155-166."""
    return math.sqrt(2 * (1000.0 * dt) ** 2.0 + dm_smear(dm, bw / numchan, f_ctr) ** 2.0 +
                     subband_smear(sub_dmstep, numsub, bw, f_ctr) ** 2.0 +
                     bw_smear(dmstep, bw, f_ctr) ** 2.0)


class Observation:
    """ddplan.py:6-21."""

    def __init__(self, dt, f_ctr, bw, numchan):
        self.dt = dt
        self.f_ctr = f_ctr
        self.bw = bw
        self.numchan = numchan
        self.chanwidth = bw / numchan


class Pass:
    """One dedispersion method (ddplan.py:23-116): DMs [lo_dm, hi_dm) at step d_dm after
    downsampling by downsamp; with subbands, calls of dms_per_call fine DMs around sub-DMs
    spaced sub_dm."""

    def __init__(self, obs, downsamp, lo_dm, hi_dm, d_dm, numdms=0, numsub=0, smearfact=2.0):
        self.obs = obs
        self.downsamp = downsamp
        self.lo_dm = lo_dm
        self.d_dm = d_dm
        self.numsub = numsub
        self.bw_smearing = bw_smear(d_dm, obs.bw, obs.f_ctr)
        self.ncalls = 0
        self.dms_per_call = 0
        if numsub:
            per = 2
            while True:
                nxt = (per + 2) * d_dm
                ss = subband_smear(nxt, numsub, obs.bw, obs.f_ctr)
                if ss > 0.8 * min(self.bw_smearing, 1000.0 * obs.dt * downsamp):
                    self.sub_dm = per * d_dm
                    self.dms_per_call = per
                    self.sub_smearing = subband_smear(self.sub_dm, numsub, obs.bw, obs.f_ctr)
                    break
                per += 2
        else:
            self.sub_dm = d_dm
            self.sub_smearing = subband_smear(self.sub_dm, numsub, obs.bw, obs.f_ctr)
        cross = self.dm_for_smearfact(smearfact)
        if cross > hi_dm:
            cross = hi_dm
        if numdms == 0:
            self.numdms = int(math.ceil((cross - lo_dm) / d_dm))
            if numsub:
                self.ncalls = int(math.ceil(self.numdms * d_dm / self.sub_dm))
                self.numdms = self.ncalls * self.dms_per_call
        else:
            self.numdms = numdms
        self.hi_dm = lo_dm + self.numdms * d_dm

    def dm_for_smearfact(self, smearfact):
        """ddplan.py:86-95."""
        o = self.obs
        other = math.sqrt((1000.0 * o.dt) ** 2.0 + (1000.0 * o.dt * self.downsamp) ** 2.0 +
                          self.bw_smearing ** 2.0 + self.sub_smearing ** 2.0)
        return smearfact * 0.001 * other / o.chanwidth * 0.0001205 * o.f_ctr ** 3.0

    def dms(self):
        return [self.lo_dm + i * self.d_dm for i in range(self.numdms)]

    def as_tuple(self):
        return (self.lo_dm, self.hi_dm, self.d_dm, self.downsamp, self.sub_dm, self.numdms,
                self.dms_per_call, self.ncalls)


def plan(lo_dm, hi_dm, f_ctr, bw, numchan, numsub, dt, ok_smearing=0.0):
    """The passes covering [lo_dm, hi_dm) (ddplan.py:168-303, 305-312)."""
    obs = Observation(dt, f_ctr, bw, numchan)
    i_ds = i_dm = 0
    downsamp = ALLOWED_DOWNSAMPS[i_ds]
    d_dm = ALLOWED_DM_STEPS[i_dm]
    dtms = 1000.0 * obs.dt
    ff = 1.2
    min_chan = dm_smear(lo_dm + 0.5 * d_dm, obs.chanwidth, obs.f_ctr)
    min_bw = bw_smear(d_dm, obs.bw, obs.f_ctr)
    ok_smearing = max([ok_smearing, min_chan, min_bw, dtms])
    if ff * min_chan > dtms or ok_smearing > dtms:
        okval = ok_smearing if ok_smearing > ff * min_chan else ff * min_chan
        while dtms * ALLOWED_DOWNSAMPS[i_ds + 1] < okval:
            i_ds += 1
        downsamp = ALLOWED_DOWNSAMPS[i_ds]
    d_dm = guess_dmstep(obs.dt * downsamp, obs.bw, obs.f_ctr)
    while ALLOWED_DM_STEPS[i_dm + 1] < ff * d_dm:
        i_dm += 1
    passes = [Pass(obs, downsamp, lo_dm, hi_dm, ALLOWED_DM_STEPS[i_dm], numsub=numsub)]
    while passes[-1].hi_dm < hi_dm:
        i_ds += 1
        downsamp = ALLOWED_DOWNSAMPS[i_ds]
        eff_dt = dtms * downsamp
        while bw_smear(ALLOWED_DM_STEPS[i_dm + 1], obs.bw, obs.f_ctr) < ff * eff_dt:
            i_dm += 1
        passes.append(Pass(obs, downsamp, passes[-1].hi_dm, hi_dm, ALLOWED_DM_STEPS[i_dm],
                           numsub=numsub))
    return passes


def passes_xml(passes, indent="    "):
    """The <passes> section of an observation file (read by dedispersion_manager.cpp:150-185
    and by mdsm_processSurveyParameters)."""
    out = [indent + "<passes>"]
    for p in passes:
        out.append(indent * 2 + "<pass>")
        for tag, val in (("lowDm", p.lo_dm), ("highDm", p.hi_dm), ("deltaDm", p.d_dm),
                         ("downsample", int(p.downsamp)), ("subDm", p.sub_dm),
                         ("numDms", p.numdms), ("dmsPerCall", p.dms_per_call),
                         ("ncalls", p.ncalls)):
            out.append(indent * 3 + "<%s>%s</%s>" % (tag, repr(val) if isinstance(val, float)
                                                     else val, tag))
        out.append(indent * 2 + "</pass>")
    out.append(indent + "</passes>")
    return "\n".join(out)


def to_segments(passes):
    """Brute-force segments (lowdm, dmstep, ndms) of a plan, ignoring downsampling."""
    return [(p.lo_dm, p.d_dm, p.numdms) for p in passes]


def adds_per_sample(passes, numchan, numsub):
    """Adds per input time sample of a plan, brute force and subband (a pass with downsample b
    runs at 1/b of the rate).  Brute force: numdms * numchan.  Subband: stage 1 sums every
    channel once per sub-DM call, stage 2 sums numsub subbands per fine trial."""
    brute = sub = 0.0
    for p in passes:
        brute += p.numdms * numchan / p.downsamp
        sub += (p.ncalls * numchan + p.numdms * numsub) / p.downsamp
    return brute, sub


def choose_algorithm(passes, numchan, numsub, min_gain=1.5):
    """'subband' when the plan has subbands and its adds are at least min_gain times fewer than
    brute force's, else 'brute' (brute force has no subband smearing)."""
    if not numsub or any(not p.numsub for p in passes):
        return "brute"
    brute, sub = adds_per_sample(passes, numchan, numsub)
    return "subband" if brute >= min_gain * sub else "brute"


def to_subband_passes(passes):
    """Subband pass dicts for SubbandPlan; a pass with downsample b > 1 dedisperses the block
    summed over b samples."""
    out = []
    for p in passes:
        if not p.numsub:
            raise ValueError("plan made without subbands")
        out.append(dict(lowdm=p.lo_dm, highdm=p.hi_dm, dmstep=p.d_dm, sub_dmstep=p.sub_dm,
                        ncalls=p.ncalls, calldms=p.dms_per_call, ndms=p.numdms,
                        binsize=int(p.downsamp)))
    return out
