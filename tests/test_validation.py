"""Argument validation of the C ABI: refused before any device work, with the status and a
message in mdsm_last_error() (the reference exits the process instead, e.g.
dedispersion_manager.cpp:46-58)."""
import pytest

EINVAL, ERANGE = 1, 6


def _brute(**kw):
    import mdsm_gb300 as m
    a = dict(nchans=64, fch1=1500.0, foff=-1.0, tsamp=64e-6, nsamp=1000,
             segments=[(0.0, 1.0, 8)])
    a.update(kw)
    return m.BrutePlan(a.pop("nchans"), a.pop("fch1"), a.pop("foff"), a.pop("tsamp"),
                       a.pop("nsamp"), a.pop("segments"), **a)


@pytest.mark.parametrize("kw,status,msg", [
    (dict(nchans=0), EINVAL, "nchans"),
    (dict(nsamp=0), EINVAL, "nsamp"),
    (dict(segments=[]), EINVAL, "segments"),
    (dict(segments=[(0.0, 1.0, 0)]), EINVAL, "no DM trials"),
    (dict(tsamp=0.0), EINVAL, "tsamp"),
    (dict(in_dtype="f32", acc="i32"), EINVAL, "integer samples"),
    (dict(nchans=40000, foff=-0.0075, in_dtype="u16", out_dtype="i32", acc="i32"), ERANGE,
     "overflow"),
])
def test_brute_plan_refusals(lib, kw, status, msg):
    from mdsm_gb300 import MdsmError
    with pytest.raises(MdsmError) as e:
        _brute(**kw)
    assert e.value.status == status
    assert msg in str(e.value)


@pytest.mark.parametrize("kw,status,msg", [
    (dict(nchans=100, nsubs=16), EINVAL, "multiple of nsubs"),
    (dict(nsamp=1001, binsize=2), EINVAL, "multiple of each downsample"),
    (dict(ncalls=0), EINVAL, "positive"),
    (dict(nsubs=0), EINVAL, "nsubs"),
])
def test_subband_plan_refusals(lib, kw, status, msg):
    import mdsm_gb300 as m
    from mdsm_gb300 import MdsmError
    nchans = kw.pop("nchans", 256)
    nsubs = kw.pop("nsubs", 16)
    nsamp = kw.pop("nsamp", 1024)
    p = dict(lowdm=0.0, highdm=10.0, dmstep=0.5, sub_dmstep=2.0, ncalls=5, calldms=4)
    p.update(kw)
    with pytest.raises(MdsmError) as e:
        m.SubbandPlan(nchans, 1500.0, -300.0 / nchans, 64e-6, nsamp, nsubs, [p],
                      in_dtype="f32", out_dtype="f32")
    assert e.value.status == status
    assert msg in str(e.value)
