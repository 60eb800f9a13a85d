"""The DM planner restated in mdsm_gb300/ddplan.py against the reference planner's own plans
(tests/golden/ddplan.json, made by tests/golden/make_ddplan_golden.py from python/ddplan.py),
and its <passes> XML read back by the observation-file parser."""
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ddplan.json")


@pytest.mark.parametrize("k", range(5))
def test_plans_equal_reference(k):
    from mdsm_gb300 import ddplan
    g = json.load(open(GOLD))[k]
    lo, hi, fctr, bw, nchan, nsub, dt, ok = g["case"]
    got = [list(p.as_tuple()) for p in ddplan.plan(lo, hi, fctr, bw, nchan, nsub, dt, ok)]
    want = g["methods"]
    assert len(got) == len(want)
    for a, b in zip(got, want):
        assert a == b


def test_passes_xml_round_trip(lib, tmp_path):
    from mdsm_gb300 import compat, ddplan
    passes = ddplan.plan(0.0, 1000.0, 1400.0, 300.0, 1024, 32, 0.000064)
    xml = ("<observation>\n    <frequencies top=\"1550.0\" offset=\"-0.29296875\" />\n"
           "    <dm lowDM=\"0\" numDMs=\"0\" dmStep=\"0\" useBruteForce=\"0\" />\n"
           "    <channels number=\"1024\" subbands=\"32\" />\n"
           "    <timing tsamp=\"0.000064\" />\n" + ddplan.passes_xml(passes) +
           "\n</observation>\n")
    path = tmp_path / "obs.xml"
    path.write_text(xml)
    s = compat.processSurveyParameters(path).contents
    assert s.num_passes == len(passes)
    assert s.tdms == sum(p.numdms for p in passes)
    for i, p in enumerate(passes):
        q = s.pass_parameters[i]
        assert np.float32(q.lowdm) == np.float32(p.lo_dm)
        assert np.float32(q.highdm) == np.float32(p.hi_dm)
        assert np.float32(q.sub_dmstep) == np.float32(p.sub_dm)
        assert (q.binsize, q.ndms, q.calldms, q.ncalls) == (int(p.downsamp), p.numdms,
                                                            p.dms_per_call, p.ncalls)
    load = __import__("mdsm_gb300")._lib.load()
    load.mdsm_free_survey(compat.processSurveyParameters(path))


def test_algorithm_choice_by_adds():
    from mdsm_gb300 import ddplan
    passes = ddplan.plan(0.0, 1000.0, 1400.0, 300.0, 4096, 64, 0.000064)
    brute, sub = ddplan.adds_per_sample(passes, 4096, 64)
    # hand count from the pass fields
    assert brute == sum(p.numdms * 4096 / p.downsamp for p in passes)
    assert sub == sum((p.ncalls * 4096 + p.numdms * 64) / p.downsamp for p in passes)
    assert sub < brute
    assert ddplan.choose_algorithm(passes, 4096, 64) == "subband"
    # no subbands: brute force; a gain below the bar: brute force
    assert ddplan.choose_algorithm(ddplan.plan(0.0, 100.0, 1400.0, 300.0, 256, 0, 64e-6),
                                   256, 0) == "brute"
    assert ddplan.choose_algorithm(passes, 4096, 64, min_gain=brute / sub * 2) == "brute"
