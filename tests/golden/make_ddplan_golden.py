"""Golden plans from the reference's own DM planner (python/ddplan.py of the MDSM tree).

The planner is Python 2 (print statements) and imports an `elementtree` module it never uses
on this path.  This script reads the source where it lies, turns its print statements into
print() calls in memory (the usage() text, never called here, is dropped), restores the
builtins that a modern `from numpy import *` shadows, stubs `elementtree`, runs calculateParams() for a set of observations and writes each method's
fields to tests/golden/ddplan.json.  Nothing of the reference is copied.

Usage:  python tests/golden/make_ddplan_golden.py   (needs the MDSM source tree)
"""
import io
import json
import os
import re
import sys
import types
from contextlib import redirect_stdout

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = "/root/reference/python/ddplan.py"

CASES = [  # loDM, hiDM, fctr, BW, numchan, numsubbands, dt, ok_smearing
    (0.0, 1000.0, 1400.0, 300.0, 1024, 0, 0.000064, 0.0),
    (0.0, 1000.0, 1400.0, 300.0, 1024, 32, 0.000064, 0.0),
    (0.0, 2000.0, 1350.0, 300.0, 4096, 64, 0.000064, 0.0),
    (0.0, 500.0, 150.0, 6.0, 256, 16, 0.0000512, 0.0),
    (10.0, 300.0, 800.0, 200.0, 2048, 128, 0.0001, 0.5),
]


def load_reference():
    src = open(SRC).read()
    src = re.sub(r"def usage\(\):.*?(?=\nif __name__)", "def usage():\n    pass\n", src,
                 flags=re.S)
    src = re.sub(r"^(\s*)print (.*)$", r"\1print(\2)", src, flags=re.M)
    # numpy of the planner's era exported neither min/max nor pow from `import *`; today's
    # does, so the builtins and math.pow the planner was written against are put back
    src = src.replace("from numpy import *",
                      "from numpy import *\nfrom builtins import min, max\nfrom math import pow", 1)
    et = types.ModuleType("elementtree")
    et.ElementTree = types.ModuleType("elementtree.ElementTree")
    sys.modules["elementtree"] = et
    sys.modules["elementtree.ElementTree"] = et.ElementTree
    ns = {"__name__": "ddplan_reference"}
    exec(compile(src, SRC, "exec"), ns)
    return ns


def main():
    ns = load_reference()
    out = []
    for case in CASES:
        with redirect_stdout(io.StringIO()):
            methods = ns["calculateParams"](*case)
        rows = []
        for m in methods:
            rows.append([m.loDM, m.hiDM, m.dDM, m.downsamp, m.dsubDM, m.numDMs,
                         getattr(m, "DMs_per_prepsub", 0) if m.numsub else 0, m.numprepsub])
        out.append({"case": list(case), "methods": rows})
    with open(os.path.join(HERE, "ddplan.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote ddplan.json: %d cases" % len(out))


if __name__ == "__main__":
    main()
