"""The C-ABI library loads and exports every symbol include/*.h declares; the SURVEY struct
and the other ABI structs have the C layout (checked against the C compiler's offsetof)."""
import ctypes
import os
import re
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")


def declared_functions():
    names = set()
    for fn in os.listdir(INC):
        if not fn.endswith(".h"):
            continue
        src = open(os.path.join(INC, fn)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        if "extern \"C\"" not in src and fn != "mdsm_gb300.h":
            continue
        for m in re.finditer(r"\b(mdsm_[A-Za-z0-9_]+|call_[A-Za-z0-9_]+|process_output)\s*\(",
                             src):
            names.add(m.group(1))
    return sorted(names)


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) > 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert {"call_dedisperse", "call_initialise_devices", "process_output"} <= set(names)
    from mdsm_gb300 import _lib
    bound = set(_lib.SIGNATURES) | set(_lib.SERVER_SYMBOLS)
    mdsm_names = {n for n in names if n.startswith("mdsm_")}
    assert mdsm_names <= bound, mdsm_names - bound


def test_library_has_no_oracle_dependency():
    """The product library links no oracle code."""
    from mdsm_gb300 import _lib
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True,
                         text=True).stdout
    assert "orc_" not in out
    ldd = subprocess.run(["ldd", _lib.LIB_PATH], capture_output=True, text=True).stdout
    assert "oracle" not in ldd


C_LAYOUT = r"""
#include <stdio.h>
#include <stddef.h>
#include "mdsm_gb300.h"
#define P(T, f) printf(#T "." #f " %zu\n", offsetof(T, f))
int main(void) {
  printf("SURVEY %zu\n", sizeof(SURVEY));
  P(SURVEY, nsamp); P(SURVEY, tsamp); P(SURVEY, useBruteForce); P(SURVEY, useL1Cache);
  P(SURVEY, lowdm); P(SURVEY, pass_parameters); P(SURVEY, num_passes); P(SURVEY, timestamp);
  P(SURVEY, noiseMean); P(SURVEY, samplesPerChunk); P(SURVEY, fp); P(SURVEY, fileprefix);
  P(SURVEY, basedir); P(SURVEY, secs_per_file); P(SURVEY, use_pc_time);
  P(SURVEY, detection_threshold); P(SURVEY, num_threads); P(SURVEY, gpu_ids); P(SURVEY, num_gpus);
  printf("SUBBAND_PASSES %zu\n", sizeof(SUBBAND_PASSES));
  printf("mdsm_brute_desc %zu\n", sizeof(mdsm_brute_desc));
  P(mdsm_brute_desc, segs); P(mdsm_brute_desc, K); P(mdsm_brute_desc, kernel);
  printf("mdsm_subband_desc %zu\n", sizeof(mdsm_subband_desc));
  P(mdsm_subband_desc, passes); P(mdsm_subband_desc, acc);
  printf("mdsm_plan_info %zu\n", sizeof(mdsm_plan_info));
  P(mdsm_plan_info, in_stride); P(mdsm_plan_info, work_bytes);
  printf("mdsm_candidate %zu\n", sizeof(mdsm_candidate));
  return 0;
}
"""


def test_struct_layouts_match_c():
    from mdsm_gb300 import _lib
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "l.c")
        exe = os.path.join(d, "l")
        open(src, "w").write(C_LAYOUT)
        subprocess.run(["gcc", "-I", INC, "-o", exe, src], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    types = {"SURVEY": _lib.SURVEY, "SUBBAND_PASSES": _lib.SUBBAND_PASSES,
             "mdsm_brute_desc": _lib.BruteDesc, "mdsm_subband_desc": _lib.SubbandDesc,
             "mdsm_plan_info": _lib.PlanInfo, "mdsm_candidate": _lib.Candidate}
    for line in out.splitlines():
        key, val = line.split()
        val = int(val)
        if "." in key:
            t, f = key.split(".")
            assert getattr(types[t], f).offset == val, key
        else:
            assert ctypes.sizeof(types[key]) == val, key


def test_cpp_compat_header_compiles_reference_call_sequence():
    """A caller written like src/MDSM.cpp:132-169 compiles and links against the library."""
    from mdsm_gb300 import _lib
    caller = r"""
#include "dedispersion_manager.h"
int main(int argc, char **argv) {
  SURVEY *survey = processSurveyParameters(argc > 1 ? argv[1] : "obs.xml");
  if (!survey) return 2;
  float *input_buffer = initialiseMDSM(survey);
  if (!input_buffer) return 3;
  unsigned x;
  next_chunk(survey->nsamp, x, 0.0, survey->tsamp);
  start_processing(survey->nsamp);
  next_chunk(0, x);
  start_processing(0);
  tearDownMDSM();
  return 0;
}
"""
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "caller.cpp")
        open(src, "w").write(caller)
        libdir = os.path.dirname(_lib.LIB_PATH)
        r = subprocess.run(["g++", "-I", INC, "-o", os.path.join(d, "caller"), src,
                            "-L" + libdir, "-lmdsm_gb300", "-Wl,-rpath," + libdir],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


THREAD_LAYOUT = r"""
#include <stdio.h>
#include <stddef.h>
#include "dedispersion_thread.h"
#define P(T, f) printf(#T "." #f " %zu\n", offsetof(T, f))
int main(void) {
  printf("DEVICE_INFO %zu\n", sizeof(DEVICE_INFO));
  P(DEVICE_INFO, clock_rate); P(DEVICE_INFO, device_id);
  printf("DEVICES %zu\n", sizeof(DEVICES));
  P(DEVICES, minTotalGlobalMem); P(DEVICES, devices);
  printf("THREAD_PARAMS %zu\n", sizeof(THREAD_PARAMS));
  P(THREAD_PARAMS, maxshift); P(THREAD_PARAMS, dmshifts); P(THREAD_PARAMS, inputsize);
  P(THREAD_PARAMS, dedispersed_size); P(THREAD_PARAMS, output); P(THREAD_PARAMS, input);
  P(THREAD_PARAMS, device_id); P(THREAD_PARAMS, thread_num); P(THREAD_PARAMS, stop);
  P(THREAD_PARAMS, rw_lock); P(THREAD_PARAMS, output_barrier); P(THREAD_PARAMS, start);
  P(THREAD_PARAMS, survey);
  return 0;
}
"""


def _reference_thread_types():
    """src/mdsm/dedispersion_thread.h:9-57 as ctypes structures, member for member."""
    c = ctypes
    class DeviceInfo(c.Structure):
        _fields_ = [(n, c.c_int) for n in ("multiprocessor_count", "constant_memory",
                                            "shared_memory", "register_count", "thread_count",
                                            "clock_rate", "device_id")]

    class Devices(c.Structure):
        _fields_ = [("num_devices", c.c_int), ("minTotalGlobalMem", c.c_ulong),
                    ("devices", c.c_void_p)]

    class ThreadParams(c.Structure):
        _fields_ = [("iterations", c.c_int), ("maxiters", c.c_int), ("maxshift", c.c_int),
                    ("binsize", c.c_int), ("dmshifts", c.c_void_p), ("inputsize", c.c_size_t),
                    ("outputsize", c.c_size_t), ("dm_output", c.c_size_t),
                    ("dedispersed_size", c.c_size_t), ("output", c.c_void_p),
                    ("input", c.c_void_p), ("device_id", c.c_int), ("thread_num", c.c_ushort),
                    ("num_threads", c.c_ushort), ("stop", c.c_ushort), ("rw_lock", c.c_void_p),
                    ("input_barrier", c.c_void_p), ("output_barrier", c.c_void_p),
                    ("start", c.c_long), ("survey", c.c_void_p)]
    return {"DEVICE_INFO": DeviceInfo, "DEVICES": Devices, "THREAD_PARAMS": ThreadParams}


def test_thread_abi_layouts_match_reference():
    """DEVICE_INFO, DEVICES and THREAD_PARAMS of include/dedispersion_thread.h have the
    reference's member order and types (src/mdsm/dedispersion_thread.h:9-57)."""
    types = _reference_thread_types()
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(src, "w").write(THREAD_LAYOUT)
        subprocess.run(["gcc", "-I", INC, "-o", exe, src], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    for line in out.splitlines():
        key, val = line.split()
        val = int(val)
        if "." in key:
            t, f = key.split(".")
            assert getattr(types[t], f).offset == val, key
        else:
            assert ctypes.sizeof(types[key]) == val, key


OUTPUT_LAYOUT = r"""
#include <stdio.h>
#include <stddef.h>
#include "dedispersion_output.h"
#define P(T, f) printf(#T "." #f " %zu\n", offsetof(T, f))
int main(void) {
  printf("OUTPUT_PARAMS %zu\n", sizeof(OUTPUT_PARAMS));
  P(OUTPUT_PARAMS, iterations); P(OUTPUT_PARAMS, maxiters); P(OUTPUT_PARAMS, output_buffer);
  P(OUTPUT_PARAMS, dedispersed_size); P(OUTPUT_PARAMS, stop); P(OUTPUT_PARAMS, rw_lock);
  P(OUTPUT_PARAMS, input_barrier); P(OUTPUT_PARAMS, output_barrier); P(OUTPUT_PARAMS, start);
  P(OUTPUT_PARAMS, survey);
  return 0;
}
"""


def test_output_abi_layout_matches_reference():
    """OUTPUT_PARAMS of include/dedispersion_output.h has the reference's member order and
    types (src/mdsm/dedispersion_output.h:8-28)."""
    c = ctypes

    class OutputParams(c.Structure):
        _fields_ = [("nthreads", c.c_int), ("iterations", c.c_int), ("maxiters", c.c_int),
                    ("output_buffer", c.c_void_p), ("dedispersed_size", c.c_size_t),
                    ("stop", c.c_ushort), ("rw_lock", c.c_void_p),
                    ("input_barrier", c.c_void_p), ("output_barrier", c.c_void_p),
                    ("start", c.c_long), ("survey", c.c_void_p)]
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(src, "w").write(OUTPUT_LAYOUT)
        subprocess.run(["gcc", "-I", INC, "-o", exe, src], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    for line in out.splitlines():
        key, val = line.split()
        if "." in key:
            assert getattr(OutputParams, key.split(".")[1]).offset == int(val), key
        else:
            assert ctypes.sizeof(OutputParams) == int(val), key


def test_qstring_overload_with_header_first():
    """src/MDSM.cpp includes dedispersion_manager.h before any Qt header (:2) and calls
    processSurveyParameters(QString(argv[++i])) (:42,79,91).  With a QString header on the
    include path (here a minimal stand-in, tests/drivers/qt_stub/QString), that call compiles
    and links against the library."""
    from mdsm_gb300 import _lib
    caller = r"""
#include "dedispersion_manager.h"
int main(int argc, char **argv) {
  int i = 0;
  SURVEY *survey = processSurveyParameters(QString(argc > 1 ? argv[++i] : "obs.xml"));
  return survey ? 0 : 1;
}
"""
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "caller.cpp")
        open(src, "w").write(caller)
        libdir = os.path.dirname(_lib.LIB_PATH)
        r = subprocess.run(["g++", "-I", INC, "-I",
                            os.path.join(ROOT, "tests", "drivers", "qt_stub"),
                            "-o", os.path.join(d, "caller"), src,
                            "-L" + libdir, "-lmdsm_gb300", "-Wl,-rpath," + libdir],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_manager_driver_compiles_against_thread_abi():
    """A C manager spawning call_dedisperse as src/mdsm/dedispersion_manager.cpp:348-374 does
    (tests/drivers/manager_driver.c) compiles and links."""
    from mdsm_gb300 import _lib
    with tempfile.TemporaryDirectory() as d:
        libdir = os.path.dirname(_lib.LIB_PATH)
        r = subprocess.run(["gcc", "-std=gnu11", "-Wall", "-Werror", "-I", INC, "-o",
                            os.path.join(d, "mgr"),
                            os.path.join(ROOT, "tests", "drivers", "manager_driver.c"),
                            "-L" + libdir, "-lmdsm_gb300", "-lpthread",
                            "-Wl,-rpath," + libdir], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
