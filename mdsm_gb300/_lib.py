"""ctypes binding of libmdsm_gb300.so (the C ABI in include/mdsm_gb300.h).

The library is built in-tree by mdsm_gb300/build.py.  Loading fails loudly when it is
missing: there is no fallback implementation.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libmdsm_gb300.so")

MDSM_OK = 0
STATUS_NAMES = {
    0: "MDSM_OK", 1: "MDSM_EINVAL", 2: "MDSM_ENOMEM", 3: "MDSM_ECUDA", 4: "MDSM_ETIMEOUT",
    5: "MDSM_ESTATE", 6: "MDSM_ERANGE", 7: "MDSM_EBUDGET", 8: "MDSM_EPARSE", 9: "MDSM_EIO",
    10: "MDSM_EAGAIN",
}

DTYPES = {"u8": 0, "u16": 1, "i16": 2, "f32": 3, "i32": 4}
OUT_DTYPES = {"f32": 0, "i32": 1}
ACC = {"auto": 0, "i32": 1, "f32": 2}
SHIFT_MODES = {"l1": 0, "l1_muladd": 1, "opt": 2, "opt_muladd": 3, "fp64_trunc": 4,
               "fp64_round": 5}


class MdsmError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), msg))
        self.status = status


class Segment(ctypes.Structure):
    _fields_ = [("lowdm", ctypes.c_float), ("dmstep", ctypes.c_float), ("ndms", ctypes.c_int)]


class SUBBAND_PASSES(ctypes.Structure):
    _fields_ = [("lowdm", ctypes.c_float), ("highdm", ctypes.c_float),
                ("dmstep", ctypes.c_float), ("sub_dmstep", ctypes.c_float),
                ("binsize", ctypes.c_int), ("ndms", ctypes.c_int), ("ncalls", ctypes.c_int),
                ("calldms", ctypes.c_int), ("mean", ctypes.c_int), ("stddev", ctypes.c_int)]


class SURVEY(ctypes.Structure):
    _fields_ = [("nsamp", ctypes.c_uint), ("nchans", ctypes.c_uint), ("tdms", ctypes.c_uint),
                ("maxshift", ctypes.c_uint), ("nbits", ctypes.c_uint),
                ("tsamp", ctypes.c_float), ("foff", ctypes.c_float), ("fch1", ctypes.c_float),
                ("useBruteForce", ctypes.c_bool), ("useL1Cache", ctypes.c_bool),
                ("lowdm", ctypes.c_float), ("dmstep", ctypes.c_float),
                ("pass_parameters", ctypes.POINTER(SUBBAND_PASSES)),
                ("num_passes", ctypes.c_uint), ("nsubs", ctypes.c_uint),
                ("timestamp", ctypes.c_double), ("blockRate", ctypes.c_double),
                ("noiseMean", ctypes.POINTER(ctypes.c_float)),
                ("noiseRMS", ctypes.POINTER(ctypes.c_float)),
                ("samplesPerChunk", ctypes.c_uint), ("fp", ctypes.c_void_p),
                ("fileprefix", ctypes.c_char * 80), ("basedir", ctypes.c_char * 120),
                ("secs_per_file", ctypes.c_uint), ("use_pc_time", ctypes.c_char),
                ("single_file_mode", ctypes.c_char), ("detection_threshold", ctypes.c_float),
                ("num_threads", ctypes.c_uint), ("gpu_ids", ctypes.POINTER(ctypes.c_uint)),
                ("num_gpus", ctypes.c_uint)]


class BruteDesc(ctypes.Structure):
    _fields_ = [("nchans", ctypes.c_int), ("fch1", ctypes.c_float), ("foff", ctypes.c_float),
                ("tsamp", ctypes.c_float), ("nsamp", ctypes.c_int),
                ("segs", ctypes.POINTER(Segment)), ("nsegs", ctypes.c_int),
                ("shift_mode", ctypes.c_int), ("K", ctypes.c_double),
                ("in_dtype", ctypes.c_int), ("out_dtype", ctypes.c_int), ("acc", ctypes.c_int),
                ("dm_block", ctypes.c_int), ("kernel", ctypes.c_int)]


class SubbandDesc(ctypes.Structure):
    _fields_ = [("nchans", ctypes.c_int), ("fch1", ctypes.c_float), ("foff", ctypes.c_float),
                ("tsamp", ctypes.c_float), ("nsamp", ctypes.c_int), ("nsubs", ctypes.c_int),
                ("passes", ctypes.POINTER(SUBBAND_PASSES)), ("npasses", ctypes.c_int),
                ("use_fma", ctypes.c_int), ("in_dtype", ctypes.c_int),
                ("out_dtype", ctypes.c_int), ("acc", ctypes.c_int)]


class PlanInfo(ctypes.Structure):
    _fields_ = [("nchans", ctypes.c_int), ("ndms", ctypes.c_int), ("nsamp", ctypes.c_int),
                ("maxshift", ctypes.c_int), ("in_stride", ctypes.c_longlong),
                ("in_bytes", ctypes.c_longlong), ("out_bytes", ctypes.c_longlong),
                ("in_dtype", ctypes.c_int), ("out_dtype", ctypes.c_int), ("acc", ctypes.c_int),
                ("dm_block", ctypes.c_int), ("time_tile", ctypes.c_int),
                ("kernel", ctypes.c_int), ("nstages", ctypes.c_int),
                ("work_bytes", ctypes.c_longlong)]


class StageInfo(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("kernel", "dm_block", "time_tile", "out_u16",
                                            "nchans", "ndms", "ngroups", "nsamp")] + \
               [("smem_bytes", ctypes.c_longlong)]


class SigprocHeader(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("nchans", "nbits", "nifs", "machine_id",
                                            "telescope_id", "data_type", "nbeams", "ibeam",
                                            "barycentric", "pulsarcentric", "nbins", "nsamples",
                                            "nfchannels")] + \
               [(n, ctypes.c_double) for n in ("tstart", "tsamp", "fch1", "foff", "refdm",
                                               "az_start", "za_start", "src_raj", "src_dej",
                                               "period")] + \
               [("npuls", ctypes.c_longlong), ("header_bytes", ctypes.c_longlong),
                ("source_name", ctypes.c_char * 81), ("rawdatafile", ctypes.c_char * 81)]


class Candidate(ctypes.Structure):
    _fields_ = [("dm_idx", ctypes.c_int32), ("sample", ctypes.c_int32), ("snr", ctypes.c_float),
                ("width", ctypes.c_int32)]


_vp = ctypes.c_void_p
_ll = ctypes.c_longlong
_i = ctypes.c_int
_f = ctypes.c_float
_d = ctypes.c_double
_st = ctypes.c_int

# name -> (restype, argtypes).  Every symbol declared in include/mdsm_gb300.h.
SIGNATURES = {
    "mdsm_dmdelay": (_f, [_f, _f]),
    "mdsm_last_error": (ctypes.c_char_p, []),
    "mdsm_version": (ctypes.c_char_p, []),
    "mdsm_brute_plan_create": (_st, [ctypes.POINTER(BruteDesc), ctypes.POINTER(_vp)]),
    "mdsm_subband_plan_create": (_st, [ctypes.POINTER(SubbandDesc), ctypes.POINTER(_vp)]),
    "mdsm_plan_destroy": (None, [_vp]),
    "mdsm_plan_get_info": (_st, [_vp, ctypes.POINTER(PlanInfo)]),
    "mdsm_plan_stage_info": (_st, [_vp, ctypes.c_int, ctypes.POINTER(StageInfo)]),
    "mdsm_plan_shift_table": (_st, [_vp, _i, _vp]),
    "mdsm_plan_dm_values": (_st, [_vp, _vp]),
    "mdsm_plan_dmshifts": (_st, [_vp, _vp]),
    "mdsm_dmshifts": (_st, [_i, _f, _f, _vp]),
    "mdsm_brute_shift_table": (_st, [ctypes.POINTER(BruteDesc), _vp, _vp, ctypes.POINTER(_i)]),
    "mdsm_subband_shift_tables": (_st, [ctypes.POINTER(SubbandDesc), _i, _vp, _vp]),
    "mdsm_dedisperse_device": (_st, [_vp, _vp, _ll, ctypes.c_size_t, _vp, _ll, _vp]),
    "mdsm_dedisperse_host": (_st, [_vp, _vp, _ll, _vp, _vp]),
    "mdsm_plan_last_launches": (_i, [_vp]),
    "mdsm_rfi_clip_device": (_st, [_vp, _i, _i, _ll, _ll, _d, _d, _vp]),
    "mdsm_ref_detect_device": (_st, [_vp, _i, _i, _f, _f, _f, ctypes.POINTER(Candidate), _ll,
                                     ctypes.POINTER(_ll), ctypes.POINTER(_f),
                                     ctypes.POINTER(_f), _vp]),
    "mdsm_ref_detect_device_noalloc": (_st, [_vp, _i, _i, _f, _f, _f, ctypes.POINTER(Candidate),
                                             _ll, ctypes.POINTER(_ll), ctypes.POINTER(_f),
                                             ctypes.POINTER(_f), _vp]),
    "mdsm_ref_detect_chunked_device": (_st, [_vp, _i, _i, _f, _f, _f, _vp, _vp, _ll, _i,
                                             ctypes.POINTER(Candidate), _ll, ctypes.POINTER(_ll),
                                             _vp]),
    "mdsm_ref_detect_subband_device": (_st, [_vp, _vp, _ll, _f, _vp, _vp, _ll, _i,
                                             ctypes.POINTER(Candidate), _ll, ctypes.POINTER(_ll),
                                             _vp]),
    "mdsm_boxcar_detect_device": (_st, [_vp, _i, _i, _i, _i, _d, ctypes.POINTER(Candidate), _ll,
                                        ctypes.POINTER(_ll), _vp]),
    "mdsm_batch_choice_info": (_st, [_i] + [ctypes.POINTER(_i)] * 5),
    "mdsm_batch_autotune_times": (_st, [_vp, ctypes.POINTER(_i), ctypes.POINTER(ctypes.c_float),
                                        _i, ctypes.POINTER(_i)]),
    "mdsm_plan_check": (_st, [_vp, _vp]),
    "mdsm_plan_wait_selftest": (_st, [_vp, ctypes.c_uint, _vp]),
    "mdsm_plan_set_stage_timing": (_st, [_vp, _i]),
    "mdsm_plan_stage_times": (_st, [_vp, ctypes.POINTER(ctypes.c_float), _i,
                                    ctypes.POINTER(_i)]),
    "mdsm_singlepulse_detect_device": (_st, [_vp, _i, _i, _i, _i, _i, _i, _d,
                                             ctypes.POINTER(Candidate), _ll, ctypes.POINTER(_ll),
                                             _vp]),
    "mdsm_downsample_device": (_st, [_vp, _i, _i, _ll, _ll, _i, _i, _vp, _i, _ll, _vp]),
    "mdsm_detrend_normalise_device": (_st, [_vp, _i, _ll, _i, _vp]),
    "mdsm_sigproc_read_header": (_st, [ctypes.c_char_p, ctypes.POINTER(SigprocHeader)]),
    "mdsm_sigproc_write_series_header": (_st, [ctypes.c_char_p, _d, _d, _d, _d]),
    "mdsm_unpack_device": (_st, [_vp, _ll, _i, _i, _i, _vp, _i, _ll, _ll, _vp]),
    "mdsm_batch_create": (_st, [ctypes.POINTER(_vp), _i, ctypes.POINTER(_vp)]),
    "mdsm_batch_set_buffers": (_st, [_vp, ctypes.POINTER(_vp), ctypes.POINTER(_ll),
                                     ctypes.POINTER(_vp), ctypes.POINTER(_ll)]),
    "mdsm_batch_enable_clip": (_st, [_vp, _d, _d]),
    "mdsm_batch_enable_detect": (_st, [_vp, _i, _d, _ll]),
    "mdsm_batch_autotune": (_st, [_vp, _vp, ctypes.POINTER(_i)]),
    "mdsm_batch_run": (_st, [_vp, _i, _vp]),
    "mdsm_batch_last_launches": (_i, [_vp]),
    "mdsm_batch_candidates": (_st, [_vp, _i, ctypes.POINTER(Candidate), _ll,
                                    ctypes.POINTER(_ll), _vp]),
    "mdsm_batch_destroy": (None, [_vp]),
    "mdsm_processSurveyParameters": (ctypes.POINTER(SURVEY), [ctypes.c_char_p]),
    "mdsm_initialiseMDSM": (ctypes.POINTER(_f), [ctypes.POINTER(SURVEY)]),
    "mdsm_next_chunk": (ctypes.POINTER(_f), [ctypes.c_uint, ctypes.POINTER(ctypes.c_uint), _d,
                                             _d, ctypes.POINTER(_f), ctypes.POINTER(_f)]),
    "mdsm_start_processing": (_i, [ctypes.c_uint]),
    "mdsm_tearDownMDSM": (None, []),
    "mdsm_compat_candidates": (_ll, [ctypes.POINTER(Candidate), _ll]),
    "mdsm_compat_blocks_8bit": (_ll, []),
    "mdsm_free_survey": (None, [ctypes.POINTER(SURVEY)]),
}

_LIB = None

# serving-form entry points are bound by mdsm_gb300/serving.py
SERVER_SYMBOLS = ("mdsm_server_create", "mdsm_server_add_beam_brute",
                  "mdsm_server_add_beam_subband", "mdsm_server_beam_info", "mdsm_server_submit",
                  "mdsm_server_poll", "mdsm_server_drain", "mdsm_server_get_stats",
                  "mdsm_server_destroy", "mdsm_server_acquire", "mdsm_server_commit")


def load(path=None):
    """Load the library (once).  Raises if it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError("libmdsm_gb300.so is not built (%s); run "
                           "`python -m mdsm_gb300.build`" % p)
    lib = ctypes.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(status):
    if status != MDSM_OK:
        msg = load().mdsm_last_error()
        raise MdsmError(status, msg.decode() if msg else "")
    return status
