"""GB300 implementation of MDSM's incoherent dedispersion search path.

Native library: mdsm_gb300/_lib/libmdsm_gb300.so (C ABI, include/mdsm_gb300.h), built by
mdsm_gb300.build.  This package is a thin Python host layer over it.
"""
from ._lib import MdsmError, load  # noqa: F401
from .api import (BrutePlan, SubbandPlan, boxcar_detect_device, detrend_normalise_device,  # noqa: F401,E501
                  dmdelay, ref_detect_chunked_device, ref_detect_device,
                  ref_detect_subband_device, rfi_clip_device, singlepulse_detect_device)
from . import compat  # noqa: F401
