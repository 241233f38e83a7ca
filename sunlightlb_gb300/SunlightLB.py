"""SunlightLB module with the interface of the reference's SWIG Python module
(src/SunlightLB.i wraps the whole of sunlightlb.h), backed by the GB300
library.  A driver written for the reference, e.g.::

    from sunlightlb_gb300.SunlightLB import *
    mylb = newlb(16, 16, 16, "sphere_python")
    mylb.tau = 0.80
    insertsph(mylb, 3.7, 7.5, 7.5, 7.5)
    lbstep(mylb)

runs unchanged.
"""

from . import binding as _binding
from . import library as _library

_lib = _library()
globals().update(_lib.globals())

TRACE_ROUTINE_EXITS = _binding.TRACE_ROUTINE_EXITS
TRACING_ROUTINE_EXITS = _binding.TRACE_ROUTINE_EXITS
OBJECT_DETAILS = _binding.OBJECT_DETAILS
MP_OBJECT_DETAILS = _binding.MP_OBJECT_DETAILS
FORCE_DETAILS = _binding.FORCE_DETAILS
POST_BBL = _binding.POST_BBL
POST_PROPAGATE = _binding.POST_PROPAGATE
POST_COLLIDE = _binding.POST_COLLIDE
SLB_FP64 = _binding.SLB_FP64
SLB_FP32 = _binding.SLB_FP32
SLB_BF16 = _binding.SLB_BF16
PI = 3.14159265358979323846
