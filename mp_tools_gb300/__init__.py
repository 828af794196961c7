"""mp_tools_gb300 — GB300 (sm_103a) engine for the S(Q,omega) hot path of MP_TOOLS mp_sqom.

The compute path is libmpsq.so (CUDA C++, C ABI in include/mpsq.h); this package holds the
host-side mirror of the reference's operator interface (Q-grid geometry, time constants,
normalisations), the .dat/.par readers, synthetic workload generators and the job scheduler.
"""
from . import _lib
from ._lib import BULK, CELL, FP32, FP64, MpsqError, load
from .sqom import QGrid, SqomJob, TimeAxis, speckle_filter

__all__ = ["load", "QGrid", "SqomJob", "TimeAxis", "speckle_filter", "MpsqError", "FP32", "FP64",
           "CELL", "BULK"]
