"""GB300-native (sm_103a) implementation of the IMPS_CPP_tools hot path.

Block-sparse H_AC / H_C / transfer-matrix applies, the Lanczos and GMRES solves built on
them, and the VUMPS driver loop that calls them, behind the C ABI in include/imps_gb300.h.
"""
from . import _native
from ._native import ImpsError, load
from .blocks import Context, Layout, Plan

__all__ = ["Context", "Layout", "Plan", "ImpsError", "load", "_native"]
