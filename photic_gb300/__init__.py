"""photic_gb300: GB300 (sm_103a) implementation of photic's per-pixel
semi-analytical inversion -- the HOPE forward model fitted per pixel by
the reference's modified AS 47 Nelder-Mead -- behind a C ABI
(include/photic.h) and this thin Python host layer over it.
"""
from . import api  # noqa: F401
from . import ncgrid  # noqa: F401
from .api import (Config, JointGraph, PhoticError, alloc_outputs, cost,  # noqa: F401
                  depth_sigma, fallbacks_first, generate_field, generate_joint, generate_scene,
                  invert, joint_invert, lut_invert, region_depth_sigma, region_fit, region_invert,
                  region_lut_invert, sync, version)
