"""GB300-native (sm_103a) FP64 staggered-grid Navier-Stokes step.

The compute path is libns_gpu.so (CUDA kernels behind a C ABI, declared in
include/ns_gpu.h); this package only loads it and mirrors the reference's
step interface on the host.
"""
from .api import AB2, AB2_CN, EULER, FACE_ORDER, NSError, Session, make_config, shapes  # noqa: F401

__all__ = ["Session", "make_config", "shapes", "NSError", "EULER", "AB2", "AB2_CN", "FACE_ORDER"]
