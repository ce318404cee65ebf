"""GB300-native (sm_103a) FP64 staggered-grid Navier-Stokes step.

The compute path is libns_gpu.so (CUDA kernels behind a C ABI, declared in
include/ns_gpu.h); this package only loads it and mirrors the reference's
step interface on the host.
"""
from .api import (AB2, AB2_CN, EULER, FACE_ORDER, SWEEP_FACE_ORDER, Batch, H5File, NSError, Session,  # noqa: F401
                  face_shapes, make_batch_config, make_config, shapes, spline_weights, tgv, write_err_csv)

__all__ = ["Session", "Batch", "make_config", "make_batch_config", "spline_weights", "shapes", "NSError", "EULER",
           "AB2", "AB2_CN", "FACE_ORDER", "write_err_csv", "H5File", "face_shapes", "tgv", "SWEEP_FACE_ORDER"]
