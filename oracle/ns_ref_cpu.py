"""ctypes binding of oracle/libns_ref_cpu.so, the C++/OpenMP restatement of
the reference's periodic step (test infrastructure and the timed CPU
baseline; never part of the product)."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libns_ref_cpu.so")
_DP = C.POINTER(C.c_double)
_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            from oracle import build_cpu
            build_cpu.build()
        lib = C.CDLL(LIB)
        lib.cpu_create.restype = C.c_void_p
        lib.cpu_create.argtypes = [C.c_int] * 3 + [C.c_double] * 5 + [C.c_int] * 3
        lib.cpu_step.restype = C.c_int
        lib.cpu_step.argtypes = [C.c_void_p] + [_DP] * 7 + [C.c_int]
        lib.cpu_destroy.argtypes = [C.c_void_p]
        lib.cpu_threads.restype = C.c_int
        lib.cpu_set_threads.restype = C.c_int
        lib.cpu_set_threads.argtypes = [C.c_int]
        _lib = lib
    return _lib


class CpuStep:
    """cfg: an oracle Config of a triply periodic box."""

    def __init__(self, cfg):
        if tuple(cfg.bc) != (1, 1, 1) or tuple(cfg.pbc) != (1, 1, 1):
            raise ValueError("the C++ restatement covers the triply periodic box")
        self.lib = load()
        self.h = self.lib.cpu_create(cfg.nx, cfg.ny, cfg.nz, cfg.lx, cfg.ly, cfg.lz, cfg.nu, cfg.dt, cfg.scheme,
                                     int(cfg.dp_flag), int(cfg.gauge))
        if not self.h:
            raise ValueError("unsupported grid")

    def step(self, st):
        """Advance the oracle State st in place (its arrays become Fortran-ordered copies)."""
        arrs = []
        for name in ("u", "v", "w", "p", "px", "py", "pz"):
            a = np.asfortranarray(getattr(st, name), dtype=np.float64).copy(order="F")
            setattr(st, name, a)
            arrs.append(a.ctypes.data_as(_DP))
        if self.lib.cpu_step(self.h, *arrs, int(st.first)) != 0:
            raise RuntimeError("cpu_step failed")
        st.first = False
        return st

    def threads(self):
        return int(self.lib.cpu_threads())

    def set_threads(self, n):
        return int(self.lib.cpu_set_threads(int(n)))

    def close(self):
        if self.h:
            self.lib.cpu_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()
