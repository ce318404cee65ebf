"""The C ABI library loads on a CPU-only host and exports every entry point
declared in include/ns_gpu.h (no compute calls: there may be no GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ns_gpu.h")
LIB = os.path.join(ROOT, "ns_3d_staggered_dp_gb300", "libns_gpu.so")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*(ns_[a-z_0-9]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(LIB):
        from ns_3d_staggered_dp_gb300 import build
        build.build()
    return ctypes.CDLL(LIB)


def test_header_declares_the_entry_points():
    names = declared_functions()
    for must in ("ns_create", "ns_destroy", "ns_set_state", "ns_get_state", "ns_step", "ns_get_diag",
                 "ns_set_faces", "ns_cal_conv", "ns_cal_diff", "ns_poisson", "ns_adi", "ns_profile"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header():
    from ns_3d_staggered_dp_gb300 import _lib
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_version_and_status_strings_without_gpu(lib):
    lib.ns_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.ns_version()
    lib.ns_status_string.restype = ctypes.c_char_p
    assert lib.ns_status_string(5) == b"unsupported boundary condition"


def test_config_default_matches_reference_driver(lib):
    from ns_3d_staggered_dp_gb300 import _lib
    L = _lib.load()
    c = _lib.NSConfig()
    assert L.ns_config_default(ctypes.byref(c), 256, 256, 256) == 0
    assert c.nu == 0.002 and c.dt == 2.5e-4 and c.scheme == 1      # big_periodic_3D.f90:10,104-105
    assert list(c.bc) == [1, 1, 1] and list(c.pbc) == [1, 1, 1] and c.dp_flag == 0 and c.gauge == 1


def test_create_rejects_bad_configs_before_touching_the_gpu(lib):
    from ns_3d_staggered_dp_gb300 import _lib
    L = _lib.load()
    c = _lib.NSConfig()
    L.ns_config_default(ctypes.byref(c), 32, 32, 32)
    c.bc[0] = 3   # Neumann velocity leaves ghosts undefined in the reference
    h = ctypes.c_void_p()
    assert L.ns_create(ctypes.byref(c), ctypes.byref(h)) == 5
    L.ns_config_default(ctypes.byref(c), 30, 32, 32)   # not a supported FFT size
    assert L.ns_create(ctypes.byref(c), ctypes.byref(h)) == 1
    assert L.ns_create(None, ctypes.byref(h)) == 6


def test_err_csv_writer_matches_the_reference_format(tmp_path):
    """ns_write_err_csv is host code: the err_vel / rms_vel files of
    re_simulation_sub_tstep_interBC_combine.f90:913-931, byte for byte as the
    oracle's restatement writes them."""
    import numpy as np

    from ns_3d_staggered_dp_gb300 import write_err_csv
    from oracle import ns_oracle as O
    rng = np.random.default_rng(3)
    for kind, ncol in ((0, 8), (1, 4)):
        rows = np.abs(rng.standard_normal((6, ncol))) * 10.0 ** rng.integers(-14, 3, (6, ncol))
        rows[0, 0] = 0.0
        rows[1, 1] = -2.5e-7
        a, b = tmp_path / f"lib_{kind}.txt", tmp_path / f"oracle_{kind}.txt"
        write_err_csv(a, kind, rows)
        O.write_err_csv(b, kind, rows)
        assert a.read_bytes() == b.read_bytes()
    first = (tmp_path / "lib_0.txt").read_text().splitlines()
    assert first[0].startswith("time_step, rel_err_u,")
    assert first[1].startswith("0, 0.00000E+00,")
