"""ns_poisson_fft_noalloc: the FFT pressure Poisson solve for callers that
must not allocate device memory (hosts whose device memory belongs to
another allocator or is reserved up front, real-time loops).

Called through the C ABI with caller-owned device buffers, twice in a row per
grid, and checked against the allocating entry point (ns_poisson) to the
routine tolerance of the parity tests.  This file sorts last so that a run
that stops at the first failure has run every other test first; it also
passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12  # relative L2, as the routine-level parity tests


def _rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.mark.parametrize("grid", [(32, 32, 32, 6.283185307179586, 6.283185307179586, 6.283185307179586),
                                  (64, 32, 16, 6.283185307179586, 3.0, 2.0)])
def test_noalloc_matches_allocating_poisson_twice(grid):
    import torch

    from ns_3d_staggered_dp_gb300 import Session, _lib, make_config
    nx, ny, nz, lx, ly, lz = grid
    lib = _lib.load()
    rng = np.random.default_rng(77)
    rhs = rng.standard_normal((nx, ny, nz))
    rhs -= rhs.mean()
    with Session(make_config(nx, ny, nz, lx=lx, ly=ly, lz=lz)) as s:
        ref = s.poisson(rhs)                                         # allocating entry point
    rhs_dev = torch.from_numpy(np.asfortranarray(rhs).ravel(order="F").copy()).cuda()
    dp_dev = torch.empty((nx + 2) * (ny + 2) * (nz + 2), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    for call in range(2):
        dp_dev.fill_(float("nan"))                                  # every output entry must be written
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        st = lib.ns_poisson_fft_noalloc(ctypes.c_void_p(rhs_dev.data_ptr()), ctypes.c_void_p(dp_dev.data_ptr()),
                                        nx, ny, nz, lx, ly, lz, ctypes.c_void_p(stream.cuda_stream))
        assert st == 0, f"call {call}: status {st}"
        torch.cuda.synchronize()
        if call > 0:
            # The static scratch is placed on the device when the driver loads the
            # library's module (lazily, at its first use); later calls take nothing.
            assert torch.cuda.mem_get_info()[0] == free_before
        got = dp_dev.cpu().numpy().reshape((nx + 2, ny + 2, nz + 2), order="F")
        assert np.isfinite(got).all()
        assert _rel(got, ref) < TOL, (call, _rel(got, ref))


def test_noalloc_rejects_grids_beyond_the_static_scratch():
    import torch

    from ns_3d_staggered_dp_gb300 import _lib
    lib = _lib.load()
    a = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = ctypes.c_void_p(a.data_ptr())
    assert lib.ns_poisson_fft_noalloc(p, p, 128, 64, 64, 1.0, 1.0, 1.0, None) == 1    # NS_ERR_SHAPE
    assert lib.ns_poisson_fft_noalloc(p, p, 48, 32, 32, 1.0, 1.0, 1.0, None) == 1
    assert lib.ns_poisson_fft_noalloc(None, p, 32, 32, 32, 1.0, 1.0, 1.0, None) == 6  # NS_ERR_ARG
    odd = ctypes.c_void_p(a.data_ptr() + 4)                                             # dp not 8-byte aligned
    assert lib.ns_poisson_fft_noalloc(p, odd, 32, 32, 32, 1.0, 1.0, 1.0, None) == 6
