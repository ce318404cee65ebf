"""The algebra of the wall-axis line solves, restated in NumPy (CPU).

The CUDA kernels solve every spectrum line along the wall axis,
  x[j-1] + b_j x[j] + x[j+1] = rs r_j,  b_j = -2 + sigma (+ e at the end rows),
(the system of DCT_poisson_solver along one axis, NS_functions.f90:1505-1630)
by a twisted factorisation: top-down multipliers m_j = 1/(b_j - m_{j-1}) above
the middle row k = N/2, bottom-up n_j = 1/(b_j - n_{j+1}) below it, the pivot
1/(b_k - m_{k-1} - n_{k+1}) at k (csrc/ns_dct.cu, tri_twist_body).  The one
singular line (sigma = 0, Neumann end rows e = +1) is solved by two prefix
sums and a mean shift (sing_line_warp), whose result the reference defines
as: rhs mean dropped, last entry pinned, then shifted to the target mean
(NS_functions.f90:1576-1577).  These tests check both restatements against
dense solves; the GPU tests check the kernels against the oracle.
"""
import numpy as np
import pytest


def tridiag(N, sigma, e):
    A = np.zeros((N, N))
    for j in range(N):
        A[j, j] = -2.0 + sigma + (e if j in (0, N - 1) else 0.0)
        if j > 0:
            A[j, j - 1] = 1.0
        if j < N - 1:
            A[j, j + 1] = 1.0
    return A


def twisted_solve(r, sigma, e, rs):
    """The table (m, n, pivot) and the two walks of tri_twist_body."""
    N = len(r)
    k = N // 2
    b = np.full(N, -2.0 + sigma)
    b[0] += e
    b[N - 1] += e
    m = np.zeros(N)
    nn = np.zeros(N)
    mr = 0.0
    for j in range(k):
        mr = 1.0 / (b[j] - mr)
        m[j] = mr
    nr = 0.0
    for j in range(N - 1, k, -1):
        nr = 1.0 / (b[j] - nr)
        nn[j] = nr
    piv = 1.0 / (b[k] - mr - nr)
    d = np.zeros(N)
    dv = 0.0
    for j in range(k):  # top lane
        dv = (r[j] * rs - dv) * m[j]
        d[j] = dv
    ev = 0.0
    for j in range(N - 1, k, -1):  # bottom lane
        ev = (r[j] * rs - ev) * nn[j]
        d[j] = ev
    x = np.zeros(N)
    x[k] = ((r[k] * rs - dv) - ev) * piv
    p = x[k]
    for j in range(k - 1, -1, -1):
        p = d[j] - m[j] * p
        x[j] = p
    q = x[k]
    for j in range(k + 1, N):
        q = d[j] - nn[j] * q
        x[j] = q
    return x


def singular_prefix(r, rs, target):
    """sing_line_warp: F_j = sum_{i<=j} R_i, x_j = sum_{i<j} F_i, mean shift."""
    R = (r - r.mean()) * rs
    F = np.cumsum(R)
    x = np.concatenate(([0.0], np.cumsum(F)[:-1]))
    return x + (target - x.mean())


def singular_reference(r, rs, target):
    """The reference's definition: rhs mean dropped, last entry pinned to 0,
    the other rows solved, then the solution shifted to the target mean."""
    N = len(r)
    A = tridiag(N, 0.0, 1.0)
    R = (r - r.mean()) * rs
    x = np.zeros(N)
    x[: N - 1] = np.linalg.solve(A[: N - 1, : N - 1], R[: N - 1])
    return x + (target - x.mean())


@pytest.mark.parametrize("N", [8, 9, 16, 21, 128, 257])
@pytest.mark.parametrize("e", [1.0, -1.0, 0.0])  # pressure codes 3, 2, 4
def test_twisted_solve_matches_dense(N, e):
    rng = np.random.default_rng(N * 7 + int(e + 1))
    for sigma in (-1e-3, -0.37, -3.9):
        r = rng.standard_normal(N)
        rs = 0.7
        x = twisted_solve(r, sigma, e, rs)
        ref = np.linalg.solve(tridiag(N, sigma, e), rs * r)
        assert np.abs(x - ref).max() <= 1e-10 * max(1.0, np.abs(ref).max()), (N, e, sigma)


@pytest.mark.parametrize("N", [8, 16, 21, 200, 256])
def test_singular_line_prefix_sums_match_the_pinned_solve(N):
    rng = np.random.default_rng(N)
    r = rng.standard_normal(N)
    for target in (0.0, 0.31):
        x = singular_prefix(r, 0.9, target)
        ref = singular_reference(r, 0.9, target)
        assert np.abs(x - ref).max() <= 1e-9 * max(1.0, np.abs(ref).max()), (N, target)
        # the rows the pinned solve keeps hold exactly; the last one up to the dropped mean
        A = tridiag(N, 0.0, 1.0)
        R = (r - r.mean()) * 0.9
        assert np.abs((A @ x - R)[: N - 1]).max() < 1e-9 * N


def test_singular_warp_segments():
    """The warp's row segments (ceil(N/32) rows a lane, the last lanes empty
    or short) cover every row once, in order."""
    for N in (8, 21, 32, 33, 200, 256, 512):
        seg = (N + 31) // 32
        rows = []
        for lane in range(32):
            j0, j1 = min(lane * seg, N), min(lane * seg + seg, N)
            rows.extend(range(j0, j1))
        assert rows == list(range(N))
