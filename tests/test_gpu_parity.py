"""CUDA path vs the CPU oracle, through the C ABI (libns_gpu.so).

Tolerances: the step is FP64 with the same algebra as the reference but
different rounding (FMA folding, MKL vs our FFT/Thomas); routine-level
results must agree to a relative L2 of 1e-12, ten full steps to 1e-10 per
field (the parity bound of the step), and max|div u| <= 1e-12 after every step.
"""
import numpy as np
import pytest

from oracle import ns_oracle as O
from tests.helpers import random_state, rel_l2, tgv_state

pytestmark = pytest.mark.gpu

ROUTINE_TOL = 1e-12
STEP_TOL = 1e-10
DIV_TOL = 1e-12


def to_ns(cfg, **kw):
    from ns_3d_staggered_dp_gb300 import make_config
    return make_config(cfg.nx, cfg.ny, cfg.nz, lx=cfg.lx, ly=cfg.ly, lz=cfg.lz, nu=cfg.nu, dt=cfg.dt,
                       scheme=cfg.scheme, bc=cfg.bc, pbc=cfg.pbc, dp_flag=cfg.dp_flag, gauge=cfg.gauge,
                       mean_dp=cfg.mean_dp, **kw)


def session(cfg, **kw):
    from ns_3d_staggered_dp_gb300 import Session
    return Session(to_ns(cfg, **kw))


GRIDS = [(32, 32, 32, 1.0, 1.0, 1.0), (32, 16, 64, 1.0, 0.5, 1.7)]


@pytest.mark.parametrize("g", GRIDS)
def test_cal_conv_diff(g):
    nx, ny, nz, fx, fy, fz = g
    cfg = O.Config(nx, ny, nz, lx=2 * np.pi * fx, ly=2 * np.pi * fy, lz=2 * np.pi * fz)
    st = random_state(cfg, 11)
    dx, dy, dz = cfg.h
    ref_c = O.cal_conv(st.u, st.v, st.w, *cfg.bc, dx, dy, dz)
    ref_d = O.cal_diff(st.u, st.v, st.w, *cfg.bc, dx * dx, dy * dy, dz * dz)
    with session(cfg) as s:
        got_c = s.cal_conv(st.u, st.v, st.w)
        got_d = s.cal_diff(st.u, st.v, st.w)
    for a, b in zip(got_c, ref_c):
        assert a.shape == b.shape
        assert rel_l2(a, b) < ROUTINE_TOL
    for a, b in zip(got_d, ref_d):
        assert rel_l2(a, b) < ROUTINE_TOL


# the largest FFT axis the library accepts (512) on each axis in turn
MAX_FFT_GRIDS = [(512, 16, 16, 2.0, 1.0, 1.0), (16, 512, 16, 1.0, 2.0, 1.0), (16, 16, 512, 1.0, 1.0, 2.0)]


@pytest.mark.parametrize("poisson_z", [0, 1])
@pytest.mark.parametrize("g", GRIDS + [(16, 16, 16, 1.0, 1.0, 1.0), (64, 32, 16, 1.0, 1.0, 1.0)] + MAX_FFT_GRIDS)
def test_fft_poisson(g, poisson_z):
    """The all-periodic Poisson solve with either z stage (0: cyclic
    tridiagonal line solves, 1: z FFT * 1/lambda * z IFFT) against the
    oracle's 3D FFT solve and the restated operator."""
    nx, ny, nz, fx, fy, fz = g
    cfg = O.Config(nx, ny, nz, lx=2 * np.pi * fx, ly=2 * np.pi * fy, lz=2 * np.pi * fz)
    rng = np.random.default_rng(5)
    R = rng.standard_normal((nx, ny, nz))
    R -= R.mean()
    dx, dy, dz = cfg.h
    ref = np.zeros((nx + 2, ny + 2, nz + 2))
    ref[1:-1, 1:-1, 1:-1] = O.fft_poisson(R, O.fft_eigenvalues(nx, ny, nz, dx, dy, dz))
    O.pr_bc_staggered(ref, O.Faces.zeros(nx, ny, nz), cfg.pbc, dx, dy, dz)
    with session(cfg, poisson_z=poisson_z) as s:
        got = s.poisson(R)
    assert rel_l2(got, ref) < ROUTINE_TOL
    # operator check: the interior solves the restated Poisson operator
    L = O.poisson_lhs_staggered(nx, ny, nz, dx * dx, dy * dy, dz * dz, (1, 1, 1))
    res = L @ got[1:-1, 1:-1, 1:-1].reshape(-1, order="F") - R.reshape(-1, order="F")
    assert np.abs(res).max() < 1e-9 * np.abs(R).max() * max(1.0, 1 / dx ** 2)


@pytest.mark.parametrize("closure", [0, 1])
@pytest.mark.parametrize("g", GRIDS)
def test_adi_periodic(g, closure):
    nx, ny, nz, fx, fy, fz = g
    cfg = O.Config(nx, ny, nz, lx=2 * np.pi * fx, ly=2 * np.pi * fy, lz=2 * np.pi * fz, nu=0.05, dt=0.01,
                   scheme=O.AB2_CN)
    st = random_state(cfg, 3)
    dx, dy, dz = cfg.h
    orig = O.mat_cn
    if closure:
        def fixed(n, bc, dx2, dt0, nu):
            A, B = orig(n, bc, dx2, dt0, nu)
            if bc == 1:
                of = A[1, 0]; A[0, n] = 0.0; A[0, n - 1] = of
            return A, B
        O.mat_cn = fixed
    try:
        cnf = O.CNFactors(nx, ny, nz, cfg.bc, dx * dx, dy * dy, dz * dz, cfg.dt, cfg.nu)
        ref = O.adi_sweeps(st.u, st.v, st.w, cnf, cfg.bc)
    finally:
        O.mat_cn = orig
    with session(cfg, cn_periodic_closure=closure) as s:
        got = s.adi(st.u, st.v, st.w)
    for a, b in zip(got, ref):
        assert rel_l2(a, b) < ROUTINE_TOL


def _run_compare(cfg, st, nsteps, **kw):
    ref = st.copy()
    with session(cfg, **kw) as s:
        s.set_state(st.u, st.v, st.w, st.p, None if st.first else (st.px, st.py, st.pz))
        for _ in range(nsteps):
            ref = O.step(ref, cfg)
            s.step(1)
            d = s.diag()
            assert d["max_div"] < DIV_TOL * max(1.0, np.abs(ref.u).max() / min(cfg.h))
        got = s.get_state()
    for k, r in (("u", ref.u), ("v", ref.v), ("w", ref.w), ("p", ref.p), ("hx", ref.px), ("hy", ref.py),
                 ("hz", ref.pz)):
        err = rel_l2(got[k], r)
        assert err < STEP_TOL, (k, err)
    return got, ref


@pytest.mark.parametrize("g", MAX_FFT_GRIDS)
def test_step_max_fft_axis(g):
    """Two AB2-CN steps with a 512-cell periodic axis (the largest FFT, the
    longest ADI lines) against the oracle."""
    nx, ny, nz, fx, fy, fz = g
    cfg = O.Config(nx, ny, nz, lx=2 * np.pi * fx, ly=2 * np.pi * fy, lz=2 * np.pi * fz, nu=0.02, dt=0.002,
                   scheme=O.AB2_CN)
    st = random_state(cfg, 17, history=True)
    _run_compare(cfg, st, 2)


def test_step_z_stages_agree():
    """Ten AB2-CN steps of a 64^3 random state with the cyclic z solve and with
    the z FFT agree to 1e-11 per field (the same operator, different rounding)."""
    cfg = O.Config(64, 64, 64, nu=0.01, dt=0.005, scheme=O.AB2_CN)
    st = random_state(cfg, 29, history=True)
    out = []
    for pz in (0, 1):
        with session(cfg, poisson_z=pz) as s:
            s.set_state(st.u, st.v, st.w, st.p, (st.px, st.py, st.pz))
            s.step(10)
            out.append(s.get_state())
    for k in ("u", "v", "w", "p"):
        assert rel_l2(out[0][k], out[1][k]) < 1e-11, k


@pytest.mark.parametrize("scheme", [O.EULER, O.AB2, O.AB2_CN])
@pytest.mark.parametrize("dp_flag", [0, 1])
def test_step_tgv_32(scheme, dp_flag):
    """32^3 Taylor-Green + noise, nu = 0.01, dt = 0.01, 10 steps from the Euler start."""
    cfg = O.Config(32, 32, 32, nu=0.01, dt=0.01, scheme=scheme, dp_flag=dp_flag)
    st = tgv_state(cfg)
    _run_compare(cfg, st, 10)


def test_step_restart_with_history():
    """Restart (history given): no Euler start, AB2-CN on a non-cubic box."""
    cfg = O.Config(32, 16, 64, lx=2 * np.pi, ly=np.pi, lz=4.0, nu=0.02, dt=0.005, scheme=O.AB2_CN)
    st = random_state(cfg, 21, amp=0.1, history=True)
    _run_compare(cfg, st, 5)


def test_step_graph_matches_eager():
    """Graph replay gives bitwise the same state as eager launches."""
    cfg = O.Config(32, 32, 32, nu=0.01, dt=0.01, scheme=O.AB2_CN)
    st = tgv_state(cfg)
    outs = []
    for g in (0, 1):
        with session(cfg, use_graph=g) as s:
            s.set_state(st.u, st.v, st.w, st.p)
            s.step(6)
            outs.append(s.get_state())
    for k in ("u", "v", "w", "p", "hx"):
        assert np.array_equal(outs[0][k], outs[1][k])


def test_determinism():
    cfg = O.Config(32, 32, 32, nu=0.01, dt=0.01, scheme=O.AB2)
    st = tgv_state(cfg)
    outs = []
    for _ in range(2):
        with session(cfg) as s:
            s.set_state(st.u, st.v, st.w, st.p)
            s.step(4)
            outs.append(s.get_state())
    assert all(np.array_equal(outs[0][k], outs[1][k]) for k in ("u", "v", "w", "p"))


@pytest.mark.parametrize("scheme,dpf,walls,n", [(O.AB2_CN, 0, None, (32, 16, 32)), (O.AB2, 1, None, (32, 16, 32)),
                                                (O.AB2_CN, 0, None, (16, 32, 128)), (O.AB2_CN, 1, "y", (32, 16, 64)),
                                                (O.EULER, 0, None, (16, 16, 64)), (O.AB2_CN, 1, "z", (32, 16, 96)),
                                                (O.AB2_CN, 0, None, (16, 16, 16))])
def test_step_host_equals_set_step_get(scheme, dpf, walls, n):
    """ns_step_host (z-slabs copied, scattered, predicted and swept in x and y
    while the next slab is in flight; with FFT x and y passes also the
    inverse passes, ghost fill and correction slab by slab, each slab copied
    out while the next is computed) gives the bits of ns_set_state + ns_step
    + ns_get_state, from an Euler start and with history."""
    kw = {"y": dict(bc=(1, 2, 1), pbc=(1, 3, 1)), "z": dict(bc=(1, 1, 2), pbc=(1, 1, 3))}.get(walls, {})
    cfg = O.Config(*n, nu=0.02, dt=0.01, scheme=scheme, dp_flag=dpf, **kw)
    st = random_state(cfg, 91, history=True)
    with session(cfg) as s:
        for hist in (None, (st.px, st.py, st.pz)):
            s.set_state(st.u, st.v, st.w, st.p, hist)
            s.step(1)
            ref = s.get_state()
            got = s.step_host(st.u, st.v, st.w, st.p, hist)
            for k in ref:
                assert np.array_equal(got[k], ref[k]), k


@pytest.mark.parametrize("n", [(32, 16, 64), (16, 16, 128)])
def test_step_host_in_place(n):
    """The Fortran driver's call passes the same arrays in and out
    (ns_step_host(h, u, v, w, p, rx, ry, rz, u, v, w, p, rx, ry, rz)): three
    in-place steps give the bits of three device-resident steps.  The copies
    out go after every copy in on the copy stream, so no output plane
    overwrites an input plane still to be read."""
    cfg = O.Config(*n, nu=0.02, dt=0.01, scheme=O.AB2_CN)
    st = random_state(cfg, 23, history=True)
    with session(cfg) as s:
        s.set_state(st.u, st.v, st.w, st.p, (st.px, st.py, st.pz))
        s.step(3)
        ref = s.get_state()
    arrs = {k: np.asfortranarray(a.copy()) for k, a in
            (("u", st.u), ("v", st.v), ("w", st.w), ("p", st.p), ("hx", st.px), ("hy", st.py), ("hz", st.pz))}
    ptrs = {k: a.ctypes.data for k, a in arrs.items()}
    with session(cfg) as s:
        for _ in range(3):
            got = s.step_host(arrs["u"], arrs["v"], arrs["w"], arrs["p"], (arrs["hx"], arrs["hy"], arrs["hz"]),
                              out=arrs)
            assert all(got[k].ctypes.data == ptrs[k] for k in arrs)  # really in place
    for k in ref:
        assert np.array_equal(arrs[k], ref[k]), k


def test_nonfinite_state_is_reported():
    """A NaN in the state spreads through the step; ns_get_diag reports it as
    NS_ERR_NONFINITE (the divergence maximum orders a NaN above every
    finite value) and the handle stays usable."""
    from ns_3d_staggered_dp_gb300 import NSError
    cfg = O.Config(16, 16, 16, nu=0.02, dt=0.01, scheme=O.AB2_CN)
    st = random_state(cfg, 5)
    bad = st.u.copy()
    bad[5, 6, 7] = np.nan
    with session(cfg) as s:
        s.set_state(bad, st.v, st.w, st.p)
        s.step(1)
        with pytest.raises(NSError) as e:
            s.diag()
        assert e.value.status == 3
        s.set_state(st.u, st.v, st.w, st.p)  # the same handle runs a clean step afterwards
        s.step(1)
        assert s.diag()["max_div"] < 1e-10


@pytest.mark.parametrize("case", [
    ((16, 16, 16), {}),                                  # one x tile, partly filled
    ((32, 16, 64), {"scheme": O.AB2, "dp_flag": 1}),
    ((48, 40, 24), {"bc": (2, 2, 2), "pbc": (3, 3, 3)}),  # ragged x and y tiles, walls everywhere
    ((64, 32, 32), {"bc": (1, 1, 2), "pbc": (1, 1, 3), "dp_flag": 1}),
])
def test_predictor_tile_loaders_agree(case, monkeypatch):
    """The predictor stages its tiles with cp.async, or with the
    tensor-memory-access loader (cp.async.bulk.tensor into an mbarrier ring)
    when NS_PREDICT_TMA=1 at ns_create: both give the same bits, for the
    device-resident step and for ns_step_host, on full and ragged tiles."""
    n, kw = case
    kw = dict(kw)
    scheme = kw.pop("scheme", O.AB2_CN)
    cfg = O.Config(*n, nu=0.02, dt=0.01, scheme=scheme, **kw)
    st = random_state(cfg, 57, history=True)
    hist = (st.px, st.py, st.pz)
    res = []
    for env in ("1", "0"):
        monkeypatch.setenv("NS_PREDICT_TMA", env)
        with session(cfg) as s:
            s.set_state(st.u, st.v, st.w, st.p, hist)
            s.step(2)
            dev = s.get_state()
            host = s.step_host(st.u, st.v, st.w, st.p, hist)
            assert s.diag()["max_div"] < DIV_TOL
        res.append((dev, host))
    for a, b in zip(res[0], res[1]):
        for k in a:
            assert np.array_equal(a[k], b[k]), k


def test_bounded_tile_wait_gives_up_and_the_device_stays_usable():
    """Failure detection of the predictor's TMA tile loader: its bounded
    mbarrier wait, run on a barrier armed for bytes that no copy delivers,
    gives up after the limit and reports NS_ERR_TIMEOUT; the context is
    usable afterwards (a step still matches the oracle)."""
    import ctypes

    from ns_3d_staggered_dp_gb300 import _lib
    lib = _lib.load()
    waited = ctypes.c_double()
    assert lib.ns_selftest_wait_timeout(5.0, ctypes.byref(waited)) == 4  # NS_ERR_TIMEOUT
    assert 5.0 <= waited.value < 500.0, waited.value
    assert lib.ns_selftest_wait_timeout(0.0, None) == 6  # NS_ERR_ARG
    cfg = O.Config(16, 16, 16, nu=0.01, dt=0.01, scheme=O.AB2_CN)
    st = tgv_state(cfg)
    ref = O.step(st.copy(), cfg)
    with session(cfg) as s:
        s.set_state(st.u, st.v, st.w, st.p)
        s.step(1)
        got = s.get_state()
    assert rel_l2(got["u"], ref.u) < 1e-10
