"""Wall-bounded boxes on the CUDA path vs the CPU oracle, through the C ABI.

Covers the non-periodic pressure solve (DCT_poisson_solver,
NS_functions.f90:1505-1630, with pr_bc_staggered_modify_rhs :1345-1400 and
pr_bc_staggered :1403-1464), its mix with periodic FFT axes, and full steps
with wall velocity BCs (vel_bc_staggered :213-310, the banded CN-ADI of
re_simulation_sub_tstep_interBC_combine.f90:656-701 with per-sweep faces).

The wall axes are transformed through FFTs (Makhoul DCT-II/III: 24, 48 and
powers of two from 32 to 512 cells, codes 2 and 3) or by exact dense pairs
(the other sizes and code 4); the last wall axis is solved line by line
(the twisted factorisation from a multiplier table, the singular line by a
warp; the one-lane Thomas solve below 8 rows).  The cases cover each.

Tolerances: the trigonometric transforms and the tridiagonal line solves
round differently from the oracle's scipy DCT/DST, and the wall Poisson
problem is less well conditioned than the periodic one, so the routine bound
is a relative L2 of 1e-11; full steps keep the 1e-10 per-field bound and
max|div u| <= 1e-12.
"""
import numpy as np
import pytest

from oracle import ns_oracle as O
from tests.helpers import random_state, rel_l2

pytestmark = pytest.mark.gpu

POISSON_TOL = 1e-11
STEP_TOL = 1e-10
DIV_TOL = 1e-12


def session(cfg, **kw):
    from ns_3d_staggered_dp_gb300 import Session, make_config
    return Session(make_config(cfg.nx, cfg.ny, cfg.nz, lx=cfg.lx, ly=cfg.ly, lz=cfg.lz, nu=cfg.nu, dt=cfg.dt,
                               scheme=cfg.scheme, bc=cfg.bc, pbc=cfg.pbc, dp_flag=cfg.dp_flag, gauge=cfg.gauge,
                               mean_dp=cfg.mean_dp, **kw))


def random_faces(cfg, seed, amp=1.0):
    rng = np.random.default_rng(seed)
    shp = O.Faces.shapes(cfg.nx, cfg.ny, cfg.nz)
    return O.Faces({k: amp * rng.standard_normal(s) for k, s in shp.items()})


# (grid, pbc): every pure wall code, mixed wall codes, and the periodic/wall mixes
POISSON_CASES = [
    ((32, 16, 24), (3, 3, 3)),
    ((32, 16, 24), (2, 2, 2)),
    ((16, 24, 32), (4, 4, 4)),
    ((24, 32, 16), (2, 3, 4)),
    ((48, 24, 16), (3, 4, 2)),
    ((32, 24, 16), (1, 3, 1)),
    ((32, 16, 32), (1, 2, 1)),
    ((16, 16, 32), (1, 4, 1)),
    ((32, 32, 24), (1, 1, 3)),
    ((16, 32, 16), (1, 1, 2)),
    ((32, 24, 16), (1, 3, 3)),
    ((64, 48, 24), (1, 2, 4)),
    ((32, 256, 16), (1, 3, 1)),
    ((16, 32, 256), (1, 1, 2)),
    ((32, 128, 200), (1, 4, 3)),
    ((64, 64, 64), (3, 3, 3)),
    # the size limits: the wall axis solved by lines (512), a dense y in front of it (512:
    # past 128 its line buffer needs the opt-in shared memory), a dense x (1024, with its
    # line axis limited to 256)
    ((16, 16, 512), (1, 1, 3)),
    ((16, 128, 512), (1, 2, 4)),
    ((16, 200, 16), (3, 3, 3)),
    ((16, 512, 16), (1, 2, 3)),
    ((1024, 16, 16), (3, 3, 3)),
    # FFT-based DCT x passes (power-of-two nx, codes 2 and 3) at their size limits
    ((512, 16, 24), (2, 3, 3)),
    ((128, 32, 16), (3, 2, 2)),
    ((256, 12, 10), (2, 4, 3)),
    # the twisted line solve: an odd solve axis (singular, periodic x), a long Neumann solve axis
    # whose singular line's warp segments do not divide evenly, and a short one on the one-lane path
    ((32, 16, 21), (1, 3, 3)),
    ((16, 16, 200), (3, 3, 3)),
    ((16, 24, 7), (3, 3, 3)),
]


@pytest.mark.parametrize("grid,pbc", POISSON_CASES)
def test_poisson_walls(grid, pbc):
    nx, ny, nz = grid
    singular = all(p in (1, 3) for p in pbc)
    bc = tuple(1 if p == 1 else 2 for p in pbc)
    cfg = O.Config(nx, ny, nz, lx=1.0, ly=0.8, lz=1.3, bc=bc, pbc=pbc, mean_dp=0.3 if singular else 0.0)
    rng = np.random.default_rng(hash((grid, pbc)) % 2**32)
    R = rng.standard_normal((nx, ny, nz))
    faces = random_faces(cfg, 7)
    dx, dy, dz = cfg.h
    ref = np.zeros((nx + 2, ny + 2, nz + 2))
    ref[1:-1, 1:-1, 1:-1] = O.poisson_solve(R, cfg, faces)
    O.pr_bc_staggered(ref, faces, pbc, dx, dy, dz)
    with session(cfg) as s:
        s.set_faces(faces.d, 0)
        got = s.poisson(R)
    assert rel_l2(got, ref) < POISSON_TOL
    # the interior solves the reference operator (the BC terms are in R already)
    L = O.poisson_lhs_staggered(nx, ny, nz, dx * dx, dy * dy, dz * dz, pbc)
    res = L @ got[1:-1, 1:-1, 1:-1].reshape(-1, order="F") - R.reshape(-1, order="F")
    scale = np.abs(got).max() * 4.0 / min(dx, dy, dz) ** 2
    if singular:  # the operator has a null space; compare against the mean-free residual
        res = res - res.mean()
    assert np.abs(res).max() < 1e-11 * scale
    if singular:
        assert abs(got[1:-1, 1:-1, 1:-1].mean() - cfg.mean_dp) < 1e-12


def _run_compare(cfg, st, nsteps, faces=None, cn_faces=None, div_free=True, **kw):
    ref = st.copy()
    cnf = None
    if cfg.scheme == O.AB2_CN:
        dx, dy, dz = cfg.h
        cnf = O.CNFactors(cfg.nx, cfg.ny, cfg.nz, cfg.bc, dx * dx, dy * dy, dz * dz, cfg.dt, cfg.nu)
    with session(cfg, **kw) as s:
        if faces is not None:
            s.set_faces(faces.d, 0)
        if cn_faces is not None:
            for d in range(3):
                s.set_faces(cn_faces[d].d, d + 1)
        s.set_state(st.u, st.v, st.w, st.p, None if st.first else (st.px, st.py, st.pz))
        umax = max(np.abs(st.u).max(), np.abs(st.v).max(), np.abs(st.w).max(), 1.0)
        for _ in range(nsteps):
            ref = O.step(ref, cfg, faces=faces, cn_faces=cn_faces, cnf=cnf)
            s.step(1)
            d = s.diag()
            if div_free:
                assert d["max_div"] < DIV_TOL * umax / min(cfg.h), d
            else:  # incompatible Neumann data: the projection leaves mean(R) dt in every cell
                ref_div = O.max_div(ref.u, ref.v, ref.w, *cfg.h)
                assert abs(d["max_div"] - ref_div) < 1e-9 * max(ref_div, 1.0), (d, ref_div)
        got = s.get_state()
    for k, r in (("u", ref.u), ("v", ref.v), ("w", ref.w), ("p", ref.p), ("hx", ref.px), ("hy", ref.py),
                 ("hz", ref.pz)):
        err = rel_l2(got[k], r)
        assert err < STEP_TOL, (k, err)
    return got, ref


def channel_state(cfg, seed=3, amp=0.05):
    """Laminar parabolic profile in x between y walls plus a seeded
    divergence-free perturbation (the small-box stand-in for the
    256x128x256 wall-bounded configuration)."""
    st = random_state(cfg, seed, amp=amp)
    y = (np.arange(cfg.ny + 2) - 0.5) * cfg.ly / cfg.ny  # cell centres, ghosts included
    prof = 4.0 * y * (cfg.ly - y) / cfg.ly ** 2
    st.u = st.u + prof[None, :, None]
    from tests.helpers import project
    return project(st, cfg)


@pytest.mark.parametrize("scheme", [O.EULER, O.AB2, O.AB2_CN])
def test_step_channel(scheme):
    """x, z periodic, y no-slip walls (bc 2) with Neumann pressure (pbc 3)."""
    cfg = O.Config(32, 16, 32, lx=2 * np.pi, ly=2.0, lz=np.pi, nu=1.0 / 180, dt=2e-3, scheme=scheme,
                   bc=(1, 2, 1), pbc=(1, 3, 1))
    _run_compare(cfg, channel_state(cfg), 10)


@pytest.mark.parametrize("scheme", [O.AB2, O.AB2_CN])
@pytest.mark.parametrize("dp_flag", [0, 1])
def test_step_open_box_faces(scheme, dp_flag):
    """All-wall subdomain (bc 2, pbc 3) driven by random faces: a re-simulation
    step with given boundary values, per-sweep ADI faces and a mean dp."""
    cfg = O.Config(24, 16, 32, lx=0.75, ly=0.5, lz=1.0, nu=0.01, dt=1e-3, scheme=scheme, bc=(2, 2, 2),
                   pbc=(3, 3, 3), dp_flag=dp_flag, mean_dp=0.05)
    faces = random_faces(cfg, 11, amp=0.1)
    cn_faces = [random_faces(cfg, 12 + d, amp=0.1) for d in range(3)] if scheme == O.AB2_CN else None
    st = random_state(cfg, 5, amp=0.2)
    # random faces carry a net flux that Neumann pressure data cannot remove
    _run_compare(cfg, st, 6, faces=faces, cn_faces=cn_faces, div_free=False)


def test_step_all_wall_box_with_a_long_dense_y():
    """An all-wall box whose dense y transform is longer than 128 points (the
    line buffer of the y passes then opts in to more shared memory): AB2-CN
    steps with wall faces against the oracle."""
    cfg = O.Config(16, 192, 24, lx=0.5, ly=6.0, lz=0.75, nu=0.01, dt=1e-3, scheme=O.AB2_CN, bc=(2, 2, 2),
                   pbc=(3, 3, 3), dp_flag=1, mean_dp=0.02)
    faces = random_faces(cfg, 21, amp=0.1)
    cn_faces = [random_faces(cfg, 22 + d, amp=0.1) for d in range(3)]
    st = random_state(cfg, 23, amp=0.2)
    _run_compare(cfg, st, 4, faces=faces, cn_faces=cn_faces, div_free=False)


@pytest.mark.parametrize("pbc", [3, 2])
def test_step_all_wall_box_fft_transforms(pbc):
    """An all-wall box whose x and y transforms go through FFTs (x 64 points,
    y 48 through the 12-point DFT) and whose z axis takes the twisted line
    solve: AB2-CN steps with wall faces against the oracle."""
    cfg = O.Config(64, 48, 32, lx=1.0, ly=0.75, lz=0.5, nu=0.01, dt=1e-3, scheme=O.AB2_CN, bc=(2, 2, 2),
                   pbc=(pbc,) * 3, dp_flag=1, mean_dp=0.02 if pbc == 3 else 0.0)
    faces = random_faces(cfg, 31, amp=0.1)
    cn_faces = [random_faces(cfg, 32 + d, amp=0.1) for d in range(3)]
    st = random_state(cfg, 33, amp=0.2)
    _run_compare(cfg, st, 4, faces=faces, cn_faces=cn_faces, div_free=False)


@pytest.mark.parametrize("bc,pbc", [((4, 2, 4), (4, 2, 4)), ((2, 4, 2), (2, 3, 2)), ((2, 2, 4), (3, 2, 4))])
def test_step_wall_codes(bc, pbc):
    """Dirichlet-on-the-ghost (4) and Dirichlet-on-the-wall (2) codes mixed,
    AB2-CN with per-sweep faces and the Euler start."""
    cfg = O.Config(16, 24, 16, lx=0.5, ly=0.75, lz=0.5, nu=0.02, dt=1e-3, scheme=O.AB2_CN, bc=bc, pbc=pbc)
    faces = random_faces(cfg, 21, amp=0.1)
    cn_faces = [random_faces(cfg, 22 + d, amp=0.1) for d in range(3)]
    st = random_state(cfg, 8, amp=0.2)
    _run_compare(cfg, st, 5, faces=faces, cn_faces=cn_faces)


def test_step_channel_graph_matches_eager():
    cfg = O.Config(32, 16, 32, lx=2 * np.pi, ly=2.0, lz=np.pi, nu=1.0 / 180, dt=2e-3, scheme=O.AB2_CN,
                   bc=(1, 2, 1), pbc=(1, 3, 1))
    st = channel_state(cfg)
    outs = []
    for g in (0, 1):
        with session(cfg, use_graph=g) as s:
            s.set_state(st.u, st.v, st.w, st.p)
            s.step(5)
            outs.append(s.get_state())
    for k in ("u", "v", "w", "p", "hx"):
        assert np.array_equal(outs[0][k], outs[1][k])


def test_unsupported_mixes_rejected():
    from ns_3d_staggered_dp_gb300 import NSError
    bad = [
        dict(nx=32, ny=16, nz=32, bc=(2, 1, 1), pbc=(3, 1, 1)),   # wall x with periodic y/z
        dict(nx=32, ny=1024, nz=32, bc=(1, 2, 1), pbc=(1, 3, 1)),  # line-solved y longer than 512
        dict(nx=32, ny=640, nz=32, bc=(1, 2, 2), pbc=(1, 3, 3)),   # dense y (wall z behind it) over 512
        dict(nx=24, ny=16, nz=32, bc=(1, 2, 1), pbc=(1, 3, 1)),   # FFT x not a power of two
        dict(nx=25, ny=16, nz=32, bc=(2, 2, 2), pbc=(3, 3, 3)),   # odd wall x
    ]
    for kw in bad:
        cfg = O.Config(kw["nx"], kw["ny"], kw["nz"], bc=kw["bc"], pbc=kw["pbc"])
        with pytest.raises(NSError):
            session(cfg)


ROUTINE_BCS = [(1, 1, 1), (1, 2, 1), (1, 1, 2), (1, 2, 2), (2, 2, 2)]  # a wall x needs walls in y and z


@pytest.mark.parametrize("bc", ROUTINE_BCS)
def test_vel_bc_routine(bc):
    """ns_vel_bc against vel_bc_staggered (NS_functions.f90:213-310) with
    random face values: periodic images and wall ghosts/faces."""
    pbc = tuple(1 if b == 1 else 3 for b in bc)
    cfg = O.Config(32, 16, 32, lx=1.0, ly=0.7, lz=1.2, bc=bc, pbc=pbc)
    st = random_state(cfg, 29)
    rng = np.random.default_rng(31)
    us, vs, ws = (rng.standard_normal(a.shape) for a in (st.u, st.v, st.w))
    faces = random_faces(cfg, 37)
    ref = [us.copy(), vs.copy(), ws.copy()]
    O.vel_bc_staggered(*ref, faces, *bc)
    with session(cfg) as s:
        s.set_faces(faces.d, 0)
        got = s.vel_bc(us, vs, ws)
    for a, b in zip(got, ref):
        assert a.shape == b.shape
        assert np.max(np.abs(a - b)) <= 1e-13 * max(1.0, np.max(np.abs(b)))


@pytest.mark.parametrize("bc", [(1, 1, 1), (1, 2, 1), (2, 2, 2)])
@pytest.mark.parametrize("dp_flag,gauge", [(0, 1), (1, 1), (1, 0)])
def test_correct_routine(bc, dp_flag, gauge):
    """ns_correct against the gauge and correction of
    big_periodic_3D.f90:562-567 over the full padded arrays."""
    pbc = tuple(1 if b == 1 else 3 for b in bc)
    cfg = O.Config(32, 16, 32, lx=1.0, ly=0.7, lz=1.2, dt=0.003, bc=bc, pbc=pbc, dp_flag=dp_flag, gauge=gauge)
    st = random_state(cfg, 41)
    rng = np.random.default_rng(43)
    us, vs, ws = (rng.standard_normal(a.shape) for a in (st.u, st.v, st.w))
    dp = rng.standard_normal(st.p.shape)
    p = rng.standard_normal(st.p.shape)
    dx, dy, dz = cfg.h
    ref = O.correct(us, vs, ws, dp, p, dx, dy, dz, cfg.dt, dp_flag, gauge)
    with session(cfg) as s:
        got = s.correct(us, vs, ws, dp, p)
    for k, b in zip(("u", "v", "w", "p"), ref):
        a = got[k]
        assert a.shape == b.shape, k
        assert np.max(np.abs(a - b)) <= 1e-13 * max(1.0, np.max(np.abs(b))), k


def test_nan_poisoned_faces_are_reported():
    """A NaN in one boundary face array (the parent data of a re-simulation)
    reaches the interior: a pressure face of set 0 enters the Poisson
    right-hand side and the pressure ghosts (with AB2-CN the velocity faces
    of set 0 are not read: the sweeps take sets 1-3).  ns_get_diag reports
    it as NS_ERR_NONFINITE, and the handle runs a clean step once the faces
    are replaced."""
    from ns_3d_staggered_dp_gb300 import NSError
    cfg = O.Config(32, 16, 32, lx=1.0, ly=0.7, lz=1.2, nu=0.02, dt=0.002, bc=(1, 2, 1), pbc=(1, 3, 1),
                   scheme=O.AB2_CN)
    st = random_state(cfg, 47)
    good = random_faces(cfg, 53, amp=0.1)
    bad = {k: v.copy() for k, v in good.d.items()}
    bad["y_p_1"][7, 9] = np.nan
    with session(cfg) as s:
        s.set_faces(bad, 0)
        s.set_state(st.u, st.v, st.w, st.p)
        s.step(1)
        with pytest.raises(NSError) as e:
            s.diag()
        assert e.value.status == 3
        s.set_faces(good.d, 0)
        s.set_state(st.u, st.v, st.w, st.p)
        s.step(1)
        assert np.isfinite(s.diag()["max_div"])
