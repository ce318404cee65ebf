"""CPU checks of the oracle itself (no GPU): the reference's own self-checks
restated, the operator identities the spectral solvers must satisfy, and the
accuracy properties the reference logs in err_file/."""
import dataclasses

import numpy as np
import pytest

from oracle import ns_oracle as O
from tests.helpers import project, random_state, rel_l2, tgv_state


@pytest.mark.parametrize("k", [1, 2, 3])
@pytest.mark.parametrize("bc", [0, 1])
def test_fd_primitives_new_equal_legacy_bitwise(k, bc):
    """test_subroutine.f90:137-185: the new avg/diff/diff2 equal the legacy ones bitwise."""
    rng = np.random.default_rng(7)
    A = rng.standard_normal((9, 8, 7))
    assert np.array_equal(O.avg(A, k, bc), O.avg_old(A, k, bc))
    assert np.array_equal(O.diff(A, 1, k), O.diff_old(A, 1, k))
    assert np.array_equal(O.diff2(A, k, bc), O.diff2_old(A, k, bc))


def test_fd_primitive_definitions():
    A = np.arange(5.0)[:, None, None] ** 2 * np.ones((5, 2, 2))
    assert np.allclose(O.diff(A, 1, 1)[:, 0, 0], [1, 3, 5, 7])
    assert np.allclose(O.diff2(A, 1, 0)[:, 0, 0], [2, 2, 2])
    # periodic diff2 wraps to A(n-1): B(1) = A(n-1) - 2A(1) + A(2)
    assert O.diff2(A, 1, 1)[0, 0, 0] == A[3, 0, 0] - 2 * A[0, 0, 0] + A[1, 0, 0]
    # periodic avg: B(1) = (A(n)+A(n-1))/2
    assert O.avg(A, 1, 1)[0, 0, 0] == (A[4, 0, 0] + A[3, 0, 0]) / 2


PBCS = [(1, 1, 1), (3, 3, 3), (2, 2, 2), (4, 4, 4), (2, 3, 4), (1, 3, 1), (1, 2, 1), (3, 1, 2)]


@pytest.mark.parametrize("pbc", PBCS)
def test_spectral_poisson_solves_the_lu_operator(pbc):
    """Poisson_LHS_staggered (NS_functions.f90:1110-1242) is the operator all
    spectral solvers invert; compare with a sparse LU solve as the reference
    prints at re_simulation_sub_tstep_interBC_combine.f90:780."""
    nx, ny, nz = 8, 6, 10
    dx, dy, dz = 0.3, 0.2, 0.25
    rng = np.random.default_rng(3)
    R = rng.standard_normal((nx, ny, nz))
    singular = all(p in (1, 3) for p in pbc)
    if singular:
        R -= R.mean()
    cfg = O.Config(nx, ny, nz, lx=nx * dx, ly=ny * dy, lz=nz * dz, pbc=pbc, bc=tuple(1 if p == 1 else 2 for p in pbc))
    a = O.poisson_solve(R, cfg, None)
    L = O.poisson_lhs_staggered(nx, ny, nz, dx * dx, dy * dy, dz * dz, pbc)
    res = L @ a.reshape(-1, order="F") - R.reshape(-1, order="F")
    assert np.abs(res).max() < 1e-12 * np.abs(R).max() / min(dx, dy, dz) ** 2
    if not singular:
        b = O.lu_poisson(R, pbc, dx, dy, dz)
        assert rel_l2(a, b) < 1e-12
    else:
        assert abs(a.mean()) < 1e-13


def test_dct_poisson_mean_mode():
    """The singular Neumann mode is set to mean_dp (NS_functions.f90:1576-1577)."""
    n = 8
    rng = np.random.default_rng(1)
    R = rng.standard_normal((n, n, n))
    R -= R.mean()
    cfg = O.Config(n, n, n, lx=1.0, ly=1.0, lz=1.0, pbc=(3, 3, 3), bc=(2, 2, 2), mean_dp=0.37)
    a = O.poisson_solve(R, cfg, None)
    assert abs(a.mean() - 0.37) < 1e-14


def test_manufactured_2d_dst_dct():
    """test_subroutine.f90:275-388: p = (1-x^2)(2y^3-3y^2+1) on [0,1]^2, Dirichlet
    (DST-2) in x and Neumann (DCT-2) in y; second-order convergence of the
    staggered solution (BC values consistent with the exact solution)."""
    errs = []
    for n in (32, 64):
        h = 1.0 / n
        xc = (np.arange(n) + 0.5) * h
        X, Y = np.meshgrid(xc, xc, indexing="ij")
        exact = (1 - X ** 2) * (2 * Y ** 3 - 3 * Y ** 2 + 1)
        rhs = -2 * (2 * Y ** 3 - 3 * Y ** 2 + 1) + 6 * (1 - X ** 2) * (2 * Y - 1)
        # as a 3D problem with one z cell and Neumann in z
        R = rhs[:, :, None].copy()
        f = {"x_p_1": (2 * xc ** 3 * 0 + (2 * xc ** 3 - 3 * xc ** 2 + 1))[:, None],   # p(0,y)
             "x_p_n": np.zeros((n, 1)),
             "y_p_1": np.zeros((n, 1)), "y_p_n": np.zeros((n, 1)),
             "z_p_1": np.zeros((n, n)), "z_p_n": np.zeros((n, n))}
        f["x_p_1"] = (2 * xc ** 3 - 3 * xc ** 2 + 1)[:, None]
        O.pr_bc_staggered_modify_rhs(R, f, (2, 3, 3), h, h, 1.0)
        cfg = O.Config(n, n, 1, lx=1.0, ly=1.0, lz=1.0, pbc=(2, 3, 3), bc=(2, 2, 2))
        a = O.poisson_solve(R, cfg, None)[:, :, 0]
        errs.append(np.abs(a - exact).max())
    order = np.log2(errs[0] / errs[1])
    assert errs[1] < 1e-3 and order > 1.8


@pytest.mark.parametrize("bc", [(1, 1, 1), (2, 2, 2), (4, 4, 4), (1, 2, 1)])
def test_cn_tridiagonal_matches_dense(bc):
    """mat_CN_tridiagonal (dttrsb path) and mat_CN (getrs path) are the same
    matrices for bc != 1 (NS_functions.f90:1245-1342)."""
    import scipy.linalg as sla
    for b in set(bc):
        if b == 1:
            continue
        A, B = O.mat_cn(12, b, 0.01, 0.01, 0.3)
        al, ad, au, bl, bd, bu = O.mat_cn_tridiagonal(12, b, 0.01, 0.01, 0.3)
        assert np.array_equal(np.diag(A), ad) and np.array_equal(np.diag(A, 1), au) and np.array_equal(np.diag(A, -1), al)
        assert np.array_equal(np.diag(B), bd) and np.array_equal(np.diag(B, 1), bu) and np.array_equal(np.diag(B, -1), bl)
        r = np.random.default_rng(0).standard_normal(13)
        x1 = np.linalg.solve(A, r)
        x2 = sla.solve_banded((1, 1), np.vstack([np.r_[0, au], ad, np.r_[al, 0]]), r)
        assert np.allclose(x1, x2, rtol=1e-13, atol=1e-14)


def test_periodic_cn_reference_closure():
    """For bc=1 the reference closes row 1 of the face matrix on the duplicate
    face (A(1,nx+1), NS_functions.f90:1273): with x(n+1) = x(1) this folds the
    off-diagonal into the diagonal of row 1."""
    A, B = O.mat_cn(8, 1, 0.01, 0.01, 0.3)
    assert A[0, 8] == A[1, 0] and A[0, 7] == 0.0
    assert A[8, 8] == 1.0 and A[8, 0] == -1.0
    assert B[0, 0] == 1.0 and B[0, 8] == -1.0 and B[9, 9] == 1.0 and B[9, 1] == -1.0


@pytest.mark.parametrize("scheme", [O.EULER, O.AB2, O.AB2_CN])
def test_step_projects_to_zero_divergence(scheme):
    cfg = O.Config(16, 16, 16, nu=0.01, dt=0.01, scheme=scheme)
    st = tgv_state(cfg)
    for _ in range(3):
        st = O.step(st, cfg)
        assert O.max_div(st.u, st.v, st.w, *cfg.h) < 1e-12


def test_tgv_2d_viscous_decay():
    """2D Taylor-Green (NS_functions.f90:18-50): u, v decay as exp(-2 nu t)."""
    n = 32
    nu, dt, steps = 0.05, 0.01, 20
    cfg = O.Config(n, n, 8, lz=2 * np.pi, nu=nu, dt=dt, scheme=O.AB2)
    c = O.staggered_coords(n, n, 8, cfg.lx, cfg.ly, cfg.lz)
    st = O.State.zeros(n, n, 8)
    st.u = O.tgv(*c["u"], 0.0, nu, "u")
    st.v = O.tgv(*c["v"], 0.0, nu, "v")
    st.p = O.tgv(*c["p"], 0.0, nu, "p")
    for _ in range(steps):
        st = O.step(st, cfg)
    ex = O.tgv(*c["u"], dt * steps, nu, "u")
    assert rel_l2(st.u[:, 1:-1, 1:-1], ex[:, 1:-1, 1:-1]) < 5e-3


def _order(scheme, dts, T=0.08, n=16):
    cfg0 = O.Config(n, n, n, nu=0.02, dt=dts[0], scheme=scheme)
    st0 = tgv_state(cfg0, noise=0.0)
    # non-trivial nonlinear flow: perturb with a smooth mode
    c = O.staggered_coords(n, n, n, cfg0.lx, cfg0.ly, cfg0.lz)
    xw, yw, zw = c["w"]
    st0.w = 0.3 * np.sin(xw)[:, None, None] * np.sin(yw)[None, :, None] * np.cos(zw)[None, None, :]
    st0 = project(st0, cfg0)
    sols = []
    for dt in list(dts) + [dts[-1] / 8]:
        cfg = O.Config(n, n, n, nu=0.02, dt=dt, scheme=scheme)
        st = st0.copy()
        for _ in range(int(round(T / dt))):
            st = O.step(st, cfg)
        sols.append(st.u)
    ref = sols[-1]
    errs = [np.abs(s - ref).max() for s in sols[:-1]]
    return np.log2(errs[0] / errs[1])


def test_temporal_order_euler_and_ab2():
    """err_file time-order logs (MATLAB err_time_scheme.m:64-65): Euler first
    order, AB2 second order in dt."""
    assert 0.8 < _order(O.EULER, [0.01, 0.005]) < 1.3
    assert 1.7 < _order(O.AB2, [0.01, 0.005]) < 2.4


def test_subdomain_index_maps():
    """big_periodic_3D.f90:20-25 (1-based parent indices), bit-exact."""
    m = O.subdomain_index_maps(16, 16, 16, 32, 32, 32)
    assert m["xu"][0] == 16 and m["xu"][-1] == 48 and len(m["xu"]) == 33
    assert len(m["yu"]) == 34 and m["yu"][-1] == 49
    assert len(m["zw"]) == 33 and len(m["xp"]) == 34
    assert m["xu"].dtype == np.int64


def test_power_spec_single_mode_and_parseval():
    """PowerSpec.m / SpecProp.m restated: a cos(2x) field puts all its energy
    in shell 2, and kin_E (spectral) equals kin_Ph (physical)."""
    n = 16
    x = (np.arange(n) + 0.5) * 2 * np.pi / n
    u = np.cos(2 * x)[:, None, None] * np.ones((n, n, n))
    z = np.zeros((n, n, n))
    k, E, c, dk, m = O.power_spec(u, z, z, 2 * np.pi)
    others = np.delete(E, 1)
    assert E[1] > 0 and np.all(np.abs(others) < 1e-25 * E[1])
    p = O.spec_prop(E, k, 0.01, u, z, z, n, dk, m)
    assert abs(p["kin_E"] - p["kin_Ph"]) < 1e-14 and abs(p["kin_Ph"] - 0.25) < 1e-14


def test_sweep_faces_are_the_parent_records():
    """O.sweep_faces restates the per-sweep records of big_periodic_3D.f90:433-489
    on a sub-block: after the x sweep bx_u_1s = u_star(idx_xu(1), ...),
    bx_v_1s = (v_star(idx_xv(1), ...) + v_star(idx_xv(2), ...)) * 0.5d0, ...;
    only the swept axis's velocity faces are set."""
    rng = np.random.default_rng(11)
    nx, ny, nz = 6, 5, 4
    u = rng.standard_normal((nx + 1, ny + 2, nz + 2))
    v = rng.standard_normal((nx + 2, ny + 1, nz + 2))
    w = rng.standard_normal((nx + 2, ny + 2, nz + 1))
    fx = O.sweep_faces(u, v, w, 0, 2)
    assert np.array_equal(fx.d["x_u_1"], u[0]) and np.array_equal(fx.d["x_u_n"], u[nx])
    assert np.array_equal(fx.d["x_v_1"], (v[0] + v[1]) * 0.5)
    assert np.array_equal(fx.d["x_w_n"], (w[nx + 1] + w[nx]) * 0.5)
    assert not fx.d["y_u_1"].any() and not fx.d["x_p_1"].any()
    fy = O.sweep_faces(u, v, w, 1, 2)
    assert np.array_equal(fy.d["y_u_1"], (u[:, 0] + u[:, 1]) * 0.5)
    assert np.array_equal(fy.d["y_v_n"], v[:, ny])
    fz = O.sweep_faces(u, v, w, 2, 2)
    assert np.array_equal(fz.d["z_w_1"], w[:, :, 0]) and np.array_equal(fz.d["z_w_n"], w[:, :, nz])
    assert np.array_equal(fz.d["z_v_n"], (v[:, :, nz + 1] + v[:, :, nz]) * 0.5)


def test_velpr_bc_u_branch_adds_the_previous_pressure_gradient():
    """get_velpr_bc with u boundary values and dp_flag = 0 adds
    dt * diff(p_previous) / h to the velocity before taking the faces
    (NS_functions.f90:434-437); with u* or dp_flag = 1 it does not."""
    rng = np.random.default_rng(12)
    nx, ny, nz = 6, 5, 4
    u = rng.standard_normal((nx + 1, ny + 2, nz + 2))
    v = rng.standard_normal((nx + 2, ny + 1, nz + 2))
    w = rng.standard_normal((nx + 2, ny + 2, nz + 1))
    p = rng.standard_normal((nx + 2, ny + 2, nz + 2))
    pp = rng.standard_normal((nx + 2, ny + 2, nz + 2))
    h, dt = 0.1, 0.01
    f0 = O.get_velpr_bc(u, v, w, p, (2, 2, 2), (3, 3, 3), h, h, h, dt, 0, False, pp)
    uc = u + O.diff(pp, 1, 1) / h * dt
    vc = v + O.diff(pp, 1, 2) / h * dt
    assert np.array_equal(f0.d["x_u_1"], uc[0])
    assert np.array_equal(f0.d["y_u_n"], (uc[:, ny + 1] + uc[:, ny]) / 2)
    assert np.array_equal(f0.d["x_v_1"], (vc[0] + vc[1]) / 2)
    for dpf, ustar in ((1, False), (0, True)):
        f1 = O.get_velpr_bc(u, v, w, p, (2, 2, 2), (3, 3, 3), h, h, h, dt, dpf, ustar, pp)
        assert np.array_equal(f1.d["x_u_1"], u[0])
    # the pressure faces come from the pressure argument either way (get_pr_bc)
    assert np.array_equal(f0.d["x_p_1"], (p[1] - p[0]) / h)


def test_resimulate_frames_steps_with_the_frame_faces():
    """resimulate_frames follows re_simulation_sub_tstep_interBC_combine.f90:436-801:
    one step per frame with that frame's faces and the mean of its pressure
    source, p_sub_pre carried from frame to frame."""
    cfg = O.Config(8, 8, 8, lx=1.0, ly=1.0, lz=1.0, nu=0.01, dt=1e-3, scheme=O.AB2, bc=(2,) * 3, pbc=(3,) * 3,
                   dp_flag=0, gauge=0)
    rng = np.random.default_rng(13)
    st = O.State.zeros(8, 8, 8)
    st.u = 0.1 * rng.standard_normal(st.u.shape); st.v = 0.1 * rng.standard_normal(st.v.shape)
    st.w = 0.1 * rng.standard_normal(st.w.shape)
    st.first = False
    frames = []
    for _ in range(2):
        fr = {k: 0.1 * rng.standard_normal(getattr(st, k).shape) for k in ("u", "v", "w", "p")}
        fr.update(us=fr["u"], vs=fr["v"], ws=fr["w"], dp=fr["p"])
        frames.append(fr)
    p0 = 0.1 * rng.standard_normal(st.p.shape)
    got = O.resimulate_frames(st, cfg, frames, p0, using_ustar=False, dp_flag=0, restart=True)
    ref = st.copy()
    prev = p0
    h = cfg.h[0]
    for fr in frames:
        faces = O.get_velpr_bc(fr["u"], fr["v"], fr["w"], fr["p"], cfg.bc, cfg.pbc, h, h, h, cfg.dt, 0, False, prev)
        c = dataclasses.replace(cfg, mean_dp=float(np.mean(fr["p"][1:-1, 1:-1, 1:-1])))
        ref = O.step(ref, c, faces=faces)
        prev = fr["p"]
    for k in ("u", "v", "w", "p"):
        assert np.array_equal(getattr(got, k), getattr(ref, k))
