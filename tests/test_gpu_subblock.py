"""Sub-block extraction on the device, bit for bit.

The reference's sub-block is an integer gather, u_sub = u(idx_xu, idx_yu,
idx_zu) with idx_xu = x0 + (0..nx0) (big_periodic_3D.f90:20-25, 665-669), and
its boundary arrays come from get_velpr_bc / get_pr_bc on that sub-block
(NS_functions.f90:414-562) in two branches
(re_simulation_sub_tstep_interBC_combine.f90:506-519):
  - using_Ustar: faces from the parent's u*, pressure from dp;
  - u: faces from the parent's u, plus dt * diff(p_previous) / h when
    dp_flag = 0 (NS_functions.f90:434-437), pressure from p (dp_sub = p_sub).
Both are index work plus the reference's own two-operand arithmetic, so the
device results must equal the oracle's on the same parent arrays exactly
(np.array_equal).  A re-simulation driven by either branch must then agree
with the oracle's re-simulation loop to the step tolerance (1e-10 relative
L2 per field); the face means feed a reduction, compared at rtol 1e-13.
"""
import numpy as np
import pytest

from oracle import ns_oracle as O
from tests.helpers import rel_l2, tgv_state

pytestmark = pytest.mark.gpu

H = 2 * np.pi / 64
DT0 = 2e-3
NU = 0.01
STEP_TOL = 1e-10
SUBS = [(5, 9, 3, 16, 24, 16, 1), (30, 2, 20, 32, 16, 24, 1), (41, 40, 33, 24, 24, 32, 1), (1, 1, 1, 16, 16, 16, 1),
        (49, 33, 41, 16, 32, 24, 1)]  # the last two touch the parent's first and last cells


def _parent(dp_flag, n=64, steps=3):
    from ns_3d_staggered_dp_gb300 import Session, make_config
    cfg = O.Config(n, n, n, nu=NU, dt=DT0, scheme=O.AB2, dp_flag=dp_flag)
    st = tgv_state(cfg, seed=5, noise=0.05)
    s = Session(make_config(n, n, n, nu=NU, dt=DT0, scheme=O.AB2, dp_flag=dp_flag))
    s.set_state(st.u, st.v, st.w, st.p)
    s.step(steps)
    return s


def _make_batch(subs, **kw):
    from ns_3d_staggered_dp_gb300 import Batch
    return Batch(subs, scheme=O.AB2, bc=2, pbc=3, nu=NU, dt0=DT0, dx=H, dy=H, dz=H, n_slots=4, **kw)


def _interior_mask(shape_key, n):
    """1 where the parent's history is inside its interior ranges (ns_get_state
    returns 0 elsewhere): periodic own axis 1..n, other axes 2..n+1."""
    from ns_3d_staggered_dp_gb300 import shapes
    m = np.zeros(shapes(n, n, n)[shape_key], dtype=bool)
    ax = "uvw".index(shape_key)
    sl = [slice(1, n + 1)] * 3
    sl[ax] = slice(0, n)
    m[tuple(sl)] = True
    return m


def _frames(parent, subs):
    ps = parent.get_state(history=False)
    stg = parent.get_stage()
    out = []
    for x0, y0, z0, nx, ny, nz, _ in subs:
        maps = O.subdomain_index_maps(x0, y0, z0, nx, ny, nz)
        fr = {k: O.extract_sub(ps[k], k, maps) for k in ("u", "v", "w", "p")}
        for k in ("us", "vs", "ws"):
            fr[k] = O.extract_sub(stg[k], k[0], maps)
        fr["dp"] = O.extract_sub(stg["dp"], "p", maps)
        out.append(fr)
    return out


def test_init_from_parent_is_an_exact_gather():
    """ns_batch_init_from_parent == O.extract_sub over the index maps, every
    entry of u, v, w, p and every interior entry of the AB2 history."""
    n = 64
    parent = _parent(1)
    full = parent.get_state()
    with _make_batch(SUBS, restart=1) as b:
        b.init_from_parent(parent)
        for i, (x0, y0, z0, nx, ny, nz, _) in enumerate(SUBS):
            maps = O.subdomain_index_maps(x0, y0, z0, nx, ny, nz)
            got = b.get_state(i)
            for k in ("u", "v", "w", "p"):
                assert np.array_equal(got[k], O.extract_sub(full[k], k, maps)), (i, k)
            for k, f in (("hx", "u"), ("hy", "v"), ("hz", "w")):
                m = O.extract_sub(_interior_mask(f, n), f, maps)
                ref = O.extract_sub(full[k], f, maps)
                assert m.any()
                assert np.array_equal(got[k][m], ref[m]), (i, k)
    parent.close()


def test_index_maps_are_the_reference_vectors():
    """The maps the device gathers with: idx_xu = x0 + (0..nx0), idx_yu =
    y0 + (0..ny0+1), ... (big_periodic_3D.f90:22-25), 1-based, int."""
    m = O.subdomain_index_maps(16, 16, 16, 32, 32, 32)
    assert np.array_equal(m["xu"], 16 + np.arange(33)) and np.array_equal(m["yu"], 16 + np.arange(34))
    assert np.array_equal(m["yv"], 16 + np.arange(33)) and np.array_equal(m["zw"], 16 + np.arange(33))
    assert np.array_equal(m["xp"], 16 + np.arange(34))
    assert all(v.dtype == np.int64 for v in m.values())


@pytest.mark.parametrize("using_ustar,dp_flag", [(1, 1), (0, 1), (0, 0), (1, 0)])
def test_captured_faces_are_get_velpr_bc_and_drive_the_oracle_resimulation(using_ustar, dp_flag):
    """Each ns_batch_capture of the parent equals get_velpr_bc of the
    parent's own arrays bit for bit (both branches, dp_flag 0/1), and the
    restarted sub-blocks stepped with those faces follow the oracle's
    re-simulation loop (re_simulation_sub_tstep_interBC_combine.f90:436-801)."""
    from ns_3d_staggered_dp_gb300 import FACE_ORDER
    parent = _parent(dp_flag)
    full = parent.get_state()
    init, p_prev, frames = [], [], [[] for _ in SUBS]
    for x0, y0, z0, nx, ny, nz, _ in SUBS:
        maps = O.subdomain_index_maps(x0, y0, z0, nx, ny, nz)
        e = {k: O.extract_sub(full[k], k, maps) for k in ("u", "v", "w", "p")}
        h = [O.extract_sub(full[k], f, maps) for k, f in (("hx", "u"), ("hy", "v"), ("hz", "w"))]
        init.append(O.State(e["u"], e["v"], e["w"], e["p"], *h, first=False))
        p_prev.append(e["p"])
    p_prev0 = list(p_prev)
    with _make_batch(SUBS, restart=1, using_ustar=using_ustar, dp_flag=dp_flag) as b:
        b.init_from_parent(parent)
        b.capture(parent, 0, 0.0)  # the current p becomes the next capture's p_previous
        for n in range(1, 5):
            parent.step(1)
            slot = n % 4
            b.capture(parent, slot, n * DT0)
            frs = _frames(parent, SUBS)
            for i, fr in enumerate(frs):
                got, got_mean = b.get_snapshot(slot, i)
                dp_sub = fr["dp"] if dp_flag else fr["p"]
                vel = (fr["us"], fr["vs"], fr["ws"]) if using_ustar else (fr["u"], fr["v"], fr["w"])
                ref = O.get_velpr_bc(*vel, dp_sub, (2,) * 3, (3,) * 3, H, H, H, DT0, dp_flag, bool(using_ustar),
                                     p_prev[i])
                for k in FACE_ORDER:
                    assert np.array_equal(got[k], ref.d[k]), (n, i, k)
                assert np.isclose(got_mean, np.mean(dp_sub[1:-1, 1:-1, 1:-1]), rtol=1e-13, atol=1e-17)
                frames[i].append(fr)
                p_prev[i] = fr["p"]
            b.advance((n - 1) * DT0)
        for i, (_, _, _, nx, ny, nz, _) in enumerate(SUBS):
            cfg = O.Config(nx, ny, nz, lx=nx * H, ly=ny * H, lz=nz * H, nu=NU, dt=DT0, scheme=O.AB2, bc=(2,) * 3,
                           pbc=(3,) * 3, dp_flag=dp_flag, gauge=0)
            ref = O.resimulate_frames(init[i], cfg, frames[i], p_prev0[i], using_ustar=bool(using_ustar),
                                      dp_flag=dp_flag, restart=True)
            got = b.get_state(i, history=False)
            for k in ("u", "v", "w", "p"):
                err = rel_l2(got[k], getattr(ref, k))
                assert err < STEP_TOL, (i, k, err)
            # u boundary values carry a flux the projection does not see, so the
            # divergence is not at rounding level there: it must match the oracle's
            ref_div = O.max_div(ref.u, ref.v, ref.w, H, H, H)
            assert abs(b.max_div(i) - ref_div) <= 1e-12 + 1e-6 * ref_div, (b.max_div(i), ref_div)
            if using_ustar and dp_flag:  # the exact-replay case: divergence-free to rounding
                assert ref_div < 1e-10
    parent.close()


def test_u_branch_needs_single_substeps():
    """sub_tstep > 1 with u boundary values is rejected, as the reference
    stops (re_simulation_sub_tstep_interBC_combine.f90:360-363)."""
    from ns_3d_staggered_dp_gb300 import NSError
    with pytest.raises(NSError):
        _make_batch([(1, 1, 1, 16, 16, 16, 2)], using_ustar=0)


def test_stage_export_is_the_recorded_sub_block_source():
    """ns_get_stage returns u*, v*, w* and the gauge-shifted dp of the last
    step; dp(1,1,1) is then 0 (big_periodic_3D.f90:562) and the correction
    u = u* - dt diff(dp)/dx reproduces the state (dp_flag = 0)."""
    parent = _parent(0, n=32, steps=2)
    st = parent.get_state(history=False)
    stg = parent.get_stage()
    assert stg["dp"][0, 0, 0] == 0.0
    h = 2 * np.pi / 32
    u = stg["us"] - DT0 * O.diff(stg["dp"], 1, 1) / h
    assert rel_l2(u[:, 1:-1, 1:-1], st["u"][:, 1:-1, 1:-1]) < 1e-14
    assert np.array_equal(stg["dp"], st["p"])  # dp_flag = 0: p = dp
    parent.close()


def test_tgv_matches_the_oracle():
    """TGV (NS_functions.f90:18-50) on the device against the oracle's
    evaluation: equal up to the last bits of sin/cos (4 ulp)."""
    from ns_3d_staggered_dp_gb300 import tgv
    nx, ny, nz = 33, 34, 5
    c = O.staggered_coords(32, 32, 3, 2 * np.pi, 2 * np.pi, 2 * np.pi)
    x, y = c["u"][0], c["u"][1]
    got = tgv(x, y, nz, 0.7, 0.01)
    for k in ("u", "v", "p"):
        ref = O.tgv(x, y, np.zeros(nz), 0.7, 0.01, k)
        assert got[k].shape == (nx, ny, nz)
        np.testing.assert_allclose(got[k], ref, rtol=0, atol=4 * np.finfo(float).eps)
    only_p = tgv(x, y, nz, 0.0, 0.01, u=False, v=False)
    assert set(only_p) == {"p"}


def _cn_parent(n=64, steps=3):
    from ns_3d_staggered_dp_gb300 import Session, make_config
    cfg = O.Config(n, n, n, nu=NU, dt=DT0, scheme=O.AB2_CN, dp_flag=1)
    st = tgv_state(cfg, seed=5, noise=0.05)
    s = Session(make_config(n, n, n, nu=NU, dt=DT0, scheme=O.AB2_CN, dp_flag=1, keep_sweeps=1))
    s.set_state(st.u, st.v, st.w, st.p)
    s.step(steps)
    return s


def test_ab2cn_batch_with_per_sweep_faces_replays_the_parent():
    """AB2-CN re-simulation with the u* faces of every ADI sweep ("Ustar123",
    big_periodic_3D.f90:433-489 records them, re_simulation_sub_tstep_interBC_combine.f90:656-701
    takes them as the BC rows of the sub-block's dttrsb sweeps):
    - every captured per-sweep face equals the oracle's record of the parent's
      own post-sweep arrays bit for bit;
    - restarted sub-blocks reproduce the parent's sub-blocks (property P1; the
      reference logs 3.6e-14 in err_vel_AB2-CN_4.E-3_N_Ustar123_TOffset_restart.txt),
      checked at 1e-11 relative L2;
    - the oracle's re-simulation driven by the same faces agrees to 1e-10."""
    from ns_3d_staggered_dp_gb300 import SWEEP_FACE_ORDER, Batch
    subs = SUBS[:3]
    parent = _cn_parent()
    full = parent.get_state()
    init = []
    for x0, y0, z0, nx, ny, nz, _ in subs:
        maps = O.subdomain_index_maps(x0, y0, z0, nx, ny, nz)
        e = {k: O.extract_sub(full[k], k, maps) for k in ("u", "v", "w", "p")}
        h = [O.extract_sub(full[k], f, maps) for k, f in (("hx", "u"), ("hy", "v"), ("hz", "w"))]
        init.append(O.State(e["u"], e["v"], e["w"], e["p"], *h, first=False))
    frames = [[] for _ in subs]
    with Batch(subs, scheme=O.AB2_CN, bc=2, pbc=3, nu=NU, dt0=DT0, dx=H, dy=H, dz=H, n_slots=4, restart=1) as b:
        b.init_from_parent(parent)
        for n in range(1, 6):
            parent.step(1)
            slot = n % 4
            b.capture(parent, slot, n * DT0)
            sw = parent.get_sweeps()
            stg = parent.get_stage()
            ps = parent.get_state(history=False)
            for i, (x0, y0, z0, nx, ny, nz, _) in enumerate(subs):
                maps = O.subdomain_index_maps(x0, y0, z0, nx, ny, nz)
                ex = lambda a, k: O.extract_sub(a, k, maps)
                after = [(ex(sw["ux"], "u"), ex(sw["vx"], "v"), ex(sw["wx"], "w")),
                         (ex(sw["uy"], "u"), ex(sw["vy"], "v"), ex(sw["wy"], "w")),
                         (ex(stg["us"], "u"), ex(stg["vs"], "v"), ex(stg["ws"], "w"))]
                cn = [O.sweep_faces(*after[d], d, 2) for d in range(3)]
                got = b.get_sweep_faces(slot, i)
                for k in SWEEP_FACE_ORDER:
                    d = "xyz".index(k[0])
                    assert np.array_equal(got[k], cn[d].d[k]), (n, i, k)
                fr = {k: ex(ps[k], k) for k in ("u", "v", "w", "p")}
                fr.update(us=after[2][0], vs=after[2][1], ws=after[2][2], dp=ex(stg["dp"], "p"), cn=cn)
                frames[i].append(fr)
            b.advance((n - 1) * DT0)
        ps = parent.get_state(history=False)
        for i, (x0, y0, z0, nx, ny, nz, _) in enumerate(subs):
            maps = O.subdomain_index_maps(x0, y0, z0, nx, ny, nz)
            got = b.get_state(i, history=False)
            for k in ("u", "v", "w", "p"):
                err = rel_l2(got[k], O.extract_sub(ps[k], k, maps))
                assert err < 1e-11, ("P1", i, k, err)
            cfg = O.Config(nx, ny, nz, lx=nx * H, ly=ny * H, lz=nz * H, nu=NU, dt=DT0, scheme=O.AB2_CN,
                           bc=(2,) * 3, pbc=(3,) * 3, dp_flag=1, gauge=0)
            ref = O.resimulate_frames(init[i], cfg, frames[i], init[i].p, using_ustar=True, dp_flag=1, restart=True)
            for k in ("u", "v", "w", "p"):
                err = rel_l2(got[k], getattr(ref, k))
                assert err < STEP_TOL, ("oracle", i, k, err)
            assert b.max_div(i) < 1e-10
    parent.close()


def test_ab2cn_batch_needs_a_keep_sweeps_parent():
    from ns_3d_staggered_dp_gb300 import Batch, NSError
    parent = _parent(1, n=32, steps=1)
    with Batch([(1, 1, 1, 16, 16, 16, 1)], scheme=O.AB2_CN, bc=2, pbc=3, nu=NU, dt0=DT0, dx=H, dy=H, dz=H,
               n_slots=4) as b:
        with pytest.raises(NSError):
            b.capture(parent, 0, 0.0)
    with pytest.raises(NSError):
        Batch([(1, 1, 1, 16, 16, 16, 2)], scheme=O.AB2_CN, bc=2, pbc=3, nu=NU, dt0=DT0, dx=H, dy=H, dz=H, n_slots=4)
    parent.close()
