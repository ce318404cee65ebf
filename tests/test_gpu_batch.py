"""Batched re-simulation (ns_batch_*) vs the CPU oracle and vs the parent run.

The re-simulated sub-block follows re_simulation_sub_tstep_interBC_combine.f90:
u* boundary values and dp faces from parent snapshots interpolated in time
with interp1 'spline' over 6 knots (sub_tstep_BC_combined_interpolation.m:53-64),
sub_tstep sub-steps in the first interval with the AB2 history saved and
restored (:443-454, :602-612), the DCT pressure solve with the mean of the
parent's dp (:766-768).

Tolerances: 1e-10 relative L2 per field against the oracle (the parity
bound of the step); the exact-replay property P1 of the reference's err_file
(err_vel_AB2_4.E-3_N_Ustar_TOffset_restart.txt: 4.5e-15 over the run) is
checked at 1e-11 relative L2 against the GPU parent's own sub-blocks;
batched and per-subdomain-loop launches must agree bit for bit.
"""
import numpy as np
import pytest

from oracle import ns_oracle as O
from tests.helpers import random_state, rel_l2

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-10
P1_TOL = 1e-11

H = 2 * np.pi / 64
DT0 = 2e-3
NU = 0.01
SUBS = [(5, 9, 3, 16, 24, 16, 1), (2, 2, 2, 24, 16, 32, 2), (10, 4, 7, 16, 16, 24, 4)]


def analytic(shape, t, ph, amp):
    i, j, k = (np.arange(n, dtype=float) for n in shape)
    return amp * (np.sin(0.31 * i[:, None, None] + 0.17 * j[None, :, None] + ph + 3.0 * t)
                  * np.cos(0.23 * k[None, None, :] - 2.0 * t + ph)
                  + 0.3 * np.cos(0.11 * (i[:, None, None] + k[None, None, :]) - 1.5 * t))


def knot_fields(nx, ny, nz, t, seed):
    u = analytic((nx + 1, ny + 2, nz + 2), t, 0.1 * seed, 0.5)
    v = analytic((nx + 2, ny + 1, nz + 2), t, 0.2 * seed + 1.0, 0.5)
    w = analytic((nx + 2, ny + 2, nz + 1), t, 0.3 * seed + 2.0, 0.5)
    dp = analytic((nx + 2, ny + 2, nz + 2), t, 0.4 * seed + 3.0, 0.02)
    return u, v, w, dp


def sub_cfg(nx, ny, nz, bc=2, pbc=3):
    return O.Config(nx, ny, nz, lx=nx * H, ly=ny * H, lz=nz * H, nu=NU, dt=DT0, scheme=O.AB2, bc=(bc,) * 3,
                    pbc=(pbc,) * 3, dp_flag=1, gauge=0)


def make_batch(subs, n_slots, bc=2, pbc=3, **kw):
    from ns_3d_staggered_dp_gb300 import Batch
    return Batch(subs, scheme=O.AB2, bc=bc, pbc=pbc, nu=NU, dt0=DT0, dx=H, dy=H, dz=H, n_slots=n_slots, **kw)


def run_case(subs, restart, n_intervals=4, stride=2, bc=2, pbc=3, autotune=False, **kw):
    """Synthetic parent data at knots every `stride` parent steps, the batch
    on the GPU and the oracle's re-simulation of every subdomain."""
    t_start = 1.0
    knot_t = [t_start + (q - 2) * stride * DT0 for q in range(2 + (n_intervals // stride) + 5)]
    rng = np.random.default_rng(7)
    states, knots = [], []
    for idx, (_, _, _, nx, ny, nz, r) in enumerate(subs):
        u, v, w, _ = knot_fields(nx, ny, nz, t_start, idx)
        p = analytic((nx + 2, ny + 2, nz + 2), t_start, 0.7 * idx, 0.1)
        st = O.State(u, v, w, p, 0.1 * rng.standard_normal(u.shape), 0.1 * rng.standard_normal(v.shape),
                     0.1 * rng.standard_normal(w.shape), first=not restart)
        states.append(st)
        knots.append([knot_fields(nx, ny, nz, t, idx) for t in knot_t])
    refs = []
    for idx, (_, _, _, nx, ny, nz, r) in enumerate(subs):
        cfg = sub_cfg(nx, ny, nz, bc, pbc)
        refs.append(O.resimulate(states[idx], cfg, knot_t, knots[idx], t_start, n_intervals, sub_tstep=r,
                                 restart=restart))
    with make_batch(subs, len(knot_t), bc=bc, pbc=pbc, restart=int(restart), **kw) as b:
        for idx, (_, _, _, nx, ny, nz, r) in enumerate(subs):
            st = states[idx]
            b.set_state(idx, st.u, st.v, st.w, st.p, (st.px, st.py, st.pz))
            for q, t in enumerate(knot_t):
                u, v, w, dp = knots[idx][q]
                f = O.get_velpr_bc(u, v, w, dp, (bc,) * 3, (pbc,) * 3, H, H, H, DT0, 1, True, None)
                b.set_snapshot(q, t, idx, f.d, float(np.mean(dp[1:-1, 1:-1, 1:-1])))
        if autotune:
            assert len(b.autotune(reps=2)) == 16
        for m in range(n_intervals):
            b.advance(t_start + m * DT0)
        got = [b.get_state(i) for i in range(len(subs))]
        launches = b.launch_count()
    return got, refs, launches


def _compare(got, ref):
    for k, r in (("u", ref.u), ("v", ref.v), ("w", ref.w), ("p", ref.p)):
        err = rel_l2(got[k], r)
        assert err < STEP_TOL, (k, err)


@pytest.mark.parametrize("restart", [False, True])
def test_batch_matches_oracle(restart):
    got, refs, _ = run_case(SUBS, restart)
    for g, r in zip(got, refs):
        _compare(g, r)


# x and y edges of 24, 32, 48 and 64 take the FFT-based DCT passes (codes 2 and 3),
# beside a 16-wide box on the dense products in the same launch sequence
DCT_SUBS = [(1, 1, 1, 32, 64, 16, 1), (3, 2, 5, 64, 32, 24, 2), (7, 1, 2, 16, 32, 16, 1), (2, 3, 1, 48, 24, 16, 1),
            (1, 2, 3, 24, 48, 32, 4)]


@pytest.mark.parametrize("pbc", [3, 2])
def test_batch_fft_dct_sizes(pbc):
    got, refs, _ = run_case(DCT_SUBS, False, n_intervals=3, pbc=pbc)
    for g, r in zip(got, refs):
        _compare(g, r)


@pytest.mark.parametrize("bc,pbc", [(2, 2), (4, 4)])
def test_batch_wall_codes(bc, pbc):
    got, refs, _ = run_case(SUBS[:2], False, n_intervals=3, bc=bc, pbc=pbc)
    for g, r in zip(got, refs):
        _compare(g, r)


@pytest.mark.parametrize("subs", [SUBS, DCT_SUBS])
def test_batch_loop_mode_is_bitwise_identical(subs):
    a, _, la = run_case(subs, False, n_intervals=3, mode=0)
    b, _, lb = run_case(subs, False, n_intervals=3, mode=1)
    for x, y in zip(a, b):
        for k in ("u", "v", "w", "p", "hx", "hy", "hz"):
            assert np.array_equal(x[k], y[k]), k
    assert lb > la  # one launch per subdomain and stage


def test_batch_graph_matches_eager():
    a, _, _ = run_case(SUBS, True, n_intervals=3, use_graph=1)
    b, _, _ = run_case(SUBS, True, n_intervals=3, use_graph=0)
    for x, y in zip(a, b):
        for k in ("u", "v", "w", "p"):
            assert np.array_equal(x[k], y[k]), k


def _parent(n=64, steps=3):
    from ns_3d_staggered_dp_gb300 import Session, make_config
    from tests.helpers import tgv_state
    cfg = O.Config(n, n, n, nu=NU, dt=DT0, scheme=O.AB2, dp_flag=1)
    st = tgv_state(cfg, seed=5, noise=0.05)
    s = Session(make_config(n, n, n, nu=NU, dt=DT0, scheme=O.AB2, dp_flag=1))
    s.set_state(st.u, st.v, st.w, st.p)
    s.step(steps)
    return s


P1_SUBS = [(5, 9, 3, 16, 24, 16, 1), (30, 2, 20, 32, 16, 24, 1), (41, 40, 33, 24, 24, 32, 1)]


@pytest.mark.parametrize("pbc", [3, 2])
def test_batch_p1_replay_of_the_parent(pbc):
    """Property P1: restarted sub-blocks driven by the parent's own u* and dp
    at every step reproduce the parent's sub-block (err_file ..._restart.txt)."""
    parent = _parent()
    with make_batch(P1_SUBS, 4, pbc=pbc, restart=1) as b:
        b.init_from_parent(parent)
        for nstep in range(1, 6):
            parent.step(1)
            b.capture(parent, nstep % 4, nstep * DT0)
            b.advance((nstep - 1) * DT0)
            for i in range(len(P1_SUBS)):
                assert b.max_div(i) < 1e-10
        ps = parent.get_state(history=False)
        for i, (x0, y0, z0, nx, ny, nz, _) in enumerate(P1_SUBS):
            maps = O.subdomain_index_maps(x0, y0, z0, nx, ny, nz)
            got = b.get_state(i, history=False)
            for k in ("u", "v", "w", "p"):
                ref = O.extract_sub(ps[k], k, maps)
                err = rel_l2(got[k], ref)
                assert err < P1_TOL, (i, k, err)
        # the err_vel columns the reference logs for this replay (max and mean
        # relative errors, vorticity error) stay at rounding level
        m = b.error_metrics(parent)
        assert np.all(m[:, 4:] < 1e-9), m[:, 4:]
    parent.close()


def test_batch_autotune_keeps_state():
    """The autotuner times the stage kernels on a copy of the state and
    restores it; tuned grid sizes change the schedule, not the results."""
    a, _, _ = run_case(SUBS[:2], False, n_intervals=2)
    b, _, _ = run_case(SUBS[:2], False, n_intervals=2, autotune=True)
    for x, y in zip(a, b):
        for k in ("u", "v", "w", "p"):
            assert np.array_equal(x[k], y[k])


def test_batch_rejects_bad_input():
    from ns_3d_staggered_dp_gb300 import NSError
    with pytest.raises(NSError):
        make_batch([(1, 1, 1, 15, 16, 16, 1)], 4)  # odd nx
    with pytest.raises(NSError):
        make_batch([(1, 1, 1, 16, 16, 16, 0)], 4)  # sub_tstep 0
    with make_batch([(1, 1, 1, 16, 16, 16, 1)], 4) as b:
        with pytest.raises(NSError):
            b.advance(0.0)  # no snapshot yet


def test_error_metrics_session_and_batch_match_the_oracle():
    """rms_vel / err_vel of re_simulation_sub_tstep_interBC_combine.f90:813-834
    reduced on the device: a session against perturbed host arrays, and every
    subdomain of a batch against the parent over its index maps."""
    from ns_3d_staggered_dp_gb300 import Batch, Session, make_config
    n = 32
    h = 2 * np.pi / n
    cfg = O.Config(n, n, n, nu=0.01, dt=0.01, scheme=O.AB2)
    st = random_state(cfg, 71)
    rng = np.random.default_rng(72)
    pert = [a + 1e-3 * rng.standard_normal(a.shape) for a in (st.u, st.v, st.w, st.p)]
    with Session(make_config(n, n, n, nu=0.01, dt=0.01, scheme=1, dp_flag=1)) as par:
        par.set_state(st.u, st.v, st.w, st.p)
        got = par.error_metrics(*pert)
        ref = O.error_metrics(st.u, st.v, st.w, st.p, *pert, h, h)
        assert np.allclose(got, ref, rtol=1e-12, atol=0)
        par.step(2)
        subs = [(3, 5, 2, 16, 8, 24, 1), (10, 1, 9, 8, 16, 16, 2)]
        with Batch(subs, scheme=1, bc=2, pbc=3, nu=0.01, dt0=0.01, dx=h, dy=h, dz=h, n_slots=4) as b:
            b.init_from_parent(par)
            par.step(1)  # the parent moves on: the subdomains now differ from it
            got = b.error_metrics(par)
            full = par.get_state(history=False)
            for i, (x0, y0, z0, nx, ny, nz, _) in enumerate(subs):
                sd = b.get_state(i, history=False)
                maps = O.subdomain_index_maps(x0, y0, z0, nx, ny, nz)
                parent_sub = [O.extract_sub(full[k], k, maps) for k in ("u", "v", "w", "p")]
                ref = O.error_metrics(sd["u"], sd["v"], sd["w"], sd["p"], *parent_sub, h, h)
                assert np.allclose(got[i], ref, rtol=1e-12, atol=0), (i, got[i], ref)


def test_batch_bench_set_of_64_boxes_matches_oracle():
    """The 64 sub-blocks the batched bench runs (edges from {16, 24, 32, 48,
    64} per axis, sub-step ratios {1, 2, 4}, seed 4096) against the oracle's
    re-simulation of each: the first parent interval with its sub-steps and
    one regular interval, restarted AB2 from a given history."""
    import bench
    subs = bench.resim_subdomains()
    assert {s[3] for s in subs} | {s[4] for s in subs} | {s[5] for s in subs} >= {48, 64}
    assert {s[6] for s in subs} == {1, 2, 4}
    got, refs, _ = run_case(subs, True, n_intervals=2, stride=1)
    for i, (g, r) in enumerate(zip(got, refs)):
        for k, rr in (("u", r.u), ("v", r.v), ("w", r.w), ("p", r.p)):
            err = rel_l2(g[k], rr)
            assert err < STEP_TOL, (i, subs[i], k, err)


def test_plain_session_loop_matches_the_batch():
    """The plain path of the re-simulation (one session per subdomain, faces
    and mean dp set every step with ns_set_faces / ns_set_mean_dp, the graph
    kept across face changes) follows the batch's result from the same start
    and the same captured faces to 1e-10."""
    from ns_3d_staggered_dp_gb300 import FACE_ORDER, Session, make_config
    parent = _parent()
    subs = P1_SUBS
    with make_batch(subs, 8, restart=1) as b:
        b.init_from_parent(parent)
        for k in range(1, 7):
            parent.step(1)
            b.capture(parent, k, k * DT0)
        b.advance(0.0)
        init = [b.get_state(i) for i in range(len(subs))]
        sess = []
        for (x0, y0, z0, nx, ny, nz, _), st in zip(subs, init):
            s = Session(make_config(nx, ny, nz, lx=nx * H, ly=ny * H, lz=nz * H, nu=NU, dt=DT0, scheme=1,
                                    bc=(2, 2, 2), pbc=(3, 3, 3), dp_flag=1, gauge=0))
            s.set_state(st["u"], st["v"], st["w"], st["p"], (st["hx"], st["hy"], st["hz"]))
            sess.append(s)
        for q in range(1, 5):
            b.advance(q * DT0)
            for i, s in enumerate(sess):
                faces, mean = b.get_snapshot(q + 1, i)
                s.set_faces({k: faces[k] for k in FACE_ORDER})
                s.set_mean_dp(mean)
                s.step(1)
        for i, s in enumerate(sess):
            a = s.get_state(history=False)
            g = b.get_state(i, history=False)
            for k in ("u", "v", "w", "p"):
                assert rel_l2(a[k], g[k]) < STEP_TOL, (i, k, rel_l2(a[k], g[k]))
            s.close()
    parent.close()
