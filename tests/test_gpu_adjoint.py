"""Discrete adjoint on the GPU (ns_adj_forward / ns_adj_backward) against the
adjoint oracle, through the C ABI.

Tolerances: the gradient agrees with the oracle's adjoint to a relative L2
of 1e-10 per field (the step's parity bound); the dot-product test against
the oracle's tangent-linear model to 1e-10; central finite differences of
the GPU forward run to 1e-6 (the gradient bound of the adjoint workload).
"""
import numpy as np
import pytest

from oracle import ns_adjoint as A
from oracle import ns_oracle as O
from tests.helpers import project, random_state, rel_l2

pytestmark = pytest.mark.gpu

GRAD_TOL = 1e-10
FD_TOL = 1e-6


def session(cfg, **kw):
    from ns_3d_staggered_dp_gb300 import Session, make_config
    return Session(make_config(cfg.nx, cfg.ny, cfg.nz, lx=cfg.lx, ly=cfg.ly, lz=cfg.lz, nu=cfg.nu, dt=cfg.dt,
                               scheme=cfg.scheme, bc=cfg.bc, pbc=cfg.pbc, dp_flag=cfg.dp_flag, **kw))


def _state(cfg, seed, history=False):
    st = project(random_state(cfg, seed), cfg)
    if history:
        h = random_state(cfg, seed + 1, history=True)
        st.px, st.py, st.pz = h.px, h.py, h.pz
    st.first = not history
    return st


def _set(s, st, history):
    s.set_state(st.u, st.v, st.w, st.p, (st.px, st.py, st.pz) if history else None)


def _seed_arrays(cfg, lam):
    """Reference-shaped seeds: slot values on their own entries, zero on the copies."""
    return [A.embed(lam[q], k, cfg) for q, k in enumerate("uvw")]


def _gpu_grad(cfg, st, history, nsteps, ckpt, lam, hist_grad=False, **kw):
    with session(cfg, **kw) as s:
        _set(s, st, history)
        s.adj_forward(nsteps, ckpt)
        fin = s.get_state()
        g = s.adj_backward(*_seed_arrays(cfg, lam), history=hist_grad)
        fin2 = s.get_state()
    for k in fin:
        assert np.array_equal(fin[k], fin2[k]), f"state after the backward pass differs in {k}"
    return g


CASES = [
    (O.AB2_CN, (16, 16, 16), (1.0, 1.0, 1.0)),
    (O.AB2_CN, (32, 16, 64), (1.0, 0.6, 1.9)),
    (O.AB2, (16, 32, 16), (1.0, 1.3, 0.8)),
    (O.EULER, (16, 16, 32), (1.0, 1.0, 1.0)),
]


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("history", [False, True])
def test_gradient_matches_oracle_adjoint(case, history):
    scheme, n, f = case
    cfg = O.Config(*n, lx=2 * np.pi * f[0], ly=2 * np.pi * f[1], lz=2 * np.pi * f[2], nu=0.02, dt=0.01,
                   scheme=scheme)
    st = _state(cfg, 21, history)
    S0 = A.state_to_slots(st, cfg)
    nsteps, ckpt = 7, 3
    lam = tuple(np.random.default_rng(22).standard_normal(S0[0].shape) for _ in range(3))
    lamT = lam + tuple(np.zeros_like(S0[0]) for _ in range(3))
    ref = A.adjoint(S0, lamT, cfg, nsteps, first=not history)
    g = _gpu_grad(cfg, st, history, nsteps, ckpt, lam, hist_grad=True)
    for q, k in enumerate("uvw"):
        assert rel_l2(A.restrict(g[k], k, cfg), ref[q]) < GRAD_TOL
        # the periodic copies carry no gradient
        assert np.array_equal(g[k], A.embed(A.restrict(g[k], k, cfg), k, cfg))
    for q, k in enumerate(("hx", "hy", "hz")):
        r = ref[3 + q]
        got = A.restrict(g[k], "uvw"[q], cfg)
        if history and scheme != O.EULER:
            assert rel_l2(got, r) < GRAD_TOL
        else:
            assert not np.any(g[k])


@pytest.mark.parametrize("closure", [0, 1])
def test_dot_product_with_oracle_tangent_linear(closure):
    """<TLM_oracle d, l> = <d, ADJ_gpu l> over 5 AB2-CN steps, both line closures."""
    cfg = O.Config(32, 32, 32, nu=0.01, dt=0.02, scheme=O.AB2_CN)
    st = _state(cfg, 31)
    S0 = A.state_to_slots(st, cfg)
    rng = np.random.default_rng(32)
    d = tuple(rng.standard_normal(S0[0].shape) for _ in range(3)) + tuple(np.zeros_like(S0[0]) for _ in range(3))
    lam = tuple(rng.standard_normal(S0[0].shape) for _ in range(3))
    lamT = lam + tuple(np.zeros_like(S0[0]) for _ in range(3))
    nsteps = 5
    lines = A.CNLines(cfg, closure)
    traj = A.forward(S0, cfg, nsteps, True, lines)
    dS = d
    for n in range(nsteps):
        dS = A.tlm_step(traj[n], dS, cfg, n == 0, lines)
    lhs = A.dot(dS, lamT)
    g = _gpu_grad(cfg, st, False, nsteps, 2, lam, cn_periodic_closure=closure)
    rhs = sum(float(np.vdot(d[q], A.restrict(g[k], k, cfg))) for q, k in enumerate("uvw"))
    assert abs(lhs - rhs) <= GRAD_TOL * abs(lhs)


def test_checkpoint_interval_does_not_change_the_gradient():
    """Recomputation is deterministic: every checkpoint interval gives the same bits."""
    cfg = O.Config(16, 16, 16, nu=0.02, dt=0.01, scheme=O.AB2_CN)
    st = _state(cfg, 41)
    lam = tuple(np.random.default_rng(42).standard_normal((16, 16, 16)) for _ in range(3))
    grads = [_gpu_grad(cfg, st, False, 8, k, lam) for k in (1, 3, 8)]
    for g in grads[1:]:
        for k in "uvw":
            assert np.array_equal(g[k], grads[0][k])


def test_seed_on_periodic_copies_folds_into_the_owner():
    """dJ/du given on a duplicate entry (u(nx+1,:,:), ghost rows) counts for the value it copies."""
    cfg = O.Config(16, 16, 16, nu=0.02, dt=0.01, scheme=O.AB2)
    st = _state(cfg, 51)
    rng = np.random.default_rng(52)
    lam = tuple(rng.standard_normal((16, 16, 16)) for _ in range(3))
    with session(cfg) as s:
        _set(s, st, False)
        s.adj_forward(3, 3)
        g_own = s.adj_backward(*_seed_arrays(cfg, lam))
        # half on the owner, half spread over its copies through expand / count
        seeds = []
        for q, k in enumerate("uvw"):
            full = A.expand(lam[q], k, cfg)
            count = A.expand(np.ones_like(lam[q]), k, cfg)
            count = A.expand(A.fold(count, k, cfg), k, cfg)  # copies per owner, at every alias
            seeds.append(full / count)
        g_split = s.adj_backward(*seeds)
    for k in "uvw":
        assert rel_l2(g_split[k], g_own[k]) < 1e-14


def test_gradient_against_central_differences_of_the_gpu_run():
    """J = 1/2 |u(T) - u_target|^2 over the central 16^3 of a 32^3 box, 10 AB2-CN
    steps, checkpoint every 5: dJ/du0 . d against (J(u0 + e d) - J(u0 - e d)) / 2e
    of the GPU forward run in 4 seeded directions."""
    cfg = O.Config(32, 32, 32, nu=0.01, dt=0.02, scheme=O.AB2_CN)
    st = _state(cfg, 61)
    target = _state(cfg, 62)
    nsteps = 10
    reg = A.region(cfg)
    with session(cfg) as s:
        def run(u, v, w):
            s.set_state(u, v, w, st.p)
            s.step(nsteps)
            o = s.get_state(history=False)
            return tuple(A.restrict(o[k], k, cfg) for k in "uvw")

        tgt = run(target.u, target.v, target.w)
        s.set_state(st.u, st.v, st.w, st.p)
        s.adj_forward(nsteps, 5)
        o = s.get_state(history=False)
        UT = tuple(A.restrict(o[k], k, cfg) for k in "uvw")
        seed = A.objective_seed(UT + UT, tgt + tgt, reg)[:3]
        g = s.adj_backward(*_seed_arrays(cfg, seed))
        rng = np.random.default_rng(63)
        scale = np.sqrt(np.mean(A.state_to_slots(st, cfg)[0] ** 2))
        for _ in range(4):
            d = [rng.standard_normal((32, 32, 32)) for _ in range(3)]
            eps = 1e-5 * scale
            up = [A.expand(A.restrict(x, k, cfg) + eps * dd, k, cfg) for x, k, dd in zip((st.u, st.v, st.w), "uvw", d)]
            um = [A.expand(A.restrict(x, k, cfg) - eps * dd, k, cfg) for x, k, dd in zip((st.u, st.v, st.w), "uvw", d)]
            Jp = A.objective(run(*up), tgt, reg)
            Jm = A.objective(run(*um), tgt, reg)
            fd = (Jp - Jm) / (2 * eps)
            ad = sum(float(np.vdot(A.restrict(g[k], k, cfg), dd)) for k, dd in zip("uvw", d))
            assert abs(fd - ad) <= FD_TOL * abs(ad)


@pytest.mark.parametrize("kw", [dict(bc=(1, 2, 1), pbc=(1, 3, 1)), dict(dp_flag=1)])
def test_unsupported_configurations_are_rejected(kw):
    from ns_3d_staggered_dp_gb300.api import NSError
    cfg = O.Config(16, 16, 16, nu=0.02, dt=0.01, scheme=O.AB2_CN, **kw)
    with session(cfg) as s:
        with pytest.raises(NSError) as e:
            s.adj_forward(2, 1)
        assert e.value.status == 5  # NS_ERR_UNSUPPORTED_BC


def test_gradient_matches_central_differences_of_the_cpu_reference_solver():
    """The gradient-check workload: J = 1/2 |u(T) - u_target|^2 over the
    central 64^3 of a 128^3 periodic box, T = 50 AB2-CN steps, checkpoint
    every 10, seeded decaying-turbulence initial field.  The reference
    gradient is built from central differences of the C++ restatement of the
    reference solver (oracle/ns_ref_cpu.cpp: dense mat_CN LU sweeps, r2c FFT
    Poisson) in 4 seeded directions; the GPU adjoint gradient must agree to
    1e-6 relative in each direction."""
    import bench
    from oracle.ns_ref_cpu import CpuStep
    n, T, K = 128, 50, 10
    nu = 1.0 / 1600.0
    u, v, w, p, umax = bench.hit_initial_field(n, seed=2024)
    u5, v5, w5, _, _ = bench.hit_initial_field(n, seed=5)
    dt = 0.3 * (2 * np.pi / n) / umax
    cfg = O.Config(n, n, n, nu=nu, dt=dt, scheme=O.AB2_CN)
    lo, hi = n // 4, 3 * n // 4
    reg = (slice(lo, hi),) * 3
    cpu = CpuStep(cfg)

    def cpu_final(uu, vv, ww):
        st = O.State(np.array(uu, order="F"), np.array(vv, order="F"), np.array(ww, order="F"),
                     np.array(p, order="F"), np.zeros(uu.shape), np.zeros(vv.shape), np.zeros(ww.shape), first=True)
        for _ in range(T):
            cpu.step(st)
        return [np.ascontiguousarray(bench._slots(a, k, n)) for a, k in zip((st.u, st.v, st.w), "uvw")]

    def J_of(U, tgt):
        return 0.5 * sum(float(np.sum((U[q][reg] - tgt[q][reg]) ** 2)) for q in range(3))

    tgt = cpu_final(u + 0.1 * u5, v + 0.1 * v5, w + 0.1 * w5)
    with session(cfg) as s:
        s.set_state(u, v, w, p)
        s.adj_forward(T, K)
        o = s.get_state(history=False)
        UT = [np.ascontiguousarray(bench._slots(o[k], k, n)) for k in "uvw"]
        seed = []
        for q, k in enumerate("uvw"):
            g = np.zeros_like(UT[q])
            g[reg] = UT[q][reg] - tgt[q][reg]
            seed.append(bench._embed(g, k, n))
        grad = s.adj_backward(*seed)
    G = [np.ascontiguousarray(bench._slots(grad[k], k, n)) for k in "uvw"]
    base = [np.ascontiguousarray(bench._slots(a, k, n)) for a, k in zip((u, v, w), "uvw")]
    eps = 1e-5 * float(np.sqrt(np.mean(base[0] ** 2)))
    rng = np.random.default_rng(55)
    for _ in range(4):
        d = [rng.standard_normal((n, n, n)) for _ in range(3)]
        Js = []
        for sg in (1.0, -1.0):
            f = [bench._expand(b + sg * eps * dd, k, n) for b, dd, k in zip(base, d, "uvw")]
            Js.append(J_of(cpu_final(*f), tgt))
        fd = (Js[0] - Js[1]) / (2 * eps)
        ad = sum(float(np.vdot(Gq, dq)) for Gq, dq in zip(G, d))
        assert abs(fd - ad) <= FD_TOL * abs(ad), (fd, ad)
