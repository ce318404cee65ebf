"""CPU checks of the adjoint oracle (no GPU): the slot-form step restates the
oracle's step, its tangent-linear model matches central finite differences,
and the adjoint is the transpose of the tangent-linear model (dot-product test)."""
import numpy as np
import pytest

from oracle import ns_adjoint as A
from oracle import ns_oracle as O
from tests.helpers import project, random_state, rel_l2

SCHEMES = [O.AB2_CN, O.AB2, O.EULER]


def _cfg(scheme, n=(8, 6, 10), closure_lengths=(1.0, 0.8, 1.3)):
    nx, ny, nz = n
    fx, fy, fz = closure_lengths
    return O.Config(nx, ny, nz, lx=2 * np.pi * fx, ly=2 * np.pi * fy, lz=2 * np.pi * fz, nu=0.05, dt=0.02,
                    scheme=scheme)


def _state(cfg, seed, history):
    st = project(random_state(cfg, seed), cfg)
    if history:
        h = random_state(cfg, seed + 1, history=True)
        st.px, st.py, st.pz = h.px, h.py, h.pz
    st.first = not history
    return st


def _rand(S, seed):
    rng = np.random.default_rng(seed)
    return tuple(rng.standard_normal(x.shape) for x in S)


def test_conv_slot_is_cal_conv():
    cfg = _cfg(O.AB2)
    st = random_state(cfg, 2)
    S = A.state_to_slots(st, cfg)
    got = A.conv_slot(*S[:3], cfg.h)
    ref = O.cal_conv(st.u, st.v, st.w, 1, 1, 1, *cfg.h)
    for g, r, k in zip(got, ref, "uvw"):
        assert rel_l2(g, A.restrict(A.expand(g, k, cfg), k, cfg)) == 0.0
        # cal_conv's interior ranges are the slots themselves on a periodic box
        assert rel_l2(g, r) < 1e-14


@pytest.mark.parametrize("scheme", SCHEMES)
@pytest.mark.parametrize("history", [False, True])
def test_step_slot_restates_the_oracle_step(scheme, history):
    cfg = _cfg(scheme)
    st = _state(cfg, 3, history)
    got = A.step_slot(A.state_to_slots(st, cfg), cfg, st.first)
    ref = A.state_to_slots(O.step(st, cfg), cfg)
    for g, r in zip(got, ref):
        assert rel_l2(g, r) < 1e-14


@pytest.mark.parametrize("scheme", SCHEMES)
@pytest.mark.parametrize("history", [False, True])
def test_tlm_matches_central_differences(scheme, history):
    cfg = _cfg(scheme)
    st = _state(cfg, 4, history)
    S = A.state_to_slots(st, cfg)
    d = _rand(S, 5)
    eps = 1e-6
    Sp = A.step_slot(tuple(x + eps * y for x, y in zip(S, d)), cfg, st.first)
    Sm = A.step_slot(tuple(x - eps * y for x, y in zip(S, d)), cfg, st.first)
    tl = A.tlm_step(S, d, cfg, st.first)
    for t, a, b in zip(tl, Sp, Sm):
        fd = (a - b) / (2 * eps)
        if np.linalg.norm(fd) > 0:
            assert rel_l2(t, fd) < 1e-8


@pytest.mark.parametrize("closure", [0, 1])
@pytest.mark.parametrize("scheme", SCHEMES)
@pytest.mark.parametrize("history", [False, True])
def test_adjoint_step_dot_product(scheme, history, closure):
    """<TLM d, l> = <d, ADJ l> for one step."""
    cfg = _cfg(scheme)
    st = _state(cfg, 6, history)
    S = A.state_to_slots(st, cfg)
    lines = A.CNLines(cfg, closure) if scheme == O.AB2_CN else None
    d, lam = _rand(S, 7), _rand(S, 8)
    lhs = A.dot(A.tlm_step(S, d, cfg, st.first, lines), lam)
    rhs = A.dot(d, A.adj_step(S, lam, cfg, st.first, lines))
    assert abs(lhs - rhs) <= 1e-13 * abs(lhs)


def test_reference_closure_line_matrix_is_not_symmetric():
    """mat_CN's A(1,n+1) closure (NS_functions.f90:1273) makes the reduced
    normal-component matrix non-symmetric, so the adjoint sweep needs M^T."""
    cfg = _cfg(O.AB2_CN)
    M0 = A.cn_reduced(8, 0.3, cfg, True, 0)
    M1 = A.cn_reduced(8, 0.3, cfg, True, 1)
    assert not np.allclose(M0, M0.T)
    assert np.allclose(M1, M1.T)
    assert np.allclose(A.cn_reduced(8, 0.3, cfg, False), A.cn_reduced(8, 0.3, cfg, False).T)


@pytest.mark.parametrize("scheme", SCHEMES)
def test_multi_step_dot_product_and_gradient(scheme):
    """Over 6 steps from an Euler start: the dot-product test of the whole run,
    and dJ/du0 against central differences of J in 3 seeded directions."""
    cfg = _cfg(scheme, n=(8, 8, 8), closure_lengths=(1.0, 1.0, 1.0))
    st = _state(cfg, 9, False)
    S0 = A.state_to_slots(st, cfg)
    nsteps = 6
    d, lam = _rand(S0, 10), _rand(S0, 11)
    d = d[:3] + tuple(np.zeros_like(x) for x in d[3:])  # the history of an Euler start is not a control
    lhs = A.dot(A.tlm(S0, d, cfg, nsteps), lam)
    rhs = A.dot(d, A.adjoint(S0, lam, cfg, nsteps))
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
    # J = 1/2 |u(T) - target|^2 over the central half of each axis
    tgt = A.forward(A.state_to_slots(_state(cfg, 12, False), cfg), cfg, nsteps)[-1]
    reg = A.region(cfg)
    ST = A.forward(S0, cfg, nsteps)[-1]
    grad = A.adjoint(S0, A.objective_seed(ST, tgt, reg), cfg, nsteps)
    for q in range(3):
        dirn = _rand(S0, 20 + q)[:3] + tuple(np.zeros_like(x) for x in S0[3:])
        eps = 1e-4
        Jp = A.objective(A.forward(tuple(x + eps * y for x, y in zip(S0, dirn)), cfg, nsteps)[-1], tgt, reg)
        Jm = A.objective(A.forward(tuple(x - eps * y for x, y in zip(S0, dirn)), cfg, nsteps)[-1], tgt, reg)
        fd = (Jp - Jm) / (2 * eps)
        ad = A.dot(grad, dirn)
        assert abs(fd - ad) <= 1e-7 * abs(ad)


def test_fold_is_the_adjoint_of_expand():
    cfg = _cfg(O.AB2)
    rng = np.random.default_rng(13)
    for k in "uvw":
        X = rng.standard_normal((cfg.nx, cfg.ny, cfg.nz))
        y = rng.standard_normal(A.expand(X, k, cfg).shape)
        assert abs(float(np.vdot(A.expand(X, k, cfg), y)) - float(np.vdot(X, A.fold(y, k, cfg)))) < 1e-12 * np.abs(y).sum()
