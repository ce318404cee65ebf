"""Parity at the full size of the headline workload: the 256^3 periodic
AB2-CN step on the GPU against the C++/OpenMP restatement of the reference
step (oracle/ns_ref_cpu.cpp, itself checked against the NumPy oracle), 3
steps from an Euler start on a seeded solenoidal field of unit rms.

Tolerance: relative L2 1e-10 per field (the step's parity bound) and
max|div u| <= 1e-12 after the steps."""
import numpy as np
import pytest

from oracle import ns_oracle as O
from tests.helpers import rel_l2

pytestmark = pytest.mark.gpu


def solenoidal_field(n, seed):
    """Seeded random-phase field with a k^4 exp(-2 (k/4)^2) spectrum, made
    discretely divergence-free by the oracle's projection, unit rms."""
    rng = np.random.default_rng(seed)
    cfg = O.Config(n, n, n)
    st = O.State.zeros(n, n, n)
    k = np.fft.fftfreq(n, 1.0 / n)
    K = np.sqrt(k[:, None, None] ** 2 + k[None, :, None] ** 2 + k[None, None, :] ** 2)
    amp = K * np.exp(-((K / 4.0) ** 2))
    for name, shape in (("u", st.u.shape), ("v", st.v.shape), ("w", st.w.shape)):
        phase = np.exp(2j * np.pi * rng.random((n, n, n)))
        f = np.real(np.fft.ifftn(amp * phase))
        ix = [np.arange(s) % n for s in shape]
        setattr(st, name, f[np.ix_(*ix)])
    from tests.helpers import project
    st = project(st, cfg)
    rms = np.sqrt(np.mean(st.u[:-1, 1:-1, 1:-1] ** 2 + st.v[1:-1, :-1, 1:-1] ** 2 + st.w[1:-1, 1:-1, :-1] ** 2) / 3)
    st.u, st.v, st.w = st.u / rms, st.v / rms, st.w / rms
    return st


def test_256_cubed_three_steps_match_the_cpu_restatement():
    from ns_3d_staggered_dp_gb300 import Session, make_config
    from oracle.ns_ref_cpu import CpuStep
    n = 256
    st = solenoidal_field(n, 2024)
    umax = max(np.abs(st.u).max(), np.abs(st.v).max(), np.abs(st.w).max())
    dt = 0.3 * (2 * np.pi / n) / umax
    cfg = O.Config(n, n, n, nu=1.0 / 1600.0, dt=dt, scheme=O.AB2_CN)
    ref = st.copy()
    cpu = CpuStep(cfg)
    for _ in range(3):
        cpu.step(ref)
    with Session(make_config(n, n, n, nu=cfg.nu, dt=dt, scheme=2)) as s:
        s.set_state(st.u, st.v, st.w, st.p)
        s.step(3)
        got = s.get_state()
        d = s.diag()
    for k, r in (("u", ref.u), ("v", ref.v), ("w", ref.w), ("p", ref.p), ("hx", ref.px), ("hy", ref.py), ("hz", ref.pz)):
        assert rel_l2(got[k], r) < 1e-10, k
    assert d["max_div"] < 1e-12
