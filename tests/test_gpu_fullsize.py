"""Parity at the full sizes of the workloads the step is quoted on.

- 256^3 periodic decaying turbulence, AB2-CN: the GPU against the C++/OpenMP
  restatement of the reference step (oracle/ns_ref_cpu.cpp, itself checked
  against the NumPy oracle), 10 steps from an Euler start on a seeded
  solenoidal field of unit rms.
- 256x128x256 wall-bounded box (x, z periodic; y no-slip walls, Neumann
  pressure), AB2-CN, Re = 180, dt = 2e-3: the GPU against the NumPy oracle,
  10 steps from the laminar profile plus a seeded divergence-free
  perturbation of amplitude 0.05.

- 256^3 all-wall box (no-slip on every face, Neumann pressure), AB2-CN: the
  GPU against the NumPy oracle, 2 steps from the decaying-turbulence field
  with the wall ghosts of vel_bc_staggered.

Tolerance: relative L2 1e-10 per field after the steps (the step's parity
bound) and max|div u| <= 1e-12."""
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


def test_256_cubed_ten_steps_match_the_cpu_restatement():
    from ns_3d_staggered_dp_gb300 import Session, make_config
    from oracle.ns_ref_cpu import CpuStep
    n = 256
    st = solenoidal_field(n, 2024)
    umax = max(np.abs(st.u).max(), np.abs(st.v).max(), np.abs(st.w).max())
    dt = 0.3 * (2 * np.pi / n) / umax
    cfg = O.Config(n, n, n, nu=1.0 / 1600.0, dt=dt, scheme=O.AB2_CN)
    ref = st.copy()
    cpu = CpuStep(cfg)
    for _ in range(10):
        cpu.step(ref)
    with Session(make_config(n, n, n, nu=cfg.nu, dt=dt, scheme=2)) as s:
        s.set_state(st.u, st.v, st.w, st.p)
        s.step(10)
        got = s.get_state()
        d = s.diag()
    for k, r in (("u", ref.u), ("v", ref.v), ("w", ref.w), ("p", ref.p), ("hx", ref.px), ("hy", ref.py), ("hz", ref.pz)):
        assert rel_l2(got[k], r) < 1e-10, k
    assert d["max_div"] < 1e-12


def test_wall_box_256x128x256_ten_steps_match_the_oracle():
    """The wall-bounded configuration at its own size: FFT in x and z, the
    wall-normal line solve in y (DCT_poisson_solver's operator,
    NS_functions.f90:1505-1630), no-slip ADI rows (vel_bc_staggered_CN2)."""
    import bench
    from ns_3d_staggered_dp_gb300 import Session, make_config
    nx, ny, nz = 256, 128, 256
    cfg = O.Config(nx, ny, nz, lx=2 * np.pi, ly=2.0, lz=2 * np.pi, nu=1.0 / 180.0, dt=2e-3, scheme=O.AB2_CN,
                   bc=(1, 2, 1), pbc=(1, 3, 1))
    u, v, w, p = bench.channel_initial_field(nx, ny, nz)
    O.vel_bc_staggered(u, v, w, O.Faces.zeros(nx, ny, nz), *cfg.bc)
    st = O.State(u, v, w, p, np.zeros_like(u), np.zeros_like(v), np.zeros_like(w), first=True)
    with Session(make_config(nx, ny, nz, lx=cfg.lx, ly=cfg.ly, lz=cfg.lz, nu=cfg.nu, dt=cfg.dt, scheme=2,
                             bc=cfg.bc, pbc=cfg.pbc)) as s:
        s.set_state(u, v, w, p)
        s.step(10)
        got = s.get_state()
        d = s.diag()
    ref = O.run(st, cfg, 10)
    for k, r in (("u", ref.u), ("v", ref.v), ("w", ref.w), ("p", ref.p), ("hx", ref.px), ("hy", ref.py), ("hz", ref.pz)):
        assert rel_l2(got[k], r) < 1e-10, k
    assert d["max_div"] < 1e-12


def test_all_wall_box_256_cubed_matches_the_oracle():
    """The 256^3 all-wall box at its own size (no-slip walls on every face,
    Neumann pressure): the x and y wall transforms through 256-point FFTs
    (Makhoul), the z axis by the twisted line solve with the singular line,
    two AB2-CN steps against the NumPy oracle."""
    import bench
    from ns_3d_staggered_dp_gb300 import Session, make_config
    O_, cfg, st, cnf, _ = bench.oracle_setup("box", 256)
    W = bench.workload("box", 256)
    ref = st.copy()
    for _ in range(2):
        ref = O.step(ref, cfg, cnf=cnf)
    with Session(make_config(256, 256, 256, **W["kw"])) as s:
        s.set_state(st.u, st.v, st.w, st.p)
        s.step(2)
        got = s.get_state()
        d = s.diag()
    for k, r in (("u", ref.u), ("v", ref.v), ("w", ref.w), ("p", ref.p), ("hx", ref.px), ("hy", ref.py), ("hz", ref.pz)):
        assert rel_l2(got[k], r) < 1e-10, k
    assert d["max_div"] < 1e-12
