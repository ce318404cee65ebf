"""Shared helpers of the parity tests (seeded synthetic states, error norms)."""
import numpy as np

from oracle import ns_oracle as O


def rel_l2(a, b):
    a = np.asarray(a); b = np.asarray(b)
    den = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0))


def random_state(cfg, seed, amp=1.0, history=False):
    """Random fields with reference-consistent ghosts for cfg's bc."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = cfg.nx, cfg.ny, cfg.nz
    st = O.State.zeros(nx, ny, nz)
    st.u = amp * rng.standard_normal(st.u.shape)
    st.v = amp * rng.standard_normal(st.v.shape)
    st.w = amp * rng.standard_normal(st.w.shape)
    st.p = amp * rng.standard_normal(st.p.shape)
    faces = O.Faces.zeros(nx, ny, nz)
    O.vel_bc_staggered(st.u, st.v, st.w, faces, *cfg.bc)
    O.pr_bc_staggered(st.p, faces, cfg.pbc, *cfg.h)
    if history:
        for name in ("px", "py", "pz"):
            setattr(st, name, amp * rng.standard_normal(getattr(st, name).shape))
        st.first = False
        # the history outside the interior ranges is never read; zero it as the library returns it
        r0, r1 = O._ranges(cfg)
        for name, sl in (("px", (r0[0], r1[1], r1[2])), ("py", (r1[0], r0[1], r1[2])), ("pz", (r1[0], r1[1], r0[2]))):
            a = getattr(st, name)
            m = np.zeros_like(a); m[sl] = a[sl]
            setattr(st, name, m)
    return st


def tgv_state(cfg, seed=1234, noise=1e-3):
    """3D Taylor-Green (u = sin x cos y cos z, v = -cos x sin y cos z, w = 0)
    plus seeded uniform noise, projected to zero divergence with the oracle's
    own Poisson solve (the synthetic stand-in for the 32^3 TGV config)."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = cfg.nx, cfg.ny, cfg.nz
    c = O.staggered_coords(nx, ny, nz, cfg.lx, cfg.ly, cfg.lz)
    xu, yu, zu = c["u"]; xv, yv, zv = c["v"]
    st = O.State.zeros(nx, ny, nz)
    st.u = np.sin(xu)[:, None, None] * np.cos(yu)[None, :, None] * np.cos(zu)[None, None, :]
    st.v = -np.cos(xv)[:, None, None] * np.sin(yv)[None, :, None] * np.cos(zv)[None, None, :]
    st.u = st.u + rng.uniform(-noise, noise, st.u.shape)
    st.v = st.v + rng.uniform(-noise, noise, st.v.shape)
    st.w = st.w + rng.uniform(-noise, noise, st.w.shape)
    return project(st, cfg)


def project(st, cfg):
    """Make the velocity discretely divergence-free with the oracle's Poisson solve."""
    faces = O.Faces.zeros(cfg.nx, cfg.ny, cfg.nz)
    O.vel_bc_staggered(st.u, st.v, st.w, faces, *cfg.bc)
    dx, dy, dz = cfg.h
    I = slice(1, -1)
    R = O.diff(st.u[:, I, I], 1, 1) / dx + O.diff(st.v[I, :, I], 1, 2) / dy + O.diff(st.w[I, I, :], 1, 3) / dz
    phi = np.zeros(st.p.shape)
    phi[1:-1, 1:-1, 1:-1] = O.poisson_solve(R, cfg, faces)
    O.pr_bc_staggered(phi, faces, cfg.pbc, dx, dy, dz)
    st.u = st.u - O.diff(phi, 1, 1) / dx
    st.v = st.v - O.diff(phi, 1, 2) / dy
    st.w = st.w - O.diff(phi, 1, 3) / dz
    return st
