"""CPU oracle of the discrete adjoint of the periodic FP64 staggered step (test infrastructure).

THIS MODULE IS TEST INFRASTRUCTURE.  Only ``tests/``, ``__graft_entry__.smoke()``
and ``bench.py``'s CPU legs may import it, and only as the checker.  The
product path (``libns_gpu.so``) never calls it.

The reference (zzwz02/NS_3D_Staggered_dp) has no adjoint.  What is
differentiated here is the reference's own periodic time step as the oracle
restates it (``ns_oracle.step``, big_periodic_3D.f90:326-567): convection
``cal_conv`` (NS_functions.f90:53-158), diffusion ``cal_diff`` (:161-210),
the Euler / AB2 / AB2-CN predictor (big_periodic_3D.f90:350-423), the CN-ADI
sweeps with ``mat_CN`` (NS_functions.f90:1245-1294, big_periodic_3D.f90:425-489),
the FFT pressure projection (:498-567), with ``dp_flag = 0`` so that p does
not feed back into the next step.

Slot form.  On a triply periodic box the step is a map of the independent
values only: the ``n`` faces (or cells) per axis of u, v, w and of the AB2
history.  They are held as periodic arrays ``(nx, ny, nz)`` indexed by
``slot - 1``, where slot m is "cell m" or "the low face of cell m" (the
reference's u(I,J,K) is slot (I, J-1, K-1), v(I,J,K) is (I-1, J, K-1),
w(I,J,K) is (I-1, J-1, K), p(I,J,K) is (I-1, J-1, K-1)).  ``step_slot``
restates ``ns_oracle.step`` in that form (a test checks the two agree),
``tlm_step`` is its tangent-linear model and ``adj_step`` the transpose of
``tlm_step``, operator by operator:

* convection: the divergence form is a sum of differences of products of
  two-point means; its adjoint scatters each product's weight back through
  the means (``conv_adj``);
* diffusion: the periodic 7-point Laplacian is symmetric;
* ADI: each sweep solves ``M x = r`` on every line with the n x n matrix that
  ``mat_CN`` reduces to once its periodic ghost rows are eliminated; the
  adjoint solves ``M^T`` in the reverse sweep order (z, y, x).  The reference
  closes row 1 of the normal-component matrix on the duplicate face
  (NS_functions.f90:1273), which makes M non-symmetric;
* projection: ``P = I - G L^+ D`` with ``D = -G^T`` on the periodic staggered
  grid, so P is symmetric.

Parity of this module: ``step_slot`` against ``ns_oracle.step`` (rounding),
``<tlm(d), l> = <d, adj(l)>`` to rounding, and central finite differences of
``step_slot`` against ``tlm_step``.
"""
from __future__ import annotations

import numpy as np

from oracle import ns_oracle as O

EULER, AB2, AB2_CN = O.EULER, O.AB2, O.AB2_CN


# ---------------------------------------------------------------------------
# Reference arrays <-> slot arrays
# ---------------------------------------------------------------------------
def _maps(cfg):
    nx, ny, nz = cfg.nx, cfg.ny, cfg.nz
    fx, fy, fz = np.arange(nx + 1) % nx, np.arange(ny + 1) % ny, np.arange(nz + 1) % nz  # face axis (slots 1..n+1)
    cx, cy, cz = (np.arange(nx + 2) - 1) % nx, (np.arange(ny + 2) - 1) % ny, (np.arange(nz + 2) - 1) % nz
    return {"u": (fx, cy, cz), "v": (cx, fy, cz), "w": (cx, cy, fz), "p": (cx, cy, cz)}


def _interior(cfg):
    nx, ny, nz = cfg.nx, cfg.ny, cfg.nz
    return {"u": (slice(0, nx), slice(1, ny + 1), slice(1, nz + 1)),
            "v": (slice(1, nx + 1), slice(0, ny), slice(1, nz + 1)),
            "w": (slice(1, nx + 1), slice(1, ny + 1), slice(0, nz))}


def restrict(a, which, cfg):
    """The independent values of a reference-shaped periodic array."""
    return np.ascontiguousarray(a[_interior(cfg)[which]])


def expand(A, which, cfg):
    """Reference-shaped array with every periodic copy filled from the slots."""
    return A[np.ix_(*_maps(cfg)[which])]


def embed(A, which, cfg):
    """Reference-shaped array with the slots at their own entries and zero
    elsewhere (history arrays; gradients with respect to the independent values)."""
    shp = {"u": (cfg.nx + 1, cfg.ny + 2, cfg.nz + 2), "v": (cfg.nx + 2, cfg.ny + 1, cfg.nz + 2),
           "w": (cfg.nx + 2, cfg.ny + 2, cfg.nz + 1)}[which]
    out = np.zeros(shp)
    out[_interior(cfg)[which]] = A
    return out


def fold(a, which, cfg):
    """Adjoint of ``expand``: every entry added into the slot it copies."""
    mx, my, mz = _maps(cfg)[which]
    out = np.zeros((cfg.nx, cfg.ny, cfg.nz))
    np.add.at(out, np.ix_(mx, my, mz), a)
    return out


def state_to_slots(st, cfg):
    return tuple(restrict(a, k, cfg) for a, k in ((st.u, "u"), (st.v, "v"), (st.w, "w"),
                                                  (st.px, "u"), (st.py, "v"), (st.pz, "w")))


def slots_to_state(S, cfg, first):
    U, V, W, HX, HY, HZ = S
    st = O.State.zeros(cfg.nx, cfg.ny, cfg.nz)
    st.u, st.v, st.w = expand(U, "u", cfg), expand(V, "v", cfg), expand(W, "w", cfg)
    st.px, st.py, st.pz = embed(HX, "u", cfg), embed(HY, "v", cfg), embed(HZ, "w", cfg)
    st.first = first
    return st


# ---------------------------------------------------------------------------
# Slot-form operators (np.roll(A, 1, ax)[i] = A[i-1], np.roll(A, -1, ax)[i] = A[i+1])
# ---------------------------------------------------------------------------
def _r(A, s, ax):
    return np.roll(A, s, axis=ax)


def conv_slot(U, V, W, h):
    """cal_conv (NS_functions.f90:53-158) on a periodic box, in slots.

    SX(c) = U(c)+U(c+1) at x-cell c; QXY(i,J) = (U(i,J-1)+U(i,J)) (V(i-1,J)+V(i,J))
    at the edge of x-face i and y-face J; likewise QXZ, QYZ, SY, SZ.
    conv_x(i) = (SX(i)^2 - SX(i-1)^2)/(4dx) + (QXY(J+1) - QXY(J))/(4dy) + (QXZ(K+1) - QXZ(K))/(4dz).
    """
    dx, dy, dz = h
    SX = U + _r(U, -1, 0); SY = V + _r(V, -1, 1); SZ = W + _r(W, -1, 2)
    QXY = (_r(U, 1, 1) + U) * (_r(V, 1, 0) + V)
    QXZ = (_r(U, 1, 2) + U) * (_r(W, 1, 0) + W)
    QYZ = (_r(V, 1, 2) + V) * (_r(W, 1, 1) + W)
    sx2, sy2, sz2 = SX * SX, SY * SY, SZ * SZ
    cx = (sx2 - _r(sx2, 1, 0)) / (4 * dx) + (_r(QXY, -1, 1) - QXY) / (4 * dy) + (_r(QXZ, -1, 2) - QXZ) / (4 * dz)
    cy = (_r(QXY, -1, 0) - QXY) / (4 * dx) + (sy2 - _r(sy2, 1, 1)) / (4 * dy) + (_r(QYZ, -1, 2) - QYZ) / (4 * dz)
    cz = (_r(QXZ, -1, 0) - QXZ) / (4 * dx) + (_r(QYZ, -1, 1) - QYZ) / (4 * dy) + (sz2 - _r(sz2, 1, 2)) / (4 * dz)
    return cx, cy, cz


def conv_tl(U, V, W, dU, dV, dW, h):
    """Tangent of conv_slot at (U, V, W) in direction (dU, dV, dW)."""
    dx, dy, dz = h
    SX = U + _r(U, -1, 0); SY = V + _r(V, -1, 1); SZ = W + _r(W, -1, 2)
    dSX = dU + _r(dU, -1, 0); dSY = dV + _r(dV, -1, 1); dSZ = dW + _r(dW, -1, 2)
    Uy, Vx = _r(U, 1, 1) + U, _r(V, 1, 0) + V
    Uz, Wx = _r(U, 1, 2) + U, _r(W, 1, 0) + W
    Vz, Wy = _r(V, 1, 2) + V, _r(W, 1, 1) + W
    dUy, dVx = _r(dU, 1, 1) + dU, _r(dV, 1, 0) + dV
    dUz, dWx = _r(dU, 1, 2) + dU, _r(dW, 1, 0) + dW
    dVz, dWy = _r(dV, 1, 2) + dV, _r(dW, 1, 1) + dW
    QXY = dUy * Vx + Uy * dVx
    QXZ = dUz * Wx + Uz * dWx
    QYZ = dVz * Wy + Vz * dWy
    sx2, sy2, sz2 = 2 * SX * dSX, 2 * SY * dSY, 2 * SZ * dSZ
    cx = (sx2 - _r(sx2, 1, 0)) / (4 * dx) + (_r(QXY, -1, 1) - QXY) / (4 * dy) + (_r(QXZ, -1, 2) - QXZ) / (4 * dz)
    cy = (_r(QXY, -1, 0) - QXY) / (4 * dx) + (sy2 - _r(sy2, 1, 1)) / (4 * dy) + (_r(QYZ, -1, 2) - QYZ) / (4 * dz)
    cz = (_r(QXZ, -1, 0) - QXZ) / (4 * dx) + (_r(QYZ, -1, 1) - QYZ) / (4 * dy) + (sz2 - _r(sz2, 1, 2)) / (4 * dz)
    return cx, cy, cz


def conv_adj(U, V, W, gx, gy, gz, h):
    """Transpose of conv_tl at (U, V, W) applied to the weights (gx, gy, gz).

    Weight of each product: A_SX(c) = (gx(c) - gx(c+1))/(4dx);
    A_XY(i,J) = (gx(i,J-1) - gx(i,J))/(4dy) + (gy(i-1,J) - gy(i,J))/(4dx); ...
    then back through the two-point sums (SX(c) holds U(c) and U(c+1), the
    y-sum of QXY at J holds U(J-1) and U(J), its x-sum V(i-1) and V(i)).
    """
    dx, dy, dz = h
    SX = U + _r(U, -1, 0); SY = V + _r(V, -1, 1); SZ = W + _r(W, -1, 2)
    Uy, Vx = _r(U, 1, 1) + U, _r(V, 1, 0) + V
    Uz, Wx = _r(U, 1, 2) + U, _r(W, 1, 0) + W
    Vz, Wy = _r(V, 1, 2) + V, _r(W, 1, 1) + W
    a_sx = 2 * SX * (gx - _r(gx, -1, 0)) / (4 * dx)
    a_sy = 2 * SY * (gy - _r(gy, -1, 1)) / (4 * dy)
    a_sz = 2 * SZ * (gz - _r(gz, -1, 2)) / (4 * dz)
    A_xy = (_r(gx, 1, 1) - gx) / (4 * dy) + (_r(gy, 1, 0) - gy) / (4 * dx)
    A_xz = (_r(gx, 1, 2) - gx) / (4 * dz) + (_r(gz, 1, 0) - gz) / (4 * dx)
    A_yz = (_r(gy, 1, 2) - gy) / (4 * dz) + (_r(gz, 1, 1) - gz) / (4 * dy)
    Ub = a_sx + _r(a_sx, 1, 0)
    Vb = a_sy + _r(a_sy, 1, 1)
    Wb = a_sz + _r(a_sz, 1, 2)
    t = A_xy * Vx; Ub = Ub + t + _r(t, -1, 1)
    t = A_xy * Uy; Vb = Vb + t + _r(t, -1, 0)
    t = A_xz * Wx; Ub = Ub + t + _r(t, -1, 2)
    t = A_xz * Uz; Wb = Wb + t + _r(t, -1, 0)
    t = A_yz * Wy; Vb = Vb + t + _r(t, -1, 2)
    t = A_yz * Vz; Wb = Wb + t + _r(t, -1, 1)
    return Ub, Vb, Wb


def lap_slot(X, h):
    """cal_diff (NS_functions.f90:161-210) on a periodic box: symmetric 7-point Laplacian."""
    dx, dy, dz = h
    return ((_r(X, 1, 0) - 2 * X + _r(X, -1, 0)) / (dx * dx) + (_r(X, 1, 1) - 2 * X + _r(X, -1, 1)) / (dy * dy)
            + (_r(X, 1, 2) - 2 * X + _r(X, -1, 2)) / (dz * dz))


def project_slot(U, V, W, cfg):
    """u - G L^+ D u: the divergence RHS, FFT Poisson solve and correction of
    big_periodic_3D.f90:498-567 (the 1/dt of the RHS and the dt of the
    correction cancel; the gauge constant does not reach the velocity)."""
    dx, dy, dz = cfg.h
    R = (_r(U, -1, 0) - U) / dx + (_r(V, -1, 1) - V) / dy + (_r(W, -1, 2) - W) / dz
    phi = O.fft_poisson(R, O.fft_eigenvalues(cfg.nx, cfg.ny, cfg.nz, dx, dy, dz))
    return U - (phi - _r(phi, 1, 0)) / dx, V - (phi - _r(phi, 1, 1)) / dy, W - (phi - _r(phi, 1, 2)) / dz


def cn_reduced(n, h, cfg, normal, closure=0):
    """The n x n line matrix of one periodic ADI sweep: mat_CN (NS_functions.f90:1245-1294)
    with its ghost rows (x(n+1) = x(1) for the normal component; x(0) = x(n),
    x(n+1) = x(1) for the tangential ones) eliminated.  closure=1 gives the
    cyclic A(1,n) in place of the reference's A(1,n+1)."""
    A, B = O.mat_cn(n, 1, h * h, cfg.dt, cfg.nu)
    if normal:
        M = A[:n, :n].copy()
        col = A[:n, n].copy()          # coefficients of face n+1
        if closure:
            M[0, n - 1] += col[0]      # row 1 tied to face n instead
            col[0] = 0.0
        M[:, 0] += col                 # slot n+1 is slot 1
        return M
    M = B[1:n + 1, 1:n + 1].copy()
    M[:, n - 1] += B[1:n + 1, 0]       # slot 0 is slot n
    M[:, 0] += B[1:n + 1, n + 1]       # slot n+1 is slot 1
    return M


class CNLines:
    """Reduced line matrices of the three sweeps: m[axis][normal]."""

    def __init__(self, cfg, closure=0):
        dx, dy, dz = cfg.h
        self.m = [[cn_reduced(n, hh, cfg, nm == 1, closure) for nm in (0, 1)]
                  for n, hh in ((cfg.nx, dx), (cfg.ny, dy), (cfg.nz, dz))]


def _solve_lines(M, X, ax):
    Xm = np.moveaxis(X, ax, 0)
    shp = Xm.shape
    return np.moveaxis(np.linalg.solve(M, Xm.reshape(shp[0], -1)).reshape(shp), 0, ax)


def adi_slot(U, V, W, lines, transpose=False):
    """The x, y, z sweeps (big_periodic_3D.f90:425-489); transpose: M^T in the order z, y, x."""
    F = [U, V, W]
    order = (2, 1, 0) if transpose else (0, 1, 2)
    for ax in order:
        for f in range(3):
            M = lines.m[ax][1 if f == ax else 0]
            F[f] = _solve_lines(M.T if transpose else M, F[f], ax)
    return tuple(F)


# ---------------------------------------------------------------------------
# One step: forward, tangent-linear, adjoint
# ---------------------------------------------------------------------------
def _check(cfg):
    if tuple(cfg.bc) != (1, 1, 1) or tuple(cfg.pbc) != (1, 1, 1) or cfg.dp_flag != 0:
        raise ValueError("the adjoint covers the triply periodic step with dp_flag = 0")


def step_slot(S, cfg, first, lines=None):
    """ns_oracle.step in slot form.  S = (U, V, W, HX, HY, HZ)."""
    _check(cfg)
    U, V, W, HX, HY, HZ = S
    h = cfg.h
    nu, dt = cfg.nu, cfg.dt
    conv = conv_slot(U, V, W, h)
    lap = [lap_slot(X, h) for X in (U, V, W)]
    F, H = (U, V, W), (HX, HY, HZ)
    if cfg.scheme == AB2_CN:
        b = 1.0 if first else 1.5
        us = [F[q] + dt * (0.5 * nu * lap[q] - b * conv[q]) - (0.0 if first else 0.5 * dt) * H[q] for q in range(3)]
        Hn = tuple(-c for c in conv)
        us = adi_slot(*us, lines or CNLines(cfg))
    else:
        rhs = [nu * lap[q] - conv[q] for q in range(3)]
        if cfg.scheme == AB2 and not first:
            us = [F[q] + dt * (1.5 * rhs[q] - 0.5 * H[q]) for q in range(3)]
        else:
            us = [F[q] + dt * rhs[q] for q in range(3)]
        Hn = tuple(rhs) if cfg.scheme == AB2 else tuple(np.zeros_like(U) for _ in range(3))
    return tuple(project_slot(*us, cfg)) + Hn


def tlm_step(S, dS, cfg, first, lines=None):
    """Tangent-linear model of step_slot at S in direction dS."""
    _check(cfg)
    U, V, W = S[:3]
    dU, dV, dW, dHX, dHY, dHZ = dS
    h = cfg.h
    nu, dt = cfg.nu, cfg.dt
    dconv = conv_tl(U, V, W, dU, dV, dW, h)
    dF, dH = (dU, dV, dW), (dHX, dHY, dHZ)
    dlap = [lap_slot(X, h) for X in dF]
    if cfg.scheme == AB2_CN:
        b = 1.0 if first else 1.5
        dus = [dF[q] + dt * (0.5 * nu * dlap[q] - b * dconv[q]) - (0.0 if first else 0.5 * dt) * dH[q]
               for q in range(3)]
        dHn = tuple(-c for c in dconv)
        dus = adi_slot(*dus, lines or CNLines(cfg))
    else:
        drhs = [nu * dlap[q] - dconv[q] for q in range(3)]
        if cfg.scheme == AB2 and not first:
            dus = [dF[q] + dt * (1.5 * drhs[q] - 0.5 * dH[q]) for q in range(3)]
        else:
            dus = [dF[q] + dt * drhs[q] for q in range(3)]
        dHn = tuple(drhs) if cfg.scheme == AB2 else tuple(np.zeros_like(U) for _ in range(3))
    return tuple(project_slot(*dus, cfg)) + dHn


def adj_step(S, lam, cfg, first, lines=None):
    """Transpose of tlm_step at S: lam = adjoints of the outputs (U', V', W', H')
    -> adjoints of the inputs (U, V, W, H)."""
    _check(cfg)
    U, V, W = S[:3]
    lU, lV, lW, lHX, lHY, lHZ = lam
    h = cfg.h
    nu, dt = cfg.nu, cfg.dt
    la = project_slot(lU, lV, lW, cfg)                    # P is symmetric
    lH = (lHX, lHY, lHZ)
    if cfg.scheme == AB2_CN:
        ls = adi_slot(*la, lines or CNLines(cfg), transpose=True)
        b = 1.0 if first else 1.5
        g = [b * dt * ls[q] + lH[q] for q in range(3)]   # weights on conv (h' = -conv)
        cb = conv_adj(U, V, W, *g, h)
        out = [ls[q] + 0.5 * dt * nu * lap_slot(ls[q], h) - cb[q] for q in range(3)]
        hb = [np.zeros_like(U) if first else -0.5 * dt * ls[q] for q in range(3)]
    else:
        ls = la
        if cfg.scheme == AB2:
            r = [(dt if first else 1.5 * dt) * ls[q] + lH[q] for q in range(3)]
            hb = [np.zeros_like(U) if first else -0.5 * dt * ls[q] for q in range(3)]
        else:
            r = [dt * ls[q] for q in range(3)]
            hb = [np.zeros_like(U) for _ in range(3)]
        cb = conv_adj(U, V, W, *r, h)
        out = [ls[q] + nu * lap_slot(r[q], h) - cb[q] for q in range(3)]
    return tuple(out) + tuple(hb)


# ---------------------------------------------------------------------------
# Whole runs and the objective
# ---------------------------------------------------------------------------
def forward(S0, cfg, nsteps, first=True, lines=None):
    """States S_0 .. S_nsteps (step 1 is the Euler start when first)."""
    lines = lines or (CNLines(cfg) if cfg.scheme == AB2_CN else None)
    traj = [S0]
    S = S0
    for n in range(nsteps):
        S = step_slot(S, cfg, first and n == 0, lines)
        traj.append(S)
    return traj


def tlm(S0, dS0, cfg, nsteps, first=True):
    lines = CNLines(cfg) if cfg.scheme == AB2_CN else None
    traj = forward(S0, cfg, nsteps, first, lines)
    dS = dS0
    for n in range(nsteps):
        dS = tlm_step(traj[n], dS, cfg, first and n == 0, lines)
    return dS


def adjoint(S0, lamT, cfg, nsteps, first=True):
    """Adjoint of the inputs S_0 given the adjoint lamT of S_nsteps."""
    lines = CNLines(cfg) if cfg.scheme == AB2_CN else None
    traj = forward(S0, cfg, nsteps, first, lines)
    lam = lamT
    for n in reversed(range(nsteps)):
        lam = adj_step(traj[n], lam, cfg, first and n == 0, lines)
    return lam


def region(cfg, frac=0.5):
    """Slot index ranges of the central box of the given fraction of each axis
    (the central 64^3 of a 128^3 grid for frac = 0.5)."""
    out = []
    for n in (cfg.nx, cfg.ny, cfg.nz):
        m = int(round(n * frac))
        lo = (n - m) // 2
        out.append(slice(lo, lo + m))
    return tuple(out)


def objective(S, target, reg):
    """J = 1/2 sum over the region of |u - u_target|^2 (u, v, w slots)."""
    return 0.5 * sum(float(np.sum((S[q][reg] - target[q][reg]) ** 2)) for q in range(3))


def objective_seed(S, target, reg):
    """dJ/dS: (u - u_target) on the region, zero elsewhere and on the history."""
    out = []
    for q in range(3):
        g = np.zeros_like(S[q])
        g[reg] = S[q][reg] - target[q][reg]
        out.append(g)
    return tuple(out) + tuple(np.zeros_like(S[0]) for _ in range(3))


def dot(a, b):
    return sum(float(np.vdot(x, y)) for x, y in zip(a, b))
