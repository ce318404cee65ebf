"""CPU oracle for the FP64 staggered-grid Navier-Stokes step (test infrastructure).

THIS MODULE IS TEST INFRASTRUCTURE.  Only ``tests/``, ``__graft_entry__.smoke()``
and the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import
it, and only as the checker or the timed CPU baseline.  The product path
(``ns_3d_staggered_dp_gb300`` and ``libns_gpu.so``) never calls it.

It is a NumPy/SciPy restatement of the reference's algorithm
(zzwz02/NS_3D_Staggered_dp, Fortran 90).  Every function cites the reference
file:line it follows.  Arrays keep the reference's padded Fortran shapes:

    u  (nx+1, ny+2, nz+2)   v  (nx+2, ny+1, nz+2)   w  (nx+2, ny+2, nz+1)
    p, dp (nx+2, ny+2, nz+2)

NumPy index ``[i-1, j-1, k-1]`` is Fortran ``(i, j, k)``.  The Intel MKL calls
of the reference (DFTI, trigonometric transforms, getrf/getrs, dttrfb/dttrsb,
PARDISO; MKL 2019.1.144, not in the reference tree) are restated from their
published definitions: the 3D real FFT by ``numpy.fft.rfftn``; the staggered
cosine/sine transforms by ``scipy.fft.dct/dst`` with the MKL normalisation
written out in ``mkl_tt_*``; the dense LU by ``scipy.linalg.lu_factor``; the
sparse LU by ``scipy.sparse.linalg.splu``.

Parity unpinned: no output of the reference itself pins this restatement.
The reference cannot be built here (Fortran + Intel MKL + HDF5; no Fortran
compiler or MKL on either machine), its ``test_subroutine.f90`` only prints,
and its ``err_file/`` logs come from a JHTDB-initialised run whose data is
not in the repository.  In place of golden vectors the oracle is checked by (i) the
reference's own bitwise check that the new and legacy stencil primitives
agree (test_subroutine.f90:137-185), restated here as ``avg_old`` and friends;
(ii) the spectral Poisson solves agreeing with a sparse LU solve of the
restated operator ``poisson_lhs_staggered`` (NS_functions.f90:1110-1242), as
the reference itself prints at re_simulation_sub_tstep_interBC_combine.f90:780;
(iii) the CN-ADI sweeps agreeing with the dense ``mat_CN`` matrices; (iv) the
properties logged in the reference's err_file/ (exact re-simulation replay,
linear response to boundary noise, temporal order); (v) 2D Taylor-Green decay.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

# ---------------------------------------------------------------------------
# Codes.  bc / pbc: 1 periodic, 2 Dirichlet on the wall, 3 Neumann on the wall,
# 4 Dirichlet on the ghost cell (NS_functions.f90:219-220).
# ---------------------------------------------------------------------------
EULER, AB2, AB2_CN = 0, 1, 2
SCHEME_NAMES = {EULER: "Euler", AB2: "AB2", AB2_CN: "AB2-CN"}


def _sl(ndim, ax, s):
    t = [slice(None)] * ndim
    t[ax] = s
    return tuple(t)


# ---------------------------------------------------------------------------
# Stencil primitives -- FD_functions.f90
# ---------------------------------------------------------------------------
def avg(A, k, bc):
    """Two-point mean along axis k (1-based).  FD_functions.f90:222-342.

    bc == 1: same size; B(1) = (A(n)+A(n-1))/2, B(i) = (A(i)+A(i-1))/2.
    otherwise: size n-1 along k; B(i) = (A(i+1)+A(i))/2.
    """
    ax = k - 1
    n = A.shape[ax]
    nd = A.ndim
    if bc == 1:
        B = np.empty_like(A)
        B[_sl(nd, ax, 0)] = (A[_sl(nd, ax, n - 1)] + A[_sl(nd, ax, n - 2)]) / 2.0
        B[_sl(nd, ax, slice(1, n))] = (A[_sl(nd, ax, slice(1, n))] + A[_sl(nd, ax, slice(0, n - 1))]) / 2.0
        return B
    return (A[_sl(nd, ax, slice(1, n))] + A[_sl(nd, ax, slice(0, n - 1))]) / 2.0


def diff(A, n_unused, k):
    """Forward difference along k, size n-1.  FD_functions.f90:345-410 (argument n unused)."""
    ax = k - 1
    n = A.shape[ax]
    nd = A.ndim
    return A[_sl(nd, ax, slice(1, n))] - A[_sl(nd, ax, slice(0, n - 1))]


def diff2(A, k, bc):
    """Three-point second difference along k.  FD_functions.f90:413-527.

    bc == 1: size n-1; B(1) = A(n-1) - 2A(1) + A(2), B(i) = A(i-1) - 2A(i) + A(i+1).
    otherwise: size n-2; B(i) = A(i) - 2A(i+1) + A(i+2).
    """
    ax = k - 1
    n = A.shape[ax]
    nd = A.ndim
    if bc == 1:
        shp = list(A.shape)
        shp[ax] = n - 1
        B = np.empty(shp, dtype=A.dtype)
        B[_sl(nd, ax, 0)] = A[_sl(nd, ax, n - 2)] - 2.0 * A[_sl(nd, ax, 0)] + A[_sl(nd, ax, 1)]
        B[_sl(nd, ax, slice(1, n - 1))] = (A[_sl(nd, ax, slice(0, n - 2))]
                                           - 2.0 * A[_sl(nd, ax, slice(1, n - 1))]
                                           + A[_sl(nd, ax, slice(2, n))])
        return B
    return (A[_sl(nd, ax, slice(0, n - 2))] - 2.0 * A[_sl(nd, ax, slice(1, n - 1))]
            + A[_sl(nd, ax, slice(2, n))])


def avg_old(A, k, bc):
    """Legacy two-point mean.  FD_functions.f90:8-88 (B(1) = B(n) for bc=1)."""
    ax = k - 1
    n = A.shape[ax]
    nd = A.ndim
    if bc == 1:
        B = np.empty_like(A)
        for i in range(n - 1):
            B[_sl(nd, ax, i + 1)] = (A[_sl(nd, ax, i + 1)] + A[_sl(nd, ax, i)]) / 2.0
        B[_sl(nd, ax, 0)] = B[_sl(nd, ax, n - 1)]
        return B
    shp = list(A.shape)
    shp[ax] = n - 1
    B = np.empty(shp, dtype=A.dtype)
    for i in range(n - 1):
        B[_sl(nd, ax, i)] = (A[_sl(nd, ax, i + 1)] + A[_sl(nd, ax, i)]) / 2.0
    return B


def diff_old(A, n_unused, k):
    """Legacy forward difference.  FD_functions.f90:91-130."""
    ax = k - 1
    n = A.shape[ax]
    nd = A.ndim
    shp = list(A.shape)
    shp[ax] = n - 1
    B = np.empty(shp, dtype=A.dtype)
    for i in range(n - 1):
        B[_sl(nd, ax, i)] = A[_sl(nd, ax, i + 1)] - A[_sl(nd, ax, i)]
    return B


def diff2_old(A, k, bc):
    """Legacy second difference.  FD_functions.f90:133-219."""
    ax = k - 1
    n = A.shape[ax]
    nd = A.ndim
    if bc == 1:
        shp = list(A.shape)
        shp[ax] = n - 1
        B = np.empty(shp, dtype=A.dtype)
        for i in range(1, n - 1):
            B[_sl(nd, ax, i)] = A[_sl(nd, ax, i - 1)] - 2.0 * A[_sl(nd, ax, i)] + A[_sl(nd, ax, i + 1)]
        B[_sl(nd, ax, 0)] = A[_sl(nd, ax, n - 2)] - 2.0 * A[_sl(nd, ax, 0)] + A[_sl(nd, ax, 1)]
        return B
    shp = list(A.shape)
    shp[ax] = n - 2
    B = np.empty(shp, dtype=A.dtype)
    for i in range(n - 2):
        B[_sl(nd, ax, i)] = A[_sl(nd, ax, i)] - 2.0 * A[_sl(nd, ax, i + 1)] + A[_sl(nd, ax, i + 2)]
    return B


# ---------------------------------------------------------------------------
# Convection and diffusion -- NS_functions.f90:53-210
# ---------------------------------------------------------------------------
def cal_conv(u, v, w, bc_x, bc_y, bc_z, dx, dy, dz):
    """Divergence-form convection on the staggered grid.  NS_functions.f90:53-158.

    Returns conv_x (nx or nx-1, ny, nz), conv_y, conv_z (sizes per bc as in
    big_periodic_3D.f90:166-181).
    """
    ux = avg(u, 1, bc_x)
    uy = avg(u, 2, 0)
    uz = avg(u, 3, 0)
    vx = avg(v, 1, 0)
    vy = avg(v, 2, bc_y)
    vz = avg(v, 3, 0)
    wx = avg(w, 1, 0)
    wy = avg(w, 2, 0)
    wz = avg(w, 3, bc_z)
    I = slice(1, -1)
    if bc_x == 1:
        a = ux[:, I, I]
        cx = diff(a * a, 1, 1) / dx
        cx = cx + diff(uy[:-1, :, I] * vx[:-1, :, I], 1, 2) / dy
        cx = cx + diff(uz[:-1, I, :] * wx[:-1, I, :], 1, 3) / dz
    else:
        a = ux[:, I, I]
        cx = diff(a * a, 1, 1) / dx
        cx = cx + diff(uy[I, :, I] * vx[I, :, I], 1, 2) / dy
        cx = cx + diff(uz[I, I, :] * wx[I, I, :], 1, 3) / dz
    if bc_y == 1:
        cy = diff(vx[:, :-1, I] * uy[:, :-1, I], 1, 1) / dx
        b = vy[I, :, I]
        cy = cy + diff(b * b, 1, 2) / dy
        cy = cy + diff(vz[I, :-1, :] * wy[I, :-1, :], 1, 3) / dz
    else:
        cy = diff(vx[:, I, I] * uy[:, I, I], 1, 1) / dx
        b = vy[I, :, I]
        cy = cy + diff(b * b, 1, 2) / dy
        cy = cy + diff(vz[I, I, :] * wy[I, I, :], 1, 3) / dz
    if bc_z == 1:
        cz = diff(wx[:, I, :-1] * uz[:, I, :-1], 1, 1) / dx
        cz = cz + diff(wy[I, :, :-1] * vz[I, :, :-1], 1, 2) / dy
        c = wz[I, I, :]
        cz = cz + diff(c * c, 1, 3) / dz
    else:
        cz = diff(wx[:, I, I] * uz[:, I, I], 1, 1) / dx
        cz = cz + diff(wy[I, :, I] * vz[I, :, I], 1, 2) / dy
        c = wz[I, I, :]
        cz = cz + diff(c * c, 1, 3) / dz
    return cx, cy, cz


def cal_diff(u, v, w, bc_x, bc_y, bc_z, dx2, dy2, dz2):
    """Seven-point Laplacian per component.  NS_functions.f90:161-210."""
    I = slice(1, -1)
    if bc_x == 1:
        dxx = diff2(u[:, I, I], 1, bc_x) / dx2
        dxx = dxx + diff2(u[:-1, :, I], 2, 0) / dy2
        dxx = dxx + diff2(u[:-1, I, :], 3, 0) / dz2
    else:
        dxx = diff2(u[:, I, I], 1, bc_x) / dx2
        dxx = dxx + diff2(u[I, :, I], 2, 0) / dy2
        dxx = dxx + diff2(u[I, I, :], 3, 0) / dz2
    if bc_y == 1:
        dyy = diff2(v[:, :-1, I], 1, 0) / dx2
        dyy = dyy + diff2(v[I, :, I], 2, bc_y) / dy2
        dyy = dyy + diff2(v[I, :-1, :], 3, 0) / dz2
    else:
        dyy = diff2(v[:, I, I], 1, 0) / dx2
        dyy = dyy + diff2(v[I, :, I], 2, bc_y) / dy2
        dyy = dyy + diff2(v[I, I, :], 3, 0) / dz2
    if bc_z == 1:
        dzz = diff2(w[:, I, :-1], 1, 0) / dx2
        dzz = dzz + diff2(w[I, :, :-1], 2, 0) / dy2
        dzz = dzz + diff2(w[I, I, :], 3, bc_z) / dz2
    else:
        dzz = diff2(w[:, I, I], 1, 0) / dx2
        dzz = dzz + diff2(w[I, :, I], 2, 0) / dy2
        dzz = dzz + diff2(w[I, I, :], 3, bc_z) / dz2
    return dxx, dyy, dzz


# ---------------------------------------------------------------------------
# Boundary faces
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class Faces:
    """The 24 boundary face arrays of the reference (big_periodic_3D.f90:53-56).

    Keys are the reference names without the ``b`` prefix, e.g. ``x_u_1`` is
    ``bx_u_1`` (ny+2, nz+2) and ``z_w_nz`` is ``bz_w_nz`` (nx+2, ny+2).
    """
    d: dict

    @staticmethod
    def shapes(nx, ny, nz):
        return {
            "x_u_1": (ny + 2, nz + 2), "x_u_n": (ny + 2, nz + 2),
            "y_u_1": (nx + 1, nz + 2), "y_u_n": (nx + 1, nz + 2),
            "z_u_1": (nx + 1, ny + 2), "z_u_n": (nx + 1, ny + 2),
            "x_v_1": (ny + 1, nz + 2), "x_v_n": (ny + 1, nz + 2),
            "y_v_1": (nx + 2, nz + 2), "y_v_n": (nx + 2, nz + 2),
            "z_v_1": (nx + 2, ny + 1), "z_v_n": (nx + 2, ny + 1),
            "x_w_1": (ny + 2, nz + 1), "x_w_n": (ny + 2, nz + 1),
            "y_w_1": (nx + 2, nz + 1), "y_w_n": (nx + 2, nz + 1),
            "z_w_1": (nx + 2, ny + 2), "z_w_n": (nx + 2, ny + 2),
            "x_p_1": (ny + 2, nz + 2), "x_p_n": (ny + 2, nz + 2),
            "y_p_1": (nx + 2, nz + 2), "y_p_n": (nx + 2, nz + 2),
            "z_p_1": (nx + 2, ny + 2), "z_p_n": (nx + 2, ny + 2),
        }

    @classmethod
    def zeros(cls, nx, ny, nz):
        return cls({k: np.zeros(s) for k, s in cls.shapes(nx, ny, nz).items()})

    def __getitem__(self, k):
        return self.d[k]


def vel_bc_staggered(us, vs, ws, f, bc_x, bc_y, bc_z):
    """Ghost/face fill of u*, v*, w* per bc code (in place).  NS_functions.f90:213-310."""
    if bc_x == 1:
        us[-1] = us[0]
        vs[0] = vs[-2]
        vs[-1] = vs[1]
        ws[0] = ws[-2]
        ws[-1] = ws[1]
    elif bc_x == 2:
        us[0] = f["x_u_1"]
        us[-1] = f["x_u_n"]
        vs[0] = 2 * f["x_v_1"] - vs[1]
        vs[-1] = 2 * f["x_v_n"] - vs[-2]
        ws[0] = 2 * f["x_w_1"] - ws[1]
        ws[-1] = 2 * f["x_w_n"] - ws[-2]
    elif bc_x == 4:
        us[0] = f["x_u_1"]; us[-1] = f["x_u_n"]
        vs[0] = f["x_v_1"]; vs[-1] = f["x_v_n"]
        ws[0] = f["x_w_1"]; ws[-1] = f["x_w_n"]
    if bc_y == 1:
        us[:, 0] = us[:, -2]
        us[:, -1] = us[:, 1]
        vs[:, -1] = vs[:, 0]
        ws[:, 0] = ws[:, -2]
        ws[:, -1] = ws[:, 1]
    elif bc_y == 2:
        us[:, 0] = 2 * f["y_u_1"] - us[:, 1]
        us[:, -1] = 2 * f["y_u_n"] - us[:, -2]
        vs[:, 0] = f["y_v_1"]
        vs[:, -1] = f["y_v_n"]
        ws[:, 0] = 2 * f["y_w_1"] - ws[:, 1]
        ws[:, -1] = 2 * f["y_w_n"] - ws[:, -2]
    elif bc_y == 4:
        us[:, 0] = f["y_u_1"]; us[:, -1] = f["y_u_n"]
        vs[:, 0] = f["y_v_1"]; vs[:, -1] = f["y_v_n"]
        ws[:, 0] = f["y_w_1"]; ws[:, -1] = f["y_w_n"]
    if bc_z == 1:
        us[:, :, 0] = us[:, :, -2]
        us[:, :, -1] = us[:, :, 1]
        vs[:, :, 0] = vs[:, :, -2]
        vs[:, :, -1] = vs[:, :, 1]
        ws[:, :, -1] = ws[:, :, 0]
    elif bc_z == 2:
        us[:, :, 0] = 2 * f["z_u_1"] - us[:, :, 1]
        us[:, :, -1] = 2 * f["z_u_n"] - us[:, :, -2]
        vs[:, :, 0] = 2 * f["z_v_1"] - vs[:, :, 1]
        vs[:, :, -1] = 2 * f["z_v_n"] - vs[:, :, -2]
        ws[:, :, 0] = f["z_w_1"]
        ws[:, :, -1] = f["z_w_n"]
    elif bc_z == 4:
        us[:, :, 0] = f["z_u_1"]; us[:, :, -1] = f["z_u_n"]
        vs[:, :, 0] = f["z_v_1"]; vs[:, :, -1] = f["z_v_n"]
        ws[:, :, 0] = f["z_w_1"]; ws[:, :, -1] = f["z_w_n"]


def vel_bc_staggered_cn2(us, vs, ws, f, bc, d):
    """BC rows of one ADI sweep (in place).  NS_functions.f90:313-410.

    ``f`` holds this sweep's faces (keys x_u_1 ... as in ``Faces``; only the
    axis ``d`` keys are read).  bc=1 zeroes the periodic closure rows.
    """
    a = "xyz"[d - 1]
    if d == 1:
        if bc == 1:
            us[-1] = 0.0; vs[0] = 0.0; vs[-1] = 0.0; ws[0] = 0.0; ws[-1] = 0.0
        elif bc in (2, 4):
            us[0] = f[a + "_u_1"]; us[-1] = f[a + "_u_n"]
            vs[0] = f[a + "_v_1"]; vs[-1] = f[a + "_v_n"]
            ws[0] = f[a + "_w_1"]; ws[-1] = f[a + "_w_n"]
    elif d == 2:
        if bc == 1:
            us[:, 0] = 0.0; us[:, -1] = 0.0; vs[:, -1] = 0.0; ws[:, 0] = 0.0; ws[:, -1] = 0.0
        elif bc in (2, 4):
            us[:, 0] = f[a + "_u_1"]; us[:, -1] = f[a + "_u_n"]
            vs[:, 0] = f[a + "_v_1"]; vs[:, -1] = f[a + "_v_n"]
            ws[:, 0] = f[a + "_w_1"]; ws[:, -1] = f[a + "_w_n"]
    else:
        if bc == 1:
            us[:, :, 0] = 0.0; us[:, :, -1] = 0.0; vs[:, :, 0] = 0.0; vs[:, :, -1] = 0.0; ws[:, :, -1] = 0.0
        elif bc in (2, 4):
            us[:, :, 0] = f[a + "_u_1"]; us[:, :, -1] = f[a + "_u_n"]
            vs[:, :, 0] = f[a + "_v_1"]; vs[:, :, -1] = f[a + "_v_n"]
            ws[:, :, 0] = f[a + "_w_1"]; ws[:, :, -1] = f[a + "_w_n"]


def get_pr_bc(p_bc, pbc, dx, dy, dz):
    """Pressure faces from a (sub-)block.  NS_functions.f90:514-562 (returns dict)."""
    out = {}
    for a, (pb, h) in zip("xyz", zip(pbc, (dx, dy, dz))):
        ax = "xyz".index(a)
        lo = np.take(p_bc, 0, axis=ax); lo2 = np.take(p_bc, 1, axis=ax)
        hi = np.take(p_bc, -1, axis=ax); hi2 = np.take(p_bc, -2, axis=ax)
        if pb == 2:
            out[a + "_p_1"] = (lo + lo2) / 2
            out[a + "_p_n"] = (hi + hi2) / 2
        elif pb == 4:
            out[a + "_p_1"] = lo.copy()
            out[a + "_p_n"] = hi.copy()
        elif pb == 3:
            out[a + "_p_1"] = (lo2 - lo) / h
            out[a + "_p_n"] = (hi - hi2) / h
    return out


def get_velpr_bc(u_bc, v_bc, w_bc, p_bc, bc, pbc, dx, dy, dz, dt, dp_flag, using_ustar, p_previous):
    """Velocity and pressure faces from a parent sub-block.  NS_functions.f90:414-510.

    Returns a ``Faces`` with the faces the bc codes define (others zero).
    """
    nx = u_bc.shape[0] - 1
    ny = v_bc.shape[1] - 1
    nz = w_bc.shape[2] - 1
    f = Faces.zeros(nx, ny, nz)
    if not (bc[0] == 1 and bc[1] == 1 and bc[2] == 1):
        if not (dp_flag or using_ustar):
            uc = u_bc + diff(p_previous, 1, 1) / dx * dt
            vc = v_bc + diff(p_previous, 1, 2) / dy * dt
            wc = w_bc + diff(p_previous, 1, 3) / dz * dt
        else:
            uc, vc, wc = u_bc, v_bc, w_bc
        if bc[0] == 2:
            f.d["x_u_1"] = uc[0].copy(); f.d["x_u_n"] = uc[nx].copy()
            f.d["x_v_1"] = (vc[0] + vc[1]) / 2; f.d["x_v_n"] = (vc[nx + 1] + vc[nx]) / 2
            f.d["x_w_1"] = (wc[0] + wc[1]) / 2; f.d["x_w_n"] = (wc[nx + 1] + wc[nx]) / 2
        elif bc[0] == 4:
            f.d["x_u_1"] = uc[0].copy(); f.d["x_u_n"] = uc[nx].copy()
            f.d["x_v_1"] = vc[0].copy(); f.d["x_v_n"] = vc[nx + 1].copy()
            f.d["x_w_1"] = wc[0].copy(); f.d["x_w_n"] = wc[nx + 1].copy()
        if bc[1] == 2:
            f.d["y_u_1"] = (uc[:, 0] + uc[:, 1]) / 2; f.d["y_u_n"] = (uc[:, ny + 1] + uc[:, ny]) / 2
            f.d["y_v_1"] = vc[:, 0].copy(); f.d["y_v_n"] = vc[:, ny].copy()
            f.d["y_w_1"] = (wc[:, 0] + wc[:, 1]) / 2; f.d["y_w_n"] = (wc[:, ny + 1] + wc[:, ny]) / 2
        elif bc[1] == 4:
            f.d["y_u_1"] = uc[:, 0].copy(); f.d["y_u_n"] = uc[:, ny + 1].copy()
            f.d["y_v_1"] = vc[:, 0].copy(); f.d["y_v_n"] = vc[:, ny].copy()
            f.d["y_w_1"] = wc[:, 0].copy(); f.d["y_w_n"] = wc[:, ny + 1].copy()
        if bc[2] == 2:
            f.d["z_u_1"] = (uc[:, :, 0] + uc[:, :, 1]) / 2; f.d["z_u_n"] = (uc[:, :, nz + 1] + uc[:, :, nz]) / 2
            f.d["z_v_1"] = (vc[:, :, 0] + vc[:, :, 1]) / 2; f.d["z_v_n"] = (vc[:, :, nz + 1] + vc[:, :, nz]) / 2
            f.d["z_w_1"] = wc[:, :, 0].copy(); f.d["z_w_n"] = wc[:, :, nz].copy()
        elif bc[2] == 4:
            f.d["z_u_1"] = uc[:, :, 0].copy(); f.d["z_u_n"] = uc[:, :, nz + 1].copy()
            f.d["z_v_1"] = vc[:, :, 0].copy(); f.d["z_v_n"] = vc[:, :, nz + 1].copy()
            f.d["z_w_1"] = wc[:, :, 0].copy(); f.d["z_w_n"] = wc[:, :, nz].copy()
    f.d.update(get_pr_bc(p_bc, pbc, dx, dy, dz))
    return f


# ---------------------------------------------------------------------------
# Crank-Nicolson matrices -- NS_functions.f90:1245-1342
# ---------------------------------------------------------------------------
def mat_cn(n, bc, dx2, dt0, nu):
    """Dense CN matrices A (n+1, normal component) and B (n+2, tangential).

    NS_functions.f90:1245-1294.  For bc=1 the reference closes row 1 of A
    with A(1,n+1) (the duplicate periodic face) rather than A(1,n); the
    oracle keeps that exactly.
    """
    idx2 = 1.0 / dx2
    dg = 1.0 + 0.5 * dt0 * nu * 2.0 * idx2
    of = -0.5 * dt0 * nu * 1.0 * idx2
    A = np.zeros((n + 1, n + 1))
    B = np.zeros((n + 2, n + 2))
    for i in range(1, n):            # Fortran i = 2..n
        A[i, i] = dg; A[i, i - 1] = of; A[i, i + 1] = of
    for i in range(1, n + 1):        # Fortran i = 2..n+1
        B[i, i] = dg; B[i, i - 1] = of; B[i, i + 1] = of
    if bc == 1:
        A[0, 0] = dg; A[0, 1] = of; A[0, n] = of
        A[n, n] = 1.0; A[n, 0] = -1.0
        B[0, 0] = 1.0; B[0, n] = -1.0
        B[n + 1, n + 1] = 1.0; B[n + 1, 1] = -1.0
    elif bc == 2:
        A[0, 0] = 1.0; A[n, n] = 1.0
        B[0, 0] = 0.5; B[0, 1] = 0.5
        B[n + 1, n + 1] = 0.5; B[n + 1, n] = 0.5
    elif bc == 4:
        A[0, 0] = 1.0; A[n, n] = 1.0
        B[0, 0] = 1.0; B[n + 1, n + 1] = 1.0
    return A, B


def mat_cn_tridiagonal(n, bc, dx2, dt0, nu):
    """Banded CN matrices (bc != 1).  NS_functions.f90:1297-1342.

    Returns (A_low, A_d, A_up, B_low, B_d, B_up).  For bc=1 the reference
    leaves the closure rows unset (non-cyclic); callers must not use it there.
    """
    A, B = mat_cn(n, bc, dx2, dt0, nu)
    return (np.diag(A, -1).copy(), np.diag(A).copy(), np.diag(A, 1).copy(),
            np.diag(B, -1).copy(), np.diag(B).copy(), np.diag(B, 1).copy())


def _lu(M):
    import scipy.linalg as sla
    return sla.lu_factor(M)


def _lu_solve_axis(lu, X, ax):
    """getrs on every line of X along axis ax (big_periodic_3D.f90:425-482)."""
    import scipy.linalg as sla
    Xm = np.moveaxis(X, ax, 0)
    shp = Xm.shape
    sol = sla.lu_solve(lu, Xm.reshape(shp[0], -1))
    return np.moveaxis(sol.reshape(shp), 0, ax)


class CNFactors:
    """getrf of the six CN matrices (big_periodic_3D.f90:171-187)."""

    def __init__(self, nx, ny, nz, bc, dx2, dy2, dz2, dt0, nu):
        self.lu = []
        for n, b, h2 in ((nx, bc[0], dx2), (ny, bc[1], dy2), (nz, bc[2], dz2)):
            A, B = mat_cn(n, b, h2, dt0, nu)
            self.lu.append((_lu(A), _lu(B)))


def adi_sweeps(us, vs, ws, cnf, bc, faces_per_sweep=None):
    """The three CN-ADI sweeps with their BC rows (in place).

    big_periodic_3D.f90:425-489 (getrs) and
    re_simulation_sub_tstep_interBC_combine.f90:656-701 (dttrsb) compute the
    same thing for bc != 1.  ``faces_per_sweep[d]`` are the faces for sweep d
    (default zero, as in big_periodic_3D where the b* arrays stay 0).
    Returns the arrays (new objects).
    """
    nx, ny, nz = us.shape[0] - 1, vs.shape[1] - 1, ws.shape[2] - 1
    if faces_per_sweep is None:
        z = Faces.zeros(nx, ny, nz)
        faces_per_sweep = (z, z, z)
    us = us.copy(); vs = vs.copy(); ws = ws.copy()
    # x sweep: u normal (A), v, w tangential (B)
    vel_bc_staggered_cn2(us, vs, ws, faces_per_sweep[0], bc[0], 1)
    (luA, luB) = cnf.lu[0]
    us = _lu_solve_axis(luA, us, 0)
    vs = _lu_solve_axis(luB, vs, 0)
    ws = _lu_solve_axis(luB, ws, 0)
    # y sweep: v normal (C), u, w tangential (D)
    vel_bc_staggered_cn2(us, vs, ws, faces_per_sweep[1], bc[1], 2)
    (luC, luD) = cnf.lu[1]
    us = _lu_solve_axis(luD, us, 1)
    vs = _lu_solve_axis(luC, vs, 1)
    ws = _lu_solve_axis(luD, ws, 1)
    # z sweep: w normal (E), u, v tangential (F)
    vel_bc_staggered_cn2(us, vs, ws, faces_per_sweep[2], bc[2], 3)
    (luE, luF) = cnf.lu[2]
    us = _lu_solve_axis(luF, us, 2)
    vs = _lu_solve_axis(luF, vs, 2)
    ws = _lu_solve_axis(luE, ws, 2)
    return us, vs, ws


# ---------------------------------------------------------------------------
# Pressure BCs -- NS_functions.f90:1345-1464
# ---------------------------------------------------------------------------
def pr_bc_staggered_modify_rhs(R, f, pbc, dx, dy, dz):
    """Move the pressure BC into the Poisson RHS (in place).  NS_functions.f90:1345-1400.

    ``f`` holds the interior parts of the p faces (e.g. x_p_1 of shape (ny, nz)),
    as the reference passes bx_p_1(2:nyp-1, 2:nzp-1) (big_periodic_3D.f90:503-505).
    """
    for ax, (pb, h) in enumerate(zip(pbc, (dx, dy, dz))):
        a = "xyz"[ax]
        lo = _sl(3, ax, 0)
        hi = _sl(3, ax, -1)
        if pb == 2:
            R[lo] = R[lo] - 2 * f[a + "_p_1"] / (h * h)
            R[hi] = R[hi] - 2 * f[a + "_p_n"] / (h * h)
        elif pb == 3:
            R[lo] = R[lo] + f[a + "_p_1"] / h
            R[hi] = R[hi] - f[a + "_p_n"] / h
        elif pb == 4:
            R[lo] = R[lo] - f[a + "_p_1"] / (h * h)
            R[hi] = R[hi] - f[a + "_p_n"] / (h * h)


def pr_bc_staggered(dp, f, pbc, dx, dy, dz):
    """dp ghost fill (in place).  NS_functions.f90:1403-1464."""
    for ax, (pb, h) in enumerate(zip(pbc, (dx, dy, dz))):
        a = "xyz"[ax]
        lo, lo2 = _sl(3, ax, 0), _sl(3, ax, 1)
        hi, hi2 = _sl(3, ax, -1), _sl(3, ax, -2)
        if pb == 1:
            dp[lo] = dp[hi2]
            dp[hi] = dp[lo2]
        elif pb == 2:
            dp[lo] = 2 * f[a + "_p_1"] - dp[lo2]
            dp[hi] = 2 * f[a + "_p_n"] - dp[hi2]
        elif pb == 3:
            dp[lo] = -h * f[a + "_p_1"] + dp[lo2]
            dp[hi] = h * f[a + "_p_n"] + dp[hi2]
        elif pb == 4:
            dp[lo] = f[a + "_p_1"]
            dp[hi] = f[a + "_p_n"]


def interior_p_faces(f, nx, ny, nz):
    """The interior parts passed to pr_bc_staggered_modify_rhs (big_periodic_3D.f90:503-505)."""
    out = {}
    for k, v in f.d.items():
        if "_p_" in k:
            out[k] = v[1:-1, 1:-1]
    return out


# ---------------------------------------------------------------------------
# Poisson operator and solvers
# ---------------------------------------------------------------------------
def poisson_lhs_staggered(nx, ny, nz, dx2, dy2, dz2, pbc):
    """Sparse discrete Laplacian (CSR).  NS_functions.f90:1110-1242.

    -kron(Iz,Iy,Ax) - ... in the reference's comment is realised there as the
    positive sum kron(kron(Iz,Iy),Ax) + kron(kron(Iz,Ay),Ix) + kron(kron(Az,Iy),Ix)
    (the COO adds at :1223-1232); x is the fastest index.
    """
    import scipy.sparse as sp

    def a1(n, pb, h2):
        A = (np.diag(-2.0 * np.ones(n)) + np.diag(np.ones(n - 1), 1) + np.diag(np.ones(n - 1), -1))
        if pb == 1:
            A[0, n - 1] = 1; A[n - 1, 0] = 1
        elif pb == 2:
            A[0, 0] = -3; A[n - 1, n - 1] = -3
        elif pb == 3:
            A[0, 0] = -1; A[n - 1, n - 1] = -1
        return sp.csr_matrix(A / h2)

    Ax = a1(nx, pbc[0], dx2)
    Ay = a1(ny, pbc[1], dy2)
    Az = a1(nz, pbc[2], dz2)
    Ix, Iy, Iz = sp.identity(nx), sp.identity(ny), sp.identity(nz)
    L = sp.kron(sp.kron(Iz, Iy), Ax) + sp.kron(sp.kron(Iz, Ay), Ix) + sp.kron(sp.kron(Az, Iy), Ix)
    return L.tocsr()


def fft_eigenvalues(nx, ny, nz, dx, dy, dz):
    """poisson_eigv (nx/2+1, ny, nz) with the +Inf mean mode.  big_periodic_3D.f90:242-255."""
    pi = 3.1415926535897932
    ex = (np.sin(pi * np.arange(nx // 2 + 1) / nx) / dx) ** 2
    ey = (np.sin(pi * np.arange(ny) / ny) / dy) ** 2
    ez = (np.sin(pi * np.arange(nz) / nz) / dz) ** 2
    e = ex[:, None, None] + ey[None, :, None]
    e = e + ez[None, None, :]
    e = -4.0 * e
    e[0, 0, 0] = np.inf
    return e


def fft_poisson(R, eig):
    """r2c 3D DFT, divide, c2r with 1/N.  big_periodic_3D.f90:526-541.

    MKL DFTI with x the fastest index equals numpy rfftn over axes (2,1,0)
    with the half axis first, i.e. rfftn on the transposed array.
    """
    Rt = np.ascontiguousarray(R.transpose(2, 1, 0))
    F = np.fft.rfftn(Rt)                      # (nz, ny, nx/2+1)
    F = F / eig.transpose(2, 1, 0)
    out = np.fft.irfftn(F, s=Rt.shape, axes=(0, 1, 2))  # includes 1/N
    return np.ascontiguousarray(out.transpose(2, 1, 0))


# MKL trigonometric transforms (MKL 2019 definitions, restated):
#   backward staggered cosine  f(i) = sum_{k=0}^{n-1} F(k) cos((2k+1) i pi / (2n))    (as used: = DCT-II/2)
#   forward  staggered cosine  F(k) = f(0)/n + (2/n) sum_{i=1}^{n-1} f(i) cos((2k+1) i pi/(2n))  (= DCT-III/n)
# The reference applies "backward" to spatial data (index k = cell) and
# "forward" to spectral data, so the pair is an exact inverse.
def mkl_tt_backward_cos(x, axis):
    import scipy.fft as sfft
    return sfft.dct(x, type=2, axis=axis) / 2.0


def mkl_tt_forward_cos(X, axis):
    import scipy.fft as sfft
    n = X.shape[axis]
    return sfft.dct(X, type=3, axis=axis) / n


def _flip_odd_1based(x, axis):
    y = x.copy()
    y[_sl(x.ndim, axis, slice(0, None, 2))] *= -1.0
    return y


def dct_eigenvalues(nx, ny, nz, dx2, dy2, dz2, pbc):
    """eig_tt (nx, ny, nz).  re_simulation_sub_tstep_interBC_combine.f90:320-353.

    The z table is kept in the natural wavenumber order; the reference stores it
    z-reversed for pbc_z=2 (:343) to skip the z reversal in DCT_poisson_solver
    (NS_functions.f90:1561,1584), an equivalent permutation.  pbc=4 uses
    sin(i pi/(2(n+1))) as the reference does.
    """
    pi = 3.1415926535897932

    def e1(n, pb, h2):
        i = np.arange(1, n + 1)
        if pb == 2:
            return np.sin(i * pi / 2 / n) ** 2 / h2
        if pb == 3:
            return np.sin((i - 1) * pi / 2 / n) ** 2 / h2
        if pb == 4:
            return np.sin(i * pi / 2 / (n + 1)) ** 2 / h2
        raise ValueError("pbc must be 2, 3 or 4 for the DCT solver")

    e = e1(nx, pbc[0], dx2)[:, None, None] + e1(ny, pbc[1], dy2)[None, :, None]
    e = e + e1(nz, pbc[2], dz2)[None, None, :]
    e = -4.0 * e
    if e[0, 0, 0] == 0.0:
        e[0, 0, 0] = np.inf
    return e


def _tt_fwd(x, axis, pb):
    """Forward trigonometric transform of one axis as DCT_poisson_solver does it."""
    import scipy.fft as sfft
    if pb == 2:   # DST-2: flip every other input, iDCT-3 (MKL backward), reverse
        y = mkl_tt_backward_cos(_flip_odd_1based(x, axis), axis)
        return np.flip(y, axis=axis).copy()
    if pb == 3:   # DCT-2 (MKL backward staggered cosine)
        return mkl_tt_backward_cos(x, axis)
    if pb == 4:   # DST-1 (restated on n points; see DESIGN notes on pbc=4)
        return sfft.dst(x, type=1, axis=axis) / 2.0
    raise ValueError(pb)


def _tt_inv(X, axis, pb):
    import scipy.fft as sfft
    if pb == 2:   # reverse, MKL forward staggered cosine, flip every other output
        y = mkl_tt_forward_cos(np.flip(X, axis=axis), axis)
        return _flip_odd_1based(y, axis)
    if pb == 3:
        return mkl_tt_forward_cos(X, axis)
    if pb == 4:
        n = X.shape[axis]
        return sfft.dst(X, type=1, axis=axis) / (n + 1)
    raise ValueError(pb)


def dct_poisson(R, eig, pbc, mean_dp):
    """DCT/DST Poisson solve.  NS_functions.f90:1505-1630.

    x, y, z forward transforms, divide by eig, the (1,1,1) mode set to
    mean_dp*nx*ny*nz when eig(1,1,1) is infinite (:1576-1577), inverse z, y, x.
    """
    nx, ny, nz = R.shape
    F = _tt_fwd(R, 0, pbc[0])
    F = _tt_fwd(F, 1, pbc[1])
    F = _tt_fwd(F, 2, pbc[2])
    F = F / eig
    if np.isinf(eig[0, 0, 0]):
        F[0, 0, 0] = mean_dp * nx * ny * nz
    F = _tt_inv(F, 2, pbc[2])
    F = _tt_inv(F, 1, pbc[1])
    F = _tt_inv(F, 0, pbc[0])
    return F


def spectral_poisson(R, pbc, dx, dy, dz, mean_dp=0.0):
    """Per-axis spectral solve of poisson_lhs_staggered for any pbc mix.

    Periodic axes use a complex DFT, the others the transforms of
    ``dct_poisson``.  For all-periodic pbc this is the same math as
    ``fft_poisson``; for pbc in {2,3,4} it is ``dct_poisson``.  The mixed
    case (e.g. x,z periodic with y walls) has no reference solver; it is
    checked against ``poisson_lhs_staggered`` with a sparse LU.  The
    singular mode (all axes periodic/Neumann) is set to mean_dp.
    """
    pi = 3.1415926535897932
    n = R.shape
    hs = (dx, dy, dz)
    F = R.astype(complex)
    lam = np.zeros(n)
    for ax in range(3):
        pb = pbc[ax]
        m = n[ax]
        h2 = hs[ax] ** 2
        if pb == 1:
            F = np.fft.fft(F, axis=ax)
            e = -4.0 * (np.sin(pi * np.arange(m) / m)) ** 2 / h2
        else:
            F = _tt_fwd(F.real, ax, pb) + 1j * _tt_fwd(F.imag, ax, pb)
            i = np.arange(1, m + 1)
            if pb == 2:
                e = -4.0 * np.sin(i * pi / 2 / m) ** 2 / h2
            elif pb == 3:
                e = -4.0 * np.sin((i - 1) * pi / 2 / m) ** 2 / h2
            else:
                e = -4.0 * np.sin(i * pi / 2 / (m + 1)) ** 2 / h2
        shp = [1, 1, 1]
        shp[ax] = m
        lam = lam + e.reshape(shp)
    sing = lam[0, 0, 0] == 0.0
    if sing:
        lam[0, 0, 0] = np.inf
    F = F / lam
    if sing:
        F[0, 0, 0] = mean_dp * n[0] * n[1] * n[2]
    for ax in (2, 1, 0):
        pb = pbc[ax]
        if pb == 1:
            F = np.fft.ifft(F, axis=ax)
        else:
            F = _tt_inv(F.real, ax, pb) + 1j * _tt_inv(F.imag, ax, pb)
    return F.real.copy()


def lu_poisson(R, pbc, dx, dy, dz):
    """Sparse LU solve of poisson_lhs_staggered (big_periodic_3D.f90:507-523)."""
    import scipy.sparse.linalg as spla
    nx, ny, nz = R.shape
    L = poisson_lhs_staggered(nx, ny, nz, dx * dx, dy * dy, dz * dz, pbc)
    b = R.reshape(-1, order="F")
    return spla.splu(L.tocsc()).solve(b).reshape((nx, ny, nz), order="F")


# ---------------------------------------------------------------------------
# Initial conditions and metrics
# ---------------------------------------------------------------------------
def tgv(x, y, z, t, nu, which):
    """2D Taylor-Green vortex.  NS_functions.f90:18-50."""
    f = math.exp(-2 * nu * t)
    X, Y = np.meshgrid(x, y, indexing="ij")
    if which == "u":
        a = np.cos(X) * np.sin(Y) * f
    elif which == "v":
        a = -np.sin(X) * np.cos(Y) * f
    else:
        a = -0.25 * (np.cos(2.0 * X) + np.cos(2.0 * Y)) * f * f
    return np.repeat(a[:, :, None], len(z), axis=2)


def mean(a):
    """other_utility.f90:110-118."""
    return float(np.sum(a) / a.size)


def rms(a):
    """other_utility.f90:121-129."""
    return float(np.sqrt(np.sum(a * a) / a.size))


def staggered_coords(nx, ny, nz, lx, ly, lz):
    """xu, yu, ... as at big_periodic_3D.f90:15-18."""
    dx, dy, dz = lx / nx, ly / ny, lz / nz
    face = lambda n, h: np.arange(0, n + 1) * h
    cell = lambda n, h: (np.arange(-1, n + 1) + 0.5) * h
    return {
        "u": (face(nx, dx), cell(ny, dy), cell(nz, dz)),
        "v": (cell(nx, dx), face(ny, dy), cell(nz, dz)),
        "w": (cell(nx, dx), cell(ny, dy), face(nz, dz)),
        "p": (cell(nx, dx), cell(ny, dy), cell(nz, dz)),
    }


def max_div(u, v, w, dx, dy, dz):
    """max|div u| diagnostic.  big_periodic_3D.f90:576-579."""
    I = slice(1, -1)
    d = diff_old(u[:, I, I], 1, 1) / dx + diff_old(v[I, :, I], 1, 2) / dy + diff_old(w[I, I, :], 1, 3) / dz
    return float(np.max(np.abs(d)))


def subdomain_index_maps(x0, y0, z0, nx0, ny0, nz0):
    """1-based parent indices of a sub-block.  big_periodic_3D.f90:20-25."""
    r = lambda o, n: np.arange(o, o + n, dtype=np.int64)
    return {
        "xu": r(x0, nx0 + 1), "yu": r(y0, ny0 + 2), "zu": r(z0, nz0 + 2),
        "xv": r(x0, nx0 + 2), "yv": r(y0, ny0 + 1), "zv": r(z0, nz0 + 2),
        "xw": r(x0, nx0 + 2), "yw": r(y0, ny0 + 2), "zw": r(z0, nz0 + 1),
        "xp": r(x0, nx0 + 2), "yp": r(y0, ny0 + 2), "zp": r(z0, nz0 + 2),
    }


def extract_sub(field, which, maps):
    """u_sub = u(idx_xu, idx_yu, idx_zu) etc.  big_periodic_3D.f90:665-669."""
    ix, iy, iz = maps["x" + which] - 1, maps["y" + which] - 1, maps["z" + which] - 1
    return field[np.ix_(ix, iy, iz)].copy()


def error_metrics(u, v, w, p, u_sub, v_sub, w_sub, p_sub, dx, dy):
    """Post-processing of a re-simulated step against the parent's sub-block.
    re_simulation_sub_tstep_interBC_combine.f90:826-833 with mean/rms of
    other_utility.f90:110-129.  Returns rms_vel(1..4) + err_vel(1..8)."""
    oz = diff(v, 1, 1) / dx - diff(u, 1, 2) / dy
    oz_sub = diff(v_sub, 1, 1) / dx - diff(u_sub, 1, 2) / dy
    r = [rms(a) for a in (u_sub, v_sub, w_sub, p_sub)]
    e = [np.max(np.abs(a - b)) / rr for a, b, rr in zip((u, v, w, p), (u_sub, v_sub, w_sub, p_sub), r)]
    e += [mean(np.abs(a - b)) / rr for a, b, rr in zip((u, v, w), (u_sub, v_sub, w_sub), r[:3])]
    e.append(np.max(np.abs(oz - oz_sub)) / rms(oz_sub))
    return np.array(r + e)


def write_err_csv(path, kind, rows):
    """err_vel (kind 0) / rms_vel (kind 1) text files.  re_simulation_sub_tstep_interBC_combine.f90:913-931:
    a header, then 'j,' and ES12.5E2 fields per row."""
    head = ("time_step, rel_err_u, rel_err_v, rel_err_w, rel_err_p, rel_err_u_m, rel_err_v_m, rel_err_w_m, rel_err_p_m"
            if kind == 0 else "time_step, rms_u, rms_v, rms_w, rms_p")
    with open(path, "w") as f:
        f.write(head + "\n")
        for j, row in enumerate(rows):
            f.write(str(j) + "".join("," + es12_5e2(x) for x in row) + "\n")


def es12_5e2(x):
    """Fortran ES12.5E2: d.ddddd mantissa, two-digit exponent, right-justified in 12 columns."""
    m, e = f"{float(x):.5E}".split("E")
    return f"{m}E{int(e):+03d}".rjust(12)


def cell_centred(u, v, w):
    """u_p, v_p, w_p: face averages at the interior cells.  Post_processing_main.m:29-31."""
    return ((u[:-1, 1:-1, 1:-1] + u[1:, 1:-1, 1:-1]) / 2, (v[1:-1, :-1, 1:-1] + v[1:-1, 1:, 1:-1]) / 2,
            (w[1:-1, 1:-1, :-1] + w[1:-1, 1:-1, 1:]) / 2)


def power_spec(u, v, w, L):
    """Shell-summed energy spectrum of an even-sized cube.  PowerSpec.m (MATLAB_post_processing),
    with its shell tests evaluated in floating point as the script does."""
    dim = u.shape[0]
    m = [(np.abs(np.fft.fftn(a)) / dim ** 3) ** 2 for a in (u, v, w)]
    rx = np.arange(dim) - dim / 2 + 1
    R = np.roll(rx, dim // 2 + 1)                       # circshift(rx', dim/2+1)
    r = np.sqrt(R[:, None, None] ** 2 + R[None, :, None] ** 2 + R[None, None, :] ** 2)
    dx = 2 * np.pi / L
    k_end = dim // 2
    k = np.arange(1, k_end + 1) * dx
    spectrum = np.zeros(k_end)
    count = np.zeros(k_end, dtype=np.int64)
    rd = r * dx

    def put(N, pick):
        spectrum[N] = sum(float(np.sum(mm[pick])) for mm in m)
        count[N] = int(np.count_nonzero(pick))

    for N in range(1, k_end - 1):                      # MATLAB N = 2 .. k_end-1
        put(N, (rd <= (k[N + 1] + k[N]) / 2) & (rd > (k[N] + k[N - 1]) / 2))
    put(0, rd <= (k[1] + k[0]) / 2)
    put(k_end - 1, (rd > (k[-1] + k[-2]) / 2) & (rd <= k[-1]))
    E = spectrum * 2 * np.pi * k ** 2 / (count * dx ** 3)
    return k, E, count, dx, m


def spec_prop(E, k, nu, u, v, w, dim, dx, m):
    """SpecProp.m, KolmoScale.m and the Taylor-scale lines of Post_processing_main.m:36-40."""
    kin_sp = float(np.sum(E) * dx)
    diss = float(np.sum(2 * nu * k ** 2 * E) * dx)
    s = float(np.sum(u ** 2 + v ** 2 + w ** 2))
    up = np.sqrt(s / 3 / dim ** 3)
    kin_ph = 0.5 * s / dim ** 3
    kin_e = 0.5 * sum(float(np.sum(mm)) for mm in m)
    eta = (nu ** 3 / diss) ** 0.25
    lam = np.sqrt(15 * nu * up ** 2 / diss)
    return {"dissipation": diss, "kin_Sp": kin_sp, "kin_Ph": kin_ph, "kin_E": kin_e, "up": up, "eta": eta,
            "u_eta": (nu * diss) ** 0.25, "tau": (nu / diss) ** 0.5, "lambda": lam, "Re_lambda": up * lam / nu}


# ---------------------------------------------------------------------------
# The step
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class Config:
    nx: int
    ny: int
    nz: int
    lx: float = 2.0 * 3.1415926535897932
    ly: float = 2.0 * 3.1415926535897932
    lz: float = 2.0 * 3.1415926535897932
    nu: float = 0.002
    dt: float = 2.5e-4
    scheme: int = AB2
    bc: tuple = (1, 1, 1)
    pbc: tuple = (1, 1, 1)
    dp_flag: int = 0
    gauge: int = 1          # 1: dp -= dp(1,1,1) (big_periodic_3D.f90:562)
    mean_dp: float = 0.0    # singular-mode mean (NS_functions.f90:1576-1577)

    @property
    def h(self):
        return self.lx / self.nx, self.ly / self.ny, self.lz / self.nz


@dataclasses.dataclass
class State:
    u: np.ndarray
    v: np.ndarray
    w: np.ndarray
    p: np.ndarray
    px: np.ndarray  # rhs_x_previous
    py: np.ndarray
    pz: np.ndarray
    first: bool = True   # next step is the Euler start (big_periodic_3D.f90:377)

    def copy(self):
        return State(self.u.copy(), self.v.copy(), self.w.copy(), self.p.copy(),
                     self.px.copy(), self.py.copy(), self.pz.copy(), self.first)

    @staticmethod
    def zeros(nx, ny, nz):
        z = np.zeros
        return State(z((nx + 1, ny + 2, nz + 2)), z((nx + 2, ny + 1, nz + 2)), z((nx + 2, ny + 2, nz + 1)),
                     z((nx + 2, ny + 2, nz + 2)), z((nx + 1, ny + 2, nz + 2)), z((nx + 2, ny + 1, nz + 2)),
                     z((nx + 2, ny + 2, nz + 1)))


def _ranges(cfg):
    r0 = [slice(0, n) if b == 1 else slice(1, n) for n, b in zip((cfg.nx, cfg.ny, cfg.nz), cfg.bc)]
    r1 = [slice(1, n + 1) for n in (cfg.nx, cfg.ny, cfg.nz)]
    return r0, r1


def correct(us, vs, ws, dp, p, dx, dy, dz, dt, dp_flag, gauge=1):
    """Gauge and correction, big_periodic_3D.f90:562-567: dp -= dp(1,1,1);
    u = -dt diff(dp,1,1)/dx + u_star (v, w likewise); p = dp_flag p + dp.
    Returns (u, v, w, p); the inputs are not modified."""
    if gauge:
        dp = dp - dp[0, 0, 0]
    return (-dt * diff(dp, 1, 1) / dx + us, -dt * diff(dp, 1, 2) / dy + vs, -dt * diff(dp, 1, 3) / dz + ws,
            dp_flag * p + dp)


def poisson_solve(R, cfg, faces, solver="auto"):
    """Interior dp from the (BC-modified) RHS for any pbc mix."""
    dx, dy, dz = cfg.h
    pbc = tuple(cfg.pbc)
    if solver == "lu":
        return lu_poisson(R, pbc, dx, dy, dz)
    if all(p == 1 for p in pbc):
        return fft_poisson(R, fft_eigenvalues(cfg.nx, cfg.ny, cfg.nz, dx, dy, dz))
    if all(p != 1 for p in pbc):
        return dct_poisson(R, dct_eigenvalues(cfg.nx, cfg.ny, cfg.nz, dx * dx, dy * dy, dz * dz, pbc), pbc, cfg.mean_dp)
    return spectral_poisson(R, pbc, dx, dy, dz, cfg.mean_dp)


def step(st, cfg, faces=None, cn_faces=None, cnf=None, solver="auto", return_parts=False):
    """One time step.  big_periodic_3D.f90:326-567 (and the same sequence in
    re_simulation_sub_tstep_interBC_combine.f90:510-802 for non-periodic bc).

    ``faces`` are the velocity/pressure faces (zero by default, as in
    big_periodic_3D.f90 where they are never set); ``cn_faces`` the per-sweep
    faces of the AB2-CN ADI (default: zero).  ``st.first`` selects the Euler
    start of AB2/AB2-CN (big_periodic_3D.f90:377,400).
    """
    nx, ny, nz = cfg.nx, cfg.ny, cfg.nz
    dx, dy, dz = cfg.h
    dx2, dy2, dz2 = dx * dx, dy * dy, dz * dz
    bx, by, bz = cfg.bc
    nu, dt, dpf = cfg.nu, cfg.dt, cfg.dp_flag
    if faces is None:
        faces = Faces.zeros(nx, ny, nz)
    u, v, w, p = st.u, st.v, st.w, st.p
    cx, cy, cz = cal_conv(u, v, w, bx, by, bz, dx, dy, dz)
    fx, fy, fz = cal_diff(u, v, w, bx, by, bz, dx2, dy2, dz2)
    dpdx = diff(p, 1, 1) / dx
    dpdy = diff(p, 1, 2) / dy
    dpdz = diff(p, 1, 3) / dz
    r0, r1 = _ranges(cfg)
    X = (r0[0], r1[1], r1[2])
    Y = (r1[0], r0[1], r1[2])
    Z = (r1[0], r1[1], r0[2])
    # rhs arrays: only the interior ranges are ever defined by the reference;
    # outside them the predictor output is overwritten by the BC fill.
    rx = np.zeros_like(u); ry = np.zeros_like(v); rz = np.zeros_like(w)
    px, py, pz = st.px.copy(), st.py.copy(), st.pz.copy()
    if cfg.scheme == EULER:
        rx[X] = nu * fx - cx; ry[Y] = nu * fy - cy; rz[Z] = nu * fz - cz
        us = dt * (1.0 * rx - dpf * dpdx) + u
        vs = dt * (1.0 * ry - dpf * dpdy) + v
        ws = dt * (1.0 * rz - dpf * dpdz) + w
        px[:] = 0; py[:] = 0; pz[:] = 0
        vel_bc_staggered(us, vs, ws, faces, bx, by, bz)
    elif cfg.scheme == AB2:
        rx[X] = nu * fx - cx; ry[Y] = nu * fy - cy; rz[Z] = nu * fz - cz
        if st.first:
            us = dt * (1.0 * rx - dpf * dpdx) + u
            vs = dt * (1.0 * ry - dpf * dpdy) + v
            ws = dt * (1.0 * rz - dpf * dpdz) + w
        else:
            us = dt * (1.5 * rx - 0.5 * px - dpf * dpdx) + u
            vs = dt * (1.5 * ry - 0.5 * py - dpf * dpdy) + v
            ws = dt * (1.5 * rz - 0.5 * pz - dpf * dpdz) + w
        px, py, pz = rx.copy(), ry.copy(), rz.copy()
        vel_bc_staggered(us, vs, ws, faces, bx, by, bz)
    else:
        if st.first:
            rx[X] = 0.5 * nu * fx - cx; ry[Y] = 0.5 * nu * fy - cy; rz[Z] = 0.5 * nu * fz - cz
            us = dt * (rx - dpf * dpdx) + u
            vs = dt * (ry - dpf * dpdy) + v
            ws = dt * (rz - dpf * dpdz) + w
        else:
            rx[X] = 0.5 * nu * fx - 1.5 * cx; ry[Y] = 0.5 * nu * fy - 1.5 * cy; rz[Z] = 0.5 * nu * fz - 1.5 * cz
            us = dt * (rx - 0.5 * px - dpf * dpdx) + u
            vs = dt * (ry - 0.5 * py - dpf * dpdy) + v
            ws = dt * (rz - 0.5 * pz - dpf * dpdz) + w
        px[X] = -cx; py[Y] = -cy; pz[Z] = -cz
        if cnf is None:
            cnf = CNFactors(nx, ny, nz, cfg.bc, dx2, dy2, dz2, dt, nu)
        us, vs, ws = adi_sweeps(us, vs, ws, cnf, cfg.bc, cn_faces)
    I = slice(1, -1)
    R = diff(us[:, I, I], 1, 1) / dx
    R = R + diff(vs[I, :, I], 1, 2) / dy
    R = R + diff(ws[I, I, :], 1, 3) / dz
    R = R / dt
    pf = interior_p_faces(faces, nx, ny, nz)
    pr_bc_staggered_modify_rhs(R, pf, cfg.pbc, dx, dy, dz)
    dp = np.zeros((nx + 2, ny + 2, nz + 2))
    dp[1:-1, 1:-1, 1:-1] = poisson_solve(R, cfg, faces, solver)
    pr_bc_staggered(dp, faces, cfg.pbc, dx, dy, dz)
    un, vn, wn, pn = correct(us, vs, ws, dp, p, dx, dy, dz, dt, dpf, cfg.gauge)
    # history outside the interior ranges is never read; keep it zero
    hx = np.zeros_like(px); hy = np.zeros_like(py); hz = np.zeros_like(pz)
    hx[X] = px[X]; hy[Y] = py[Y]; hz[Z] = pz[Z]
    out = State(un, vn, wn, pn, hx, hy, hz, first=False)
    if return_parts:
        return out, {"us": us, "vs": vs, "ws": ws, "R": R, "dp": dp, "conv": (cx, cy, cz), "diff": (fx, fy, fz)}
    return out


def run(st, cfg, nsteps, faces=None, solver="auto"):
    cnf = None
    if cfg.scheme == AB2_CN:
        dx, dy, dz = cfg.h
        cnf = CNFactors(cfg.nx, cfg.ny, cfg.nz, cfg.bc, dx * dx, dy * dy, dz * dz, cfg.dt, cfg.nu)
    for _ in range(nsteps):
        st = step(st, cfg, faces=faces, cnf=cnf, solver=solver)
    return st


# ---------------------------------------------------------------------------
# Sub-block re-simulation -- re_simulation_sub_tstep_interBC_combine.f90:415-811
# ---------------------------------------------------------------------------
def spline_window(knot_t, t, tol=1e-12):
    """First index of the 6 knots interp1 uses around t
    (sub_tstep_BC_combined_interpolation.m:59: the last knot <= t, two before it,
    three after it)."""
    k = np.nonzero(np.asarray(knot_t) <= t + tol)[0]
    if k.size == 0:
        raise ValueError("t before the first knot")
    first = int(k[-1]) - 2
    if first < 0 or first + 6 > len(knot_t):
        raise ValueError("no 6-knot window around t")
    return first


def interp_spline(knot_t, knot_vals, t, tol=1e-12):
    """interp1(t0(win), y(win, ...), t, 'spline'): not-a-knot cubic spline over
    the 6-knot window, elementwise over the arrays in knot_vals."""
    from scipy.interpolate import CubicSpline
    kt = np.asarray(knot_t, dtype=float)
    at = np.nonzero(np.abs(kt - t) <= tol)[0]
    if at.size:  # a knot: the data value
        return np.array(knot_vals[int(at[0])], copy=True)
    f = spline_window(kt, t, tol)
    y = np.stack([knot_vals[f + q] for q in range(6)], axis=0)
    return CubicSpline(kt[f:f + 6], y, axis=0, bc_type="not-a-knot")(t)


def resimulate(st, cfg, knot_t, knot_data, t_start, n_intervals, sub_tstep=1, restart=False):
    """Re-simulate one sub-block driven by parent data.

    ``knot_data[k] = (u_star_sub, v_star_sub, w_star_sub, dp_sub)`` is the
    parent's sub-block at time ``knot_t[k]`` (the HDF5 groups of
    big_periodic_3D.f90:664-712).  Each step takes the spline-interpolated
    u*/dp sub-blocks at its end time (:496-504), builds the faces with
    get_velpr_bc (using_Ustar, dp_flag = 1; :510-520) and steps with the
    DCT pressure solve whose mean is the interpolated dp's interior mean
    (:766-768).  The first parent interval is covered by ``sub_tstep``
    sub-steps with the AB2 history saved after the first and restored after
    the last (:443-454, :602-612).  ``st.first`` is the Euler start
    (``not restart``, :565).
    """
    dx, dy, dz = cfg.h
    st = st.copy()
    st.first = not restart
    saved = None
    for m in range(n_intervals):
        nsub = sub_tstep if m == 0 else 1
        dt = cfg.dt / nsub
        for s in range(1, nsub + 1):
            t = t_start + (s * dt if m == 0 else (m + 1) * cfg.dt)
            u_s, v_s, w_s, dp_s = (interp_spline(knot_t, [kd[q] for kd in knot_data], t) for q in range(4))
            faces = get_velpr_bc(u_s, v_s, w_s, dp_s, cfg.bc, cfg.pbc, dx, dy, dz, dt, 1, True, None)
            c = dataclasses.replace(cfg, dt=dt, mean_dp=float(np.mean(dp_s[1:-1, 1:-1, 1:-1])), gauge=0, dp_flag=1)
            st = step(st, c, faces=faces)
            if nsub > 1 and s == 1:
                saved = (st.px.copy(), st.py.copy(), st.pz.copy())
            if nsub > 1 and s == nsub:
                st.px, st.py, st.pz = (a.copy() for a in saved)
    return st


def sweep_faces(u_d, v_d, w_d, d, bc):
    """The faces of ADI sweep d (0 x, 1 y, 2 z) of a sub-block, from the
    parent's sub-block u*, v*, w* after that sweep.  big_periodic_3D.f90:433-489
    records them (bx_u_1s = u_star(idx_xu(1), ...), bx_v_1s = (v_star(idx_xv(1),
    ...) + v_star(idx_xv(2), ...)) * 0.5d0, ...): the velocity part of
    get_velpr_bc on the axis d only.  Returns a Faces with the axis-d keys."""
    nx, ny, nz = u_d.shape[0] - 1, v_d.shape[1] - 1, w_d.shape[2] - 1
    dummy = np.zeros((nx + 2, ny + 2, nz + 2))
    b3 = [1, 1, 1]
    b3[d] = bc
    f = get_velpr_bc(u_d, v_d, w_d, dummy, tuple(b3), (1, 1, 1), 1.0, 1.0, 1.0, 0.0, 1, True, None)
    out = Faces.zeros(nx, ny, nz)
    a = "xyz"[d]
    for k in out.d:
        if k[0] == a and k[2] in "uvw":
            out.d[k] = f.d[k]
    return out


def resimulate_frames(st, cfg, frames, p_prev0, using_ustar=True, dp_flag=1, restart=True):
    """Re-simulate one sub-block stepped at the parent's own time step, one
    parent record per step, with either boundary source of
    re_simulation_sub_tstep_interBC_combine.f90:436-519.

    ``frames[m]`` is the parent's sub-block after parent step m+1: a dict with
    u, v, w, p (u_sub ... p_sub) and us, vs, ws, dp (u_star_sub ... dp_sub).
    ``p_prev0`` is p_sub of the record before frames[0].  Per step, as the
    reference's loop does: p_sub_pre = p_sub (:439-441); dp_sub = p_sub when
    dp_flag = 0 (:506-508); faces from get_velpr_bc on u*_sub (using_Ustar)
    or u_sub (:510-520), whose u branch adds dt * diff(p_sub_pre) / h with
    dp_flag = 0 (NS_functions.f90:434-437); the DCT solve with the mean of
    dp_sub (:766-768); p = dp_flag * p + dp (:801).  With AB2-CN a frame also
    holds "cn": the faces of the three ADI sweeps (``sweep_faces``), the BC
    rows of the sub-block's sweeps (:656-701).
    """
    dx, dy, dz = cfg.h
    st = st.copy()
    st.first = not restart
    p_sub_pre = p_prev0
    for fr in frames:
        dp_sub = fr["dp"] if dp_flag else fr["p"]
        if using_ustar:
            faces = get_velpr_bc(fr["us"], fr["vs"], fr["ws"], dp_sub, cfg.bc, cfg.pbc, dx, dy, dz, cfg.dt, dp_flag,
                                 True, p_sub_pre)
        else:
            faces = get_velpr_bc(fr["u"], fr["v"], fr["w"], dp_sub, cfg.bc, cfg.pbc, dx, dy, dz, cfg.dt, dp_flag,
                                 False, p_sub_pre)
        c = dataclasses.replace(cfg, mean_dp=float(np.mean(dp_sub[1:-1, 1:-1, 1:-1])), gauge=0, dp_flag=dp_flag)
        st = step(st, c, faces=faces, cn_faces=fr.get("cn"))
        p_sub_pre = fr["p"]
    return st
