"""Host-side mirror of the reference's step interface over the C ABI.

The Fortran drivers of the reference (big_periodic_3D.f90,
re_simulation*.f90) call NS_functions.f90 routines on column-major padded
arrays.  ``Session`` replaces the time-loop body with GPU-resident state;
the module-level functions replace single routines.  Arrays are NumPy
float64 in the reference's shapes; they are passed to the library in
Fortran order.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib

EULER, AB2, AB2_CN = 0, 1, 2
PI = 3.1415926535897932

SWEEP_FACE_ORDER = [  # per-sweep AB2-CN faces, as big_periodic_3D.f90:433-489 records them
    "x_u_1", "x_u_n", "x_v_1", "x_v_n", "x_w_1", "x_w_n",
    "y_u_1", "y_u_n", "y_v_1", "y_v_n", "y_w_1", "y_w_n",
    "z_u_1", "z_u_n", "z_v_1", "z_v_n", "z_w_1", "z_w_n",
]

FACE_ORDER = [  # get_velpr_bc output order (NS_functions.f90:414-420)
    "x_u_1", "x_u_n", "y_u_1", "y_u_n", "z_u_1", "z_u_n",
    "x_v_1", "x_v_n", "y_v_1", "y_v_n", "z_v_1", "z_v_n",
    "x_w_1", "x_w_n", "y_w_1", "y_w_n", "z_w_1", "z_w_n",
    "x_p_1", "x_p_n", "y_p_1", "y_p_n", "z_p_1", "z_p_n",
]


def face_shapes(nx, ny, nz):
    """Shapes of the 24 get_velpr_bc outputs (NS_functions.f90:418-421): the
    face of field f on axis a spans f's extents on the two other axes."""
    n = (nx, ny, nz)
    out = {}
    for name in FACE_ORDER:
        a = "xyz".index(name[0])
        f = "uvwp".index(name[2])
        out[name] = tuple(n[b] + (1 if f == b else 2) for b in range(3) if b != a)
    return out


class NSError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{_lib.STATUS.get(status, status)}: {msg}")
        self.status = status


def _f(a, shape=None):
    a = np.asarray(a, dtype=np.float64)
    if shape is not None and tuple(a.shape) != tuple(shape):
        raise NSError(1, f"shape {a.shape} != {shape}")
    return np.asfortranarray(a)


def _ptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def shapes(nx, ny, nz):
    return {"u": (nx + 1, ny + 2, nz + 2), "v": (nx + 2, ny + 1, nz + 2), "w": (nx + 2, ny + 2, nz + 1),
            "p": (nx + 2, ny + 2, nz + 2)}


def make_config(nx, ny, nz, **kw) -> _lib.NSConfig:
    """ns_config with the big_periodic_3D defaults, overridden by keywords
    (bc/pbc take 3-tuples)."""
    lib = _lib.load()
    c = _lib.NSConfig()
    lib.ns_config_default(C.byref(c), nx, ny, nz)
    for k, v in kw.items():
        if k in ("bc", "pbc"):
            for i in range(3):
                getattr(c, k)[i] = int(v[i])
        else:
            setattr(c, k, v)
    return c


class Session:
    """One GPU-resident simulation (ns_create / ns_step / ns_destroy)."""

    def __init__(self, cfg=None, **kw):
        self.lib = _lib.load()
        if cfg is None:
            cfg = make_config(kw.pop("nx"), kw.pop("ny"), kw.pop("nz"), **kw)
        self.cfg = cfg
        self.h = C.c_void_p()
        s = self.lib.ns_create(C.byref(cfg), C.byref(self.h))
        if s != 0:
            raise NSError(s, "ns_create failed")
        self.shapes = shapes(cfg.nx, cfg.ny, cfg.nz)

    def _check(self, s):
        if s != 0:
            raise NSError(s, self.lib.ns_last_error(self.h).decode())

    def close(self):
        if self.h:
            self.lib.ns_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_state(self, u, v, w, p, rhs_prev=None):
        sh = self.shapes
        u, v, w, p = _f(u, sh["u"]), _f(v, sh["v"]), _f(w, sh["w"]), _f(p, sh["p"])
        if rhs_prev is None:
            hx = hy = hz = None
        else:
            hx, hy, hz = _f(rhs_prev[0], sh["u"]), _f(rhs_prev[1], sh["v"]), _f(rhs_prev[2], sh["w"])
        self._keep = (u, v, w, p, hx, hy, hz)
        self._check(self.lib.ns_set_state(self.h, _ptr(u), _ptr(v), _ptr(w), _ptr(p), _ptr(hx), _ptr(hy), _ptr(hz)))

    def get_state(self, history=True):
        sh = self.shapes
        out = {k: np.zeros(sh[k], order="F") for k in ("u", "v", "w", "p")}
        hist = [np.zeros(sh[k], order="F") for k in ("u", "v", "w")] if history else [None] * 3
        self._check(self.lib.ns_get_state(self.h, _ptr(out["u"]), _ptr(out["v"]), _ptr(out["w"]), _ptr(out["p"]),
                                          _ptr(hist[0]), _ptr(hist[1]), _ptr(hist[2])))
        if history:
            out["hx"], out["hy"], out["hz"] = hist
        return out

    def set_faces(self, faces: dict, which=0):
        """faces: {name: 2D array} using FACE_ORDER names; missing = zero."""
        keep = []
        arr = (C.POINTER(C.c_double) * 24)()
        for i, k in enumerate(FACE_ORDER):
            if k in faces and faces[k] is not None:
                a = _f(faces[k])
                keep.append(a)
                arr[i] = _ptr(a)
            else:
                arr[i] = None
        self._check(self.lib.ns_set_faces(self.h, which, arr))

    def set_mean_dp(self, mean_dp):
        """mean(dp_sub) of the DCT solve's singular mode from the next step on (ns_set_mean_dp)."""
        self._check(self.lib.ns_set_mean_dp(self.h, float(mean_dp)))

    def step(self, n=1):
        self._check(self.lib.ns_step(self.h, n))

    def step_host(self, u, v, w, p, rhs_prev=None, out=None):
        """One step of host-resident state (ns_step_host): returns the state
        dict (u, v, w, p, hx, hy, hz); `out` may hold preallocated arrays."""
        sh = self.shapes
        ins = [_f(u, sh["u"]), _f(v, sh["v"]), _f(w, sh["w"]), _f(p, sh["p"])]
        hist = [None] * 3 if rhs_prev is None else [_f(rhs_prev[0], sh["u"]), _f(rhs_prev[1], sh["v"]),
                                                     _f(rhs_prev[2], sh["w"])]
        keys = ("u", "v", "w", "p", "hx", "hy", "hz")
        shp = (sh["u"], sh["v"], sh["w"], sh["p"], sh["u"], sh["v"], sh["w"])
        res = {k: (out[k] if out is not None and k in out else np.zeros(sp, order="F")) for k, sp in zip(keys, shp)}
        self._check(self.lib.ns_step_host(self.h, *[_ptr(a) for a in ins + hist], *[_ptr(res[k]) for k in keys]))
        return res

    def synchronize(self):
        self._check(self.lib.ns_synchronize(self.h))

    def set_stream(self, stream_handle: int):
        self._check(self.lib.ns_set_stream(self.h, C.c_void_p(stream_handle)))

    def diag(self):
        d = _lib.NSDiag()
        self._check(self.lib.ns_get_diag(self.h, C.byref(d)))
        return {"max_div": d.max_div, "probe": d.probe, "steps": d.steps_done,
                "euler_start_pending": bool(d.euler_start_pending)}

    def get_sweeps(self):
        """u*, v*, w* after the x sweep and after the y sweep of the last
        AB2-CN step (keep_sweeps sessions; ns_get_sweeps)."""
        sh = self.shapes
        keys = ("ux", "vx", "wx", "uy", "vy", "wy")
        out = {k: np.zeros(sh[k[0]], order="F") for k in keys}
        self._check(self.lib.ns_get_sweeps(self.h, *[_ptr(out[k]) for k in keys]))
        return out

    def get_stage(self):
        """u*, v*, w* and the gauge-shifted dp of the last step (ns_get_stage):
        the u_star_sub ... dp_sub arrays the reference records."""
        sh = self.shapes
        out = {k: np.zeros(sh[k[0]], order="F") for k in ("us", "vs", "ws")}
        out["dp"] = np.zeros(sh["p"], order="F")
        self._check(self.lib.ns_get_stage(self.h, _ptr(out["us"]), _ptr(out["vs"]), _ptr(out["ws"]),
                                          _ptr(out["dp"])))
        return out

    def profile(self, nsteps=1):
        """Per-kernel device time (ms) over nsteps eager steps: {name: (ms, launches)}."""
        arr = (_lib.NSKernelTime * 64)()
        n = C.c_int()
        self._check(self.lib.ns_profile(self.h, nsteps, arr, 64, C.byref(n)))
        return {arr[i].name.decode(): (arr[i].ms, arr[i].launches) for i in range(n.value)}

    def launch_count(self):
        v = C.c_longlong()
        self._check(self.lib.ns_launch_count(self.h, C.byref(v)))
        return v.value

    # routine tier -----------------------------------------------------------
    def _conv_shapes(self):
        c = self.cfg
        sx = (c.nx if c.bc[0] == 1 else c.nx - 1, c.ny, c.nz)
        sy = (c.nx, c.ny if c.bc[1] == 1 else c.ny - 1, c.nz)
        sz = (c.nx, c.ny, c.nz if c.bc[2] == 1 else c.nz - 1)
        return sx, sy, sz

    def cal_conv(self, u, v, w):
        """cal_conv (NS_functions.f90:53-158)."""
        sh = self.shapes
        u, v, w = _f(u, sh["u"]), _f(v, sh["v"]), _f(w, sh["w"])
        outs = [np.zeros(s, order="F") for s in self._conv_shapes()]
        self._check(self.lib.ns_cal_conv(self.h, _ptr(u), _ptr(v), _ptr(w), *[_ptr(o) for o in outs]))
        return tuple(outs)

    def cal_diff(self, u, v, w):
        """cal_diff (NS_functions.f90:161-210)."""
        sh = self.shapes
        u, v, w = _f(u, sh["u"]), _f(v, sh["v"]), _f(w, sh["w"])
        outs = [np.zeros(s, order="F") for s in self._conv_shapes()]
        self._check(self.lib.ns_cal_diff(self.h, _ptr(u), _ptr(v), _ptr(w), *[_ptr(o) for o in outs]))
        return tuple(outs)

    def poisson(self, rhs):
        """Poisson solve of a BC-modified RHS (nx, ny, nz) -> dp with ghosts."""
        c = self.cfg
        r = _f(rhs, (c.nx, c.ny, c.nz))
        dp = np.zeros(self.shapes["p"], order="F")
        self._check(self.lib.ns_poisson(self.h, _ptr(r), _ptr(dp)))
        return dp

    def adi(self, us, vs, ws):
        """The three CN-ADI sweeps on u*, v*, w* (returns new arrays)."""
        sh = self.shapes
        us, vs, ws = (np.array(_f(us, sh["u"]), order="F"), np.array(_f(vs, sh["v"]), order="F"),
                      np.array(_f(ws, sh["w"]), order="F"))
        self._check(self.lib.ns_adi(self.h, _ptr(us), _ptr(vs), _ptr(ws)))
        return us, vs, ws

    def vel_bc(self, us, vs, ws):
        """vel_bc_staggered on u*, v*, w* with the session's bc and face set 0 (returns new arrays)."""
        sh = self.shapes
        us, vs, ws = (np.array(_f(us, sh["u"]), order="F"), np.array(_f(vs, sh["v"]), order="F"),
                      np.array(_f(ws, sh["w"]), order="F"))
        self._check(self.lib.ns_vel_bc(self.h, _ptr(us), _ptr(vs), _ptr(ws)))
        return us, vs, ws

    def correct(self, us, vs, ws, dp, p):
        """Gauge and correction (big_periodic_3D.f90:562-567): returns u, v, w, p."""
        sh = self.shapes
        ins = [_f(us, sh["u"]), _f(vs, sh["v"]), _f(ws, sh["w"]), _f(dp, sh["p"])]
        out = {k: np.zeros(sh[k], order="F") for k in ("u", "v", "w")}
        out["p"] = np.array(_f(p, sh["p"]), order="F")
        self._check(self.lib.ns_correct(self.h, *[_ptr(a) for a in ins], _ptr(out["u"]), _ptr(out["v"]),
                                        _ptr(out["w"]), _ptr(out["p"])))
        return out

    def error_metrics(self, u_ref, v_ref, w_ref, p_ref):
        """rms_vel(1..4) + err_vel(1..8) of the current state against reference
        arrays (ns_error_metrics, re_simulation_sub_tstep_interBC_combine.f90:813-834)."""
        sh = self.shapes
        arrs = [_f(u_ref, sh["u"]), _f(v_ref, sh["v"]), _f(w_ref, sh["w"]), _f(p_ref, sh["p"])]
        out = np.zeros(12)
        self._check(self.lib.ns_error_metrics(self.h, *[_ptr(a) for a in arrs], _ptr(out)))
        return out

    SPECTRUM_PROPS = ("dissipation", "kin_Sp", "kin_Ph", "kin_E", "up", "eta", "u_eta", "tau", "lambda",
                      "Re_lambda")

    def spectrum(self):
        """(k, E, count, props) of the current velocity (ns_spectrum): the shell
        spectrum of PowerSpec.m and the statistics of SpecProp.m / KolmoScale.m."""
        n = self.cfg.nx // 2
        k, E, props = np.zeros(n), np.zeros(n), np.zeros(10)
        cnt = np.zeros(n, dtype=np.int64)
        self._check(self.lib.ns_spectrum(self.h, _ptr(k), _ptr(E), cnt.ctypes.data_as(C.POINTER(C.c_longlong)),
                                         _ptr(props)))
        return k, E, cnt, dict(zip(self.SPECTRUM_PROPS, props))

    # adjoint tier ------------------------------------------------------------
    def adj_forward(self, nsteps, ckpt_every):
        """Run nsteps steps keeping a checkpoint every ckpt_every steps (ns_adj_forward)."""
        self._check(self.lib.ns_adj_forward(self.h, int(nsteps), int(ckpt_every)))

    def adj_backward(self, dJ_du, dJ_dv, dJ_dw, history=False, out=None):
        """Gradient of J(u(T)) with respect to the initial u, v, w (ns_adj_backward).

        Returns {"u", "v", "w"} (and "hx", "hy", "hz" with history=True) in the
        reference shapes, zero on the entries that are periodic copies.  `out`
        may hold preallocated Fortran-ordered arrays "u", "v", "w" (e.g. in
        pinned host memory) that receive the gradient."""
        sh = self.shapes
        seeds = [_f(dJ_du, sh["u"]), _f(dJ_dv, sh["v"]), _f(dJ_dw, sh["w"])]
        if out is None:
            out = {k: np.zeros(sh[k], order="F") for k in ("u", "v", "w")}
        else:
            for k in ("u", "v", "w"):
                a = out[k]
                if a.shape != sh[k] or a.dtype != np.float64 or not a.flags.f_contiguous:
                    raise NSError(6, f"out[{k!r}] must be a Fortran-ordered float64 array of shape {sh[k]}")
            out = dict(out)
        hist = [np.zeros(sh[k], order="F") for k in ("u", "v", "w")] if history else [None] * 3
        self._check(self.lib.ns_adj_backward(self.h, *[_ptr(a) for a in seeds], _ptr(out["u"]), _ptr(out["v"]),
                                             _ptr(out["w"]), _ptr(hist[0]), _ptr(hist[1]), _ptr(hist[2])))
        if history:
            out["hx"], out["hy"], out["hz"] = hist
        return out


def tgv(x, y, nz, t, nu, u=True, v=True, p=True):
    """TGV (NS_functions.f90:18-50) on the GPU (ns_tgv): {name: (nx, ny, nz)
    array} for the requested fields of the 2D Taylor-Green vortex at time t."""
    lib = _lib.load()
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    shp = (len(x), len(y), int(nz))
    out = {k: np.zeros(shp, order="F") for k, want in (("u", u), ("v", v), ("p", p)) if want}
    s = lib.ns_tgv(_ptr(x), len(x), _ptr(y), len(y), int(nz), float(t), float(nu), _ptr(out.get("u")),
                   _ptr(out.get("v")), None, _ptr(out.get("p")))
    if s != 0:
        raise NSError(s, "ns_tgv failed")
    return out


def spline_weights(knots, t):
    """(first, w[6]) of MATLAB interp1(knots, y, t, 'spline') on the 6-knot
    window (ns_spline_weights): value = sum_q w[q] * y[first + q]."""
    lib = _lib.load()
    k = np.ascontiguousarray(knots, dtype=np.float64)
    first = C.c_int()
    w = np.zeros(6)
    s = lib.ns_spline_weights(_ptr(k), len(k), float(t), C.byref(first), _ptr(w))
    if s != 0:
        raise NSError(s, "no 6-knot window around t")
    return first.value, w


def make_batch_config(**kw) -> _lib.NSBatchConfig:
    lib = _lib.load()
    c = _lib.NSBatchConfig()
    lib.ns_batch_config_default(C.byref(c))
    for k, v in kw.items():
        if k == "grid":
            for i, g in enumerate(v):
                c.grid[i] = int(g)
        else:
            setattr(c, k, v)
    return c


class Batch:
    """Batched re-simulation of sub-blocks of a parent Session (ns_batch_*).

    subs: iterable of (x0, y0, z0, nx, ny, nz, sub_tstep) with 1-based
    parent origins (idx_xu = x0 + (0..nx), big_periodic_3D.f90:20-25)."""

    def __init__(self, subs, cfg=None, **kw):
        self.lib = _lib.load()
        self.cfg = cfg if cfg is not None else make_batch_config(**kw)
        subs = list(subs)
        arr = (_lib.NSSubdomain * len(subs))()
        for i, sd in enumerate(subs):
            x0, y0, z0, nx, ny, nz, r = sd
            arr[i] = _lib.NSSubdomain(x0, y0, z0, nx, ny, nz, r, 0)
        self.subs = subs
        self.h = C.c_void_p()
        s = self.lib.ns_batch_create(C.byref(self.cfg), arr, len(subs), C.byref(self.h))
        if s != 0:
            raise NSError(s, "ns_batch_create failed")

    def _check(self, s):
        if s != 0:
            raise NSError(s, self.lib.ns_batch_last_error(self.h).decode())

    def close(self):
        if self.h:
            self.lib.ns_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def shapes(self, i):
        _, _, _, nx, ny, nz, _ = self.subs[i]
        return shapes(nx, ny, nz)

    def init_from_parent(self, parent: "Session"):
        self._check(self.lib.ns_batch_init_from_parent(self.h, parent.h))

    def set_state(self, i, u, v, w, p, rhs_prev=None):
        sh = self.shapes(i)
        arrs = [_f(u, sh["u"]), _f(v, sh["v"]), _f(w, sh["w"]), _f(p, sh["p"])]
        if rhs_prev is None:
            arrs += [None] * 3
        else:
            arrs += [_f(rhs_prev[0], sh["u"]), _f(rhs_prev[1], sh["v"]), _f(rhs_prev[2], sh["w"])]
        self._check(self.lib.ns_batch_set_state(self.h, i, *[_ptr(a) for a in arrs]))

    def get_state(self, i, history=True):
        sh = self.shapes(i)
        out = {k: np.zeros(sh[k], order="F") for k in ("u", "v", "w", "p")}
        hist = [np.zeros(sh[k], order="F") for k in ("u", "v", "w")] if history else [None] * 3
        self._check(self.lib.ns_batch_get_state(self.h, i, _ptr(out["u"]), _ptr(out["v"]), _ptr(out["w"]),
                                                _ptr(out["p"]), _ptr(hist[0]), _ptr(hist[1]), _ptr(hist[2])))
        if history:
            out["hx"], out["hy"], out["hz"] = hist
        return out

    def capture(self, parent: "Session", slot, t):
        self._check(self.lib.ns_batch_capture(self.h, parent.h, int(slot), float(t)))

    def set_snapshot(self, slot, t, i, faces: dict, mean_dp):
        keep = []
        arr = (C.POINTER(C.c_double) * 24)()
        for q, k in enumerate(FACE_ORDER):
            if k in faces and faces[k] is not None:
                a = _f(faces[k])
                keep.append(a)
                arr[q] = _ptr(a)
            else:
                arr[q] = None
        self._check(self.lib.ns_batch_set_snapshot(self.h, int(slot), float(t), int(i), arr, float(mean_dp)))

    def get_snapshot(self, slot, i):
        """(faces dict in FACE_ORDER names, mean) of snapshot slot `slot` of
        subdomain i (ns_batch_get_snapshot)."""
        _, _, _, nx, ny, nz, _ = self.subs[i]
        fs = face_shapes(nx, ny, nz)
        faces = {k: np.zeros(fs[k], order="F") for k in FACE_ORDER}
        arr = (C.POINTER(C.c_double) * 24)()
        for q, k in enumerate(FACE_ORDER):
            arr[q] = _ptr(faces[k])
        m = C.c_double()
        self._check(self.lib.ns_batch_get_snapshot(self.h, int(slot), int(i), arr, C.byref(m)))
        return faces, m.value

    def get_sweep_faces(self, slot, i):
        """AB2-CN: {name: array} of the 18 per-sweep faces of snapshot slot
        `slot` of subdomain i (SWEEP_FACE_ORDER names, ns_batch_get_sweep_faces)."""
        _, _, _, nx, ny, nz, _ = self.subs[i]
        fs = face_shapes(nx, ny, nz)
        faces = {k: np.zeros(fs[k], order="F") for k in SWEEP_FACE_ORDER}
        arr = (C.POINTER(C.c_double) * 18)(*[_ptr(faces[k]) for k in SWEEP_FACE_ORDER])
        self._check(self.lib.ns_batch_get_sweep_faces(self.h, int(slot), int(i), arr))
        return faces

    def set_sweep_faces(self, slot, i, faces: dict):
        """AB2-CN: the per-sweep faces of slot `slot` of subdomain i (missing = zero)."""
        keep = [_f(faces[k]) if faces.get(k) is not None else None for k in SWEEP_FACE_ORDER]
        arr = (C.POINTER(C.c_double) * 18)(*[_ptr(a) if a is not None else None for a in keep])
        self._check(self.lib.ns_batch_set_sweep_faces(self.h, int(slot), int(i), arr))

    def advance(self, t0):
        self._check(self.lib.ns_batch_advance(self.h, float(t0)))

    def max_div(self, i):
        d = C.c_double()
        self._check(self.lib.ns_batch_max_div(self.h, int(i), C.byref(d)))
        return d.value

    def launch_count(self):
        n = C.c_longlong()
        self._check(self.lib.ns_batch_launch_count(self.h, C.byref(n)))
        return n.value

    def autotune(self, reps=3):
        self._check(self.lib.ns_batch_autotune(self.h, int(reps)))
        c = _lib.NSBatchConfig()
        self._check(self.lib.ns_batch_get_config(self.h, C.byref(c)))
        return list(c.grid)

    def set_stream(self, stream_handle: int):
        self._check(self.lib.ns_batch_set_stream(self.h, C.c_void_p(stream_handle)))

    STAGES = ("interp", "predict", "vel_bc_x", "vel_bc_y", "vel_bc_z", "x_fwd", "y_fwd", "z_solve", "y_inv",
              "x_inv", "pr_bc_x", "pr_bc_y", "pr_bc_z", "correct")

    def profile(self, reps=3):
        """{stage: ms} of one regular step's stage kernels (ns_batch_profile)."""
        out = np.zeros(16)
        self._check(self.lib.ns_batch_profile(self.h, int(reps), _ptr(out)))
        return dict(zip(self.STAGES, out[:len(self.STAGES)]))

    def error_metrics(self, parent: "Session"):
        """(n, 12): rms_vel(1..4) + err_vel(1..8) of every subdomain against the
        parent's current state over its index maps (ns_batch_error_metrics)."""
        out = np.zeros((len(self.subs), 12))
        self._check(self.lib.ns_batch_error_metrics(self.h, parent.h, _ptr(out)))
        return out


def write_err_csv(path, kind, rows):
    """err_vel (kind 0, 8 columns) or rms_vel (kind 1, 4 columns) file in the
    reference's format (ns_write_err_csv)."""
    lib = _lib.load()
    r = np.ascontiguousarray(rows, dtype=np.float64)
    ncol = 8 if kind == 0 else 4
    if r.ndim != 2 or r.shape[1] != ncol:
        raise NSError(6, f"rows must be (n, {ncol})")
    s = lib.ns_write_err_csv(str(path).encode(), int(kind), r.shape[0], _ptr(r))
    if s != 0:
        raise NSError(s, f"cannot write {path}")


class H5File:
    """A file of the reference's HDF5 subset (ns_h5_*; needs no GPU).

    ``H5File(path, "w")`` creates (``"w!"`` overwrites), ``"r"`` opens read-only,
    ``"a"`` opens for adding groups, datasets and attributes.  Arrays are
    written and read in their Fortran shapes, as h5ltmake_dataset_double_f and
    h5ltread_dataset_double_f take them."""

    def __init__(self, path, mode="r"):
        self.lib = _lib.load()
        self.h = C.c_void_p()
        p = str(path).encode()
        if mode in ("w", "w!"):
            s = self.lib.ns_h5_create(p, int(mode == "w!"), C.byref(self.h))
        elif mode in ("r", "a"):
            s = self.lib.ns_h5_open(p, int(mode == "a"), C.byref(self.h))
        else:
            raise NSError(6, f"mode {mode!r}")
        if s != 0:
            raise NSError(s, self.lib.ns_h5_last_error(None).decode())

    def _check(self, s):
        if s != 0:
            raise NSError(s, self.lib.ns_h5_last_error(self.h).decode())

    def close(self):
        if self.h:
            h, self.h = self.h, C.c_void_p()
            s = self.lib.ns_h5_close(h)
            if s != 0:
                raise NSError(s, self.lib.ns_h5_last_error(None).decode())

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def flush(self):
        self._check(self.lib.ns_h5_flush(self.h))

    def group(self, path):
        self._check(self.lib.ns_h5_group(self.h, path.encode()))

    def set_attr(self, obj, name, value):
        """An int, float or str attribute on obj ("/" is the root)."""
        o, n = obj.encode(), name.encode()
        if isinstance(value, str):
            self._check(self.lib.ns_h5_attr_string(self.h, o, n, value.encode()))
        elif isinstance(value, (int, np.integer)) and not isinstance(value, bool):
            self._check(self.lib.ns_h5_attr_int(self.h, o, n, int(value)))
        else:
            self._check(self.lib.ns_h5_attr_double(self.h, o, n, float(value)))

    def attr(self, obj, name, kind=float):
        o, n = obj.encode(), name.encode()
        if kind is str:
            buf = C.create_string_buffer(4096)
            self._check(self.lib.ns_h5_get_attr_string(self.h, o, n, buf, len(buf)))
            return buf.value.decode()
        if kind is int:
            v = C.c_longlong()
            self._check(self.lib.ns_h5_get_attr_int(self.h, o, n, C.byref(v)))
            return v.value
        v = C.c_double()
        self._check(self.lib.ns_h5_get_attr_double(self.h, o, n, C.byref(v)))
        return v.value

    def write(self, path, a):
        a = np.asfortranarray(a, dtype=np.float64)
        dims = (C.c_longlong * a.ndim)(*a.shape)
        self._check(self.lib.ns_h5_write_double(self.h, path.encode(), a.ndim, dims, _ptr(a)))

    def shape(self, path):
        r = C.c_int()
        d = (C.c_longlong * 32)()
        self._check(self.lib.ns_h5_dims(self.h, path.encode(), C.byref(r), d))
        return tuple(d[i] for i in range(r.value))

    def read(self, path, shape=None):
        shape = tuple(shape) if shape is not None else self.shape(path)
        out = np.zeros(shape, order="F")
        dims = (C.c_longlong * max(1, len(shape)))(*shape)
        self._check(self.lib.ns_h5_read_double(self.h, path.encode(), len(shape), dims, _ptr(out)))
        return out

    def members(self, group="/"):
        need = C.c_longlong()
        self._check(self.lib.ns_h5_members(self.h, group.encode(), None, 0, C.byref(need)))
        buf = C.create_string_buffer(need.value)
        self._check(self.lib.ns_h5_members(self.h, group.encode(), buf, need.value, None))
        return [x for x in buf.value.decode().split("\n") if x]


def _session_h5_write_state(self, path, time=0.0, time_step=0, overwrite=False):
    """The state as a reference snapshot (big_periodic_3D.f90:630-651)."""
    self._check(self.lib.ns_h5_write_state(self.h, str(path).encode(), float(time), int(time_step), int(overwrite)))


def _session_h5_read_state(self, path):
    """Restart from a snapshot (big_periodic_3D.f90:309-324); returns (time, time_step)."""
    t = C.c_double()
    ts = C.c_int()
    self._check(self.lib.ns_h5_read_state(self.h, str(path).encode(), C.byref(t), C.byref(ts)))
    return t.value, ts.value


Session.h5_write_state = _session_h5_write_state
Session.h5_read_state = _session_h5_read_state
