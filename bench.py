"""Benchmark of the FP64 staggered Navier-Stokes step (one JSON line on stdout).

Workload (the headline configuration): triply periodic decaying turbulence
on a 256^3 staggered grid, FP64, AB2 + Crank-Nicolson ADI + FFT pressure
Poisson (big_periodic_3D.f90 step with timescheme "AB2-CN"), Re = 1600
(nu = 1/1600), dt fixed from CFL 0.3 on the initial field.  The initial
field is a seeded random-phase solenoidal field with E(k) ~ k^4
exp(-2 (k/k0)^2), k0 = 4, scaled to unit rms velocity and sampled at the
staggered u/v/w locations (synthetic; the reference's JHTDB-initialised
256^3 state is not available).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload hit|channel]

--workload channel measures the wall-bounded box instead: 256x128x256
(x, z periodic; y no-slip walls with Neumann pressure), domain 2pi x 2 x 2pi,
laminar profile u = 1 - (y-1)^2 plus a seeded divergence-free perturbation
of amplitude 0.05, Re = 180, dt = 2e-3, AB2-CN with the mixed FFT-x/z and
wall-y Poisson solve.

metric: grid cell-steps per second (nx*ny*nz*steps / seconds), whole job.
value : state resident in HBM, K steps replayed from a captured CUDA graph,
        CUDA events on the session's stream, barrier + synchronize around.
e2e   : the same metric through the C ABI with host buffers: every step
        is one ns_step_host call that copies the state in from pinned host
        memory, steps, and copies the state out (the copies of the history
        overlap the step).
--impl reference: the CPU restatement of the reference step on every host
        thread (oracle/ns_ref_cpu.cpp: the reference's algorithm in C++ and
        OpenMP; the Fortran/MKL reference cannot be built on these machines),
        a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import functools
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "FP64 grid cell-steps/s (256^3 periodic decaying turbulence, AB2-CN + FFT Poisson)"
UNIT = "cell-steps/s"

# Algorithmic HBM traffic per cell of each kernel (doubles read + written,
# dp_flag = 0, AB2-CN), the pass model of the step:
ALG_DOUBLES = {
    "predict": 12.0,      # read u, v, w, 3 history; write u*, v*, w*, 3 history
    "adi_x": 6.0, "adi_y": 6.0, "adi_z": 6.0,  # read + write u*, v*, w*
    "fft_x_fwd": 4.0,     # read u*, v*, w*; write half spectrum (16 B per 2 cells)
    "fft_y_fwd": 2.0,     # read + write half spectrum
    "fft_z_solve": 2.5,   # read + write half spectrum, read 1/lambda (8 B per 2 cells)
    "fft_y_inv": 2.0,
    "fft_x_inv": 2.0,     # read half spectrum, write dp
    "pr_bc": 0.0,         # ghost planes only
    "correct": 8.0,       # read u*, v*, w*, dp; write u, v, w, p
    "fft_z_fwd": 2.0, "fft_z_inv": 2.0,        # wall-y box: z transforms of the half spectrum
    "tri_y_solve": 2.0,   # read + write half spectrum (line solves along the wall axis)
}

# FP64 instructions per cell of each kernel (thread-level, adds and multiplies
# issued as DFMA), from ncu's sm__sass_thread_inst_executed_op_dfma_pred_on.sum
# of this build's kernels at 256^3 divided by the cells of one launch.
FP64_PER_CELL = {
    "predict": 62.7, "adi_x": 9.5, "adi_y": 9.5, "adi_z": 9.5, "fft_x_fwd": 18.8, "fft_y_fwd": 11.2,
    "fft_z_solve": 23.4, "fft_y_inv": 11.2, "fft_x_inv": 12.7, "correct": 7.2,
}


def fp64_per_cell(kernel, n):
    """FP64 instructions per cell of a step kernel at n^3; the cyclic z line
    solves do 10 per complex unknown, (n/2+1)/n complex unknowns per cell."""
    if kernel == "cyc_z_solve":
        return 10.0 * (n // 2 + 1) / n
    return FP64_PER_CELL.get(kernel, 0.0)
FP64_LANES_PER_CLK_SM = 2  # DFMA issue rate of this part (ncu ..._op_dfma_pred_on.sum.peak_sustained)

# DRAM bytes per launch at 256^3 (dram__bytes_read.sum + dram__bytes_write.sum)
# from one ncu capture of each kernel of this build's step.
NCU_TRAFFIC_256 = {
    "predict": 1659.0e6, "adi_x": 1574.2e6, "adi_y": 1486.3e6, "adi_z": 1480.0e6,
    "fft_x_fwd": 533.7e6, "fft_y_fwd": 213.0e6, "fft_z_solve": 293.6e6, "fft_y_inv": 213.0e6,
    "fft_x_inv": 219.9e6, "correct": 1112.1e6,
}


@functools.lru_cache(maxsize=2)
def hit_initial_field(n, k0=4.0, seed=2024):
    """Random-phase solenoidal field with E(k) ~ k^4 exp(-2 (k/k0)^2) on [0, 2pi]^3,
    unit rms velocity, sampled at the staggered locations, in the reference's
    padded shapes (periodic ghosts)."""
    rng = np.random.default_rng(seed)
    k = np.fft.fftfreq(n, 1.0 / n)
    kh = np.fft.rfftfreq(n, 1.0 / n)
    KX, KY, KZ = np.meshgrid(k, k, kh, indexing="ij")  # field axes (x, y, z); z is the half axis
    K2 = KX ** 2 + KY ** 2 + KZ ** 2
    K = np.sqrt(K2)
    K2[0, 0, 0] = 1.0
    amp = K * np.exp(-((K / k0) ** 2)) / np.sqrt(4.0 * np.pi)
    amp[0, 0, 0] = 0.0
    a = [(rng.standard_normal(K.shape) + 1j * rng.standard_normal(K.shape)) * amp for _ in range(3)]
    kdota = (KX * a[0] + KY * a[1] + KZ * a[2]) / K2
    a = [a[0] - KX * kdota, a[1] - KY * kdota, a[2] - KZ * kdota]
    del kdota, K, K2
    h = 2.0 * np.pi / n
    # staggered sample points: u at (x-face, y-cell, z-cell) = (i h, (j+1/2) h, (k+1/2) h)
    shifts = [(0.0, 0.5, 0.5), (0.5, 0.0, 0.5), (0.5, 0.5, 0.0)]
    comps = []
    for c in range(3):
        sx, sy, sz = (s * h for s in shifts[c])
        ph = np.exp(1j * (KX * sx + KY * sy + KZ * sz))
        comps.append(np.fft.irfftn(a[c] * ph, s=(n, n, n), axes=(0, 1, 2)))
        del ph
    del a, KX, KY, KZ
    rms = np.sqrt((np.mean(comps[0] ** 2) + np.mean(comps[1] ** 2) + np.mean(comps[2] ** 2)) / 3.0)
    comps = [c / rms for c in comps]
    face = np.r_[np.arange(n), 0]                     # faces 1..n+1 -> samples 0..n-1, 0
    cell = np.r_[n - 1, np.arange(n), 0]              # cells 1..n+2 (with ghosts) -> n-1, 0..n-1, 0
    u = np.asfortranarray(comps[0][np.ix_(face, cell, cell)])
    v = np.asfortranarray(comps[1][np.ix_(cell, face, cell)])
    w = np.asfortranarray(comps[2][np.ix_(cell, cell, face)])
    p = np.zeros((n + 2, n + 2, n + 2), order="F")
    umax = max(np.abs(comps[0]).max(), np.abs(comps[1]).max(), np.abs(comps[2]).max())
    return u, v, w, p, float(umax)


def channel_initial_field(nx, ny, nz, ly=2.0, amp=0.05, seed=180):
    """Laminar profile u = 1 - (y - 1)^2 between no-slip walls at y = 0, ly
    plus a divergence-free perturbation: the discrete curl of a smooth seeded
    vector potential (a_y, a_z) that vanishes on the walls, so the staggered
    divergence is zero to rounding.  Reference padded shapes, ghosts filled
    as vel_bc_staggered does with zero wall values: by the library's
    ns_vel_bc on the GPU arm, by the oracle on the CPU legs (bc_fill)."""
    rng = np.random.default_rng(seed)
    lx = lz = 2.0 * np.pi
    dx, dy, dz = lx / nx, ly / ny, lz / nz
    xf = dx * np.arange(nx + 1)             # x faces 1..nx+1
    yf = dy * np.arange(ny + 1)
    yc = dy * (np.arange(ny + 2) - 0.5)
    zf = dz * np.arange(nz + 1)
    zc = dz * (np.arange(nz + 2) - 0.5)
    modes = [(rng.integers(1, 5), rng.integers(1, 5), rng.uniform(0, 2 * np.pi), rng.uniform(0, 2 * np.pi),
              rng.standard_normal()) for _ in range(8)]

    def pot(x, y, z, off):
        env = (y * (ly - y)) ** 2
        a = np.zeros((x.size, y.size, z.size))
        for kx, kz, px, pz, c in modes:
            a += c * (np.sin(kx * x + px + off)[:, None, None] * np.sin(kz * z + pz)[None, None, :])
        return a * env[None, :, None]

    # a_z on (x face, y face, z cell), a_y on (x face, y cell, z face):
    # u = D_y a_z - D_z a_y, v = -D_x a_z, w = D_x a_y (exact discrete curl)
    az = pot(xf, yf, zc, 0.0)
    ay = pot(xf, yc, zf, 1.0)
    u = np.zeros((nx + 1, ny + 2, nz + 2))
    v = np.zeros((nx + 2, ny + 1, nz + 2))
    w = np.zeros((nx + 2, ny + 2, nz + 1))
    u[:, 1:ny + 1, :] = np.diff(az, axis=1) / dy
    u[:, :, 1:nz + 1] -= np.diff(ay, axis=2) / dz
    v[1:nx + 1] = -np.diff(az, axis=0) / dx
    w[1:nx + 1] = np.diff(ay, axis=0) / dx
    scale = amp / max(np.abs(u).max(), np.abs(v).max(), np.abs(w).max(), 1e-300)
    u *= scale; v *= scale; w *= scale
    u = u + (1.0 - (yc - 1.0) ** 2)[None, :, None]
    u, v, w = np.asfortranarray(u), np.asfortranarray(v), np.asfortranarray(w)
    p = np.zeros((nx + 2, ny + 2, nz + 2), order="F")
    return u, v, w, p


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x, world, device="cuda"):
    """The largest x over all ranks (the slowest replica sets the job's time)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(world, units_per_rank, seconds):
    """Whole-job throughput of `world` replicas that each did units_per_rank
    in `seconds` (the max over ranks)."""
    return world * units_per_rank / seconds


def workload(name, n):
    """Grid, initial state, step parameters and JSON config of a workload."""
    if name == "channel":
        nx, ny, nz = n, n // 2, n
        nu, dt = 1.0 / 180.0, 2e-3
        kw = dict(lx=2 * np.pi, ly=2.0, lz=2 * np.pi, nu=nu, dt=dt, scheme=2, bc=(1, 2, 1), pbc=(1, 3, 1))
        cfgd = {"workload": f"{nx}x{ny}x{nz} wall-bounded box (x, z periodic; y no-slip walls, Neumann pressure), "
                            "AB2-CN + FFT-x/z, line-solved y Poisson",
                "grid": [nx, ny, nz], "domain": "2pi x 2 x 2pi", "scheme": "AB2-CN", "poisson": "FFT x/z + wall y",
                "Re": 180, "nu": nu, "dt": dt, "seed": 180, "perturbation": 0.05, "dp_flag": 0,
                "l2": f"inputs larger than L2 (state 7 x {(nx + 2) * (ny + 2) * (nz + 2) * 8 / 1e6:.0f} MB)"}
        return dict(grid=(nx, ny, nz), kw=kw, config=cfgd,
                    metric="FP64 grid cell-steps/s (256x128x256 wall-bounded box, AB2-CN + mixed FFT/wall Poisson)",
                    init=lambda: channel_initial_field(nx, ny, nz), bc_fill=True)
    nu = 1.0 / 1600.0
    u, v, w, p, umax = hit_initial_field(n)
    dt = 0.3 * (2 * np.pi / n) / umax
    if name == "box":
        kw = dict(nu=nu, dt=dt, scheme=2, bc=(2, 2, 2), pbc=(3, 3, 3))
        cfgd = {"workload": f"{n}^3 all-wall box (no-slip walls on every face, Neumann pressure), AB2-CN, "
                            "FFT-based DCT x and y transforms + line-solved z Poisson",
                "grid": [n, n, n], "scheme": "AB2-CN",
                "poisson": "DCT x and y through FFTs (Makhoul), twisted tridiagonal z",
                "nu": nu, "dt": dt, "seed": 2024, "dp_flag": 0,
                "initial": "the decaying-turbulence field with the wall ghosts of vel_bc_staggered"}
        return dict(grid=(n, n, n), kw=kw, config=cfgd,
                    metric=f"FP64 grid cell-steps/s ({n}^3 all-wall box, AB2-CN + DCT Poisson)",
                    init=lambda: (u.copy(order="F"), v.copy(order="F"), w.copy(order="F"), p), bc_fill=True)
    return dict(grid=(n, n, n), kw=dict(nu=nu, dt=dt, scheme=2), config=workload_config(n, dt), metric=METRIC,
                init=lambda: (u, v, w, p))


def oracle_setup(name, n):
    from oracle import ns_oracle as O
    W = workload(name, n)
    nx, ny, nz = W["grid"]
    kw = dict(W["kw"])
    cfg = O.Config(nx, ny, nz, **kw)
    u, v, w, p = W["init"]()
    if W.get("bc_fill"):
        O.vel_bc_staggered(u, v, w, O.Faces.zeros(nx, ny, nz), *cfg.bc)
    st = O.State(u, v, w, p, np.zeros_like(u), np.zeros_like(v), np.zeros_like(w), first=True)
    dx, dy, dz = cfg.h
    cnf = O.CNFactors(nx, ny, nz, cfg.bc, dx * dx, dy * dy, dz * dz, cfg.dt, cfg.nu)
    return O, cfg, st, cnf, nx * ny * nz


def cpu_stepper(name, n, nthreads=None):
    """(advance_one_step, ncell, description, threads) of the timed CPU baseline:
    the C++/OpenMP restatement of the reference step (oracle/ns_ref_cpu.cpp,
    the reference's own algorithm: dense mat_CN LU solves for the ADI, FFT
    Poisson) on every host thread for the periodic workload; the NumPy/SciPy
    restatement otherwise (or if the C++ library cannot be built).  nthreads
    (C++ restatement only) limits the OpenMP threads of the steps; the
    returned restore() puts the process-wide setting back."""
    O, cfg, st, cnf, ncell = oracle_setup(name, n)
    if name == "hit":
        try:
            from oracle.ns_ref_cpu import CpuStep
            cpu = CpuStep(cfg)
            holder = {"st": st}
            before = cpu.threads()
            if nthreads:
                cpu.set_threads(nthreads)

            def adv():
                cpu.step(holder["st"])

            def restore():
                cpu.set_threads(before)

            return adv, ncell, ("C++/OpenMP restatement of the reference step (dense mat_CN LU line solves "
                                "as getrs, r2c FFT Poisson)"), cpu.threads(), restore
        except Exception:
            pass
    holder = {"st": st}

    def adv_np():
        holder["st"] = O.step(holder["st"], cfg, cnf=cnf)

    return (adv_np, ncell, "NumPy/SciPy restatement of the reference step (threaded BLAS)", os.cpu_count(),
            lambda: None)


def cpu_baseline_sample(name, n, steps, nthreads=None):
    """The CPU restatement on the host cores (or nthreads of them), on `steps`
    steps of the workload at grid size n after one untimed Euler-start step."""
    adv, ncell, desc, threads, restore = cpu_stepper(name, n, nthreads)
    try:
        adv()  # warm (Euler start)
        t0 = time.perf_counter()
        for _ in range(steps):
            adv()
        sec = time.perf_counter() - t0
    finally:
        restore()
    return ncell * steps / sec, sec, desc, threads


def run_reference(args):
    """The CPU restatement of the reference step on the host cores (rank 0 only)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    n = args.n
    W = workload(args.workload, n)
    adv, ncell, desc, threads, _restore = cpu_stepper(args.workload, n)
    t_w = time.perf_counter()
    warm = 0
    for _ in range(max(1, args.warmup)):
        adv()  # untimed (the first is the Euler start)
        warm += 1
        if time.perf_counter() - t_w > args.ref_budget_s / 2:
            break
    per_step = []
    for _ in range(max(1, args.steps)):
        t0 = time.perf_counter()
        adv()
        per_step.append(time.perf_counter() - t0)
        if sum(per_step) > args.ref_budget_s:
            break
    sec = float(np.median(per_step))
    value = ncell / sec
    line = {
        "impl": "reference", "metric": W["metric"], "value": value, "unit": UNIT, "n_gpus": world,
        "steps": len(per_step), "warmup": warm, "ms_per_step": 1e3 * sec,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": W["config"],
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{len(per_step)} step(s) of the full workload after {warm} untimed "
                                   f"step(s), the first an Euler start; {desc} (the Fortran/MKL reference "
                                   f"cannot be built here)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def workload_config(n, dt):
    return {"workload": f"{n}^3 triply periodic decaying turbulence, AB2-CN + FFT Poisson",
            "grid": [n, n, n], "scheme": "AB2-CN", "poisson": "FFT", "Re": 1600, "nu": 1.0 / 1600.0,
            "dt": dt, "cfl": 0.3, "k0": 4, "seed": 2024, "dp_flag": 0,
            "l2": "inputs larger than L2 (state 7 x 137 MB)"}


def resim_subdomains(n_parent=128, count=64, seed=4096):
    """64 sub-blocks: edges per axis from {16, 24, 32, 48, 64}, sub-step ratio
    from {1, 2, 4}, origins uniform so that every box fits in the parent."""
    rng = np.random.default_rng(seed)
    edges = np.array([16, 24, 32, 48, 64])
    subs = []
    for _ in range(count):
        nx, ny, nz = (int(e) for e in rng.choice(edges, 3))
        r = int(rng.choice([1, 2, 4]))
        x0, y0, z0 = (int(rng.integers(1, n_parent + 2 - e)) for e in (nx, ny, nz))
        subs.append((x0, y0, z0, nx, ny, nz, r))
    return subs


def run_resim(args):
    """Batched re-simulation of 64 sub-blocks of a 128^3 periodic parent
    (AB2, dp_flag = 1) over `steps` parent intervals, against (1) the same
    kernels launched once per subdomain and stage (mode 1), and (2) the plain
    path: one session per subdomain, advanced one by one with ns_set_faces,
    ns_set_mean_dp and ns_step, the faces of each interval read back from the
    batch's snapshots beforehand (untimed).  --resim-scheme ab2cn runs the
    AB2-CN re-simulation instead: parent and sub-blocks AB2-CN, the sub-blocks'
    ADI sweeps bounded by the parent's u* after each sweep, sub_tstep 1 (the
    reference's restriction for AB2-CN)."""
    import torch
    from ns_3d_staggered_dp_gb300 import Batch, Session, make_config

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    n = 128
    T = args.steps
    cn = getattr(args, "resim_scheme", "ab2") == "ab2cn"
    scheme = 2 if cn else 1
    u, v, w, p, umax = hit_initial_field(n, seed=64)
    nu = 1.0 / 1600.0
    h = 2 * np.pi / n
    dt = 0.3 * h / umax
    subs = resim_subdomains(n)
    if cn:
        subs = [s[:6] + (1,) for s in subs]
    cells = [nx * ny * nz for (_, _, _, nx, ny, nz, _) in subs]
    # cell-steps of the run: the first interval takes sub_tstep sub-steps
    work = sum(c * (r + (T - 1)) for c, (*_, r) in zip(cells, subs))
    n0 = 3
    n_slots = T + n0 + 8
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    out = {}
    with Session(make_config(n, n, n, nu=nu, dt=dt, scheme=scheme, dp_flag=1, keep_sweeps=int(cn))) as par:
        par.set_stream(stream.cuda_stream)
        par.set_state(u, v, w, p)
        batches = {m: Batch(subs, scheme=scheme, bc=2, pbc=3, nu=nu, dt0=dt, dx=h, dy=h, dz=h, n_slots=n_slots,
                            mode=m, use_graph=1) for m in (0, 1)}
        for b in batches.values():
            b.set_stream(stream.cuda_stream)
        tuned = batches[0].autotune(reps=3) if args.autotune else None
        stage_ms = None
        t_job0 = time.perf_counter()
        for k in range(1, T + n0 + 7):
            par.step(1)
            for b in batches.values():
                b.capture(par, k, k * dt)
            if k == n0:
                for b in batches.values():
                    b.init_from_parent(par)
        torch.cuda.synchronize()
        init_states = None
        for m, b in batches.items():
            l0 = b.launch_count()
            b.advance(n0 * dt)  # first interval (sub-steps; graph capture happens here)
            torch.cuda.synchronize()
            if m == 0:
                init_states = [b.get_state(i) for i in range(len(subs))]
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            with ClockSampler(local) as clk:
                e0.record(stream)
                for q in range(1, T):
                    b.advance((n0 + q) * dt)
                e1.record(stream)
                torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            steady = sum(c * (T - 1) for c in cells)
            out[m] = {"ms": ms, "value": steady / (ms / 1e3), "launches": b.launch_count() - l0,
                      "clocks": clk.summary()}
        job_sec = time.perf_counter() - t_job0
        plain = run_plain_loop(subs, init_states, batches[0], stream, n0, T, nu, dt, h, cn=cn)
        stage_ms = batches[0].profile(reps=3)
        st = [batches[m].get_state(0, history=False) for m in (0, 1)]
        same = all(np.array_equal(st[0][k], st[1][k]) for k in ("u", "v", "w", "p"))
        divs = [batches[0].max_div(i) for i in range(len(subs))]
        for b in batches.values():
            b.close()
    if rank != 0:
        return None
    line = {
        "metric": ("FP64 subdomain cell-steps/s, batched re-simulation of 64 sub-blocks (128^3 periodic parent)"
                   + (", AB2-CN with per-sweep u* faces" if cn else "")),
        "value": out[0]["value"], "unit": UNIT, "n_gpus": world, "steps": T - 1, "warmup": 1,
        "ms_per_step": out[0]["ms"] / (T - 1), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded k^4 exp(-2(k/4)^2) parent field, seed 64)",
        "config": {"workload": ("64 sub-blocks, edges {16,24,32,48,64} (seed 4096), AB2-CN, sub_tstep 1, bc 2 / "
                                "pbc 3, dp_flag 1, u* BCs of every ADI sweep, parent snapshots every step" if cn else
                                "64 sub-blocks, edges {16,24,32,48,64} and sub_tstep {1,2,4} (seed 4096), "
                                "AB2, bc 2 / pbc 3, dp_flag 1, u* BCs, spline-interpolated parent snapshots"),
                   "parent": [n, n, n], "subdomain_cells": int(sum(cells)), "intervals": T,
                   "first_interval_substeps": True},
        "loop": {"value": out[1]["value"], "ms_per_step": out[1]["ms"] / (T - 1), "launches": out[1]["launches"],
                 "what": "the batch's stage kernels launched once per subdomain and stage (mode 1)"},
        "speedup_vs_loop": out[0]["value"] / out[1]["value"],
        "plain_path_loop": plain,
        "speedup_vs_plain_path_loop": (plain["ms_per_step"] / (out[0]["ms"] / (T - 1))) if plain.get("ms_per_step")
        else None,
        "gpu_launches": out[0]["launches"],
        "bitwise_equal_to_loop": same,
        "max_div": max(divs),
        "autotuned_grid": tuned,
        "stage_ms": stage_ms,
        "clocks": out[0]["clocks"],
        "e2e": {"value": work / job_sec, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
                "path": "whole job: parent steps + snapshot captures + both batches (mode 0 and 1)"},
    }
    return line


def run_plain_loop(subs, init_states, batch, stream, n0, T, nu, dt, h, cn=False):
    """The plain path of the re-simulation: one session per subdomain (DCT
    pressure solve of the all-wall box), stepped one subdomain after another
    with its faces and mean dp for the interval (ns_set_faces, ns_set_mean_dp,
    ns_step), as a driver loop over the sub-blocks would.  Starts from the
    batch's state after its first interval; the faces of each interval are the
    batch's captured snapshot at the interval's end time, read back before the
    interval is timed.  The first regular interval is untimed (graph capture);
    returns ms per interval over the remaining T - 2 and the largest relative
    L2 difference of the final states from the batched run."""
    import ctypes as C

    import torch
    from ns_3d_staggered_dp_gb300 import FACE_ORDER, Session, make_config
    sess = []
    try:
        for (x0, y0, z0, nx, ny, nz, r), st in zip(subs, init_states):
            s = Session(make_config(nx, ny, nz, lx=nx * h, ly=ny * h, lz=nz * h, nu=nu, dt=dt, scheme=2 if cn else 1,
                                    bc=(2, 2, 2), pbc=(3, 3, 3), dp_flag=1, gauge=0))
            s.set_stream(stream.cuda_stream)
            s.set_state(st["u"], st["v"], st["w"], st["p"], (st["hx"], st["hy"], st["hz"]))
            sess.append(s)
        lib = sess[0].lib
        P = C.POINTER(C.c_double)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ms, timed, launches = 0.0, 0, 0
        for q in range(1, T):
            slot = n0 + q + 1  # the snapshot at the interval's end time (n0 + q + 1) dt
            prepared = []
            for i, s in enumerate(sess):
                faces, mean = batch.get_snapshot(slot, i)
                keep = [np.asfortranarray(faces[k]) for k in FACE_ORDER]
                arrs = [(P * 24)(*[a.ctypes.data_as(P) for a in keep])]
                if cn:  # the per-sweep faces go in face sets 1-3 (axis d's u, v, w entries)
                    sw = batch.get_sweep_faces(slot, i)
                    for d in range(3):
                        ks = [k if k[0] == "xyz"[d] and k[2] in "uvw" else None for k in FACE_ORDER]
                        a_d = [np.asfortranarray(sw[k]) if k else None for k in ks]
                        keep += [a for a in a_d if a is not None]
                        arrs.append((P * 24)(*[a.ctypes.data_as(P) if a is not None else None for a in a_d]))
                prepared.append((s.h, arrs, keep, mean))
            l0 = sum(s.launch_count() for s in sess)
            torch.cuda.synchronize()
            e0.record(stream)
            rcs = 0
            for hh, arrs, _keep, mean in prepared:
                for which, arr in enumerate(arrs):
                    rcs |= lib.ns_set_faces(hh, which, arr)
                rcs |= lib.ns_set_mean_dp(hh, mean)
                rcs |= lib.ns_step(hh, 1)
            e1.record(stream)
            torch.cuda.synchronize()
            if rcs:
                return {"error": "a session call failed"}
            if q > 1:
                ms += e0.elapsed_time(e1)
                timed += 1
                launches += sum(s.launch_count() for s in sess) - l0
        diff = 0.0
        for i, s in enumerate(sess):
            a = s.get_state(history=False)
            b = batch.get_state(i, history=False)
            for k in ("u", "v", "w", "p"):
                diff = max(diff, float(np.linalg.norm(a[k] - b[k]) / np.linalg.norm(b[k])))
        cells = sum(nx * ny * nz for (_, _, _, nx, ny, nz, _) in subs)
        return {"ms_per_step": ms / max(1, timed), "value": cells * timed / (ms / 1e3) if ms > 0 else None,
                "intervals_timed": timed, "launches": launches, "max_rel_l2_vs_batched": diff,
                "what": "64 sessions (ns_create with the subdomain's box, DCT/DST pressure solve), each interval "
                        "ns_set_faces (set 0, and sets 1-3 with AB2-CN) + ns_set_mean_dp + ns_step(1) per "
                        "subdomain, one after another"}
    finally:
        for s in sess:
            s.close()


def _slots(a, which, n):
    """Independent values of a periodic reference-shaped field."""
    sl = {"u": (slice(0, n), slice(1, n + 1), slice(1, n + 1)), "v": (slice(1, n + 1), slice(0, n), slice(1, n + 1)),
          "w": (slice(1, n + 1), slice(1, n + 1), slice(0, n))}[which]
    return a[sl]


def _embed(A, which, n):
    shp = {"u": (n + 1, n + 2, n + 2), "v": (n + 2, n + 1, n + 2), "w": (n + 2, n + 2, n + 1)}[which]
    out = np.zeros(shp, order="F")
    _slots(out, which, n)[...] = A
    return out


def _expand(A, which, n):
    face, cell = np.r_[np.arange(n), 0], np.r_[n - 1, np.arange(n), 0]
    ix = {"u": (face, cell, cell), "v": (cell, face, cell), "w": (cell, cell, face)}[which]
    return np.asfortranarray(A[np.ix_(*ix)])


def run_adjoint(args):
    """Gradient of J = 1/2 |u(T) - u_target|^2 over the central 64^3 of a 128^3
    periodic box with respect to the initial velocity: T = 50 AB2-CN steps
    (nu = 1/1600, dt from CFL 0.3), checkpoint every 10 steps.  The initial
    field has the decaying-turbulence spectrum (seed 2024); u_target is the
    forward run from the initial field plus 0.1 x a second field (seed 5).
    Reports the backward pass's cell-steps/s, its cost per step against a
    plain forward step, and central differences of J of the forward run in
    32 seeded directions against the gradient."""
    import torch
    from ns_3d_staggered_dp_gb300 import Session, make_config

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    n, T, K = 128, args.adj_steps, args.adj_ckpt
    nu = 1.0 / 1600.0
    u, v, w, p, umax = hit_initial_field(n, seed=2024)
    u5, v5, w5, _, _ = hit_initial_field(n, seed=5)
    dt = 0.3 * (2 * np.pi / n) / umax
    ncell = n ** 3
    lo, hi = n // 4, 3 * n // 4
    reg = (slice(lo, hi),) * 3
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    with Session(make_config(n, n, n, nu=nu, dt=dt, scheme=2)) as s:
        s.set_stream(stream.cuda_stream)

        def final_slots():
            o = s.get_state(history=False)
            return [np.ascontiguousarray(_slots(o[k], k, n)) for k in "uvw"]

        def J_of(U, tgt):
            return 0.5 * sum(float(np.sum((U[q][reg] - tgt[q][reg]) ** 2)) for q in range(3))

        # target: forward run from the perturbed field
        s.set_state(u + 0.1 * u5, v + 0.1 * v5, w + 0.1 * w5, p)
        s.step(T)
        tgt = final_slots()
        # plain forward step time (graph replay, CUDA events)
        s.set_state(u, v, w, p)
        s.step(3)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s.step(T)
        e1.record(stream)
        torch.cuda.synchronize()
        fwd_ms = e0.elapsed_time(e1) / T
        # warm run of the adjoint pair (allocations, graph capture)
        s.set_state(u, v, w, p)
        s.adj_forward(T, K)
        UT = final_slots()
        # seed and gradient in pinned host memory
        sh = s.shapes
        pin = lambda shp: torch.zeros(int(np.prod(shp)), dtype=torch.float64, pin_memory=True).numpy().reshape(
            shp, order="F")
        seed = [pin(sh[k]) for k in "uvw"]
        gout = {k: pin(sh[k]) for k in "uvw"}
        for q, k in enumerate("uvw"):
            g = np.zeros_like(UT[q])
            g[reg] = UT[q][reg] - tgt[q][reg]
            seed[q][...] = _embed(g, k, n)
        s.adj_backward(*seed, out=gout)
        # timed: forward with checkpoints, then the backward pass
        l0 = s.launch_count()
        s.set_state(u, v, w, p)
        torch.cuda.synchronize()
        with ClockSampler(local) as clk:
            t0 = time.perf_counter()
            s.adj_forward(T, K)
            t1 = time.perf_counter()
            grad = s.adj_backward(*seed, out=gout)
            t2 = time.perf_counter()
        launches = s.launch_count() - l0
        fwdk_ms, bwd_ms = 1e3 * (t1 - t0) / T, 1e3 * (t2 - t1) / T
        J0 = J_of(final_slots(), tgt)
        # central differences of the forward run in seeded directions
        G = [np.ascontiguousarray(_slots(grad[k], k, n)) for k in "uvw"]
        rng = np.random.default_rng(5)
        rms = float(np.sqrt(np.mean(_slots(u, "u", n) ** 2)))
        eps = args.adj_eps * rms
        base = [np.ascontiguousarray(_slots(a, k, n)) for a, k in zip((u, v, w), "uvw")]
        errs = []
        t_fd = time.perf_counter()
        for _ in range(args.adj_dirs):
            d = [rng.standard_normal((n, n, n)) for _ in range(3)]
            Js = []
            for sg in (1.0, -1.0):
                f = [_expand(b + sg * eps * dd, k, n) for b, dd, k in zip(base, d, "uvw")]
                s.set_state(f[0], f[1], f[2], p)
                s.step(T)
                Js.append(J_of(final_slots(), tgt))
            fd = (Js[0] - Js[1]) / (2 * eps)
            ad = sum(float(np.vdot(Gq, dq)) for Gq, dq in zip(G, d))
            errs.append(abs(fd - ad) / abs(ad))
        fd_sec = time.perf_counter() - t_fd
    if rank != 0:
        return None
    line = {
        "metric": "FP64 adjoint cell-steps/s (dJ/du0 over 50 AB2-CN steps of a 128^3 periodic box, checkpoint every 10)",
        "value": ncell * T / (bwd_ms * T / 1e3), "unit": UNIT, "n_gpus": world, "steps": T, "warmup": 1,
        "ms_per_step": bwd_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded k^4 exp(-2(k/4)^2) initial field, seed 2024; target from + 0.1 x seed 5 field)",
        "config": {"workload": "adjoint: J = 1/2 |u(T) - u_target|^2 over the central 64^3 of a 128^3 periodic box",
                   "grid": [n, n, n], "scheme": "AB2-CN", "nu": nu, "dt": dt, "steps": T, "ckpt_every": K,
                   "l2": "state 7 x 19 MB, checkpoints and stored inputs > L2 in total"},
        "forward_ms_per_step": fwd_ms,
        "forward_with_checkpoints_ms_per_step": fwdk_ms,
        "backward_ms_per_step": bwd_ms,
        "adjoint_cost_vs_forward": bwd_ms / fwd_ms,
        "gradient_run_cost_vs_forward": (fwdk_ms + bwd_ms) / fwd_ms,
        "J": J0,
        "fd_check": {"directions": args.adj_dirs, "eps": eps, "max_rel_err": max(errs) if errs else None,
                     "median_rel_err": float(np.median(errs)) if errs else None, "seconds": fd_sec},
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "e2e": {"value": ncell * T / (t2 - t0), "unit": UNIT, "h2d_bytes_per_step": 3 * 8 * (n + 1) * (n + 2) ** 2 / T,
                "d2h_bytes_per_step": 3 * 8 * (n + 1) * (n + 2) ** 2 / T,
                "path": "ns_adj_forward + ns_adj_backward (pinned host seed in, pinned host gradient out)"},
    }
    return line


def run_wall_extra(args, name="channel", steps=30):
    """Device-resident steps of a wall-bounded workload (the 256x128x256
    channel of the wall-bounded config), timed with CUDA events on the
    session's stream after 3 untimed steps."""
    import torch
    from ns_3d_staggered_dp_gb300 import Session, make_config

    W = workload(name, args.n)
    nx, ny, nz = W["grid"]
    u, v, w, p = W["init"]()
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    with Session(make_config(nx, ny, nz, **W["kw"])) as s:
        s.set_stream(stream.cuda_stream)
        if W.get("bc_fill"):
            u, v, w = s.vel_bc(u, v, w)
        s.set_state(u, v, w, p)
        s.step(3)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s.step(steps)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        d = s.diag()
    torch.cuda.set_stream(torch.cuda.default_stream())
    return {"metric": W["metric"], "value": nx * ny * nz * steps / (ms / 1e3), "unit": UNIT,
            "ms_per_step": ms / steps, "steps": steps, "workload": W["config"]["workload"],
            "max_div": d["max_div"]}


def run_ours(args):
    import torch

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from ns_3d_staggered_dp_gb300 import Session, make_config

    n = args.n
    W = workload(args.workload, n)
    nx, ny, nz = W["grid"]
    u, v, w, p = W["init"]()
    cfg = make_config(nx, ny, nz, **W["kw"])
    ncell = nx * ny * nz
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    with Session(cfg) as s:
        s.set_stream(stream.cuda_stream)
        if W.get("bc_fill"):
            u, v, w = s.vel_bc(u, v, w)  # ghosts as vel_bc_staggered sets them (ns_vel_bc, zero wall faces)
        s.set_state(u, v, w, p)
        s.step(max(3, args.warmup))  # Euler start, eager step, graph capture + replays
        torch.cuda.synchronize()

        def barrier():
            if world > 1:
                import torch.distributed as dist
                dist.barrier()

        # ---- device-resident throughput ----
        l0 = s.launch_count()
        barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with ClockSampler(local) as clk:
            e0.record(stream)
            s.step(args.steps)
            e1.record(stream)
            torch.cuda.synchronize()
        barrier()
        ms = max_over_ranks(e0.elapsed_time(e1), world)
        launches = s.launch_count() - l0
        ms_per_step = ms / args.steps
        value = job_rate(world, ncell * args.steps, ms / 1e3)
        d = s.diag()

        # ---- per-kernel times (events between launches, eager) ----
        prof = s.profile(2)

        # ---- end to end through the C ABI with pinned host buffers ----
        sh = s.shapes
        pin = lambda shp: torch.empty(int(np.prod(shp)), dtype=torch.float64, pin_memory=True).numpy().reshape(
            shp, order="F")
        hin = {k: pin(sh[k]) for k in ("u", "v", "w", "p")}
        hhist = [pin(sh[k]) for k in ("u", "v", "w")]
        st0 = s.get_state()
        for k in hin:
            hin[k][...] = st0[k]
        for a, k in zip(hhist, ("hx", "hy", "hz")):
            a[...] = st0[k]
        hout = {k: pin(sh[k]) for k in ("u", "v", "w", "p")}
        hout_h = [pin(sh[k]) for k in ("u", "v", "w")]
        import ctypes as C
        P = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        lib = s.lib
        e2e_steps = max(1, min(args.steps, args.e2e_steps))
        # ns_step_host reads p only with dp_flag = 1 (the step overwrites it otherwise)
        dpf = int(W["config"].get("dp_flag", 0))
        h2d = sum(a.nbytes for k, a in hin.items() if k != "p" or dpf) + sum(a.nbytes for a in hhist)
        d2h = sum(a.nbytes for a in hout.values()) + sum(a.nbytes for a in hout_h)
        # one untimed call first: it allocates the per-field staging buffers
        s._check(lib.ns_step_host(s.h, P(hin["u"]), P(hin["v"]), P(hin["w"]), P(hin["p"]),
                                  P(hhist[0]), P(hhist[1]), P(hhist[2]),
                                  P(hout["u"]), P(hout["v"]), P(hout["w"]), P(hout["p"]),
                                  P(hout_h[0]), P(hout_h[1]), P(hout_h[2])))
        torch.cuda.synchronize()
        barrier()
        # ns_step_host returns once the step's outputs are in host memory, so
        # every call is timed on its own; the rate is taken on the median call
        # (a stall of the host, e.g. page-cache work of another process, moves
        # one call, not the figure) and the extremes are reported beside it
        e2e_calls = []
        for _ in range(e2e_steps):
            t0 = time.perf_counter()
            s._check(lib.ns_step_host(s.h, P(hin["u"]), P(hin["v"]), P(hin["w"]), P(hin["p"]),
                                      P(hhist[0]), P(hhist[1]), P(hhist[2]),
                                      P(hout["u"]), P(hout["v"]), P(hout["w"]), P(hout["p"]),
                                      P(hout_h[0]), P(hout_h[1]), P(hout_h[2])))
            e2e_calls.append(time.perf_counter() - t0)
        torch.cuda.synchronize()
        e2e_sec = float(np.median(e2e_calls)) * e2e_steps
        # one more round, phase by phase (each phase ends synchronised)
        tp = [time.perf_counter()]
        s._check(lib.ns_set_state(s.h, P(hin["u"]), P(hin["v"]), P(hin["w"]), P(hin["p"]),
                                  P(hhist[0]), P(hhist[1]), P(hhist[2])))
        tp.append(time.perf_counter())
        s._check(lib.ns_step(s.h, 1))
        s._check(lib.ns_synchronize(s.h))
        tp.append(time.perf_counter())
        s._check(lib.ns_get_state(s.h, P(hout["u"]), P(hout["v"]), P(hout["w"]), P(hout["p"]),
                                  P(hout_h[0]), P(hout_h[1]), P(hout_h[2])))
        tp.append(time.perf_counter())
        e2e_phases = {"set_state_ms": 1e3 * (tp[1] - tp[0]), "step_ms": 1e3 * (tp[2] - tp[1]),
                      "get_state_ms": 1e3 * (tp[3] - tp[2])}
        barrier()
        e2e_sec = max_over_ranks(e2e_sec, world)
        e2e_value = job_rate(world, ncell * e2e_steps, e2e_sec)

    if rank != 0:
        return 0
    # roofline of the dominant kernel
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        with open(pk) as f:
            peaks = json.load(f)
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    dom = max(prof.items(), key=lambda kv: kv[1][0])
    dname, (dms, dl) = dom
    per_launch_ms = dms / max(1, dl)
    alg_bytes = ALG_DOUBLES.get(dname, 0.0) * 8.0 * ncell
    achieved = alg_bytes / (per_launch_ms / 1e3) / 1e9
    traffic = NCU_TRAFFIC_256.get(dname) if (n == 256 and args.workload == "hit") else None
    total_prof = sum(v[0] for v in prof.values())
    # FP64 roof: DFMA lanes per clock x SMs x the SM clock sampled in the timed region
    clk_s = clk.summary()
    sm_mhz = clk_s.get("sm_mhz") or 2070.0
    nsm = torch.cuda.get_device_properties(local).multi_processor_count
    fp64_peak = FP64_LANES_PER_CLK_SM * nsm * sm_mhz * 1e6 / 1e9  # G FP64 inst/s
    fp64_roof = None
    if args.workload == "hit":
        dom_fp = fp64_per_cell(dname, n) * ncell / (per_launch_ms / 1e3) / 1e9
        step_fp = sum(fp64_per_cell(k, n) * ncell * v[1] / 2 for k, v in prof.items()) / (ms_per_step / 1e3) / 1e9
        fp64_roof = {"bound": "fp64", "kernel": dname, "achieved": dom_fp, "peak": fp64_peak, "unit": "G FP64 inst/s",
                     "frac": dom_fp / fp64_peak, "step_achieved": step_fp, "step_frac": step_fp / fp64_peak,
                     "peak_source": f"{FP64_LANES_PER_CLK_SM} DFMA lanes/clk/SM x {nsm} SMs x {sm_mhz:.0f} MHz"}
    line = {
        "metric": W["metric"], "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64",
        "data": ("synthetic (seeded k^4 exp(-2(k/4)^2) solenoidal field, unit rms; no dataset)"
                 if args.workload in ("hit", "box") else
                 "synthetic (laminar profile + seeded divergence-free perturbation)"),
        "config": W["config"] | ({"parallelism": f"replicas x{world}"} if world > 1 else {}),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "steps": e2e_steps, "rate_on": "median call",
                "call_ms": {"median": 1e3 * float(np.median(e2e_calls)), "min": 1e3 * min(e2e_calls),
                            "max": 1e3 * max(e2e_calls)},
                "path": "ns_step_host: pinned host state in, one step, pinned host state out (copies overlap the step)",
                "separate_calls": {"set_state_get_state_phases": e2e_phases}},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": dname, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": traffic, "peak_source": peak_src,
                     "alg_bytes_per_launch": alg_bytes, "ms_per_launch": per_launch_ms,
                     "note": "the step is bound by the FP64 pipe, not HBM, on this part: see the fp64 object"},
        "fp64": fp64_roof,
        "kernel_ms_per_step": {k: v[0] / 2 for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])},
        "kernel_share": {k: v[0] / total_prof for k, v in prof.items()},
        "clocks": clk_s,
        "diag": {"max_div": d["max_div"], "probe": d["probe"]},
    }
    if args.extras and world == 1 and args.workload == "hit":
        # the other targets of the step, measured in the same run
        try:
            line["channel"] = run_wall_extra(args, "channel")
        except Exception as e:  # an extra never blocks the headline line
            line["channel"] = {"error": str(e)}
        try:
            a = argparse.Namespace(**vars(args))
            a.steps, a.autotune = 20, False
            r = run_resim(a)
            line["batched"] = {k: r[k] for k in ("metric", "value", "ms_per_step", "speedup_vs_plain_path_loop",
                                                 "speedup_vs_loop", "bitwise_equal_to_loop", "max_div")} | {
                "loop_ms_per_step": r["loop"]["ms_per_step"],
                "plain_path_loop_ms_per_step": r["plain_path_loop"].get("ms_per_step"),
                "plain_path_max_rel_l2_vs_batched": r["plain_path_loop"].get("max_rel_l2_vs_batched")}
        except Exception as e:  # an extra never blocks the headline line
            line["batched"] = {"error": str(e)}
        try:
            a = argparse.Namespace(**vars(args))
            a.steps, a.autotune, a.resim_scheme = 20, False, "ab2cn"
            r = run_resim(a)
            line["batched_ab2cn"] = {k: r[k] for k in ("metric", "value", "ms_per_step", "speedup_vs_plain_path_loop",
                                                       "speedup_vs_loop", "bitwise_equal_to_loop", "max_div")} | {
                "plain_path_loop_ms_per_step": r["plain_path_loop"].get("ms_per_step"),
                "plain_path_max_rel_l2_vs_batched": r["plain_path_loop"].get("max_rel_l2_vs_batched")}
        except Exception as e:
            line["batched_ab2cn"] = {"error": str(e)}
        try:
            a = argparse.Namespace(**vars(args))
            a.adj_dirs = 32
            r = run_adjoint(a)
            line["adjoint"] = {k: r[k] for k in ("metric", "value", "forward_ms_per_step", "backward_ms_per_step",
                                                 "adjoint_cost_vs_forward", "gradient_run_cost_vs_forward",
                                                 "fd_check")}
        except Exception as e:
            line["adjoint"] = {"error": str(e)}
        torch.cuda.set_stream(torch.cuda.default_stream())
    if args.cpu_baseline:
        try:
            cn = min(n, args.cpu_n)
            cv, csec, desc, threads = cpu_baseline_sample(args.workload, cn, 2)
            g = workload(args.workload, cn)["grid"]
            line["cpu_baseline"] = {"value": cv, "unit": UNIT, "cores": threads, "kind": "port",
                                    "sample": f"2 steps of the workload at {g[0]}x{g[1]}x{g[2]} "
                                              f"({csec:.1f} s) after one untimed step; {desc}"}
            if args.workload == "hit" and threads > 1:
                sv, ssec, _, st1 = cpu_baseline_sample(args.workload, cn, 1, nthreads=1)
                line["cpu_baseline"]["single_thread"] = {
                    "value": sv, "cores": st1,
                    "sample": f"1 step at {g[0]}x{g[1]}x{g[2]} ({ssec:.1f} s) after one untimed step"}
        except Exception as e:  # the baseline never blocks the GPU line
            line["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                                    "sample": f"failed: {e}"}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--cpu-n", type=int, default=256)
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--ref-budget-s", type=float, default=60.0)
    ap.add_argument("--workload", default="hit", choices=["hit", "channel", "box", "resim", "adjoint"])
    ap.add_argument("--adj-steps", type=int, default=50)
    ap.add_argument("--adj-ckpt", type=int, default=10)
    ap.add_argument("--adj-dirs", type=int, default=32)
    ap.add_argument("--adj-eps", type=float, default=1e-5)
    ap.add_argument("--no-extras", dest="extras", action="store_false",
                    help="skip the batched and adjoint summaries of the default line")
    ap.add_argument("--autotune", action="store_true", help="resim: autotune the batched stage kernels first")
    ap.add_argument("--resim-scheme", default="ab2", choices=["ab2", "ab2cn"],
                    help="resim: AB2 (sub-steps, spline BCs) or AB2-CN (per-sweep u* BCs, sub_tstep 1)")
    args = ap.parse_args()
    if args.workload in ("resim", "adjoint") and args.impl != "reference":
        line = run_resim(args) if args.workload == "resim" else run_adjoint(args)
        if line is not None:
            print(json.dumps(line), flush=True)
        return 0
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
