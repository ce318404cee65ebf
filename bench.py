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

metric: grid cell-steps per second (nx*ny*nz*steps / seconds), whole job.
value : state resident in HBM, K steps replayed from a captured CUDA graph,
        CUDA events on the session's stream, barrier + synchronize around.
e2e   : the same metric through the C ABI with host buffers: every step
        copies the state in from pinned host memory (ns_set_state), steps,
        and copies the state out (ns_get_state).
--impl reference: the CPU restatement of the reference step (the oracle
        port; the Fortran/MKL reference cannot be built on this machine) on
        the host cores, a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
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
}

# DRAM bytes per launch at 256^3 (dram__bytes_read.sum + dram__bytes_write.sum)
# from one ncu capture of each kernel of this build's step.
NCU_TRAFFIC_256 = {
    "predict": 1649.1e6, "adi_x": 1469.8e6, "adi_y": 1588.6e6, "adi_z": 1588.6e6,
    "fft_x_fwd": 533.7e6, "fft_y_fwd": 213.0e6, "fft_z_solve": 293.6e6, "fft_y_inv": 213.0e6,
    "fft_x_inv": 219.9e6, "correct": 1112.1e6,
}


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


def cpu_baseline_sample(n, steps, nu, dt):
    """The oracle step (a NumPy/SciPy restatement of big_periodic_3D's loop body)
    on the host cores, on `steps` steps of the n^3 workload."""
    from oracle import ns_oracle as O
    u, v, w, p, _ = hit_initial_field(n)
    cfg = O.Config(n, n, n, nu=nu, dt=dt, scheme=O.AB2_CN)
    st = O.State(u, v, w, p, np.zeros_like(u), np.zeros_like(v), np.zeros_like(w), first=True)
    dx = cfg.h[0]
    cnf = O.CNFactors(n, n, n, cfg.bc, dx * dx, dx * dx, dx * dx, dt, nu)
    st = O.step(st, cfg, cnf=cnf)  # warm (Euler start)
    t0 = time.perf_counter()
    for _ in range(steps):
        st = O.step(st, cfg, cnf=cnf)
    sec = time.perf_counter() - t0
    return n ** 3 * steps / sec, sec


def run_reference(args):
    """The oracle port of the reference step on the host cores (rank 0 only)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import ns_oracle as O
    n = args.n
    u, v, w, p, umax = hit_initial_field(n)
    nu = 1.0 / 1600.0
    dt = 0.3 * (2 * np.pi / n) / umax
    cfg = O.Config(n, n, n, nu=nu, dt=dt, scheme=O.AB2_CN)
    st = O.State(u, v, w, p, np.zeros_like(u), np.zeros_like(v), np.zeros_like(w), first=True)
    dx = cfg.h[0]
    cnf = O.CNFactors(n, n, n, cfg.bc, dx * dx, dx * dx, dx * dx, dt, nu)
    for _ in range(max(1, min(args.warmup, 1))):
        st = O.step(st, cfg, cnf=cnf)  # untimed (includes the Euler start)
    per_step = []
    for _ in range(max(1, args.steps)):
        t0 = time.perf_counter()
        st = O.step(st, cfg, cnf=cnf)
        per_step.append(time.perf_counter() - t0)
        if sum(per_step) > args.ref_budget_s:
            break
    sec = float(np.median(per_step))
    value = n ** 3 / sec
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": len(per_step), "warmup": 1, "ms_per_step": 1e3 * sec,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": workload_config(n, dt),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                         "sample": f"{len(per_step)} step(s) of the {n}^3 AB2-CN workload after one untimed "
                                   "Euler-start step; NumPy/SciPy restatement of the reference step "
                                   "(the Fortran/MKL reference cannot be built here), threaded BLAS"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def workload_config(n, dt):
    return {"workload": f"{n}^3 triply periodic decaying turbulence, AB2-CN + FFT Poisson",
            "grid": [n, n, n], "scheme": "AB2-CN", "poisson": "FFT", "Re": 1600, "nu": 1.0 / 1600.0,
            "dt": dt, "cfl": 0.3, "k0": 4, "seed": 2024, "dp_flag": 0,
            "l2": "inputs larger than L2 (state 7 x 137 MB)"}


def run_ours(args):
    import torch

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from ns_3d_staggered_dp_gb300 import Session, make_config

    n = args.n
    u, v, w, p, umax = hit_initial_field(n)
    nu = 1.0 / 1600.0
    dt = 0.3 * (2 * np.pi / n) / umax
    cfg = make_config(n, n, n, nu=nu, dt=dt, scheme=2)
    ncell = n ** 3
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    with Session(cfg) as s:
        s.set_stream(stream.cuda_stream)
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
        ms = e0.elapsed_time(e1)
        launches = s.launch_count() - l0
        if world > 1:
            import torch.distributed as dist
            t = torch.tensor([ms], device="cuda", dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        ms_per_step = ms / args.steps
        value = world * ncell * args.steps / (ms / 1e3)
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
        h2d = sum(a.nbytes for a in hin.values()) + sum(a.nbytes for a in hhist)
        d2h = sum(a.nbytes for a in hout.values()) + sum(a.nbytes for a in hout_h)
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            s._check(lib.ns_set_state(s.h, P(hin["u"]), P(hin["v"]), P(hin["w"]), P(hin["p"]),
                                      P(hhist[0]), P(hhist[1]), P(hhist[2])))
            s._check(lib.ns_step(s.h, 1))
            s._check(lib.ns_get_state(s.h, P(hout["u"]), P(hout["v"]), P(hout["w"]), P(hout["p"]),
                                      P(hout_h[0]), P(hout_h[1]), P(hout_h[2])))
        torch.cuda.synchronize()
        e2e_sec = time.perf_counter() - t0
        barrier()
        e2e_value = world * ncell * e2e_steps / e2e_sec

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
    traffic = NCU_TRAFFIC_256.get(dname) if n == 256 else None
    total_prof = sum(v[0] for v in prof.values())
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded k^4 exp(-2(k/4)^2) solenoidal field, unit rms; no dataset)",
        "config": workload_config(n, dt) | {"parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "steps": e2e_steps, "path": "ns_set_state (pinned host) + ns_step + ns_get_state (pinned host)"},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": dname, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": traffic, "peak_source": peak_src,
                     "alg_bytes_per_launch": alg_bytes, "ms_per_launch": per_launch_ms,
                     "note": "the step is FP64-pipe bound on this part (measured ~0.6 T DFMA/s); see fp64"},
        "kernel_ms_per_step": {k: v[0] / 2 for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])},
        "kernel_share": {k: v[0] / total_prof for k, v in prof.items()},
        "clocks": clk.summary(),
        "diag": {"max_div": d["max_div"], "probe": d["probe"]},
    }
    if args.cpu_baseline:
        try:
            cv, csec = cpu_baseline_sample(min(n, args.cpu_n), 1, nu, dt)
            line["cpu_baseline"] = {"value": cv, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                                    "sample": f"1 step of the {min(n, args.cpu_n)}^3 AB2-CN workload "
                                              f"({csec:.1f} s), NumPy/SciPy oracle restatement, threaded BLAS/FFT"}
        except Exception as e:  # the baseline never blocks the GPU line
            line["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                                    "sample": f"failed: {e}"}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--cpu-n", type=int, default=256)
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--ref-budget-s", type=float, default=60.0)
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
