"""Benchmark of the fused D2Q9 TRT lattice update (MLUPS, HBM roofline).

Workload (one GPU): the large obstacle array -- ny = 2048, nx = 8192
(16.8 M cells), 400 squares of side 0.02 ny on a seeded jittered 20 x 20
grid, parabolic Zou-He inlet, Zou-He pressure outlet, no-slip walls, IBB on
every obstacle link, drag/lift of every obstacle summed every iteration.
A "step" is one lattice iteration over all cells.  The distributions (2.4 GB
in 64-bit storage) are far larger than the 129 MB L2, so no flush is needed
between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--precision q60]
    python bench.py --impl reference        # CPU baseline arm (oracle port)

Prints one JSON line.  ``value`` is device-timed whole-job MLUPS of the
plain path (FP64 interface; ``q60``: 64-bit fixed-point state and integer
bulk collision, FP64 at wall and link cells) with the state resident in HBM;
``e2e`` is the same workload driven step by step through the host API (BC
vectors uploaded from pinned host memory and the drag/lift of every obstacle
read back every step); ``roofline`` is the bulk kernel's algorithmic bytes
(9 loads + 9 stores per cell) over its CUDA-event time against the measured
HBM copy bandwidth; ``forms`` are the other storage forms on the same
workload (``f64``: FP64 storage and arithmetic, bounded by the FP64 pipe,
reported with that second bound); ``form_errors`` runs the cylinder channel
(ny 200, nx 1100, Re 100) in every form and states the error of each against
the FP64 run; ``array_form_errors`` (``--array-errors N``, off by default)
does the same on this workload for N iterations; ``app_api`` runs the
channel through ``lbm_gb300.run`` with the app's hooks (observables, moving
averages, drag_lift lines) beside the engine-only figure; ``plain_vs_oracle`` checks
the plain forms' Cd/Cl series over the whole channel run against the C
oracle (run in a child process on the host cores meanwhile: the oracle is
the checker there, never the thing measured); ``batched_sweep`` is the
256-case sweep; ``adjoint`` is the drag-gradient cost on the ny 100 channel;
``cpu_baseline`` is the C restatement of the reference kernels driven by the
reference loop in C (oracle/, OpenMP over the host cores) on a bounded
sample of the same workload.
Under torchrun (N > 1) every rank runs one independent replica; the whole-job
figures are the slowest rank's (replica_totals).
"""
import argparse
import contextlib
import ctypes
import io
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BYTES_PER_LU = {"f64": 144, "q60": 144, "f32": 72, "f16s": 36, "bf16s": 36, "f16sr": 36,
                "bf16sr": 36}
FORMS = ["f64", "q60", "f32", "f16s", "f16sr", "bf16s", "bf16sr"]
SWEEP_FORM = "f16sr"  # FP16 shifted storage with stochastic rounding
FP64_DP_OPS_PER_LU = 67  # DP instructions of the FP64 collision (lbm_device.cuh)
ARITHMETIC = {
    "q60": "plain path, FP64 interface: populations stored as 64-bit fixed point (Q3.60, "
           "resolution 2^-60, exact sums), bulk collision on the integer pipes, wall and "
           "link cells in FP64",
    "f64": "FP64 storage and FP64 arithmetic",
    "f32": "FP32 storage of f - w rho0, FP32 arithmetic",
    "f16s": "FP16 storage of f - w rho0, FP32 arithmetic, FP64 drag sums",
    "bf16s": "BF16 storage of f - w rho0, FP32 arithmetic, FP64 drag sums",
    "f16sr": "FP16 storage of f - w rho0 with stochastic rounding, FP32 arithmetic, FP64 drag "
             "sums",
    "bf16sr": "BF16 storage of f - w rho0 with stochastic rounding, FP32 arithmetic, FP64 drag "
              "sums",
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="q60", choices=FORMS)
    ap.add_argument("--ny", type=int, default=2048)
    ap.add_argument("--forms", default="f64,f32,f16s,f16sr,bf16s,bf16sr",
                    help="other storage forms measured in the same run ('' = none)")
    ap.add_argument("--error-steps", type=int, default=200000,
                    help="iterations of the cylinder-channel form-error study (0 = skip)")
    ap.add_argument("--adjoint-steps", type=int, default=40000,
                    help="iterations of the adjoint cost measurement (0 = skip)")
    ap.add_argument("--e2e-steps", type=int, default=50)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--sweep-steps", type=int, default=10000,
                    help="iterations of the 256-case batched sweep (0 = skip)")
    ap.add_argument("--app-steps", type=int, default=200000,
                    help="iterations of the app-API run of the cylinder channel (0 = skip)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain-oracle", action="store_true",
                    help="skip the oracle run of the channel behind plain_vs_oracle")
    ap.add_argument("--array-errors", type=int, default=0,
                    help="iterations of the obstacle-array workload in every form, errors "
                         "against FP64 (0: skipped; 100000 takes ~7 minutes)")
    return ap.parse_args()


def workload_config(ny):
    return {"workload": "obstacle_array %dx%d, 400 squares (side 0.02 ny), IBB, Zou-He "
                        "inlet/outlet, drag+lift every step" % (4 * ny, ny),
            "nx": 4 * ny, "ny": ny, "n_obstacles": 400,
            "l2": "state larger than L2 (no flush needed)"}


def make_app(ny):
    from lbm_gb300.apps import obstacle_array
    app = obstacle_array(L_lbm=ny)
    app.output_freq = 10 ** 12
    return app


# ---------------------------------------------------------------------------
# nvidia-smi clock sampler
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.samples = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()
        time.sleep(0.3)

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm = []
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        smax = None
        for p in self.samples:
            try:
                sm.append(float(p[0]))
                smax = float(p[1])
            except ValueError:
                continue
            for k, n in enumerate(names):
                if p[3 + k].lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def build_engine(ny, precision, tmp):
    import lbm_gb300
    from lbm_gb300.engine import FusedEngine, trace_bc_program
    app = make_app(ny)
    with contextlib.redirect_stdout(io.StringIO()):
        lat = lbm_gb300.lattice(app, precision=precision, output_dir=tmp, verbose=False)
        lat.generate_image = lambda obstacles: None
        app.initialize(lat)
    obstacles, walls, corners = trace_bc_program(app)
    eng = FusedEngine(lat, obstacles, walls, corners, precision=precision, drag_cap=4096)
    base, vec, scale = app.bc_schedule(lat)
    eng.set_bc_schedule(base, vec, scale(np.arange(200000)), it0=0)
    eng.collide_from_g(0, macro=False)
    return app, lat, eng


def measure_form(ny, precision, steps, warmup, tmp, peak_gbs, dist=None):
    import torch
    from lbm_gb300 import _lib
    app, lat, eng = build_engine(ny, precision, tmp)
    N = lat.nx * lat.ny
    stream = torch.cuda.current_stream()
    it = 1
    # Warm-up: W steps, then one untimed K-step graph (captures the graph).
    eng.steps(it, warmup, graph=False)
    it += warmup
    eng.steps(it, steps, graph=True)
    it += steps
    eng.check_status()
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    eng.steps(it, steps, graph=True)
    e1.record(stream)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    ms = e0.elapsed_time(e1)
    it += steps
    eng.check_status()
    # Per-kernel times over K more steps (events around each kernel).
    prof = (ctypes.c_double * 4)()
    _lib.call("lbm_profile_steps", ctypes.byref(eng.P), it, steps, eng.cur,
              _lib.FLAG_CHECK_FINITE | eng.step_flags, prof, ctypes.c_void_p(stream.cuda_stream))
    eng.cur ^= (steps & 1)
    it += steps
    bulk_units = (lat.nx - 2) * (lat.ny - 2)
    bulk_ms = prof[0]
    achieved = BYTES_PER_LU[precision] * bulk_units / (bulk_ms * 1e-3) / 1e9
    res = {
        "precision": precision,
        "ms_per_step": ms / steps,
        "mlups": N * steps / (ms * 1e-3) / 1e6,
        "kernel_ms": {"bulk": prof[0], "special": prof[1], "drag": prof[2]},
        "kernels_per_step": int(prof[3]),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak_gbs, "unit": "GB/s",
                     "frac": achieved / peak_gbs, "traffic": None,
                     "bytes_per_unit": BYTES_PER_LU[precision], "units_per_launch": bulk_units},
        "n_special": eng.n_special, "n_links": eng.n_links,
    }
    return res, (app, lat, eng, it)


def measure_e2e(app, lat, eng, it, steps, depth=2):
    """Step by step through the C-ABI with host buffers: every step's BC
    vectors go up from pinned host memory and every step's drag/lift of all
    obstacles comes back to pinned host memory and is read by the host.
    The copies run on a copy stream (each step's kernels wait for its
    upload; each download waits for its step), and the host runs ``depth``
    steps ahead: step k + depth (its BC vectors computed on the host and
    copied into one of depth + 1 rotating device buffers) is enqueued before
    the host waits for step k's drag/lift, so neither the copies nor the
    host's turnaround leave the GPU idle."""
    import torch
    nx, ny = lat.nx, lat.ny
    base, vec, scale = app.bc_schedule(lat)
    n_obs = len(eng.obstacles)
    nb = depth + 1
    h_bc = [torch.empty(base.size, dtype=torch.float64).pin_memory() for _ in range(nb)]
    d_bc = [eng.bc_base] + [torch.empty_like(eng.bc_base) for _ in range(nb - 1)]
    h_drag = [torch.empty((n_obs, 2), dtype=torch.float64).pin_memory() for _ in range(nb)]
    up = [torch.cuda.Event() for _ in range(nb)]      # upload of buffer b done
    ran = [torch.cuda.Event() for _ in range(nb)]     # step using buffer b done
    down = [torch.cuda.Event() for _ in range(nb)]    # drag/lift of buffer b on the host
    eng.set_bc_constant(base)
    P = eng.P
    stream = torch.cuda.current_stream()
    copy = torch.cuda.Stream()

    def host_bc(m, buf):  # BC vectors of iteration m - 1, straight into pinned memory
        hb = buf.numpy()
        np.multiply(vec, scale([m - 1])[0], out=hb)
        np.add(hb, base, out=hb)

    def launch(m, b):  # step m with BC buffer b, then its drag/lift down into h_drag[b]
        up[b].synchronize()  # the pinned buffer's previous upload has been read
        host_bc(m, h_bc[b])
        with torch.cuda.stream(copy):
            copy.wait_event(ran[b])  # the device buffer's previous step is done
            d_bc[b].copy_(h_bc[b], non_blocking=True)
            up[b].record(copy)
        stream.wait_event(up[b])
        P.bc_base = d_bc[b].data_ptr()
        eng.steps(m, 1, graph=True)
        ran[b].record(stream)
        slot = (m - 1) % eng.drag_cap
        with torch.cuda.stream(copy):
            copy.wait_event(ran[b])
            h_drag[b].copy_(eng.drag_hist[slot, :n_obs], non_blocking=True)
            down[b].record(copy)

    # untimed steps capture the one-step graph of every BC buffer
    for k in range(nb):
        launch(it, k)
        it += 1
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    checksum = 0.0
    for k in range(steps):
        launch(it + k, k % nb)
        if k >= depth:  # step k - depth's drag/lift on the host
            down[(k - depth) % nb].synchronize()
            checksum += float(h_drag[(k - depth) % nb].numpy().sum())
    for k in range(max(0, steps - depth), steps):
        down[k % nb].synchronize()
        checksum += float(h_drag[k % nb].numpy().sum())
    stream.wait_stream(copy)
    e1.record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    ms = e0.elapsed_time(e1)
    P.bc_base = eng.bc_base.data_ptr()
    if not np.isfinite(checksum):
        raise FloatingPointError("end-to-end run: non-finite drag/lift")
    return {"value": nx * ny * steps / (ms * 1e-3) / 1e6, "unit": "MLUPS",
            "h2d_bytes_per_step": int(base.size * 8), "d2h_bytes_per_step": int(n_obs * 2 * 8),
            "wall_s": wall, "steps": steps, "pipeline_depth": depth}


def measure_sweep(steps):
    """The 256-case sweep (FP16 shifted storage): autotune (scheduling,
    vector width, threads, tile rounds, bulk kernel, then iterations per
    graph and concurrent groups; the lattices are put back in their state
    before the trials), then `steps` iterations of every case in batched
    graphs; the per-case serial loop is timed for comparison, with plain
    launches (20 iterations) and with one CUDA graph per case (50
    iterations)."""
    import torch
    from lbm_gb300.batch import Batch, autotune, serial_loop_mlups, sweep_apps, time_batch
    t0 = time.perf_counter()
    # BC schedule length: the autotuner's trials (24 configurations x 250
    # iterations, then 5 x (K + 200) and 6 x (K + 200), rolled back
    # afterwards), the timed iterations and the serial loops.
    b = Batch(sweep_apps(seed=2024), precision=SWEEP_FORM, max_steps=steps + 12000)
    setup_s = time.perf_counter() - t0
    best, trials = autotune(b, steps=200)
    b.check()
    ms = time_batch(b, steps, k=best["k_steps"])
    b.check()
    mlups = b.cells * steps / (ms * 1e-3) / 1e6
    serial, _ = serial_loop_mlups(b, steps=20)
    serial_g, _ = serial_loop_mlups(b, steps=50, graph=True)
    info = b.info()
    b.close()
    k_trials = {t[0]["k_steps"]: t[1] for t in trials if t[0].get("_stage") == 2}
    group_trials = {"%d groups, bulk_tma %d" % (t[0]["streams"], t[0].get("bulk_tma", 0)): t[1]
                    for t in trials if t[0].get("_stage") == 3}
    return {"cases": info["lattices"], "cells": b.cells, "steps": steps, "mlups": mlups,
            "ms_per_step": ms / steps, "serial_loop_mlups": serial,
            "x_vs_serial": mlups / serial, "serial_graph_loop_mlups": serial_g,
            "x_vs_serial_graphs": mlups / serial_g, "config": best,
            "k_steps_trials_mlups": k_trials, "concurrent_groups_trials_mlups": group_trials,
            "setup_s": setup_s,
            "autotune_trials": len(trials), "precision": SWEEP_FORM,
            "all_finite": True}


def channel_app(ny, steps):
    """Turek cylinder channel with nx = 5.5 ny (x_max = 2.055), Re 100 on the
    cylinder diameter 0.244 ny, centred 0.49 ny from the inlet and the bottom."""
    from lbm_gb300.apps import turek
    a = turek()
    a.L_lbm = ny
    a.x_max = 2.055
    a.compute_lbm_parameters()
    a.stop, a.it_max, a.output_freq = "it", steps - 1, 10 ** 12
    return a


def run_channel(precision, ny, steps, tmp, chunk=2000):
    """Iterations 0 .. steps-1 of the channel in one form: drag/lift series
    (Cd, Cl of iterations 0 .. steps-2), final velocity field, MLUPS."""
    app = channel_app(ny, steps)
    r = run_case(app, precision, steps, tmp, chunk)
    norm = -2.0 / (app.rho_lbm * app.D_lbm * app.u_avg ** 2)
    r["cd"], r["cl"] = r.pop("fx") * norm, r.pop("fy") * norm
    return r


def run_case(app, precision, steps, tmp, chunk=2000):
    """Iterations 0 .. steps-1 of an app in one form from its initial state:
    drag/lift sums over every obstacle (iterations 0 .. steps-2), final
    velocity field on the host, MLUPS."""
    import torch
    import lbm_gb300
    from lbm_gb300.engine import FusedEngine, trace_bc_program
    with contextlib.redirect_stdout(io.StringIO()):
        lat = lbm_gb300.lattice(app, precision=precision, output_dir=tmp, verbose=False)
        lat.generate_image = lambda obstacles: None
        app.initialize(lat)
    obstacles, walls, corners = trace_bc_program(app)
    eng = FusedEngine(lat, obstacles, walls, corners, precision=precision, drag_cap=steps + 8)
    base, vec, scale = app.bc_schedule(lat)
    eng.set_bc_schedule(base, vec, scale(np.arange(steps + 2)), it0=0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    eng.collide_from_g(0, macro=False)
    it = 1
    while it <= steps - 1:
        n = min(chunk, steps - it)
        eng.steps(it, n, macro_last=(it + n == steps), graph=True)
        it += n
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    eng.check_status()
    idx = torch.arange(0, steps - 1, device=eng.drag_hist.device) % eng.drag_cap
    rows = eng.drag_hist[idx, :len(obstacles)].sum(dim=1).cpu().numpy()
    u = lat.device_field("u").cpu().numpy().copy()
    del eng
    return {"fx": rows[:, 0], "fy": rows[:, 1], "u": u,
            "mlups": lat.nx * lat.ny * steps / dt / 1e6, "nx": lat.nx, "ny": lat.ny}


def measure_array_errors(steps, forms, tmp, ny):
    """Every form on the obstacle-array workload from the same initial state,
    errors against the FP64 run: total drag (sum of fx over the obstacles)
    mean / max and total lift rms over the second half, the total-drag series,
    and the velocity field at the last iteration (L2)."""
    import torch
    ref = run_case(make_app(ny), "f64", steps, tmp)
    half = slice(len(ref["fx"]) // 2, None)

    def stats(r):
        fx, fy = r["fx"][half], r["fy"][half]
        return {"fx_mean": float(fx.mean()), "fx_max": float(np.abs(fx).max()),
                "fy_rms": float(np.sqrt((fy ** 2).mean()))}

    sref = stats(ref)
    out = {"case": "obstacle_array %dx%d, 400 squares, Re 2000 on the side, %d iterations "
                   "(all forms from the same initial state)" % (ref["nx"], ref["ny"], steps),
           "f64": dict(sref, mlups=ref["mlups"])}
    for form in forms:
        if form == "f64":
            continue
        try:
            r = run_case(make_app(ny), form, steps, tmp)
        except FloatingPointError as e:  # the form's range or precision gave out
            out[form] = {"diverged": str(e)}
            torch.cuda.empty_cache()
            continue
        st = stats(r)
        err = {k + "_rel": abs(st[k] - sref[k]) / abs(sref[k]) for k in sref}
        err["u_l2_rel"] = float(np.linalg.norm(r["u"] - ref["u"]) / np.linalg.norm(ref["u"]))
        err["fx_series_max_rel"] = float(np.max(np.abs(r["fx"] - ref["fx"])) /
                                         np.max(np.abs(ref["fx"])))
        out[form] = dict(st, mlups=r["mlups"], error_vs_f64=err)
        del r
        torch.cuda.empty_cache()
    return out


def shedding_period(cl):
    """Mean distance in iterations between upward zero crossings of the
    lift about its mean (None without at least three)."""
    s = np.sign(cl - cl.mean())
    up = np.flatnonzero((s[:-1] < 0) & (s[1:] >= 0))
    return float(np.mean(np.diff(up))) if len(up) >= 3 else None


def aligned_lag(ref, got, max_lag):
    """The shift L (|L| <= max_lag) that best aligns got[t + L] with ref[t]
    (largest mean product of the mean-free series over their overlap; the
    correlations by FFT)."""
    a = ref - ref.mean()
    b = got - got.mean()
    n = len(a)
    m = 1 << int(np.ceil(np.log2(2 * n)))
    c = np.fft.irfft(np.fft.rfft(b, m) * np.conj(np.fft.rfft(a, m)), m)
    lags = np.arange(-max_lag, max_lag + 1)
    # mean product over the overlap of each shift
    return int(lags[np.argmax(c[lags % m] / (n - np.abs(lags)))])


def smooth(x, w=101):
    """Centred moving average over w iterations (w odd; the ends dropped)."""
    c = np.cumsum(np.insert(np.asarray(x, dtype=np.float64), 0, 0.0))
    return (c[w:] - c[:-w]) / w


def series_errors(ref_cd, ref_cl, cd, cl, period):
    """Max deviation of the Cd / Cl series relative to the series' maximum
    magnitude, as they are and after shifting the form's series by the lag
    that aligns its shedding phase with the reference's."""
    out = {"cd_series_max_rel": float(np.max(np.abs(cd - ref_cd)) / np.max(np.abs(ref_cd))),
           "cl_series_max_rel": float(np.max(np.abs(cl - ref_cl)) / np.max(np.abs(ref_cl)))}
    if period:
        # the phase is defined up to whole periods: the smallest shift, then
        # the least-squares shift of Cl near it
        lag0 = aligned_lag(ref_cl, cl, int(period // 2))

        def sq(L):
            n = len(ref_cl) - abs(L)
            a0, b0 = (0, L) if L >= 0 else (-L, 0)
            return float(np.mean((cl[b0:b0 + n] - ref_cl[a0:a0 + n]) ** 2))

        lag = min(range(lag0 - 32, lag0 + 33), key=sq)
        n = len(ref_cl) - abs(lag)
        r0, g0 = (0, lag) if lag >= 0 else (-lag, 0)
        out["phase_lag_iterations"] = lag
        for k, rs, gs in (("cd", ref_cd, cd), ("cl", ref_cl, cl)):
            d = np.abs(gs[g0:g0 + n] - rs[r0:r0 + n])
            out[k + "_aligned_max_rel"] = float(d.max() / np.max(np.abs(rs[r0:r0 + n])))
    return out


def measure_form_errors(steps, forms, tmp, ny=200):
    """Every form on the cylinder channel, errors stated against the FP64 run
    over the second half of the run: mean Cd, rms Cl, max Cd, max Cl, the
    Cd oscillation amplitude and the shedding period; the whole Cd and Cl
    series (max deviation, as they are and phase-aligned); the velocity
    field at the last iteration (L2).  Amplitude, period, max Cl and the
    series errors are also given on a 101-iteration moving average
    ("_smoothed", about 2 % of the shedding period): the 16-bit forms' drag
    and lift carry per-iteration rounding noise (a few 1e-2 of Cd) that the
    raw extremes and zero crossings pick up.  Also returns the Cd/Cl series and
    final velocity of the two plain forms (f64, q60) for plain_vs_oracle."""
    import torch
    ref = run_channel("f64", ny, steps, tmp)
    half = slice(len(ref["cd"]) // 2, None)

    def stats(r):
        cd, cl = r["cd"][half], r["cl"][half]
        cds, cls = smooth(cd), smooth(cl)
        return {"cd_mean": float(cd.mean()), "cl_rms": float(np.sqrt((cl ** 2).mean())),
                "cd_max": float(cd.max()), "cl_max": float(cl.max()),
                "cd_amplitude": float(0.5 * (cd.max() - cd.min())),
                "period": shedding_period(cl),
                "cd_amplitude_smoothed": float(0.5 * (cds.max() - cds.min())),
                "cl_max_smoothed": float(cls.max()), "period_smoothed": shedding_period(cls)}

    sref = stats(ref)
    out = {"case": "cylinder channel %dx%d, D = %d, Re 100, %d iterations (all forms from the "
                   "same initial state); statistics over the second half" %
                   (ref["nx"], ref["ny"], channel_app(ny, 2).D_lbm, steps),
           "f64": dict(sref, mlups=ref["mlups"])}
    plain = {"f64": {k: ref[k] for k in ("cd", "cl", "u")}}
    for form in forms:
        if form == "f64":
            continue
        r = run_channel(form, ny, steps, tmp)
        if form == "q60":
            plain["q60"] = {k: r[k] for k in ("cd", "cl", "u")}
        st = stats(r)
        err = {k + "_rel": (abs(st[k] - sref[k]) / abs(sref[k])
                            if st[k] is not None and sref[k] else None) for k in sref}
        err["u_l2_rel"] = float(np.linalg.norm(r["u"] - ref["u"]) / np.linalg.norm(ref["u"]))
        err.update(series_errors(ref["cd"][half], ref["cl"][half], r["cd"][half],
                                 r["cl"][half], sref["period"]))
        sm = series_errors(smooth(ref["cd"][half]), smooth(ref["cl"][half]),
                           smooth(r["cd"][half]), smooth(r["cl"][half]), sref["period_smoothed"])
        err.update({k + "_smoothed": v for k, v in sm.items()})
        out[form] = dict(st, mlups=r["mlups"], error_vs_f64=err)
        del r
        torch.cuda.empty_cache()
    return out, plain


def measure_app_api(steps, tmp, engine_mlups, ny=200):
    """The cylinder channel (config 1) through the app API: lbm_gb300.run
    with the turek app's hooks (drag/lift every iteration, the buffers'
    moving averages and convergence test, one drag_lift line per iteration),
    wall time from run() to its return, against the engine-only figure of
    the same case (run_case).  Field outputs are off (output_freq beyond the
    run): they are the app's file writes, not the lattice update.  An untimed
    2,000-iteration run first loads what a process loads once (the CUDA
    modules of the PyTorch operations the hooks use, the buffers' code
    paths): measured at ~2 s, which is not a per-run cost."""
    import lbm_gb300
    warm = channel_app(ny, 2000)
    wout = tempfile.mkdtemp(prefix="app_api_warm_", dir=tmp)
    with contextlib.redirect_stdout(io.StringIO()):
        wlat = lbm_gb300.lattice(warm, precision="q60", output_dir=wout + "/", verbose=False)
        wlat.generate_image = lambda obstacles: None
        lbm_gb300.run(wlat, warm)
    del wlat
    app = channel_app(ny, steps)
    out = tempfile.mkdtemp(prefix="app_api_", dir=tmp)
    with contextlib.redirect_stdout(io.StringIO()):
        lat = lbm_gb300.lattice(app, precision="q60", output_dir=out + "/", verbose=False)
        lat.generate_image = lambda obstacles: None
        t0 = time.perf_counter()
        lbm_gb300.run(lat, app)
        wall = time.perf_counter() - t0
    with open(os.path.join(out, "drag_lift")) as f:
        n_lines = sum(1 for _ in f)
    mlups = lat.nx * lat.ny * steps / wall / 1e6
    return {"case": "lbm_gb300.run(lattice, turek) on the cylinder channel %dx%d, %d iterations, "
                    "q60" % (lat.nx, lat.ny, steps),
            "wall_s": wall, "mlups": mlups, "engine_mlups": engine_mlups,
            "frac_of_engine": mlups / engine_mlups if engine_mlups else None,
            "drag_lift_lines": n_lines}


def measure_adjoint(steps, tmp, ny=100):
    """Gradient of the mean Cd over the last half of `steps` iterations with
    respect to the inlet profile (every inlet row) and the TRT rate, on the
    channel with ny = 100 (nx 550, Re 100), FP64: wall time of the gradient
    (checkpointed forward + reverse sweep) over one plain forward run, peak
    device memory, and a central-difference check (h = 1e-6) of dJ/d om_p and
    of dJ/d u_in at the middle inlet row."""
    import torch
    import lbm_gb300
    from lbm_gb300.adjoint import DragAdjoint, cd_weights
    app = channel_app(ny, steps)
    with contextlib.redirect_stdout(io.StringIO()):
        lat = lbm_gb300.lattice(app, precision="f64", output_dir=tmp, verbose=False)
        lat.generate_image = lambda obstacles: None
        app.initialize(lat)
    adj = DragAdjoint(lat, app)
    n_obs = len(adj.eng.obstacles)
    win = (steps - steps // 2, steps - 1)
    w = cd_weights(app, n_obs, win[1] - win[0] + 1)
    adj.forward(min(steps, 200), (0, 0), w, checkpoint=False)  # warm-up (graph capture)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    J_plain = adj.forward(steps, win, w, checkpoint=False)
    torch.cuda.synchronize()
    t_fwd = time.perf_counter() - t0
    torch.cuda.reset_peak_memory_stats()
    base_mem = torch.cuda.memory_allocated()
    t0 = time.perf_counter()
    J = adj.forward(steps, win, w, checkpoint=True)
    grad = adj.gradient()
    torch.cuda.synchronize()
    t_grad = time.perf_counter() - t0
    peak = torch.cuda.max_memory_allocated() - base_mem
    n_ckpt = len(adj.ckpt)
    h = 1e-6
    om0, vec0 = lat.om_p_lbm, adj.vec.copy()

    def J_at(om=om0, vec=vec0):
        adj.set_omega(om)
        adj.set_bc_vec(vec)
        return adj.forward(steps, win, w, checkpoint=False)

    fd_om = (J_at(om=om0 + h) - J_at(om=om0 - h)) / (2 * h)
    j = lat.ny // 2
    vp, vm = vec0.copy(), vec0.copy()
    vp[j] += h
    vm[j] -= h
    fd_u = (J_at(vec=vp) - J_at(vec=vm)) / (2 * h)
    J_at()
    return {"case": "cylinder channel %dx%d, Re 100, FP64, J = mean Cd over iterations %d..%d"
                    % (lat.nx, lat.ny, win[0], win[1]),
            "iterations": steps, "parameters": lat.ny + 1, "J": J, "J_plain_forward": J_plain,
            "forward_s": t_fwd, "gradient_s": t_grad, "gradient_over_forward": t_grad / t_fwd,
            "checkpoints": n_ckpt, "segment": adj.K,
            "peak_device_bytes": int(peak),
            "fd_check": {"h": h,
                         "omega": {"adjoint": grad["omega"], "fd": fd_om,
                                   "rel": abs(fd_om - grad["omega"]) / abs(grad["omega"])},
                         "u_in_row_%d" % j: {"adjoint": float(grad["bc_vec"][j]), "fd": fd_u,
                                             "rel": abs(fd_u - grad["bc_vec"][j]) /
                                             abs(grad["bc_vec"][j])}}}


def fp64_bound(res):
    """Second roofline of the FP64-arithmetic form: its DP instructions per
    cell over the bulk kernel time, against DFMA chains timed in this run."""
    import torch
    from lbm_gb300 import _lib
    L = _lib.load()
    nbytes = L.lbm_measure_dfma_scratch_bytes()
    buf = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    peak_dp = ctypes.c_double()
    _lib.call("lbm_measure_dfma_rate", ctypes.byref(peak_dp), ctypes.c_void_p(buf.data_ptr()),
              nbytes, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    rate = FP64_DP_OPS_PER_LU * res["roofline"]["units_per_launch"] / (res["kernel_ms"]["bulk"] * 1e-3)
    return {"bound": "fp64_alu", "dp_instr_per_lu": FP64_DP_OPS_PER_LU,
            "achieved_ginstr_s": rate / 1e9, "peak_ginstr_s": peak_dp.value,
            "peak_source": "DFMA chains timed in this run (lbm_measure_dfma_rate)",
            "frac": rate / 1e9 / peak_dp.value}


# ---------------------------------------------------------------------------
# CPU arm (oracle port, all host threads)
# ---------------------------------------------------------------------------
def _oracle_lattice(app, td):
    """The oracle's lattice with links from the vectorised builder (the cell
    loops take hours at these sizes; the builder is pinned to them by the
    geometry tests)."""
    from lbm_gb300 import geometry
    from oracle import oracle as O

    class _Lat(O.OracleLattice):
        def add_obstacle(self, obstacle):
            return geometry.add_obstacle(self, obstacle.polygon, obstacle.tag, self.IBB)

    return _Lat(app, output_dir=os.path.join(td, ""))


def cpu_reference(ny, seconds):
    """The oracle port on the host cores: the reference loop (run.py:24-54)
    in C with OpenMP cell loops, over a bounded sample of the workload."""
    from oracle import oracle as O
    app = make_app(ny)
    with tempfile.TemporaryDirectory() as td, contextlib.redirect_stdout(io.StringIO()):
        lat = _oracle_lattice(app, td)
        base, vec, scale = app.bc_schedule(lat)
        app.initialize(lat)
        # two untimed iterations (the first touches the work arrays), then a
        # bounded sample sized from the second
        O.run_program(lat, app, 1, (base, vec, scale([0])), initialize=False)
        t0 = time.perf_counter()
        O.run_program(lat, app, 1, (base, vec, scale([1])), initialize=False)
        n = max(2, int(seconds / max(time.perf_counter() - t0, 1e-3)))
        t0 = time.perf_counter()
        O.run_program(lat, app, n, (base, vec, scale(np.arange(2, n + 2))), initialize=False)
        dt = time.perf_counter() - t0
    cells = lat.nx * lat.ny
    return {"value": cells * n / dt / 1e6, "unit": "MLUPS", "cores": O.threads(),
            "kind": "port",
            "sample": "%d iterations of the full %dx%d workload (FP64, C restatement of "
                      "nb.py driven by the run.py loop in C, OpenMP cell loops), %.1f s"
                      % (n, lat.nx, lat.ny, dt)}


def _oracle_channel_series(ny, steps, path, threads):
    """Child process of the plain_vs_oracle check: the cylinder channel on
    the oracle for `steps` iterations; writes the Cd/Cl series (same
    normalisation as run_channel) and the final interior velocity."""
    os.environ["OMP_NUM_THREADS"] = str(threads)
    from oracle import oracle as O
    app = channel_app(ny, steps)
    with tempfile.TemporaryDirectory() as td, contextlib.redirect_stdout(io.StringIO()):
        lat = _oracle_lattice(app, td)
        base, vec, scale = app.bc_schedule(lat)
        t0 = time.perf_counter()
        raw = O.run_program(lat, app, steps, (base, vec, scale(np.arange(steps))))
        dt = time.perf_counter() - t0
    norm = -2.0 / (app.rho_lbm * app.D_lbm * app.u_avg ** 2)
    np.savez(path, cd=raw[:, 0, 0] * norm, cl=raw[:, 0, 1] * norm, u=lat.u[:, 1:-1, 1:-1],
             seconds=dt, threads=O.threads())


def start_oracle_channel(ny, steps, tmp):
    """Start the oracle run of the channel in a spawned process, leaving a
    few host cores to the GPU measurements that run meanwhile."""
    import multiprocessing
    threads = max(1, (os.cpu_count() or 4) - 4)
    path = os.path.join(tmp, "oracle_channel_%d.npz" % steps)
    proc = multiprocessing.get_context("spawn").Process(
        target=_oracle_channel_series, args=(ny, steps, path, threads))
    proc.start()
    return proc, path


def plain_vs_oracle(proc, path, series, steps, ny):
    """Cd/Cl series of the plain forms over the whole channel run against
    the oracle: max deviation over the run relative to the series' maximum
    magnitude, the first iteration where it exceeds 1e-12 of that maximum,
    the relative error of mean Cd and rms Cl over the second half, and the
    final interior velocity field."""
    proc.join()
    if proc.exitcode != 0 or not os.path.exists(path):
        return {"error": "oracle run failed (exit code %s)" % proc.exitcode}
    d = np.load(path)
    out = {"case": "cylinder channel %dx%d, D = %d, Re 100, %d iterations, Cd/Cl of iterations "
                   "0..%d" % (int(5.5 * ny), ny, channel_app(ny, 2).D_lbm, steps, steps - 2),
           "oracle": {"seconds": float(d["seconds"]), "threads": int(d["threads"]),
                      "kind": "C restatement of nb.py driven by the run.py loop (oracle/)"}}
    half = slice((steps - 1) // 2, None)
    for form, r in series.items():
        res = {}
        for k in ("cd", "cl"):
            ref = d[k][:steps - 1]
            got = r[k]
            dev = np.abs(got - ref)
            scale_ = np.max(np.abs(ref))
            over = np.nonzero(dev > 1e-12 * scale_)[0]
            res[k + "_series_max_rel"] = float(dev.max() / scale_)
            res[k + "_first_it_above_1e-12"] = int(over[0]) if len(over) else None
        cd_r, cl_r = d["cd"][:steps - 1][half], d["cl"][:steps - 1][half]
        cd_g, cl_g = r["cd"][half], r["cl"][half]
        res["cd_mean_rel"] = float(abs(cd_g.mean() - cd_r.mean()) / abs(cd_r.mean()))
        rms = lambda x: float(np.sqrt((x ** 2).mean()))
        res["cl_rms_rel"] = abs(rms(cl_g) - rms(cl_r)) / rms(cl_r)
        u_in = r["u"][:, 1:-1, 1:-1]
        res["u_interior_max_rel"] = float(np.max(np.abs(u_in - d["u"])) / np.max(np.abs(d["u"])))
        out[form] = res
    return out


# ---------------------------------------------------------------------------
def replica_totals(ms, e2e_value, world, dist=None, device="cuda"):
    """Whole-job figures of `world` independent replicas (one lattice per
    GPU, no data exchange): the slowest rank's time per iteration, and
    `world` x the slowest rank's end-to-end rate."""
    if dist is None or world == 1:
        return ms, e2e_value * world
    import torch
    t = torch.tensor([ms, -e2e_value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t[0]), -float(t[1]) * world


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    cfg = workload_config(args.ny)
    cfg["parallelism"] = "replicas%d" % world

    if args.impl == "reference":
        if rank != 0:
            return 0
        res = cpu_reference(args.ny, args.cpu_seconds)
        line = {"metric": "MLUPS", "value": res["value"], "unit": "MLUPS", "impl": "reference",
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic", "config": cfg,
                "cpu_baseline": res,
                "e2e": {"value": res["value"], "unit": "MLUPS", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0

    import torch
    import __graft_entry__
    __graft_entry__.build(verbose=False)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local_rank)
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak = 6789.0
    peak_src = "fallback"
    if os.path.exists(peaks_path):
        peak = float(json.load(open(peaks_path))["hbm_gbs"])
        peak_src = "measured"
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if os.path.exists(tpath):
        traffic = json.load(open(tpath))

    tmp = tempfile.mkdtemp(prefix="lbm_bench_")
    sampler = ClockSampler(local_rank)
    sampler.start()
    res, state = measure_form(args.ny, args.precision, args.steps, args.warmup, tmp, peak, dist)
    clocks = sampler.stop()
    app, lat, eng, it = state
    e2e = measure_e2e(app, lat, eng, it, args.e2e_steps)
    del app, lat, eng, state
    torch.cuda.empty_cache()

    ms, e2e["value"] = replica_totals(res["ms_per_step"], e2e["value"], world, dist)
    N = 4 * args.ny * args.ny
    value = N * world / (ms * 1e-3) / 1e6

    forms = {}
    if rank == 0 and args.forms:
        for form in [f for f in args.forms.split(",") if f and f != args.precision]:
            r, st = measure_form(args.ny, form, args.steps, args.warmup, tmp, peak)
            forms[form] = {"mlups": r["mlups"], "ms_per_step": r["ms_per_step"],
                           "roofline_frac": r["roofline"]["frac"],
                           "achieved_gbs": r["roofline"]["achieved"],
                           "kernel_ms": r["kernel_ms"]}
            if form == "f64":
                forms[form]["second_bound"] = fp64_bound(r)
            del st
            torch.cuda.empty_cache()
    ref64 = res["mlups"] if args.precision == "f64" else forms.get("f64", {}).get("mlups")
    if ref64:
        for f in forms.values():
            f["x_vs_f64"] = f["mlups"] / ref64

    # The oracle's run of the channel (plain_vs_oracle) goes on on the host
    # cores while the GPU measurements below run.
    oracle_job = None
    if rank == 0 and world == 1 and args.error_steps > 0 and not args.no_plain_oracle:
        oracle_job = start_oracle_channel(200, args.error_steps, tmp)

    form_errors = plain_series = None
    if rank == 0 and args.error_steps > 0:
        form_errors, plain_series = measure_form_errors(args.error_steps, FORMS, tmp)
        torch.cuda.empty_cache()

    array_errors = None
    if rank == 0 and args.array_errors > 0:
        array_errors = measure_array_errors(args.array_errors, FORMS, tmp, args.ny)
        torch.cuda.empty_cache()

    sweep = None
    if rank == 0 and args.sweep_steps > 0:
        sweep = measure_sweep(args.sweep_steps)
        torch.cuda.empty_cache()

    adjoint = None
    if rank == 0 and args.adjoint_steps > 0:
        adjoint = measure_adjoint(args.adjoint_steps, tmp)
        torch.cuda.empty_cache()

    plain_oracle = None
    if oracle_job is not None:
        plain_oracle = plain_vs_oracle(*oracle_job, plain_series, args.error_steps, 200)

    # The app-API run is host-bound (its hooks' replay of each chunk): it is
    # timed after the oracle child has left the host cores.
    app_api = None
    if rank == 0 and args.app_steps > 0:
        if form_errors and "q60" in form_errors and args.app_steps == args.error_steps:
            eng_mlups = form_errors["q60"]["mlups"]
        else:
            eng_mlups = run_case(channel_app(200, args.app_steps), "q60", args.app_steps,
                                 tmp)["mlups"]
        app_api = measure_app_api(args.app_steps, tmp, eng_mlups)
        torch.cuda.empty_cache()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_reference(args.ny, args.cpu_seconds)

    if sweep and SWEEP_FORM in forms:
        sweep["single_large_mlups"] = forms[SWEEP_FORM]["mlups"]
        sweep["frac_of_single_large"] = sweep["mlups"] / forms[SWEEP_FORM]["mlups"]
    roof = res["roofline"]
    if traffic and traffic.get(args.precision):
        tr = traffic[args.precision]
        roof["traffic"] = tr.get("bytes_per_launch")
        roof["traffic_read"] = tr.get("read_bytes_per_launch")
        roof["traffic_write"] = tr.get("write_bytes_per_launch")
        alg = roof["bytes_per_unit"] * roof["units_per_launch"]
        if roof["traffic_read"]:
            # reads against the algorithmic reads (half the algorithmic bytes)
            roof["read_over_algorithmic_read"] = roof["traffic_read"] / (alg / 2)
        roof["traffic_source"] = tr.get("source")
    roof["peak_source"] = peak_src
    dtype = {"q60": "int64", "f64": "f64", "f32": "f32", "f16s": "f16", "bf16s": "bf16",
             "f16sr": "f16", "bf16sr": "bf16"}
    line = {
        "metric": "MLUPS", "value": value, "unit": "MLUPS", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": dtype[args.precision], "form": args.precision,
        "arithmetic": ARITHMETIC[args.precision],
        "data": "synthetic", "config": cfg,
        "roofline": roof, "second_bound": fp64_bound(res) if args.precision == "f64" else None,
        "kernel_ms": res["kernel_ms"], "e2e": e2e,
        "gpu_launches": args.steps * res["kernels_per_step"],
        "clocks": clocks, "forms": forms, "form_errors": form_errors,
        "plain_vs_oracle": plain_oracle, "app_api": app_api,
        "array_form_errors": array_errors,
        "batched_sweep": sweep, "adjoint": adjoint, "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
