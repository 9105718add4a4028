"""Batched sweep: many independent lattices advanced by one set of kernels.

* ``sweep_apps(seed)``  the 256-case sweep: 128 lid-driven cavities with
  n ~ U{64..512} and Re ~ U[100, 1000], 128 channels with ny ~ U{64..256},
  nx = 4 ny, 1-6 random squares of side U[0.05, 0.15] ny and Re ~ U[100, 2000]
  (on the channel height), all seeded from one generator.
* ``Batch``  builds one lattice and one fused engine per app (same code as a
  single run), gathers their C-ABI descriptions into an ``lbm_batch`` and
  advances all of them with ``lbm_batch_advance_graph``: per iteration one
  persistent bulk kernel over a tile work queue of every lattice, one
  persistent special-cell kernel and one drag kernel.
* ``autotune(batch)``  picks the scheduling (persistent work queue or one
  block per tile), the vector width of the bulk kernel (cells per thread),
  block-widths per bulk tile,
  threads per block, persistent grid size, the number of iterations per
  CUDA graph and the number of concurrent groups by timing candidates on
  the batch.

With ``streams`` = n > 1 the lattices are split into n groups of about the
same number of cells, each its own ``lbm_batch`` advanced on its own CUDA
stream: the groups are independent, so the latency-bound special-cell
phase of one group runs beside the bandwidth-bound bulk phase of another.
"""
import contextlib
import ctypes
import io
import itertools
import math
import tempfile

import numpy as np
import torch

from . import _lib
from .apps import cavity
from .apps.channel import _channel
from .engine import FusedEngine, trace_bc_program
from .lattice import lattice
from .obstacle import obstacle


def samples_per_side(side, dx):
    """n_spts of generate_shape that spaces the samples of a square's side
    (ceil(n_spts sqrt(side)) points, shapes.py:104) below 0.4 dx."""
    return max(4, math.ceil(side / (0.4 * dx) / math.sqrt(side)))


class channel_squares(_channel):
    """Channel of height ny, length 4 ny, with square obstacles (cell units).

    Re is defined on the channel height with the mean inlet velocity.
    """

    def __init__(self, ny, squares, Re, u_lbm=0.1, name="channel"):
        self.name = name
        self.Re_lbm = Re
        self.L_lbm = ny
        self.u_lbm = u_lbm
        self.rho_lbm = 1.0
        self.t_max = 1.0
        self.x_min, self.x_max = 0.0, 4.0
        self.y_min, self.y_max = 0.0, 1.0
        self.IBB = True
        self.stop = "it"
        self.obs_cv_ct, self.obs_cv_nb = 1.0e-3, 1000
        self.output_freq = 10 ** 12
        self.output_it = 0
        self.dpi = 100
        self.compute_lbm_parameters()
        self.obstacles = []
        for k, (x, y, side) in enumerate(squares):
            # The IBB distance is measured to the nearest polygon sample
            # (lattice.py:350-361): sample each side finer than half a cell.
            n_spts = samples_per_side(side * self.dx, self.dx)
            self.obstacles.append(obstacle("%s_sq%d" % (name, k), 4, n_spts, "square",
                                           side * self.dx, [x * self.dx, y * self.dx]))

    def compute_lbm_parameters(self):
        self._derive(self.L_lbm)


def sweep_apps(seed=2024, n_cavity=128, n_channel=128):
    """The seeded sweep of uneven cases (cavities then channels)."""
    rng = np.random.default_rng(seed)
    apps = []
    for k in range(n_cavity):
        a = cavity()
        a.name = "cavity%d" % k
        a.L_lbm = int(rng.integers(64, 513))
        a.Re_lbm = float(rng.uniform(100.0, 1000.0))
        a.u_lbm = 0.1
        a.compute_lbm_parameters()
        a.output_freq = 10 ** 12
        apps.append(a)
    for k in range(n_channel):
        ny = int(rng.integers(64, 257))
        nx = 4 * ny
        n_sq = int(rng.integers(1, 7))
        squares = []
        tries = 0
        while len(squares) < n_sq and tries < 1000:
            tries += 1
            side = float(rng.uniform(0.05, 0.15)) * ny
            half = 0.5 * side + 4.0
            x = float(rng.uniform(0.1 * nx + half, 0.8 * nx - half))
            y = float(rng.uniform(half, ny - half))
            if all(abs(x - x2) > 0.5 * (side + s2) + 6 or abs(y - y2) > 0.5 * (side + s2) + 6
                   for (x2, y2, s2) in squares):
                squares.append((x, y, side))
        re = float(rng.uniform(100.0, 2000.0))
        # At u_lbm = 0.1 channels with tau near 0.51 diverge within 10,000
        # iterations even in FP64 (measured: tau 0.5086 at ~6,000, several at
        # tau 0.515 between 9,500 and 10,000), so Re is clipped to keep
        # tau >= 0.53 (Re <= 6.7 ny).
        re = min(re, re_max_stable(ny, 0.1))
        apps.append(channel_squares(ny, squares, re, name="channel%d" % k))
    return apps


def re_max_stable(ny, u_lbm, tau_min=0.53):
    """Largest Re (on the channel height, mean inlet velocity) with tau >= tau_min."""
    nu_min = (tau_min - 0.5) / 3.0
    return (2.0 * u_lbm / 3.0) * ny / nu_min


class Batch:
    """One fused engine per app, advanced together through lbm_batch."""

    def __init__(self, apps, precision="f16sr", config=None, max_steps=20000, verbose=False):
        self.apps = list(apps)
        self.precision = precision
        self.lattices, self.engines = [], []
        self.tmp = tempfile.mkdtemp(prefix="lbm_batch_")
        for a in self.apps:
            with contextlib.redirect_stdout(io.StringIO()):
                lat = lattice(a, precision=precision, output_dir=self.tmp, verbose=False)
                lat.generate_image = lambda obstacles: None
                a.initialize(lat)
            obstacles, walls, corners = trace_bc_program(a)
            eng = FusedEngine(lat, obstacles, walls, corners, precision=precision, drag_cap=64)
            sched = a.bc_schedule(lat)
            if sched is not None:
                base, vec, scale = sched
                eng.set_bc_schedule(base, vec, scale(np.arange(max_steps + 2)), it0=0)
            eng.collide_from_g(0, macro=False)
            self.lattices.append(lat)
            self.engines.append(eng)
        self.cells = sum(e.N for e in self.engines)
        self.it = 1          # next iteration to collide
        self.parity = 0      # every engine's f[0] holds g_up(0) after collide_from_g
        self.handles = []
        self.streams = []
        self.config = None
        self.set_config(config or default_config())

    @property
    def handle(self):
        """The lbm_batch of the first group (the only one with streams = 1)."""
        return self.handles[0] if self.handles else None

    def groups(self, n):
        """Engine indices split into n groups of about the same number of
        cells (largest lattice to the group with the fewest cells so far)."""
        order = sorted(range(len(self.engines)), key=lambda i: -self.engines[i].N)
        groups, cells = [[] for _ in range(n)], [0] * n
        for i in order:
            g = cells.index(min(cells))
            groups[g].append(i)
            cells[g] += self.engines[i].N
        return [sorted(g) for g in groups if g]

    def _destroy(self):
        for h in self.handles:
            _lib.call("lbm_batch_destroy", h)
        self.handles = []

    def set_config(self, cfg):
        self._destroy()
        self.config = dict(cfg)
        n = int(cfg.get("streams", 1))
        if n < 1:
            raise ValueError("streams must be at least 1")
        c = _lib.BatchConfig(cfg["bulk_threads"], cfg["bulk_blocks_per_sm"],
                             cfg["special_blocks_per_sm"], cfg["scalar_tile_cells"],
                             int(cfg.get("persistent", 1)), int(cfg.get("vec_bytes", 16)),
                             int(cfg.get("tile_rounds", 1)), int(cfg.get("bulk_tma", 0)))
        for g in self.groups(n):
            arr = (_lib.Problem * len(g))(*[self.engines[i].P for i in g])
            h = ctypes.c_void_p()
            _lib.call("lbm_batch_create", ctypes.byref(h), arr, len(g), ctypes.byref(c))
            self.handles.append(h)
        self.streams = [torch.cuda.Stream() for _ in self.handles] if len(self.handles) > 1 else []

    def info(self):
        tot = {"lattices": 0, "bulk_tiles": 0, "special_tiles": 0, "drag_items": 0}
        out = (ctypes.c_int64 * 6)()
        for h in self.handles:
            _lib.call("lbm_batch_info", h, out)
            for k, v in zip(("lattices", "bulk_tiles", "special_tiles", "drag_items"), out[:4]):
                tot[k] += v
        tot.update(sms=out[4], kernels_per_step=out[5], groups=len(self.handles))
        return tot

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def advance(self, n_steps, graph=True, k=None):
        """Advance every lattice by n_steps iterations, k per graph launch
        (with several groups: each group's launches on its own stream, all
        joined into the current stream at the end)."""
        k = k or self.config.get("k_steps", 50)
        fn = "lbm_batch_advance_graph" if graph else "lbm_batch_advance"
        cur = torch.cuda.current_stream()
        for s in self.streams:
            s.wait_stream(cur)
        done = 0
        while done < n_steps:
            n = min(k, n_steps - done)
            if self.streams:
                for h, s in zip(self.handles, self.streams):
                    _lib.call(fn, h, self.it, n, self.parity, ctypes.c_void_p(s.cuda_stream))
            else:
                _lib.call(fn, self.handles[0], self.it, n, self.parity, self._stream())
            self.it += n
            self.parity ^= (n & 1)
            done += n
        for s in self.streams:
            cur.wait_stream(s)
        for e in self.engines:
            e.cur = self.parity

    def check(self):
        for e in self.engines:
            e.check_status()

    def close(self):
        self._destroy()


# storage forms with a TMA-staged bulk kernel (lbm_batch_config.bulk_tma)
TMA_FORMS = ("f16s", "f16sr", "bf16s", "bf16sr")


def default_config():
    return {"bulk_threads": 128, "bulk_blocks_per_sm": 8, "special_blocks_per_sm": 8,
            "scalar_tile_cells": 2048, "k_steps": 50, "persistent": 0, "vec_bytes": 8,
            "tile_rounds": 4, "bulk_tma": 0, "streams": 1}


def time_batch(batch, n_steps, k=None):
    """Device time (ms) of n_steps batched iterations."""
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    batch.advance(n_steps, graph=True, k=k)
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def autotune(batch, steps=60, space=None, k_space=(10, 25, 50, 100, 200),
             stream_space=(2, 3), verbose=False):
    """Pick the fastest batch configuration by timing candidates.

    Every candidate runs ``steps`` iterations after one warm-up launch (which
    also captures its graph); the lattices keep advancing, which does not
    change the cost per iteration.  A second stage times the winner with
    each number of iterations per CUDA graph in ``k_space`` (over the same
    iteration count for every K), a third with the lattices split into each
    number of concurrent groups in ``stream_space``.  Returns (best config,
    table of trials); the trials of the second and third stages carry
    ``_stage`` 2 and 3.  The lattices are put back in the state they had
    before the trials (the sweep's channels at tau = 0.53 go unstable after
    ~17,000 iterations, so the trials must not age them).
    """
    snaps = [e.snapshot() for e in batch.engines]
    it0, parity0 = batch.it, batch.parity
    # one block per tile (the persistent grid size does not apply), then
    # persistent blocks, then (16-bit forms) the TMA-staged bulk kernel with
    # either schedule of the special cells; a dict of value lists or a list
    # of such dicts
    if space is None:
        space = [
            {"persistent": [0], "tile_rounds": [2, 4, 8], "vec_bytes": [16, 8],
             "bulk_threads": [64, 128], "k_steps": [50]},
            {"persistent": [1], "tile_rounds": [4, 8], "vec_bytes": [16, 8],
             "bulk_threads": [128], "bulk_blocks_per_sm": [8, 12], "k_steps": [50]},
        ]
        if batch.precision in TMA_FORMS:
            space.append({"bulk_tma": [1, 2], "persistent": [0, 1], "k_steps": [50]})
    spaces = [space] if isinstance(space, dict) else list(space)
    candidates = []
    for sp in spaces:
        keys = list(sp)
        for values in itertools.product(*(sp[k] for k in keys)):
            candidates.append(dict(zip(keys, values)))
    trials = []
    best = None
    for values in candidates:
        cfg = default_config()
        cfg.update(values)
        batch.set_config(cfg)
        k = cfg["k_steps"]
        batch.advance(k, k=k)  # warm-up + graph capture
        n = max(k, (steps // k) * k)
        ms = time_batch(batch, n, k=k)
        mlups = batch.cells * n / (ms * 1e-3) / 1e6
        trials.append((dict(cfg), mlups))
        if verbose:
            print(cfg, "%.0f MLUPS" % mlups)
        if best is None or mlups > best[1]:
            best = (dict(cfg), mlups)
    if k_space:
        n = max(k_space) * max(1, -(-steps // max(k_space)))
        stage1 = best
        best = None
        for k in k_space:
            cfg = dict(stage1[0], k_steps=k)
            batch.set_config(cfg)
            batch.advance(k, k=k)  # warm-up + graph capture
            ms = time_batch(batch, n, k=k)
            mlups = batch.cells * n / (ms * 1e-3) / 1e6
            trials.append((dict(cfg, _stage=2), mlups))
            if verbose:
                print(cfg, "%.0f MLUPS" % mlups)
            if best is None or mlups > best[1]:
                best = (dict(cfg), mlups)
    if stream_space:
        k = best[0]["k_steps"]
        n = k * max(1, -(-steps // k))
        # the winner, and for the 16-bit forms the TMA-staged bulk phase in
        # both its shapes (the half-width one leaves room on each SM for the
        # other groups' kernels; alone on the GPU it may lose to the winner)
        bases = [dict(best[0])]
        if batch.precision in TMA_FORMS:
            for tma in (1, 2):
                if best[0].get("bulk_tma", 0) != tma:
                    bases.append(dict(best[0], bulk_tma=tma))
        for g, base in itertools.product(stream_space, bases):
            cfg = dict(base, streams=g)
            batch.set_config(cfg)
            batch.advance(k, k=k)  # warm-up + graph capture
            ms = time_batch(batch, n, k=k)
            mlups = batch.cells * n / (ms * 1e-3) / 1e6
            trials.append((dict(cfg, _stage=3), mlups))
            if verbose:
                print(cfg, "%.0f MLUPS" % mlups)
            if mlups > best[1]:
                best = (dict(cfg), mlups)
    batch.set_config(best[0])
    torch.cuda.synchronize()
    for e, snap in zip(batch.engines, snaps):
        e.restore(snap)
    batch.it, batch.parity = it0, parity0
    torch.cuda.synchronize()
    return best[0], trials


def serial_loop_mlups(batch, steps=40, graph=False):
    """Aggregate MLUPS of advancing the same lattices one after another.

    Each lattice runs ``steps`` iterations with its own fused engine and its
    own kernel launches (three per iteration), the way a one-case-at-a-time
    code would drive them.
    """
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    it0 = batch.it
    for e in batch.engines:  # warm-up (graph capture)
        e.cur = batch.parity
        e.steps(it0, steps, graph=graph)
    torch.cuda.synchronize()
    e0.record()
    for e in batch.engines:
        e.steps(it0 + steps, steps, graph=graph)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    # the engines moved 2*steps iterations ahead of the batch: keep them in step
    batch.it = it0 + 2 * steps
    batch.parity = batch.engines[0].cur
    return batch.cells * steps / (ms * 1e-3) / 1e6, ms
