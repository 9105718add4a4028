"""Driver loop (lbm/src/core/run.py:12-61) with the fused GPU engine.

``run(lattice, app)`` keeps the reference contract: ``app.initialize``, then
per iteration ``printings, set_inlets, macro, outputs, equilibrium,
collision_stream, set_bc, observables, check_stop``, then ``app.finalize``.

When the app's ``set_bc`` is a sequence the fused kernels implement
(obstacle links, then Zou-He walls, then corners), iterations run in chunks
on the device (``engine.FusedEngine``), captured as CUDA graphs; the host
hooks are replayed in order after each chunk:

* ``set_inlets``  evaluated on the device from ``app.bc_schedule`` when the
  app provides it, else called on the host before every step;
* ``outputs``     chunks end at multiples of ``app.output_freq``, where the
  step writes macro rho/u, so the hook sees the reference fields;
* ``observables`` ``lattice.drag_lift`` returns the drag/lift the device
  computed for that iteration; apps with ``observables_chunk`` (turek) take
  a whole chunk at once (moving averages on the device, lines written by a
  writer thread) instead of one Python call per iteration;
* ``check_stop``  when it stops inside a chunk, the chunk is re-run from a
  snapshot up to the stop iteration.

At the end the lattice holds what the reference holds: g after the last
set_bc, g_up and g_eq of the last iteration, rho/u from its macro with the
wall rows set by the Zou-He operations.
"""
import time

import numpy as np
import torch

from . import _lib
from .engine import FusedEngine, Unfusable, pack_bc, trace_bc_program


def _host_bc(lattice):
    return pack_bc({k: getattr(lattice, k) for k in
                    ("u_left", "u_right", "u_top", "u_bot", "rho_right")}, lattice.nx, lattice.ny)


def run_methods(lattice, app, n_iter=None):
    """The reference loop, one lattice method (one kernel) at a time."""
    it = 0
    compute = True
    while compute:
        app.printings(it)
        app.set_inlets(lattice, it)
        lattice.macro()
        app.outputs(lattice, it)
        lattice.equilibrium()
        lattice.collision_stream()
        app.set_bc(lattice)
        app.observables(lattice, it)
        compute = app.check_stop(it)
        if n_iter is not None and it + 1 >= n_iter:
            compute = False
        it += 1
    return it


class _Replay:
    """lattice.drag_lift during replay: values the device computed."""

    def __init__(self, obstacles):
        self.index = {id(o): k for k, o in enumerate(obstacles)}
        self.rows = {}
        self.it = None

    def __call__(self, obs):
        k = self.index.get(id(obs))
        if k is None:
            raise Unfusable("drag_lift on an obstacle without bounce-back in set_bc")
        row = self.rows[self.it]
        return float(row[k, 0]), float(row[k, 1])


def run_fused(lattice, app, chunk=1000, graph=True, n_iter=None, verbose=True):
    """Fused-engine loop; returns the number of iterations run."""
    obstacles, walls, corners = trace_bc_program(app)
    # Apps that take a chunk of observables at once (observables_chunk) skip
    # the per-iteration replay: their outputs act only at multiples of
    # output_freq, and the hook evaluates check_stop itself.  With a known
    # final iteration their chunks are replayed while the next chunk runs
    # (the drag ring then holds two chunks).
    chunk_obs = getattr(app, "observables_chunk", None)
    known = getattr(app, "stop", None) == "it" and hasattr(app, "it_max")
    overlap = chunk_obs is not None and (known or n_iter is not None)
    eng = FusedEngine(lattice, obstacles, walls, corners,
                      drag_cap=(2 * chunk if overlap else chunk) + 8)
    sched = app.bc_schedule(lattice) if hasattr(app, "bc_schedule") else None
    out_freq = getattr(app, "output_freq", None) or None
    known_stop = None
    if getattr(app, "stop", None) == "it" and hasattr(app, "it_max"):
        known_stop = int(app.it_max)
    if n_iter is not None:
        known_stop = n_iter - 1 if known_stop is None else min(known_stop, n_iter - 1)

    state = {"scale_len": 0, "outputs_done": -1}

    def ensure_scale(upto):
        if sched is None or upto < state["scale_len"]:
            return
        base, vec, scale = sched
        new_len = max(upto + 1, 2 * state["scale_len"], 1024)
        if known_stop is not None:
            new_len = max(upto + 1, min(new_len, known_stop + 2))
        eng.set_bc_schedule(base, vec, scale(np.arange(new_len)), it0=0)
        state["scale_len"] = new_len

    def is_output(m):
        return bool(out_freq) and m % out_freq == 0

    def steps(first, last_it, macro_last, use_graph):
        """Collisions of iterations first..last_it."""
        if sched is None:
            for m in range(first, last_it + 1):
                app.set_inlets(lattice, m - 1)
                eng.set_bc_constant(_host_bc(lattice))
                eng.steps(m, 1, macro_last=macro_last and m == last_it, graph=False)
        else:
            ensure_scale(last_it + 1)
            eng.steps(first, last_it - first + 1, macro_last=macro_last, graph=use_graph)

    replay = _Replay(obstacles)

    def replay_chunk(first, last_avail, honour_stop, rows=None):
        if rows is None:
            rows = eng.drag_rows(first, last_avail)
        if out_freq:
            m = max(first, state["outputs_done"] + 1)
            m = -(-m // out_freq) * out_freq
            while m <= last_avail:
                app.outputs(lattice, m)
                state["outputs_done"] = m
                m += out_freq
        stop = chunk_obs(lattice, first, rows, obstacles, stop_check=honour_stop)
        if honour_stop and stop is None and n_iter is not None and first <= n_iter - 1 <= last_avail:
            stop = n_iter - 1
        return stop

    def replay_hooks(first, last_avail, honour_stop=True):
        """outputs/observables/check_stop of first..last_avail; stop iteration or None."""
        if last_avail < first:
            return None
        if chunk_obs is not None:
            return replay_chunk(first, last_avail, honour_stop)
        rows = eng.drag_rows(first, last_avail)
        lattice._replay = replay
        try:
            for k, m in enumerate(range(first, last_avail + 1)):
                if m > state["outputs_done"]:
                    app.outputs(lattice, m)
                    state["outputs_done"] = m
                replay.rows[m] = rows[k]
                replay.it = m
                app.observables(lattice, m)
                del replay.rows[m]
                go_on = app.check_stop(m)
                if n_iter is not None and m + 1 >= n_iter:
                    go_on = False
                if honour_stop and not go_on:
                    return m
        finally:
            lattice._replay = None
        return None

    # Iteration 0: macro (for outputs(0)), equilibrium, collision of g(0).
    app.printings(0)
    if sched is None:
        app.set_inlets(lattice, 0)
    eng.collide_from_g(0, macro=True)
    app.outputs(lattice, 0)
    state["outputs_done"] = 0
    last = 0      # last collided iteration: f[cur] = g_up(last)
    pending = 0   # first iteration whose observables/check_stop are pending
    if overlap:
        # chunk k + 1 is enqueued before chunk k's observables are replayed
        # (on a side stream that waits only for chunk k)
        side = torch.cuda.Stream()
        queued = None  # (first, last iteration, event after its step)

        def replay_queued(q):
            rows = eng.drag_rows_after(q[0], q[1], q[2], side)
            with torch.cuda.stream(side):
                stop = replay_chunk(q[0], q[1], True, rows)
            if stop is not None:
                raise RuntimeError("check_stop stopped before the known final iteration")

        while last < known_stop:
            e = min(last + chunk, known_stop)
            if out_freq:
                e = min(e, (last // out_freq + 1) * out_freq)
            steps(last + 1, e, macro_last=is_output(e) or e == known_stop, use_graph=graph)
            ev = torch.cuda.Event()
            ev.record()
            if queued is not None:
                replay_queued(queued)
            queued = (pending, e - 1, ev)
            if is_output(e):
                ev.synchronize()
                app.outputs(lattice, e)
                state["outputs_done"] = e
            pending = e
            last = e
            if verbose:
                app.printings(e)
        if queued is not None:
            replay_queued(queued)
        torch.cuda.synchronize()
    while not overlap and (known_stop is None or last < known_stop):
        e = last + chunk
        if out_freq:
            e = min(e, (last // out_freq + 1) * out_freq)
        if known_stop is not None:
            e = min(e, known_stop)
        snap = eng.snapshot() if known_stop is None else None
        first = last + 1
        steps(first, e, macro_last=is_output(e) or e == known_stop, use_graph=graph)
        torch.cuda.synchronize()  # waits without the GIL (the apps' writer threads run)
        eng.check_status()
        stop = replay_hooks(pending, e - 1)
        if stop is not None:
            # check_stop ended the run inside this chunk: redo it up to `stop`.
            if snap is None:
                raise RuntimeError("check_stop stopped before the known final iteration")
            eng.restore(snap)
            steps(first, stop, macro_last=True, use_graph=False)
            last = stop
            pending = stop + 1
            break
        if is_output(e):
            app.outputs(lattice, e)
            state["outputs_done"] = e
        pending = e
        last = e
        if verbose:
            app.printings(e)

    # Final state of iteration `last`: BCs, drag, g(last+1).
    if sched is None:
        app.set_inlets(lattice, last)
        eng.set_bc_constant(_host_bc(lattice))
    else:
        ensure_scale(last + 1)
    _finalize_state(lattice, eng, last)
    replay_hooks(pending, last, honour_stop=False)
    if chunk_obs is not None and known_stop is not None and last == known_stop:
        app.check_stop(last)  # the per-iteration replay's last call (its message)
    if sched is not None:
        app.set_inlets(lattice, last)
    lattice._engine = eng
    return last + 1


def _finalize_state(lattice, eng, stop_at):
    """g(stop_at+1), g_up(stop_at), g_eq and rho/u of the reference end state."""
    # rho/u of macro(g(stop_at)) are in the lattice when the last collision
    # ran with MACRO_LAST; recompute them otherwise from a collide-free pass.
    m = lattice._m
    stream = torch.cuda.current_stream()
    eng.g_up_into(m["g_up"].device(True))
    m["g_up"].written()
    # g_eq of iteration stop_at from its macro (before the wall rows change).
    _lib.call("lbm_equilibrium_f64", m["u"].dev.data_ptr(), m["rho"].dev.data_ptr(),
              m["g_eq"].device(True).data_ptr(), lattice.nx, lattice.ny,
              stream.cuda_stream)
    m["g_eq"].written()
    eng.finish(stop_at + 1, wall_macro=True)
    eng.check_status()


def run(lattice, app, fused=None, chunk=1000, graph=True, n_iter=None):
    """Reference driver contract; fused GPU engine when the app allows it.

    fused=None: use the fused engine if the app's set_bc can be fused, else
    the per-method kernels; True: require it; False: per-method kernels.
    n_iter: stop after that many iterations even if check_stop continues.
    """
    app.initialize(lattice)
    start = time.time()
    print("### Solving")
    ran = None
    if fused is not False:
        try:
            trace_bc_program(app)
            ok = True
        except Unfusable as ex:
            if fused:
                raise
            ok = False
            print("# fused engine not used: %s" % ex)
        if ok:
            ran = run_fused(lattice, app, chunk=chunk, graph=graph, n_iter=n_iter)
    if ran is None:
        ran = run_methods(lattice, app, n_iter=n_iter)
    torch.cuda.synchronize()
    end = time.time()
    print("# Loop time = {:f}".format(end - start))
    app.finalize(lattice)
    return ran
