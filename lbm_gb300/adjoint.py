"""Gradient of a time-averaged drag/lift objective by the discrete adjoint.

``DragAdjoint(lattice, app)`` builds the FP64 fused engine of the app (its
set_bc must give every wall a Zou-He operation and apply the four corners).

* ``forward(T, window, weights)``: iterations 0..T-1 plus the boundary pass
  of iteration T-1, with a checkpoint of the post-collision state every
  K = ceil(sqrt(T)) iterations; returns J = sum over the window of
  sum_o (w_fx[o] fx_o + w_fy[o] fy_o), fx/fy the raw drag/lift sums.
* ``gradient()``: sweeps the segments from the last to the first; each
  segment is recomputed from its checkpoint into a K-slot buffer
  (``lbm_adjoint_recompute``, on a second stream, one segment ahead of the
  sweep) and then walked backwards (``lbm_adjoint_sweep``); returns
  dJ/d om_p, dJ/d(BC vector entries) scaled like the BC schedule
  (``bc_vec``: entry k of the packed u_left | u_right | u_top | u_bot |
  rho_right vectors, value(it) = base + scale(it) vec) and dJ/d(base).

Memory: T/K checkpoints + 2 K recomputed states + two adjoint states, i.e.
about 3 sqrt(T) copies of the lattice instead of T.

``DragObjective.apply(om_p, inlet, adjoint, T, window, weights)`` is the same
objective as a ``torch.autograd.Function`` of the TRT rate and the inlet
profile (the first ny entries of the BC vector: the x-velocity of the left
wall per row, scaled by the inlet ramp): forward runs ``forward``, backward
runs ``gradient``.
"""
import ctypes
import math

import numpy as np
import torch

from . import _lib
from .engine import FusedEngine, trace_bc_program


def cd_weights(app, n_obstacles, window_len, obstacle=0):
    """Weights making J the mean drag coefficient of one obstacle over the window:
    Cd = -2 fx / (rho U^2 L) (nb.py:70, U = u_avg, L = D_lbm as in turek.py:142-143)."""
    w = np.zeros(2 * n_obstacles)
    w[obstacle] = -2.0 / (app.rho_lbm * app.u_avg ** 2 * app.D_lbm) / window_len
    return w


class DragAdjoint:
    def __init__(self, lat, app, max_iter=None):
        obstacles, walls, corners = trace_bc_program(app)
        self.lat, self.app = lat, app
        self.eng = FusedEngine(lat, obstacles, walls, corners, precision="f64", drag_cap=4096)
        self.sched = app.bc_schedule(lat)
        if self.sched is None:
            raise ValueError("the adjoint needs an app with a BC schedule (bc_schedule)")
        self.max_iter = max_iter
        self.N = lat.nx * lat.ny
        dev = lat.device
        special = np.zeros(self.N, dtype=np.uint8)
        special[self.eng.t_special.cpu().numpy()] = 1
        self.is_special = torch.from_numpy(special).to(dev)
        self.g0 = lat.device_field("g").clone()  # initial g after app.initialize
        self.nbc = self.eng.bc_base.numel()

    # ------------------------------------------------------------------ helpers
    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def _set_schedule(self, T):
        base, vec, scale = self.sched
        if not hasattr(self, "vec"):
            self.base, self.vec = base.copy(), vec.copy()
        self.scale = scale(np.arange(T + 2))
        self.eng.set_bc_schedule(self.base, self.vec, self.scale, it0=0)

    def set_omega(self, om_p):
        """Change the TRT rate (om_m follows with lambda = 1/4)."""
        tau_p = 1.0 / om_p
        tau_m = 0.25 / (tau_p - 0.5) + 0.5
        self.eng.P.om_p = om_p
        self.eng.P.om_m = 1.0 / tau_m

    def set_bc_vec(self, vec):
        self.vec = np.ascontiguousarray(vec, dtype=np.float64)
        self.eng.bc_vec.copy_(torch.from_numpy(self.vec))

    # ------------------------------------------------------------------ forward
    def forward(self, T, window, weights, checkpoint=True):
        """Run T iterations; returns J (and keeps the checkpoints)."""
        eng = self.eng
        self.T = int(T)
        self.window = (int(window[0]), int(window[1]))
        self.weights = np.ascontiguousarray(weights, dtype=np.float64)
        self._set_schedule(self.T)
        self.lat.device_field("g", True).copy_(self.g0)
        eng.collide_from_g(0, macro=False)
        self.K = max(1, int(math.ceil(math.sqrt(self.T))))
        self.ckpt = {0: eng.f[eng.cur].clone()} if checkpoint else {}
        n_obs = len(eng.obstacles)
        J = 0.0
        n = 1
        while n <= self.T:
            m = min(self.K - (n - 1) % self.K, self.T - n + 1)
            eng.steps(n, m, graph=True)
            last = n + m - 1
            # drag of iterations n-1 .. last-1 (inside the window)
            lo, hi = max(n - 1, self.window[0]), min(last - 1, self.window[1])
            if hi >= lo and n_obs:
                rows = eng.drag_rows(lo, hi)
                J += float(np.sum(rows[:, :, 0] @ self.weights[:n_obs]) +
                           np.sum(rows[:, :, 1] @ self.weights[n_obs:]))
            n = last + 1
            if checkpoint and last % self.K == 0 and last < self.T:
                self.ckpt[last] = eng.f[eng.cur].clone()
        eng.check_status()
        self.J = J
        return J

    # ----------------------------------------------------------------- backward
    def gradient(self):
        eng, dev, N = self.eng, self.lat.device, self.N
        L = _lib.load()
        n_obs = max(1, len(eng.obstacles))
        slots = int(L.lbm_adjoint_omega_slots(ctypes.byref(eng.P)))
        w = torch.from_numpy(np.concatenate([self.weights,
                                             np.zeros(max(0, 2 * n_obs - self.weights.size))]))
        w = w.to(dev)
        bufs = {
            "adj_pulled": torch.zeros(9 * N, dtype=torch.float64, device=dev),
            "link_adj": torch.zeros(max(1, 3 * eng.n_links), dtype=torch.float64, device=dev),
            "corner_seed": torch.zeros(16, dtype=torch.float64, device=dev),
            "grad_bc_base": torch.zeros(self.nbc, dtype=torch.float64, device=dev),
            "grad_bc_vec": torch.zeros(self.nbc, dtype=torch.float64, device=dev),
            "grad_omega": torch.zeros(slots, dtype=torch.float64, device=dev),
        }
        A = _lib.Adjoint()
        A.obj_it_first, A.obj_it_last = self.window
        A.obj_w = w.data_ptr()
        A.is_special = self.is_special.data_ptr()
        for k, t in bufs.items():
            setattr(A, k, t.data_ptr())
        A.grad_omega_len = slots
        lam = [torch.zeros(9 * N, dtype=torch.float64, device=dev) for _ in range(2)]
        cur = 0  # lam[cur] = lambda(n)
        # Two segment buffers: the segment before the one being swept back is
        # recomputed meanwhile on a second stream (the sweep's kernels are
        # latency-bound and leave the GPU room).
        seg_bufs = [torch.empty((self.K, 9 * N), dtype=torch.float64, device=dev)
                    for _ in range(2)]
        starts = sorted(self.ckpt)
        main = torch.cuda.current_stream()
        side = torch.cuda.Stream()
        ready = [torch.cuda.Event(), torch.cuda.Event()]
        free = [torch.cuda.Event(), torch.cuda.Event()]

        def recompute(k, b):
            s0 = starts[k]
            s1 = min(s0 + self.K, self.T)
            side.wait_event(free[b])
            with torch.cuda.stream(side):
                seg_bufs[b][0].copy_(self.ckpt[s0].reshape(-1))
                _lib.call("lbm_adjoint_recompute", ctypes.byref(eng.P), s0, s1 - s0,
                          ctypes.c_void_p(seg_bufs[b].data_ptr()), 9 * N,
                          ctypes.c_void_p(side.cuda_stream))
            ready[b].record(side)

        for b in range(2):
            free[b].record(main)
        order = list(range(len(starts)))[::-1]
        recompute(order[0], 0)
        for n, k in enumerate(order):
            b = n & 1
            if n + 1 < len(order):
                recompute(order[n + 1], b ^ 1)
            s0 = starts[k]
            s1 = min(s0 + self.K, self.T)
            main.wait_event(ready[b])
            # walk back s1 .. s0 + 1 over x(s0) .. x(s1 - 1)
            _lib.call("lbm_adjoint_sweep", ctypes.byref(eng.P), ctypes.byref(A), s0, s1 - s0,
                      ctypes.c_void_p(seg_bufs[b].data_ptr()), 9 * N,
                      ctypes.c_void_p(lam[0].data_ptr()), ctypes.c_void_p(lam[1].data_ptr()),
                      cur, ctypes.c_void_p(main.cuda_stream))
            free[b].record(main)
            cur ^= (s1 - s0) & 1
        st = self._stream()
        # the first collision x(0) = collide(g0)
        _lib.call("lbm_adjoint_initial", ctypes.byref(eng.P), ctypes.byref(A),
                  ctypes.c_void_p(self.g0.data_ptr()), ctypes.c_void_p(lam[cur].data_ptr()),
                  ctypes.c_void_p(lam[cur ^ 1].data_ptr()), st)
        torch.cuda.synchronize()
        g_om = float(np.sum(bufs["grad_omega"].cpu().numpy()))
        return {"omega": g_om, "bc_vec": bufs["grad_bc_vec"].cpu().numpy(),
                "bc_base": bufs["grad_bc_base"].cpu().numpy(),
                "g0": lam[cur ^ 1].cpu().numpy().reshape(9, self.lat.nx, self.lat.ny)}


class DragObjective(torch.autograd.Function):
    """J(om_p, inlet) of a ``DragAdjoint`` as a differentiable torch op.

    om_p: 0-d float64 tensor, the TRT rate om+ (om- follows, lambda = 1/4);
    inlet: float64 tensor of ny entries, the inlet x-velocity profile (first
    ny entries of the packed BC vector); T, window, weights as in
    ``DragAdjoint.forward``.  Returns J as a 0-d float64 tensor on the
    device of om_p; backward gives dJ/d om_p and dJ/d inlet from the
    discrete adjoint (one adjoint sweep per backward)."""

    @staticmethod
    def forward(ctx, om_p, inlet, adjoint, T, window, weights):
        ny = adjoint.lat.ny
        prof = inlet.detach().to("cpu", torch.float64).numpy().reshape(-1)
        if prof.size != ny:
            raise ValueError("inlet profile has %d entries, the lattice has ny = %d"
                             % (prof.size, ny))
        if not hasattr(adjoint, "vec"):
            base, vec, _ = adjoint.sched
            adjoint.base, adjoint.vec = base.copy(), vec.copy()
        vec = adjoint.vec.copy()
        vec[:ny] = prof
        adjoint.vec = vec
        adjoint.set_omega(float(om_p))
        J = adjoint.forward(T, window, weights)
        ctx.adjoint = adjoint
        ctx.devices = (om_p.device, inlet.device)
        return torch.tensor(J, dtype=torch.float64, device=om_p.device)

    @staticmethod
    def backward(ctx, grad_J):
        g = ctx.adjoint.gradient()
        ny = ctx.adjoint.lat.ny
        s = float(grad_J)
        g_om = torch.tensor(s * g["omega"], dtype=torch.float64, device=ctx.devices[0])
        g_in = torch.from_numpy(s * g["bc_vec"][:ny]).to(ctx.devices[1])
        return g_om, g_in, None, None, None, None
