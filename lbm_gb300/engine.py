"""Fused engine: the per-iteration lattice update as two or three kernels.

``FusedEngine`` owns the device state of one lattice run: two ping-pong
buffers of post-collision populations in the storage form (``f64``, ``q60``,
``f32``, ``f16s``, ``bf16s``, ``f16sr``, ``bf16sr``), the special-cell and link tables, the scratch that the
kernels carry from one iteration to the next, the per-iteration drag/lift
history and the BC schedule.  It drives ``lbm_advance`` /
``lbm_advance_graph`` of liblbm_gb300 (include/lbm_gb300.h).  The 16-bit
forms step through the TMA-staged bulk kernel; ``bulk_kernel = "registers"``
selects the register-pipelined one (``LBM_FLAG_BULK_REGISTERS``, same bits).

Iteration numbering follows lbm/src/core/run.py: iteration ``it`` computes
macro, equilibrium and collision of g(it); its boundary conditions and its
drag/lift are applied/computed by the step of iteration it + 1 (or by
``finish``), which is how the pull scheme orders the work.
"""
import ctypes

import numpy as np
import torch

from . import _lib

_CX = np.array([0, 1, -1, 0, 0, 1, -1, -1, 1])
_CY = np.array([0, 0, 0, 1, -1, 1, -1, 1, -1])
_NS = np.array([0, 2, 1, 4, 3, 6, 5, 8, 7])

_STORE_DTYPE = {
    "f64": torch.float64,
    "f32": torch.float32,
    "f16s": torch.float16,
    "bf16s": torch.bfloat16,
    "q60": torch.int64,
    "f16sr": torch.float16,
    "bf16sr": torch.bfloat16,
}

WALL_OPS = {
    "zou_he_left_wall_velocity": _lib.WALL_LEFT_VELOCITY,
    "zou_he_right_wall_velocity": _lib.WALL_RIGHT_VELOCITY,
    "zou_he_right_wall_pressure": _lib.WALL_RIGHT_PRESSURE,
    "zou_he_top_wall_velocity": _lib.WALL_TOP_VELOCITY,
    "zou_he_bottom_wall_velocity": _lib.WALL_BOTTOM_VELOCITY,
}
CORNER_OPS = {
    "zou_he_bottom_left_corner": _lib.CORNER_BOTTOM_LEFT,
    "zou_he_top_left_corner": _lib.CORNER_TOP_LEFT,
    "zou_he_top_right_corner": _lib.CORNER_TOP_RIGHT,
    "zou_he_bottom_right_corner": _lib.CORNER_BOTTOM_RIGHT,
}


class Unfusable(Exception):
    """The app's boundary sequence is outside what the fused kernels do."""


class BCRecorder:
    """Stand-in lattice that records the calls an app's ``set_bc`` makes."""

    def __init__(self):
        self.ops = []

    def bounce_back_obstacle(self, obs):
        self.ops.append(("bb", obs))

    def __getattr__(self, name):
        if name in WALL_OPS:
            return lambda: self.ops.append(("wall", WALL_OPS[name]))
        if name in CORNER_OPS:
            return lambda: self.ops.append(("corner", CORNER_OPS[name]))
        raise Unfusable("set_bc uses lattice.%s" % name)


def trace_bc_program(app):
    """(obstacles, wall ops, corner ops) of app.set_bc, in call order.

    The fused kernels apply obstacle links first, then walls, then corners;
    any other interleaving raises Unfusable.
    """
    rec = BCRecorder()
    app.set_bc(rec)
    phase = 0
    obstacles, walls, corners = [], [], []
    for kind, arg in rec.ops:
        if kind == "bb":
            if phase > 0:
                raise Unfusable("bounce-back after a wall or corner operation")
            obstacles.append(arg)
        elif kind == "wall":
            if phase > 1:
                raise Unfusable("wall operation after a corner operation")
            phase = 1
            walls.append(arg)
        else:
            phase = 2
            if arg not in corners:
                corners.append(arg)
    if len(walls) > 5:
        raise Unfusable("more than five wall operations")
    return obstacles, walls, corners


def pack_bc(lat_or_arrays, nx, ny):
    """Packed BC layout: u_left | u_right | u_top | u_bot | rho_right."""
    g = lat_or_arrays
    parts = [np.asarray(g["u_left"]).reshape(2 * ny), np.asarray(g["u_right"]).reshape(2 * ny),
             np.asarray(g["u_top"]).reshape(2 * nx), np.asarray(g["u_bot"]).reshape(2 * nx),
             np.asarray(g["rho_right"]).reshape(ny)]
    return np.ascontiguousarray(np.concatenate(parts), dtype=np.float64)


def _wrap(k, n):
    return np.where(k < 0, k + n, k)


def build_tables(nx, ny, obstacles, ibb_on):
    """Special-cell and link tables of the fused kernels (host, NumPy).

    Links of all obstacles are concatenated in set_bc order, each obstacle's
    links in its ``boundary`` order; link k of a cell is applied before link
    k' > k, so the last one wins as in the serial reference loop.  Special
    cells are every wall cell plus every (wrapped) link cell, sorted by
    linear index i*ny + j, with a CSR list of their link ids.
    """
    bnds, ps, starts = [], [], [0]
    for obs in obstacles:
        b = np.asarray(obs.boundary, dtype=np.int64).reshape(-1, 3)
        bnds.append(b)
        if ibb_on:
            p = np.asarray(obs.ibb, dtype=np.float64).reshape(-1)
            if len(p) < len(b):
                raise ValueError("obstacle %r: IBB distances missing" % getattr(obs, "name", "?"))
            ps.append(p[:len(b)])
        else:
            ps.append(np.zeros(len(b)))
        starts.append(starts[-1] + len(b))
    bnd = np.concatenate(bnds) if bnds else np.zeros((0, 3), np.int64)
    p = np.concatenate(ps) if ps else np.zeros(0)
    n_links = len(bnd)
    if n_links and (bnd[:, 2].min() < 1 or bnd[:, 2].max() > 8):
        raise ValueError("link direction outside 1..8")
    for name, k, n in (("i", 0, nx), ("j", 1, ny)):
        if n_links and (bnd[:, k].min() < -n or bnd[:, k].max() >= n):
            raise IndexError("link %s index outside the lattice" % name)
    li, lj, lq = _wrap(bnd[:, 0], nx), _wrap(bnd[:, 1], ny), bnd[:, 2]
    qb = _NS[lq] if n_links else lq
    link_cell = li * ny + lj
    nb1 = np.zeros(n_links, np.int64)
    nb2 = np.zeros(n_links, np.int64)
    if ibb_on and n_links:
        for mult, arr, need in ((1, nb1, np.ones(n_links, bool)), (2, nb2, p < 0.5)):
            ii = bnd[:, 0] + mult * _CX[qb]
            jj = bnd[:, 1] + mult * _CY[qb]
            ok = (ii >= -nx) & (ii < nx) & (jj >= -ny) & (jj < ny)
            if (need & ~ok).any():
                raise IndexError("IBB stencil of link %s leaves the lattice"
                                 % (bnd[np.argmax(need & ~ok)],))
            # Entries not needed (x + 2 c_qb when p >= 0.5) are never read.
            arr[ok] = _wrap(ii[ok], nx) * ny + _wrap(jj[ok], ny)

    I, J = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    wall = (I == 0) | (I == nx - 1) | (J == 0) | (J == ny - 1)
    special = np.unique(np.concatenate([(I * ny + J)[wall], link_cell]).astype(np.int64))
    n_special = len(special)
    sidx = np.searchsorted(special, link_cell)
    order = np.lexsort((np.arange(n_links), sidx)) if n_links else np.zeros(0, np.int64)
    counts = np.bincount(sidx, minlength=n_special) if n_links else np.zeros(n_special, np.int64)
    link_start = np.zeros(n_special + 1, np.int64)
    link_start[1:] = np.cumsum(counts)

    def sp(i, j):
        return int(np.searchsorted(special, i * ny + j))

    corner_special, corner_nb = [0] * 4, [0] * 4
    for c, (i, j) in {_lib.CORNER_BOTTOM_LEFT: (0, 0), _lib.CORNER_TOP_LEFT: (0, ny - 1),
                      _lib.CORNER_TOP_RIGHT: (nx - 1, ny - 1),
                      _lib.CORNER_BOTTOM_RIGHT: (nx - 1, 0)}.items():
        corner_special[c] = sp(i, j)
        corner_nb[c] = sp(1 if i == 0 else nx - 2, j)
    return dict(n_links=n_links, n_special=n_special, special=special, link_start=link_start,
                link_ids=order, link_cell=link_cell, link_q=lq, nb1=nb1, nb2=nb2, p=p,
                coef=ibb_coefficients(p),
                obs_start=np.array(starts, np.int64), corner_special=corner_special,
                corner_nb_special=corner_nb)


def ibb_coefficients(p):
    """[3][n] IBB coefficients of each link (lbm_problem.link_coef): the
    factors of the reference's interpolated bounce-back (nb.py:98-104),
    evaluated in its order in IEEE double."""
    p = np.asarray(p, dtype=np.float64)
    pp = 2.0 * p
    lo = p < 0.5
    with np.errstate(divide="ignore", invalid="ignore"):
        c1 = np.where(lo, p * (pp + 1.0), 1.0 / (p * (pp + 1.0)))
        c2 = np.where(lo, (1.0 + pp) * (1.0 - pp), (pp - 1.0) / p)
        c3 = np.where(lo, p * (1.0 - pp), (1.0 - pp) / (1.0 + pp))
    return np.ascontiguousarray(np.stack([c1, c2, c3]))


class FusedEngine:
    """Device state and launch logic of a fused run (see module docstring)."""

    def __init__(self, lat, obstacles, walls, corners, precision=None, drag_cap=4096):
        self.lat = lat
        self.nx, self.ny = lat.nx, lat.ny
        self.N = self.nx * self.ny
        self.dev = lat.device
        self.precision = precision or lat.precision
        self.prec_id = _lib.PRECISIONS[self.precision]
        self.rho0 = float(getattr(lat, "rho_lbm", 1.0))
        self.obstacles = list(obstacles)
        self._keep = []
        nx, ny, dev = self.nx, self.ny, self.dev

        st_dtype = _STORE_DTYPE[self.precision]
        # Rows of the reduced forms are padded to 16 bytes so that the bulk
        # kernel can use 16-byte vectors whatever ny is.
        elems = 16 // torch.tensor([], dtype=st_dtype).element_size()
        self.sy = ny if self.precision in ("f64", "q60") else -(-ny // elems) * elems
        self.f = [torch.zeros((9, nx, self.sy), dtype=st_dtype, device=dev) for _ in range(2)]
        self.cur = 0  # f[cur] holds g_up of the last collided iteration

        tb = build_tables(nx, ny, self.obstacles, bool(lat.IBB))
        n_links, n_special = tb["n_links"], tb["n_special"]
        special, link_start, order = tb["special"], tb["link_start"], tb["link_ids"]
        lq, p = tb["link_q"], tb["p"]

        def storage_index(x):  # i * ny + j  ->  i * sy + j
            x = np.asarray(x, dtype=np.int64)
            return (x // ny) * self.sy + x % ny

        link_cell = storage_index(tb["link_cell"])
        nb1, nb2 = storage_index(tb["nb1"]), storage_index(tb["nb2"])
        starts = tb["obs_start"]
        corner_special, corner_nb = tb["corner_special"], tb["corner_nb_special"]

        def i32(a):
            t = torch.from_numpy(np.ascontiguousarray(a, dtype=np.int32)).to(dev)
            self._keep.append(t)
            return t

        def f64(a):
            t = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(dev)
            self._keep.append(t)
            return t

        self.t_special = i32(special if n_special else np.zeros(1))
        self.t_link_start = i32(link_start)
        self.t_link_ids = i32(order if n_links else np.zeros(1))
        self.t_link_cell = i32(link_cell if n_links else np.zeros(1))
        self.t_link_q = i32(lq if n_links else np.zeros(1))
        self.t_nb1 = i32(nb1 if n_links else np.zeros(1))
        self.t_nb2 = i32(nb2 if n_links else np.zeros(1))
        self.t_link_p = f64(p if n_links else np.zeros(1))
        self.t_link_coef = f64(tb["coef"] if n_links else np.zeros(3))
        self.t_obs_start = i32(np.array(starts))
        self.n_links = n_links
        self.n_special = n_special

        # ---- BC (packed) and schedule
        self.bc_base = torch.zeros(4 * ny + 4 * nx + ny, dtype=torch.float64, device=dev)
        self.bc_vec = None
        self.bc_scale = None
        self.bc_scale_it0 = 0

        # ---- drag history, status
        self.drag_cap = int(drag_cap)
        n_obs = max(1, len(self.obstacles))
        self.drag_hist = torch.zeros((self.drag_cap, n_obs, 2), dtype=torch.float64, device=dev)
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        # 16-bit forms step through the TMA-staged bulk kernel unless
        # bulk_kernel is set to "registers" (lbm_advance flags)
        self.bulk_kernel = "tma"

        # ---- problem descriptor
        P = _lib.Problem()
        P.nx, P.ny = nx, ny
        P.precision = self.prec_id
        P.ibb = int(bool(lat.IBB))
        P.om_p, P.om_m = lat.om_p_lbm, lat.om_m_lbm
        P.rho0 = self.rho0
        P.n_wall_ops = len(walls)
        for k, w in enumerate(walls):
            P.wall_ops[k] = w
        P.n_corner_ops = len(corners)
        for k, c in enumerate(corners):
            P.corner_ops[k] = c
        for c in range(4):
            P.corner_special[c] = corner_special[c]
            P.corner_nb_special[c] = corner_nb[c]
        P.f[0], P.f[1] = self.f[0].data_ptr(), self.f[1].data_ptr()
        P.row_pitch = self.sy
        P.n_special = n_special
        P.special_cell = self.t_special.data_ptr()
        P.special_link_start = self.t_link_start.data_ptr()
        P.n_links = n_links
        P.link_cell = self.t_link_cell.data_ptr()
        P.link_q = self.t_link_q.data_ptr()
        P.link_nb1 = self.t_nb1.data_ptr()
        P.link_nb2 = self.t_nb2.data_ptr()
        P.link_p = self.t_link_p.data_ptr()
        P.link_coef = self.t_link_coef.data_ptr()
        P.special_link_ids = self.t_link_ids.data_ptr()
        P.n_obstacles = len(self.obstacles)
        P.obstacle_link_start = self.t_obs_start.data_ptr()
        P.bc_base = self.bc_base.data_ptr()
        P.drag_hist = self.drag_hist.data_ptr()
        P.drag_cap = self.drag_cap
        P.rho_out = lat.device_field("rho").data_ptr()
        P.u_out = lat.device_field("u").data_ptr()
        P.g_out = lat.device_field("g").data_ptr()
        P.status_flags = self.status.data_ptr()
        self.P = P
        nbytes = _lib.load().lbm_problem_scratch_bytes(ctypes.byref(P))
        self.scratch = torch.zeros(int(nbytes), dtype=torch.uint8, device=dev)
        P.scratch = self.scratch.data_ptr()
        P.scratch_bytes = int(nbytes)

    # ------------------------------------------------------------------ BCs
    def set_bc_constant(self, packed):
        self.bc_base.copy_(torch.from_numpy(packed))
        self.bc_vec = None
        self.P.bc_vec = None
        self.P.bc_scale = None
        self.P.bc_scale_len = 0

    def set_bc_schedule(self, base, vec, scale, it0=0):
        """BC vectors at iteration it = base + scale[it - it0] * vec."""
        self.bc_base.copy_(torch.from_numpy(np.ascontiguousarray(base, dtype=np.float64)))
        if self.bc_vec is None:
            self.bc_vec = torch.zeros_like(self.bc_base)
        self.bc_vec.copy_(torch.from_numpy(np.ascontiguousarray(vec, dtype=np.float64)))
        self.bc_scale = torch.from_numpy(np.ascontiguousarray(scale, dtype=np.float64)).to(self.dev)
        self.bc_scale_it0 = int(it0)
        self.P.bc_vec = self.bc_vec.data_ptr()
        self.P.bc_scale = self.bc_scale.data_ptr()
        self.P.bc_scale_it0 = self.bc_scale_it0
        self.P.bc_scale_len = int(self.bc_scale.numel())

    # -------------------------------------------------------------- stepping
    @property
    def step_flags(self):
        if self.bulk_kernel not in ("tma", "registers"):
            raise ValueError("bulk_kernel is 'tma' or 'registers'")
        flags = _lib.FLAG_BULK_REGISTERS if self.bulk_kernel == "registers" else 0
        if getattr(self, "test_stall", False):  # failure-path test (LBM_FLAG_TEST_STALL)
            flags |= _lib.FLAG_TEST_STALL
        return flags

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def collide_from_g(self, it, macro=True):
        """Collision of iteration ``it`` from the lattice's g (all cells)."""
        self.lat.device_field("g")  # upload if the host copy is newer
        flags = (_lib.FLAG_MACRO_LAST if macro else 0) | _lib.FLAG_CHECK_FINITE
        if macro:
            self.lat.device_field("rho", True)
            self.lat.device_field("u", True)
        _lib.call("lbm_advance", ctypes.byref(self.P), _lib.MODE_COLLIDE_FROM_G, it, 1, 1,
                  flags, self._stream())
        self.cur = 0

    def steps(self, it0, n, macro_last=False, graph=True):
        """Collisions of iterations it0 .. it0+n-1 (BCs/drag of it0-1 .. it0+n-2)."""
        if n <= 0:
            return
        flags = (_lib.FLAG_MACRO_LAST if macro_last else 0) | _lib.FLAG_CHECK_FINITE
        flags |= self.step_flags
        if macro_last:
            self.lat.device_field("rho", True)
            self.lat.device_field("u", True)
        if graph:
            _lib.call("lbm_advance_graph", ctypes.byref(self.P), it0, n, self.cur, flags,
                      self._stream())
        else:
            _lib.call("lbm_advance", ctypes.byref(self.P), _lib.MODE_STEP, it0, n, self.cur,
                      flags, self._stream())
        self.cur ^= (n & 1)

    def finish(self, it, wall_macro=True):
        """Stream + BCs of iteration it-1 into lattice.g; drag of it-1."""
        flags = _lib.FLAG_WALL_MACRO if wall_macro else 0
        self.lat.device_field("g", True)
        _lib.call("lbm_advance", ctypes.byref(self.P), _lib.MODE_FINISH, it, 1, self.cur, flags,
                  self._stream())
        self.lat.mark_written("g")
        if wall_macro:
            self.lat.mark_written("rho", "u")

    def g_up_into(self, out):
        """Unpack f[cur] (g_up of the last collided iteration) into FP64 ``out``."""
        _lib.call("lbm_unpack_f64", self.prec_id, ctypes.c_void_p(self.f[self.cur].data_ptr()),
                  ctypes.c_void_p(out.data_ptr()), self.nx, self.ny, self.sy, self.rho0,
                  self._stream())

    def drag_rows(self, it_first, it_last):
        """Raw (fx, fy) per obstacle for iterations it_first..it_last (host)."""
        if it_last < it_first:
            return np.zeros((0, max(1, len(self.obstacles)), 2))
        if not self.obstacles:
            return np.zeros((it_last - it_first + 1, 1, 2))
        idx = np.arange(it_first, it_last + 1) % self.drag_cap
        h = self.drag_hist.cpu().numpy()
        return h[idx]

    def drag_rows_after(self, it_first, it_last, event, stream):
        """drag_rows of iterations whose step precedes ``event``, copied on
        ``stream`` after it, so that later steps may run meanwhile; also
        raises what check_status would for the steps up to the event."""
        with torch.cuda.stream(stream):
            stream.wait_event(event)
            status = int(self.status.cpu().item())
            if it_last < it_first:
                rows = np.zeros((0, max(1, len(self.obstacles)), 2))
            elif not self.obstacles:
                rows = np.zeros((it_last - it_first + 1, 1, 2))
            else:
                idx = torch.arange(it_first, it_last + 1, device=self.dev) % self.drag_cap
                rows = self.drag_hist[idx].cpu().numpy()
        if status & 1:
            raise FloatingPointError("non-finite density or velocity in the lattice")
        if status & 2:
            raise RuntimeError("BC schedule table does not cover the iterations run")
        return rows

    def check_status(self):
        s = int(self.status.item())
        if s & 1:
            raise FloatingPointError("non-finite density or velocity in the lattice")
        if s & 2:
            raise RuntimeError("BC schedule table does not cover the iterations run")
        if s & 4:
            raise RuntimeError("batched step: special-cell tiles stopped waiting for "
                               "their lattice's bulk tiles")
        if s & 8:
            raise RuntimeError("bulk kernel: a shared-memory stage wait timed out")

    # --------------------------------------------------------- snapshot/restore
    def snapshot(self):
        return (self.f[self.cur].clone(), self.scratch.clone(), self.cur)

    def restore(self, snap):
        f, sc, cur = snap
        self.cur = cur
        self.f[cur].copy_(f)
        self.scratch.copy_(sc)
