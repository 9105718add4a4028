"""CPU oracle for the lattice update -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module.  It is the checker for the CUDA library,
never a fallback for it.

* ``lib()`` loads ``liblbm_oracle.so`` (built from ``lbm_oracle.c`` by
  ``build()``), a C restatement of ``lbm/src/core/nb.py``.
* ``OracleLattice`` restates the reference ``lattice`` class
  (``lbm/src/core/lattice.py:15-436``): same attributes, same methods, same
  step semantics, with the kernels executed by the C oracle.  Apps drive it
  exactly like the GPU lattice, so one app object can run on both.
* ``add_obstacle_loops`` restates ``lattice.add_obstacle``/``get_coords``/
  ``is_inside`` (``lattice.py:290-414``) cell by cell, as the checker for the
  vectorised link builder.

Parity of this restatement with the reference source is pinned by
``tests/test_oracle_golden.py`` against ``tests/golden/*.npz``.
"""
import ctypes
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liblbm_oracle.so")

C = np.array([[0, 0], [1, 0], [-1, 0], [0, 1], [0, -1],
              [1, 1], [-1, -1], [-1, 1], [1, -1]])
NS = np.array([0, 2, 1, 4, 3, 6, 5, 8, 7])
W = np.array([4. / 9.] + [1. / 9.] * 4 + [1. / 36.] * 4)

_lib = None


def build(force=False, verbose=False):
    """Compile lbm_oracle.c with gcc (no FP contraction, so x86 == Arm);
    verbose: print the gcc command line."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    src = os.path.join(HERE, "lbm_oracle.c")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src)):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O3", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
           "-o", tmp, src]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        lp = ctypes.POINTER(ctypes.c_int64)
        i = ctypes.c_int
        d = ctypes.c_double
        sig = {
            "oracle_macro": [dp, dp, dp, i, i],
            "oracle_equilibrium": [dp, dp, dp, i, i],
            "oracle_col_str": [dp, dp, dp, d, d, i, i],
            "oracle_drag_lift": [lp, ctypes.c_int64, dp, dp, i, i, d, d, d, dp],
            "oracle_bounce_back": [i, lp, ctypes.c_int64, dp, dp, dp, i, i],
            "oracle_zh_left": [dp, dp, dp, dp, i, i],
            "oracle_zh_right": [dp, dp, dp, dp, i, i],
            "oracle_zh_right_pressure": [dp, dp, dp, dp, dp, i, i],
            "oracle_zh_top": [dp, dp, dp, dp, i, i],
            "oracle_zh_bottom": [dp, dp, dp, dp, i, i],
            "oracle_corner": [i, dp, dp, dp, i, i],
            "oracle_threads": [],
            "oracle_run": [dp] * 10 + [i, i, d, d, i, ctypes.POINTER(ctypes.c_int32), i, lp, lp,
                                       dp, i, dp, dp, dp, ctypes.c_int64, dp],
        }
        for name, args in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = i if name in ("oracle_drag_lift", "oracle_bounce_back",
                                       "oracle_threads", "oracle_run") else None
        _lib = L
    return _lib


def threads():
    """OpenMP threads the oracle's cell loops use (OMP_NUM_THREADS)."""
    return int(lib().oracle_threads())


def _dp(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _lp(a):
    assert a.dtype == np.int64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))


# ---------------------------------------------------------------------------
# Kernel-level entry points (numpy in, numpy mutated in place)
# ---------------------------------------------------------------------------
def macro(g, rho, u):
    nx, ny = g.shape[1:]
    lib().oracle_macro(_dp(g), _dp(rho), _dp(u), nx, ny)


def equilibrium(u, rho, g_eq):
    nx, ny = rho.shape
    lib().oracle_equilibrium(_dp(u), _dp(rho), _dp(g_eq), nx, ny)


def col_str(g, g_eq, g_up, om_p, om_m):
    nx, ny = g.shape[1:]
    lib().oracle_col_str(_dp(g), _dp(g_eq), _dp(g_up), om_p, om_m, nx, ny)


def drag_lift(links, g_up, g, R_ref, U_ref, L_ref):
    nx, ny = g.shape[1:]
    links = np.ascontiguousarray(links, dtype=np.int64).reshape(-1, 3)
    out = np.zeros(2)
    rc = lib().oracle_drag_lift(_lp(links), links.shape[0], _dp(g_up), _dp(g), nx, ny,
                                R_ref, U_ref, L_ref, _dp(out))
    if rc != 0:
        raise IndexError("drag_lift: link index out of range")
    return out[0], out[1]


def bounce_back(ibb, links, p, g_up, g):
    nx, ny = g.shape[1:]
    links = np.ascontiguousarray(links, dtype=np.int64).reshape(-1, 3)
    p = np.ascontiguousarray(p, dtype=np.float64).reshape(-1)
    if ibb and p.shape[0] < links.shape[0]:
        raise ValueError("ibb distances missing")
    if p.shape[0] == 0:
        p = np.zeros(1)
    rc = lib().oracle_bounce_back(int(bool(ibb)), _lp(links), links.shape[0], _dp(p),
                                  _dp(g_up), _dp(g), nx, ny)
    if rc != 0:
        raise IndexError("bounce_back: link stencil leaves the lattice")


def zou_he(kind, u, rho, g, vec=None, rho_right=None):
    nx, ny = g.shape[1:]
    L = lib()
    if kind == "left":
        L.oracle_zh_left(_dp(u), _dp(vec), _dp(rho), _dp(g), nx, ny)
    elif kind == "right":
        L.oracle_zh_right(_dp(u), _dp(vec), _dp(rho), _dp(g), nx, ny)
    elif kind == "right_pressure":
        L.oracle_zh_right_pressure(_dp(u), _dp(rho_right), _dp(vec), _dp(rho), _dp(g), nx, ny)
    elif kind == "top":
        L.oracle_zh_top(_dp(u), _dp(vec), _dp(rho), _dp(g), nx, ny)
    elif kind == "bottom":
        L.oracle_zh_bottom(_dp(u), _dp(vec), _dp(rho), _dp(g), nx, ny)
    else:
        raise ValueError(kind)


CORNERS = {"bottom_left": 0, "top_left": 1, "top_right": 2, "bottom_right": 3}


def corner(name, u, rho, g):
    nx, ny = g.shape[1:]
    lib().oracle_corner(CORNERS[name], _dp(u), _dp(rho), _dp(g), nx, ny)


# ---------------------------------------------------------------------------
# Geometry (restatement of lattice.add_obstacle / get_coords / is_inside)
# ---------------------------------------------------------------------------
def get_coords(lat, i, j):
    """lbm/src/core/lattice.py:379-387."""
    dx = (lat.x_max - lat.x_min) / (lat.nx - 1)
    dy = (lat.y_max - lat.y_min) / (lat.ny - 1)
    return [lat.x_min + i * dx, lat.y_min + j * dy]


def is_inside(poly, pt):
    """Crossing-number test, lbm/src/core/lattice.py:391-414."""
    j = len(poly) - 1
    odd = False
    for i in range(len(poly)):
        if (((poly[i, 1] < pt[1] and poly[j, 1] >= pt[1]) or
             (poly[j, 1] < pt[1] and poly[i, 1] >= pt[1])) and
                (poly[i, 0] < pt[0] or poly[j, 0] < pt[0])):
            slope = (poly[j, 0] - poly[i, 0]) / (poly[j, 1] - poly[i, 1])
            if (poly[i, 0] + (pt[1] - poly[i, 1]) * slope) < pt[0]:
                odd = not odd
        j = i
    return odd


def add_obstacle_loops(lat, polygon, tag, ibb_on):
    """Cell-by-cell restatement of lattice.add_obstacle (lattice.py:290-375).

    Mutates ``lat.lattice`` (the tag mask) and returns ``(area, bnd, ibb)``.
    """
    polygon = np.asarray(polygon, dtype=np.float64)
    b = [polygon[:, 0].min(), polygon[:, 0].max(), polygon[:, 1].min(), polygon[:, 1].max()]
    obs = []
    for i in range(lat.nx):
        for j in range(lat.ny):
            pt = get_coords(lat, i, j)
            if pt[0] > b[0] and pt[0] < b[1] and pt[1] > b[2] and pt[1] < b[3]:
                if is_inside(polygon, pt):
                    lat.lattice[i, j] = tag
                    obs.append((i, j))
    bnd = []
    for (i, j) in obs:
        for q in range(1, 9):
            ii, jj = i + C[q, 0], j + C[q, 1]
            if ii > lat.nx - 1 or jj > lat.ny - 1:
                continue
            if not lat.lattice[ii, jj]:
                bnd.append((ii, jj, NS[q]))
    bnd = np.unique(np.array(bnd, dtype=np.int64).reshape(-1, 3), axis=0)
    ibb = np.empty(0)
    if ibb_on:
        vals = []
        for k in range(len(bnd)):
            i, j, q = bnd[k]
            pt = get_coords(lat, i, j)
            x = polygon[:, 0] - pt[0]
            y = polygon[:, 1] - pt[1]
            dist = np.sqrt(np.square(x) + np.square(y))
            mpt = np.argmin(dist)
            vals.append(dist[mpt] / (lat.dx * np.linalg.norm(C[q])))
        ibb = np.array(vals, dtype=np.float64)
    area = 0.0
    for i in range(lat.nx):
        for j in range(lat.ny):
            if lat.lattice[i, j] == tag:
                area += lat.dx ** 2
    return area, bnd, ibb


# ---------------------------------------------------------------------------
# Lattice restatement (CPU), same public surface as the reference class
# ---------------------------------------------------------------------------
class OracleLattice:
    """CPU restatement of the reference ``lattice`` (lbm/src/core/lattice.py).

    Parameters are copied from the app with the same ``hasattr`` rules
    (lattice.py:50-78, including ``Cr`` taking ``app.Ct``); arrays are
    float64 numpy with the reference shapes.  No output directories are
    created unless ``output_dir`` is given.
    """

    _PARAMS = ["name", "x_min", "x_max", "y_min", "y_max", "nx", "ny", "tau_lbm",
               "dx", "dt", "Cx", "Ct", "Cn", "Cu", "Cf", "dpi", "u_lbm", "L_lbm",
               "nu_lbm", "Re_lbm", "rho_lbm", "IBB", "stop", "t_max", "it_max",
               "obs_cv_ct", "obs_cv_nb"]

    def __init__(self, app, output_dir=None):
        self.name, self.x_min, self.x_max, self.y_min, self.y_max = "lattice", 0.0, 1.0, 0.0, 1.0
        self.nx = self.ny = 100
        self.tau_lbm, self.dx, self.dt = 1.0, 1.0, 1.0
        self.Cx, self.Ct, self.Cr = self.dx, self.dt, 1.0
        self.Cn, self.Cu, self.Cf = self.Cx ** 2 / self.Ct, self.Cx / self.Ct, self.Cr * self.Cx ** 2 / self.Ct
        self.dpi, self.u_lbm, self.L_lbm, self.nu_lbm, self.Re_lbm = 100, 0.03, 100, 0.01, 100.0
        self.rho_lbm, self.IBB, self.stop, self.t_max, self.it_max = 1.0, False, "it", 1.0, 1000
        self.obs_cv_ct, self.obs_cv_nb = 1.0e-1, 500
        for k in self._PARAMS:
            if hasattr(app, k):
                setattr(self, k, getattr(app, k))
        if hasattr(app, "Cr"):
            self.Cr = app.Ct
        self.output_dir = output_dir if output_dir is not None else "./"
        self.png_dir = self.output_dir
        self.output_it = 0
        self.lx, self.ly, self.q = self.nx - 1, self.ny - 1, 9
        self.Cs = 1.0 / math.sqrt(3.0)
        self.tau_p_lbm = self.tau_lbm
        self.lambda_trt = 1.0 / 4.0
        self.tau_m_lbm = self.lambda_trt / (self.tau_p_lbm - 0.5) + 0.5
        self.om_p_lbm = 1.0 / self.tau_p_lbm
        self.om_m_lbm = 1.0 / self.tau_m_lbm
        self.om_lbm = 1.0 / self.tau_lbm
        self.c, self.w, self.ns = C.copy(), W.copy(), NS.copy()
        shp = (9, self.nx, self.ny)
        self.g, self.g_eq, self.g_up = np.zeros(shp), np.zeros(shp), np.zeros(shp)
        self.u_left, self.u_right = np.zeros((2, self.ny)), np.zeros((2, self.ny))
        self.u_top, self.u_bot = np.zeros((2, self.nx)), np.zeros((2, self.nx))
        self.rho_right = np.zeros(self.ny)
        self.lattice = np.zeros((self.nx, self.ny))
        self.rho = np.ones((self.nx, self.ny))
        self.u = np.zeros((2, self.nx, self.ny))

    def _c(self, name):
        a = getattr(self, name)
        if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous):
            a = np.ascontiguousarray(a, dtype=np.float64)
            setattr(self, name, a)
        return a

    def macro(self):
        macro(self._c("g"), self._c("rho"), self._c("u"))

    def equilibrium(self):
        equilibrium(self._c("u"), self._c("rho"), self._c("g_eq"))

    def collision_stream(self):
        col_str(self._c("g"), self._c("g_eq"), self._c("g_up"), self.om_p_lbm, self.om_m_lbm)

    def drag_lift(self, obs, R_ref, U_ref, L_ref):
        return drag_lift(obs.boundary, self._c("g_up"), self._c("g"), R_ref, U_ref, L_ref)

    def bounce_back_obstacle(self, obstacle):
        bounce_back(self.IBB, obstacle.boundary, obstacle.ibb, self._c("g_up"), self._c("g"))

    def zou_he_left_wall_velocity(self):
        zou_he("left", self._c("u"), self._c("rho"), self._c("g"), vec=self._c("u_left"))

    def zou_he_right_wall_velocity(self):
        zou_he("right", self._c("u"), self._c("rho"), self._c("g"), vec=self._c("u_right"))

    def zou_he_right_wall_pressure(self):
        zou_he("right_pressure", self._c("u"), self._c("rho"), self._c("g"),
               vec=self._c("u_right"), rho_right=self._c("rho_right"))

    def zou_he_top_wall_velocity(self):
        zou_he("top", self._c("u"), self._c("rho"), self._c("g"), vec=self._c("u_top"))

    def zou_he_bottom_wall_velocity(self):
        zou_he("bottom", self._c("u"), self._c("rho"), self._c("g"), vec=self._c("u_bot"))

    def zou_he_bottom_left_corner(self):
        corner("bottom_left", self._c("u"), self._c("rho"), self._c("g"))

    def zou_he_top_left_corner(self):
        corner("top_left", self._c("u"), self._c("rho"), self._c("g"))

    def zou_he_top_right_corner(self):
        corner("top_right", self._c("u"), self._c("rho"), self._c("g"))

    def zou_he_bottom_right_corner(self):
        corner("bottom_right", self._c("u"), self._c("rho"), self._c("g"))

    def get_coords(self, i, j):
        return get_coords(self, i, j)

    def is_inside(self, poly, pt):
        return is_inside(poly, pt)

    def add_obstacle(self, obstacle):
        return add_obstacle_loops(self, obstacle.polygon, obstacle.tag, self.IBB)

    def generate_image(self, obstacles):
        pass


_WALLS = {"zou_he_left_wall_velocity": 0, "zou_he_right_wall_velocity": 1,
          "zou_he_right_wall_pressure": 2, "zou_he_top_wall_velocity": 3,
          "zou_he_bottom_wall_velocity": 4}


class _Program:
    """Records the lattice calls of an app's set_bc as (kind, arg) pairs:
    0 = bounce-back of obstacle arg, 1 = Zou-He wall, 2 = corner."""

    def __init__(self, obstacles):
        self.obstacles = list(obstacles)
        self.ops = []

    def bounce_back_obstacle(self, obs):
        self.ops.append((0, next(k for k, o in enumerate(self.obstacles) if o is obs)))

    def __getattr__(self, name):
        if name in _WALLS:
            return lambda: self.ops.append((1, _WALLS[name]))
        if name.startswith("zou_he_") and name.endswith("_corner"):
            return lambda: self.ops.append((2, CORNERS[name[len("zou_he_"):-len("_corner")]]))
        raise AttributeError(name)


def run_program(lat, app, n_iter, schedule, initialize=True):
    """Iterations of ``run`` (below) in one C call (oracle_run): the same
    kernels in the same order, for an app whose ``outputs`` does nothing in
    those iterations and whose ``set_inlets(lat, it)`` sets the BC vectors to
    ``base + scale[it] * vec`` (packed u_left | u_right | u_top | u_bot |
    rho_right), given as ``schedule = (base, vec, scale)``.

    initialize: call ``app.initialize(lat)`` first and run iterations
    0 .. n_iter-1; False: continue from the lattice's current state, with
    ``scale[k]`` the scale of the k-th iteration run.  Returns the raw
    drag/lift sums (fx, fy) of every obstacle in ``app.obstacles`` after
    every iteration's set_bc, shape (n_iter, n_obs, 2): ``lattice.drag_lift``
    is ``-2 (fx, fy) / (R L U^2)`` of these.
    """
    if initialize:
        app.initialize(lat)
    obstacles = list(getattr(app, "obstacles", ()))
    rec = _Program(obstacles)
    app.set_bc(rec)
    prog = np.ascontiguousarray(np.array(rec.ops, dtype=np.int32).reshape(-1, 2))
    starts = np.zeros(len(obstacles) + 1, dtype=np.int64)
    links, ps = [], []
    for k, o in enumerate(obstacles):
        b = np.asarray(o.boundary, dtype=np.int64).reshape(-1, 3)
        links.append(b)
        starts[k + 1] = starts[k] + len(b)
        ps.append(np.asarray(o.ibb, dtype=np.float64).reshape(-1)[:len(b)] if lat.IBB
                  else np.zeros(len(b)))
    links = np.ascontiguousarray(np.concatenate(links) if links else np.zeros((1, 3), np.int64))
    ps = np.ascontiguousarray(np.concatenate(ps) if ps else np.zeros(1))
    if lat.IBB and len(ps) < starts[-1]:
        raise ValueError("ibb distances missing")
    base, vec, scale = schedule
    base = np.ascontiguousarray(base, dtype=np.float64)
    vec = None if vec is None else np.ascontiguousarray(vec, dtype=np.float64)
    scale = np.ascontiguousarray(np.asarray(scale, dtype=np.float64)[:n_iter])
    nx, ny = lat.nx, lat.ny
    if base.shape != (5 * ny + 4 * nx,) or (vec is not None and vec.shape != base.shape) \
            or scale.shape != (n_iter,):
        raise ValueError("schedule shapes")
    drag = np.zeros((n_iter, max(len(obstacles), 1), 2))
    names = ["g", "g_eq", "g_up", "rho", "u", "u_left", "u_right", "u_top", "u_bot", "rho_right"]
    arrs = [lat._c(k) for k in names]
    rc = lib().oracle_run(*[_dp(a) for a in arrs], nx, ny, lat.om_p_lbm, lat.om_m_lbm,
                          int(bool(lat.IBB)),
                          prog.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), len(prog),
                          _lp(links), _lp(starts), _dp(ps), len(obstacles), _dp(base),
                          _dp(vec) if vec is not None else None, _dp(scale), n_iter, _dp(drag))
    if rc != 0:
        raise IndexError("oracle_run: link or program entry out of range")
    return drag[:, :len(obstacles)]


def run(lattice, app, n_iter=None):
    """Driver loop of lbm/src/core/run.py:12-61 (printing omitted)."""
    app.initialize(lattice)
    it = 0
    compute = True
    while compute:
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
    app.finalize(lattice)
    return it
