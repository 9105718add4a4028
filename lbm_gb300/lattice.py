"""GPU lattice: drop-in for the reference ``lattice`` class.

Same constructor (``lattice(app)``), same attributes and the same methods as
lbm/src/core/lattice.py:15-436.  The distribution and field arrays live in
device memory (torch tensors, float64) and are mirrored to NumPy when the
host touches them:

* reading an attribute (``lattice.g``, ``lattice.u``, ``lattice.u_top``...)
  returns a NumPy array synchronised from the device; the array may be
  modified in place (``lattice.u[:, mask] = 0``) and is uploaded again before
  the next device operation that reads it;
* assigning an attribute (``lattice.g = lattice.g_eq.copy()``) replaces the
  host copy, uploaded on next use.

Each lattice method launches the matching CUDA kernel of liblbm_gb300
(lbm_macro_f64, lbm_equilibrium_f64, ...).  ``lbm_gb300.run`` drives the
fused engine (``lbm_gb300.engine``) instead when the app's step can be fused.
An array kept from an earlier read and modified later, without reading the
attribute again, is not seen by the device.
"""
import ctypes
import math
import os
from datetime import datetime

import numpy as np
import torch

from . import _lib
from . import geometry

_C = np.array([[0, 0], [1, 0], [-1, 0], [0, 1], [0, -1],
               [1, 1], [-1, -1], [-1, 1], [1, -1]])


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class _Mirror:
    """A float64 device tensor with a lazily synchronised NumPy copy."""

    def __init__(self, shape, device, fill=0.0):
        self.shape = tuple(shape)
        self.dev = torch.full(self.shape, fill, dtype=torch.float64, device=device)
        self.host = None
        self.dev_ok = True
        self.host_ok = False

    def get(self):
        if not self.host_ok:
            self.host = self.dev.cpu().numpy().copy()
            self.host_ok = True
        # The caller may modify the array in place: re-upload before next use.
        self.dev_ok = False
        return self.host

    def set(self, value):
        a = np.array(value, dtype=np.float64, copy=True)
        if a.shape != self.shape:
            a = np.broadcast_to(a, self.shape).copy()
        self.host = np.ascontiguousarray(a)
        self.host_ok = True
        self.dev_ok = False

    def device(self, overwrite=False):
        """Device tensor, uploaded if the host copy is newer.

        overwrite=True: the caller writes every element, no upload needed.
        """
        if overwrite:
            self.dev_ok = True
            self.host_ok = False
        elif not self.dev_ok:
            self.dev.copy_(torch.from_numpy(self.host), non_blocking=False)
            self.dev_ok = True
        return self.dev

    def written(self):
        """The device copy was modified by a kernel."""
        self.dev_ok = True
        self.host_ok = False


def _mirror_property(name):
    def getter(self):
        return self._m[name].get()

    def setter(self, value):
        self._m[name].set(value)

    return property(getter, setter)


def default_precision(rho0, om_p, om_m):
    """The plain path's default form: "q60" (64-bit fixed-point state, integer
    bulk collision; at least FP64's resolution for populations above 2^-7)
    when the case is inside its range, else "f64"."""
    ok = 0.75 <= rho0 <= 1.5 and all(1.0 / 1024 <= om <= 1.999 for om in (om_p, om_m))
    return "q60" if ok else "f64"


class lattice:
    """Device-resident D2Q9 TRT lattice with the reference lattice API."""

    g = _mirror_property("g")
    g_eq = _mirror_property("g_eq")
    g_up = _mirror_property("g_up")
    rho = _mirror_property("rho")
    u = _mirror_property("u")
    u_left = _mirror_property("u_left")
    u_right = _mirror_property("u_right")
    u_top = _mirror_property("u_top")
    u_bot = _mirror_property("u_bot")
    rho_right = _mirror_property("rho_right")

    _PARAMS = ["name", "x_min", "x_max", "y_min", "y_max", "nx", "ny", "tau_lbm", "dx", "dt",
               "Cx", "Ct", "Cn", "Cu", "Cf", "dpi", "u_lbm", "L_lbm", "nu_lbm", "Re_lbm",
               "rho_lbm", "IBB", "stop", "t_max", "it_max", "obs_cv_ct", "obs_cv_nb"]

    def __init__(self, app, device=None, precision=None, output_dir=None, verbose=True):
        if not torch.cuda.is_available():
            raise RuntimeError("lbm_gb300.lattice needs a CUDA device (no CPU fallback)")
        _lib.load()
        # Defaults and app overrides (lbm/src/core/lattice.py:20-78).
        self.name = "lattice"
        self.x_min, self.x_max, self.y_min, self.y_max = 0.0, 1.0, 0.0, 1.0
        self.nx = self.ny = 100
        self.tau_lbm = 1.0
        self.dx = self.dt = 1.0
        self.Cx, self.Ct, self.Cr = self.dx, self.dt, 1.0
        self.Cn = self.Cx ** 2 / self.Ct
        self.Cu = self.Cx / self.Ct
        self.Cf = self.Cr * self.Cx ** 2 / self.Ct
        self.dpi = 100
        self.u_lbm, self.L_lbm, self.nu_lbm, self.Re_lbm, self.rho_lbm = 0.03, 100, 0.01, 100.0, 1.0
        self.IBB = False
        self.stop = "it"
        self.t_max = 1.0
        self.it_max = 1000
        self.obs_cv_ct, self.obs_cv_nb = 1.0e-1, 500
        for k in self._PARAMS:
            if hasattr(app, k):
                setattr(self, k, getattr(app, k))
        if hasattr(app, "Cr"):
            self.Cr = app.Ct  # the reference copies Ct into Cr (lattice.py:63)

        # Storage form of the fused engine, checked once the TRT rates are set.
        self.precision = precision or getattr(app, "precision", None)
        if self.precision is not None and self.precision not in _lib.PRECISIONS:
            raise ValueError("precision must be one of %s" % sorted(_lib.PRECISIONS))

        # Output directories (lattice.py:80-91).
        if output_dir is None:
            stamp = datetime.now().strftime("%Y-%m-%d_%H_%M_%S")
            self.results_dir = "./results/"
            self.output_dir = self.results_dir + stamp + "/"
        else:
            self.results_dir = output_dir
            self.output_dir = os.path.join(output_dir, "")
        self.png_dir = self.output_dir + "./png/"
        for d in (self.results_dir, self.output_dir, self.png_dir):
            os.makedirs(d, exist_ok=True)

        self.device = torch.device(device if device is not None else "cuda")
        if self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        self.set_default_lbm()
        if self.precision is None:
            self.precision = default_precision(self.rho_lbm, self.om_p_lbm, self.om_m_lbm)
        self._obs_cache = {}
        self._replay = None
        self._drag_scratch = None
        self._drag_out = torch.zeros(2, dtype=torch.float64, device=self.device)

        if verbose:
            print("##################")
            print("### LBM solver ###")
            print("##################")
            print("")
            print("# name       = " + self.name)
            print("# u_lbm      = " + "{:f}".format(self.u_lbm))
            print("# L_lbm      = " + "{:f}".format(self.L_lbm))
            print("# nu_lbm     = " + "{:f}".format(self.nu_lbm))
            print("# Re_lbm     = " + "{:f}".format(self.Re_lbm))
            print("# tau_p_lbm  = " + "{:f}".format(self.tau_p_lbm))
            print("# tau_m_lbm  = " + "{:f}".format(self.tau_m_lbm))
            print("# dt         = " + "{:f}".format(self.dt))
            print("# dx         = " + "{:f}".format(self.dx))
            print("# nx         = " + str(self.nx))
            print("# ny         = " + str(self.ny))
            print("# IBB        = " + str(self.IBB))
            print("# precision  = " + self.precision)
            print("")

    def set_default_lbm(self):
        """Constants and arrays of lattice.py:117-174, arrays on the device."""
        self.output_it = 0
        self.lx = self.nx - 1
        self.ly = self.ny - 1
        self.q = 9
        self.Cs = 1.0 / math.sqrt(3.0)
        self.tau_p_lbm = self.tau_lbm
        self.lambda_trt = 1.0 / 4.0
        self.tau_m_lbm = self.lambda_trt / (self.tau_p_lbm - 0.5) + 0.5
        self.om_p_lbm = 1.0 / self.tau_p_lbm
        self.om_m_lbm = 1.0 / self.tau_m_lbm
        self.om_lbm = 1.0 / self.tau_lbm
        self.c = _C.copy()
        self.w = np.ones(self.q)
        self.w[1:5] = 1.0 / 9.0
        self.w[5:9] = 1.0 / 36.0
        self.w[0] = 4.0 / 9.0
        self.ns = np.array([0, 2, 1, 4, 3, 6, 5, 8, 7])
        nx, ny, dev = self.nx, self.ny, self.device
        self._m = {
            "g": _Mirror((9, nx, ny), dev),
            "g_eq": _Mirror((9, nx, ny), dev),
            "g_up": _Mirror((9, nx, ny), dev),
            "u_left": _Mirror((2, ny), dev),
            "u_right": _Mirror((2, ny), dev),
            "u_top": _Mirror((2, nx), dev),
            "u_bot": _Mirror((2, nx), dev),
            "rho_right": _Mirror((ny,), dev),
            "rho": _Mirror((nx, ny), dev, fill=1.0),
            "u": _Mirror((2, nx, ny), dev),
        }
        self.lattice = np.zeros((nx, ny))

    # ------------------------------------------------------------------ kernels
    def macro(self):
        """lattice.py:178-189 on the device."""
        m = self._m
        _lib.call("lbm_macro_f64", _ptr(m["g"].device()), _ptr(m["rho"].device(True)),
                  _ptr(m["u"].device(True)), self.nx, self.ny, _stream())

    def equilibrium(self):
        """nb_equilibrium (nb.py:7-17) on the device."""
        m = self._m
        _lib.call("lbm_equilibrium_f64", _ptr(m["u"].device()), _ptr(m["rho"].device()),
                  _ptr(m["g_eq"].device(True)), self.nx, self.ny, _stream())

    def collision_stream(self):
        """nb_col_str (nb.py:21-45) on the device."""
        m = self._m
        _lib.call("lbm_collision_stream_f64", _ptr(m["g"].device()), _ptr(m["g_eq"].device()),
                  _ptr(m["g_up"].device(True)), self.om_p_lbm, self.om_m_lbm, self.nx, self.ny,
                  _stream())
        m["g"].written()

    def _obstacle_links(self, obs):
        """Device copy of an obstacle's links (cached per obstacle object)."""
        key = id(obs)
        ent = self._obs_cache.get(key)
        bnd = np.asarray(obs.boundary)
        ibb = np.asarray(getattr(obs, "ibb", np.empty(0)))
        if ent is not None and ent[0] is obs.boundary and ent[1] is getattr(obs, "ibb", None):
            return ent[2]
        bnd = np.ascontiguousarray(bnd, dtype=np.int64).reshape(-1, 3)
        p = np.ascontiguousarray(ibb, dtype=np.float64).reshape(-1)
        # Keep only the last link per (wrapped cell, q): the serial reference
        # loop lets that one win when NumPy wraps two indices onto one cell.
        wi = np.where(bnd[:, 0] < 0, bnd[:, 0] + self.nx, bnd[:, 0])
        wj = np.where(bnd[:, 1] < 0, bnd[:, 1] + self.ny, bnd[:, 1])
        key3 = (wi * self.ny + wj) * 9 + bnd[:, 2]
        last = np.ones(len(bnd), dtype=bool)
        if len(bnd):
            _, first_rev = np.unique(key3[::-1], return_index=True)
            last[:] = False
            last[len(bnd) - 1 - first_rev] = True
        bb_links = torch.from_numpy(bnd[last].astype(np.int32)).to(self.device)
        bb_p = torch.from_numpy(p[last] if len(p) == len(bnd) else np.zeros(int(last.sum()))).to(self.device)
        all_links = torch.from_numpy(bnd.astype(np.int32)).to(self.device)
        dev = (bb_links, bb_p, all_links, len(bnd))
        self._obs_cache[key] = (obs.boundary, getattr(obs, "ibb", None), dev)
        return dev

    def bounce_back_obstacle(self, obstacle):
        """nb_bounce_back_obstacle (nb.py:77-117) on the device."""
        links, p, _, _ = self._obstacle_links(obstacle)
        if self.IBB and len(np.asarray(obstacle.ibb)) < len(np.asarray(obstacle.boundary)):
            raise ValueError("bounce_back_obstacle: IBB distances missing")
        self._check_ibb_stencil(obstacle)
        m = self._m
        _lib.call("lbm_bounce_back_f64", int(bool(self.IBB)), _ptr(links), links.shape[0],
                  _ptr(p), _ptr(m["g_up"].device()), _ptr(m["g"].device()), self.nx, self.ny,
                  _stream())
        m["g"].written()

    def _check_ibb_stencil(self, obstacle):
        """Reject links whose IBB stencil leaves the lattice (IndexError in the reference)."""
        if not self.IBB:
            return
        bnd = np.asarray(obstacle.boundary).reshape(-1, 3)
        p = np.asarray(obstacle.ibb).reshape(-1)
        qb = np.array([0, 2, 1, 4, 3, 6, 5, 8, 7])[bnd[:, 2]]
        for mult, need in ((1, np.ones(len(bnd), bool)), (2, p < 0.5)):
            ii = bnd[:, 0] + mult * _C[qb, 0]
            jj = bnd[:, 1] + mult * _C[qb, 1]
            bad = need & ((ii < -self.nx) | (ii >= self.nx) | (jj < -self.ny) | (jj >= self.ny))
            if bad.any():
                raise IndexError("IBB stencil of link %s leaves the lattice" % (bnd[np.argmax(bad)],))

    def drag_lift(self, obs, R_ref, U_ref, L_ref):
        """nb_drag_lift (nb.py:49-73): momentum exchange over the obstacle links."""
        if self._replay is not None:
            fx, fy = self._replay(obs)
        else:
            _, _, links, n = self._obstacle_links(obs)
            need = _lib.load().lbm_drag_lift_scratch_bytes(n)
            if self._drag_scratch is None or self._drag_scratch.numel() < need:
                self._drag_scratch = torch.empty(need, dtype=torch.uint8, device=self.device)
            m = self._m
            _lib.call("lbm_drag_lift_f64", _ptr(links), n, _ptr(m["g_up"].device()),
                      _ptr(m["g"].device()), self.nx, self.ny, _ptr(self._drag_out),
                      _ptr(self._drag_scratch), _stream())
            fx, fy = self._drag_out.cpu().tolist()
        Cx = -2.0 * fx / (R_ref * L_ref * U_ref ** 2)
        Cy = -2.0 * fy / (R_ref * L_ref * U_ref ** 2)
        return Cx, Cy

    def _zou_he(self, wall, vec_name):
        m = self._m
        rr = m["rho_right"].device() if wall == _lib.WALL_RIGHT_PRESSURE else None
        _lib.call("lbm_zou_he_f64", wall, _ptr(m["u"].device()), _ptr(m["rho"].device()),
                  _ptr(m["g"].device()), _ptr(m[vec_name].device()),
                  _ptr(rr) if rr is not None else None, self.nx, self.ny, _stream())
        for k in ("u", "rho", "g"):
            m[k].written()

    def zou_he_left_wall_velocity(self):
        self._zou_he(_lib.WALL_LEFT_VELOCITY, "u_left")

    def zou_he_right_wall_velocity(self):
        self._zou_he(_lib.WALL_RIGHT_VELOCITY, "u_right")

    def zou_he_right_wall_pressure(self):
        self._zou_he(_lib.WALL_RIGHT_PRESSURE, "u_right")

    def zou_he_top_wall_velocity(self):
        self._zou_he(_lib.WALL_TOP_VELOCITY, "u_top")

    def zou_he_bottom_wall_velocity(self):
        self._zou_he(_lib.WALL_BOTTOM_VELOCITY, "u_bot")

    def _corner(self, corner):
        m = self._m
        _lib.call("lbm_zou_he_corner_f64", corner, _ptr(m["u"].device()), _ptr(m["rho"].device()),
                  _ptr(m["g"].device()), self.nx, self.ny, _stream())
        for k in ("u", "rho", "g"):
            m[k].written()

    def zou_he_bottom_left_corner(self):
        self._corner(_lib.CORNER_BOTTOM_LEFT)

    def zou_he_top_left_corner(self):
        self._corner(_lib.CORNER_TOP_LEFT)

    def zou_he_top_right_corner(self):
        self._corner(_lib.CORNER_TOP_RIGHT)

    def zou_he_bottom_right_corner(self):
        self._corner(_lib.CORNER_BOTTOM_RIGHT)

    # ----------------------------------------------------------------- geometry
    def add_obstacle(self, obstacle):
        """lattice.py:290-375, vectorised (lbm_gb300.geometry.add_obstacle)."""
        print("# Obstacle ", str(obstacle.tag))
        area, bnd, ibb = geometry.add_obstacle(self, obstacle.polygon, obstacle.tag, self.IBB)
        print("# " + str(bnd.shape[0]) + " locations on boundary")
        print("# Area = " + "{:f}".format(area))
        print("")
        return area, bnd, ibb

    def get_coords(self, i, j):
        dx = (self.x_max - self.x_min) / (self.nx - 1)
        dy = (self.y_max - self.y_min) / (self.ny - 1)
        return [self.x_min + i * dx, self.y_min + j * dy]

    def is_inside(self, poly, pt):
        return bool(geometry.points_inside(poly, np.array([pt[0]]), np.array([pt[1]]))[0])

    def generate_image(self, obstacles):
        """Headless: the lattice/link map is saved as .npy instead of a PNG."""
        lat = self.lattice.astype(float)
        for obs in obstacles:
            b = np.asarray(obs.boundary).reshape(-1, 3)
            lat[b[:, 0], b[:, 1]] = -1.0
        np.save(self.output_dir + self.name + "_lattice.npy", np.rot90(lat))

    # ------------------------------------------------------------ device access
    def device_field(self, name, overwrite=False):
        """The float64 device tensor behind ``name`` (synchronised first)."""
        return self._m[name].device(overwrite)

    def mark_written(self, *names):
        for n in names:
            self._m[n].written()
