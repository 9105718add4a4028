"""Channel apps: turek, poiseuille, array, step (lbm/src/app/{turek,poiseuille,
array,step}.py) and the large obstacle array.

All share the ramped parabolic Zou-He inlet, the Zou-He pressure outlet and
no-slip top/bottom walls; they differ in geometry, obstacles and
observables.
"""
import math
import os

import numpy as np

from .base_app import base_app, poiseuille_profile
from ..buff import buff
from ..obstacle import obstacle
from ..plot import plot_norm


class _channel(base_app):
    """Ramped parabolic inlet, pressure outlet, walls, optional obstacles."""

    obstacles = ()

    def _derive(self, nu_length):
        self.Cs = 1.0 / math.sqrt(3.0)
        self.ny = self.L_lbm
        self.u_avg = 2.0 * self.u_lbm / 3.0
        self.nu_lbm = self.u_avg * nu_length / self.Re_lbm
        self.tau_lbm = 0.5 + self.nu_lbm / (self.Cs ** 2)
        self.dt = self.Re_lbm * self.nu_lbm / nu_length ** 2
        self.dx = (self.y_max - self.y_min) / self.ny
        self.dy = self.dx
        self.nx = math.floor(self.ny * (self.x_max - self.x_min) / (self.y_max - self.y_min))
        self.it_max = math.floor(self.t_max / self.dt)
        self.sigma = math.floor(10 * self.nx)

    def initialize(self, lattice):
        if self.obstacles:
            self.add_obstacles(lattice, self.obstacles)
        self.set_inlets(lattice, 0)
        if self.obstacles:
            lattice.u[:, np.where(lattice.lattice > 0.0)] = 0.0
        lattice.rho *= self.rho_lbm
        lattice.generate_image(list(self.obstacles))
        self.init_observables(lattice)
        lattice.equilibrium()
        lattice.g = lattice.g_eq.copy()

    def init_observables(self, lattice):
        pass

    def poiseuille(self, pt):
        y = pt[1]
        H = self.y_max - self.y_min
        u = np.zeros(2)
        u[0] = 4.0 * (self.y_max - y) * (y - self.y_min) / H ** 2
        return u

    def set_inlets(self, lattice, it):
        ret = self.ramp(it)
        lattice.u_left = (ret * self.u_lbm) * poiseuille_profile(self, lattice)
        lattice.u_top[0, :] = 0.0
        lattice.u_bot[0, :] = 0.0
        lattice.u_right[1, :] = 0.0
        lattice.rho_right[:] = self.rho_lbm

    def inlet_vectors(self, lattice):
        return {"u_left": poiseuille_profile(self, lattice)}

    def set_bc(self, lattice):
        for obs in self.obstacles:
            lattice.bounce_back_obstacle(obs)
        lattice.zou_he_bottom_wall_velocity()
        lattice.zou_he_left_wall_velocity()
        lattice.zou_he_top_wall_velocity()
        lattice.zou_he_right_wall_pressure()
        lattice.zou_he_bottom_left_corner()
        lattice.zou_he_top_left_corner()
        lattice.zou_he_top_right_corner()
        lattice.zou_he_bottom_right_corner()

    def outputs(self, lattice, it):
        if it % self.output_freq != 0:
            return
        plot_norm(lattice, 0.0, 1.5, self.output_it, self.dpi)
        self.output_it += 1


class turek(_channel):
    """Turek cylinder benchmark (lbm/src/app/turek.py:10-173)."""

    def __init__(self):
        self.name = "turek"
        self.Re_lbm = 100.0
        self.L_lbm = 151
        self.u_lbm = 0.05
        self.rho_lbm = 1.0
        self.t_max = 0.02
        self.x_min, self.x_max = -0.2, 2.0
        self.y_min, self.y_max = -0.2, 0.21
        self.IBB = True
        self.stop = "obs"
        self.obs_cv_ct = 1.0e-3
        self.obs_cv_nb = 1000
        self.output_freq = 500
        self.output_it = 0
        self.dpi = 200
        self.compute_lbm_parameters()
        self.obstacles = [obstacle("turek", 200, 2, "cylinder", self.r_cyl, [0.0, 0.0])]

    def compute_lbm_parameters(self):
        self.r_cyl = 0.1
        self.D_lbm = math.floor(self.L_lbm * self.r_cyl / (self.y_max - self.y_min))
        self._derive(self.D_lbm)

    def init_observables(self, lattice):
        self.drag_buff = buff("drag", lattice.dt, lattice.obs_cv_ct, lattice.obs_cv_nb,
                              lattice.output_dir)
        self.lift_buff = buff("lift", lattice.dt, lattice.obs_cv_ct, lattice.obs_cv_nb,
                              lattice.output_dir)
        self._lines = []
        self._dl_file = lattice.output_dir + "drag_lift"

    def observables(self, lattice, it):
        drag, lift = lattice.drag_lift(self.obstacles[0], self.rho_lbm, self.u_avg, self.D_lbm)
        self.add_buff(drag, lift, lattice, it)

    def observables_chunk(self, lattice, first, rows, obstacles, stop_check=True):
        """``observables`` (and ``check_stop`` when stop_check) of iterations
        first .. first + len(rows) - 1 at once, for the fused runner.

        rows[k, o] is the raw (fx, fy) of obstacles[o] (the runner's list, in
        set_bc order) at iteration first + k: what ``lattice.drag_lift``
        normalises.  The coefficients, the buffers' moving averages (on the
        GPU, ``buff.add_chunk``) and the drag_lift lines are those of the
        per-iteration calls, bit for bit.  Returns the iteration at which
        check_stop ends the run (the observables stop there too) or None.
        """
        n = len(rows)
        if n == 0:
            return None
        o = next(k for k, ob in enumerate(obstacles) if ob is self.obstacles[0])
        den = self.rho_lbm * self.D_lbm * self.u_avg ** 2
        cx = -2.0 * rows[:, o, 0] / den
        cy = -2.0 * rows[:, o, 1] / den
        saved = [(b.it, b.obs, b.obs_cv_cnt, b.obs_cv,
                  None if b._state is None else b._state.clone())
                 for b in (self.drag_buff, self.lift_buff)]
        ax, gx, vx = self.drag_buff.add_chunk(cx)
        ay, gy, vy = self.lift_buff.add_chunk(cy)
        its = np.arange(first, first + n)
        stop = None
        if stop_check:
            if self.stop == "obs":
                hit = np.flatnonzero(vx & vy)
            elif self.stop == "it":
                hit = np.flatnonzero(its >= self.it_max)
            else:
                hit = np.zeros(0, np.int64)
            if len(hit):
                t = int(hit[0])
                stop = first + t
                if t < n - 1:
                    # the run ends inside the chunk: redo the buffers up to it
                    for b, (it0, obs, cnt, cv, st) in zip((self.drag_buff, self.lift_buff),
                                                          saved):
                        b.it, b.obs, b.obs_cv_cnt, b.obs_cv = it0, obs, cnt, cv
                        if st is not None:
                            b._state.copy_(st)
                        else:
                            b._state = None
                    ax, gx, _ = self.drag_buff.add_chunk(cx[:t + 1])
                    ay, gy, _ = self.lift_buff.add_chunk(cy[:t + 1])
                    its, cx, cy = its[:t + 1], cx[:t + 1], cy[:t + 1]
                self.check_stop(stop)
        self._write_lines(its * self.dt, cx, cy, ax, ay, gx, gy)
        return stop

    def _write_lines(self, *cols):
        """Append drag_lift lines ('{} {} {} {} {} {} {}' of the columns) from
        a writer thread, in submission order, after any pending lines."""
        import concurrent.futures
        if getattr(self, "_writer", None) is None:
            self._writer = concurrent.futures.ThreadPoolExecutor(1)
            self._writes = []
        cols = [np.asarray(c, dtype=np.float64).copy() for c in cols]
        path = self._dl_file
        pending = self._lines
        self._lines = []

        def work():
            strs = [list(map(repr, c.tolist())) for c in cols]
            text = "".join(pending) + "".join(" ".join(t) + "\n" for t in zip(*strs))
            with open(path, "a") as f:
                f.write(text)

        for w in [w for w in self._writes if w.done()]:
            w.result()  # raises a failed write here
        self._writes = [w for w in self._writes if not w.done()]
        self._writes.append(self._writer.submit(work))

    def add_buff(self, Cx, Cy, lattice, it):
        self.drag_buff.add(Cx)
        self.lift_buff.add(Cy)
        avg_Cx, dcx = self.drag_buff.mv_avg()
        avg_Cy, dcy = self.lift_buff.mv_avg()
        self._lines.append("{} {} {} {} {} {} {}\n".format(it * self.dt, Cx, Cy, avg_Cx, avg_Cy,
                                                          dcx, dcy))
        if len(self._lines) >= 4096:
            self.flush_observables()

    def flush_observables(self):
        for w in getattr(self, "_writes", ()):
            w.result()
        self._writes = []
        if getattr(self, "_lines", None):
            with open(self._dl_file, "a") as f:
                f.writelines(self._lines)
            self._lines = []

    def finalize(self, lattice):
        self.flush_observables()


class poiseuille(_channel):
    """Poiseuille channel (lbm/src/app/poiseuille.py:13-152)."""

    def __init__(self):
        self.name = "poiseuille"
        self.Re_lbm = 100.0
        self.L_lbm = 50
        self.u_lbm = 0.1
        self.rho_lbm = 1.0
        self.t_max = 15.0
        self.x_min, self.x_max = -0.2, 1.0
        self.y_min, self.y_max = -0.2, 0.2
        self.stop = "it"
        self.output_freq = 50000
        self.output_it = 0
        self.dpi = 200
        self.compute_lbm_parameters()
        self.obstacles = []

    def compute_lbm_parameters(self):
        self._derive(self.L_lbm)

    def finalize(self, lattice):
        self.compute_error(lattice)

    def compute_error(self, lattice):
        """L1 error of the mid-channel profile against the parabola."""
        u = lattice.u
        nx2 = math.floor(self.nx / 2)
        u_error = np.zeros((3, self.ny))
        l1_error = 0.0
        for j in range(self.ny):
            pt = lattice.get_coords(nx2, j)
            u_ex = self.poiseuille(pt)
            u_error[0, j] = u[0, nx2, j] / self.u_lbm
            u_error[1, j] = u_ex[0]
            u_error[2, j] = abs(u_error[0, j] - u_error[1, j])
            l1_error += u_error[2, j] * self.dx
        with open(lattice.output_dir + "poiseuille", "w") as f:
            for j in range(self.ny):
                f.write("{} {} {}\n".format(j * self.dx, u_error[0, j], u_error[1, j]))
        return l1_error


class array(_channel):
    """Ring of square obstacles (lbm/src/app/array.py:13-144)."""

    def __init__(self):
        self.name = "array"
        self.Re_lbm = 2000.0
        self.L_lbm = 200
        self.u_lbm = 0.025
        self.rho_lbm = 1.0
        self.t_max = 7.5
        self.x_min, self.x_max = -1.0, 8.0
        self.y_min, self.y_max = -1.0, 1.0
        self.IBB = True
        self.stop = "it"
        self.obs_cv_ct = 1.0e-3
        self.obs_cv_nb = 1000
        self.n_obs = 8
        self.r_obs = 0.1
        self.output_freq = 500
        self.output_it = 0
        self.dpi = 200
        self.compute_lbm_parameters()
        radius = 0.5
        self.obstacles = []
        for i in range(self.n_obs):
            pos = [radius * math.cos(2.0 * math.pi * float(i) / self.n_obs),
                   radius * math.sin(2.0 * math.pi * float(i) / self.n_obs) + 0.01]
            self.obstacles.append(obstacle("array", 4, 100, "square", self.r_obs, pos))

    def compute_lbm_parameters(self):
        self.r_cyl = 0.1
        self.D_lbm = math.floor(self.L_lbm * self.r_cyl / (self.y_max - self.y_min))
        self._derive(self.L_lbm)


class step(_channel):
    """Two squares making a step, plain bounce-back (lbm/src/app/step.py:11-139)."""

    def __init__(self):
        self.name = "step"
        self.Re_lbm = 500.0
        self.L_lbm = 150
        self.u_lbm = 0.05
        self.rho_lbm = 1.0
        self.t_max = 15.0
        self.x_min, self.x_max = -1.0, 15.0
        self.y_min, self.y_max = -1.0, 1.0
        self.IBB = False
        self.stop = "it"
        self.obs_cv_ct = 1.0e-3
        self.obs_cv_nb = 1000
        self.output_freq = 500
        self.output_it = 0
        self.dpi = 200
        self.compute_lbm_parameters()
        self.obstacles = [obstacle("square1", 4, 100, "square", 1.5, [1.5, 1.0]),
                          obstacle("square2", 4, 100, "square", 1.5, [4.0, -1.0])]

    def compute_lbm_parameters(self):
        self.r_cyl = 0.5
        self.D_lbm = math.floor(self.L_lbm * self.r_cyl / (self.y_max - self.y_min))
        self._derive(self.L_lbm)


class obstacle_array(_channel):
    """Large channel with a seeded, jittered grid of square obstacles.

    Defaults: ny = 2048, nx = 4 ny = 8192 (16.8 M cells), 20 x 20 squares of
    side 0.02 H (about 41 cells) with centres jittered by up to 20% of the
    grid pitch, Re = 2000 on the square side, parabolic Zou-He inlet,
    pressure outlet, IBB links on every square.
    """

    def __init__(self, L_lbm=2048, n_grid=(20, 20), side=0.02, Re_side=2000.0, u_lbm=0.05,
                 seed=2024, jitter=0.2, n_spts=None):
        self.name = "obstacle_array"
        self.Re_lbm = Re_side
        self.L_lbm = L_lbm
        self.u_lbm = u_lbm
        self.rho_lbm = 1.0
        self.t_max = 1.0
        self.x_min, self.x_max = 0.0, 4.0
        self.y_min, self.y_max = 0.0, 1.0
        self.IBB = True
        self.stop = "it"
        self.obs_cv_ct = 1.0e-3
        self.obs_cv_nb = 1000
        self.output_freq = 10 ** 9
        self.output_it = 0
        self.dpi = 200
        self.side = side
        self.compute_lbm_parameters()
        if n_spts is None:
            # The IBB distance is measured to the nearest polygon sample
            # (lattice.py:350-361): sample each side finer than half a cell
            # (a side gets ceil(n_spts sqrt(side)) samples, shapes.py:104).
            n_spts = max(4, math.ceil(side / (0.4 * self.dx) / math.sqrt(side)))
        rng = np.random.default_rng(seed)
        gx, gy = n_grid
        px = (self.x_max - self.x_min) / gx
        py = (self.y_max - self.y_min) / gy
        self.obstacles = []
        # keep every square at least 3 cells away from the walls so that the
        # IBB stencil (x + 2 c) stays inside the lattice
        margin = 0.5 * side + 3.0 * self.dx
        for a in range(gx):
            for b in range(gy):
                jx, jy = jitter * (rng.random(2) - 0.5) * 2.0
                pos = [self.x_min + (a + 0.5 + jx) * px, self.y_min + (b + 0.5 + jy) * py]
                pos[0] = min(max(pos[0], self.x_min + margin), self.x_max - margin)
                pos[1] = min(max(pos[1], self.y_min + margin), self.y_max - margin)
                self.obstacles.append(obstacle("sq%d_%d" % (a, b), 4, n_spts, "square", side, pos))

    def compute_lbm_parameters(self):
        self.D_lbm = max(1, math.floor(self.L_lbm * self.side / (self.y_max - self.y_min)))
        self._derive(self.D_lbm)

    def init_observables(self, lattice):
        n = len(self.obstacles)
        self.drag = np.zeros(n)
        self.lift = np.zeros(n)
        self.drag_sum = np.zeros(n)
        self.n_obs_it = 0

    def observables(self, lattice, it):
        """Drag and lift coefficient of every square, every iteration."""
        for k, obs in enumerate(self.obstacles):
            self.drag[k], self.lift[k] = lattice.drag_lift(obs, self.rho_lbm, self.u_avg,
                                                           self.D_lbm)
        self.drag_sum += self.drag
        self.n_obs_it += 1
