"""Base app: hooks called by ``lbm_gb300.run`` (lbm/src/app/base_app.py:10-69).

Besides the reference hooks (initialize, set_inlets, set_bc, outputs,
observables, finalize, printings, check_stop), apps here may implement
``bc_schedule(lattice)`` so that the fused engine can evaluate the inlet
ramp on the device instead of calling ``set_inlets`` every iteration.
"""
import math

import numpy as np

from .. import geometry
from ..engine import pack_bc


class base_app:
    def set_inlets(self, lattice, it):
        pass

    def observables(self, lattice, it):
        pass

    def outputs(self, lattice, it):
        pass

    def finalize(self, lattice):
        pass

    def add_obstacles(self, lattice, obstacles):
        """Polygon, tag, links and IBB distances of every obstacle (base_app.py:27-38)."""
        for i, obs in enumerate(obstacles):
            shape = geometry.generate_shape(obs.n_pts, obs.pos, obs.type, obs.size, obs.name,
                                            obs.n_spts, lattice.output_dir)
            obs.set_polygon(shape.curve_pts)
            obs.set_tag(i + 1)
            area, bnd, ibb = lattice.add_obstacle(obs)
            obs.fill(area, bnd, ibb)

    def printings(self, it):
        if self.stop == "it":
            print("# it = " + str(it) + " / " + str(self.it_max), end="\r")
        if self.stop == "obs":
            str_d = "{:10.6f}".format(self.drag_buff.obs)
            str_l = "{:10.6f}".format(self.lift_buff.obs)
            print("# it = " + str(it) + ", avg drag =" + str_d + ", avg lift =" + str_l, end="\r")

    def check_stop(self, it):
        compute = True
        if self.stop == "it":
            if it >= self.it_max:
                compute = False
                print("\n")
                print("# Computation ended: it>it_max")
        if self.stop == "obs":
            if self.drag_buff.obs_cv and self.lift_buff.obs_cv:
                compute = False
                print("\n")
                print("# Computation ended: converged")
        return compute

    # ---- inlet ramp shared by the apps: ret(it) = 1 - exp(-it^2 / (2 sigma^2))
    def ramp(self, it):
        return 1.0 - math.exp(-it ** 2 / (2.0 * self.sigma ** 2))

    def inlet_vectors(self, lattice):
        """BC entries scaled by u_lbm * ramp(it); None: no device schedule."""
        return None

    def bc_schedule(self, lattice):
        """(base, vec, scale) with BC(it) = base + scale(it) * vec, packed.

        ``set_inlets(lattice, 0)`` (ramp 0) leaves the constant entries in the
        lattice's BC vectors; ``inlet_vectors`` gives the ramped profile.
        """
        vec = self.inlet_vectors(lattice)
        if vec is None:
            return None
        self.set_inlets(lattice, 0)
        nx, ny = lattice.nx, lattice.ny
        base = pack_bc({k: getattr(lattice, k) for k in
                        ("u_left", "u_right", "u_top", "u_bot", "rho_right")}, nx, ny)
        full = {"u_left": np.zeros((2, ny)), "u_right": np.zeros((2, ny)),
                "u_top": np.zeros((2, nx)), "u_bot": np.zeros((2, nx)),
                "rho_right": np.zeros(ny)}
        full.update(vec)
        vpk = pack_bc(full, nx, ny)
        u_lbm = self.u_lbm

        def scale(its):
            return np.array([u_lbm * self.ramp(int(it)) for it in its], dtype=np.float64)

        return base, vpk, scale


def poiseuille_profile(app, lattice):
    """Inlet profile 4 (y_max - y)(y - y_min) / H^2 at get_coords(0, j)."""
    H = app.y_max - app.y_min
    prof = np.zeros((2, lattice.ny))
    for j in range(lattice.ny):
        y = lattice.get_coords(0, j)[1]
        prof[0, j] = 4.0 * (app.y_max - y) * (y - app.y_min) / H ** 2
    return prof
