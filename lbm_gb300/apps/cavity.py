"""Lid-driven cavity (parameters and hooks of lbm/src/app/cavity.py:11-133)."""
import math

import numpy as np

from .base_app import base_app
from ..plot import plot_norm


class cavity(base_app):
    def __init__(self):
        self.name = "cavity"
        self.Re_lbm = 100.0
        self.L_lbm = 100
        self.u_lbm = 0.2
        self.rho_lbm = 1.0
        self.t_max = 20.0
        self.x_min, self.x_max = 0.0, 1.0
        self.y_min, self.y_max = 0.0, 1.0
        self.stop = "it"
        self.output_freq = 500
        self.output_it = 0
        self.dpi = 200
        self.compute_lbm_parameters()

    def compute_lbm_parameters(self):
        self.Cs = 1.0 / math.sqrt(3.0)
        self.ny = self.L_lbm
        self.nu_lbm = self.u_lbm * self.L_lbm / self.Re_lbm
        self.tau_lbm = 0.5 + self.nu_lbm / (self.Cs ** 2)
        self.dt = self.Re_lbm * self.nu_lbm / self.L_lbm ** 2
        self.dx = (self.y_max - self.y_min) / self.ny
        self.dy = self.dx
        self.nx = math.floor(self.ny * (self.x_max - self.x_min) / (self.y_max - self.y_min))
        self.it_max = math.floor(self.t_max / self.dt)
        self.sigma = math.floor(10 * self.nx)

    def initialize(self, lattice):
        self.set_inlets(lattice, 0)
        lattice.rho *= self.rho_lbm
        lattice.generate_image([])
        lattice.equilibrium()
        lattice.g = lattice.g_eq.copy()

    def set_inlets(self, lattice, it):
        ret = self.ramp(it)
        lattice.u_top[0, :] = self.u_lbm * ret
        lattice.u_bot[0, :] = 0.0
        lattice.u_left[1, :] = 0.0
        lattice.u_right[1, :] = 0.0

    def inlet_vectors(self, lattice):
        top = np.zeros((2, lattice.nx))
        top[0, :] = 1.0
        return {"u_top": top}

    def set_bc(self, lattice):
        lattice.zou_he_bottom_wall_velocity()
        lattice.zou_he_left_wall_velocity()
        lattice.zou_he_right_wall_velocity()
        lattice.zou_he_top_wall_velocity()
        lattice.zou_he_bottom_left_corner()
        lattice.zou_he_top_left_corner()
        lattice.zou_he_top_right_corner()
        lattice.zou_he_bottom_right_corner()

    def outputs(self, lattice, it):
        if it % self.output_freq != 0:
            return
        plot_norm(lattice, 0.0, 1.0, self.output_it, self.dpi)
        self.output_it += 1

    def finalize(self, lattice):
        self.line_fields(lattice)

    def line_fields(self, lattice):
        """Centre-line profiles u_y(x) and u_x(y) over u_lbm, written to files."""
        u = lattice.u
        nx2 = math.floor(self.nx / 2)
        ny2 = math.floor(self.ny / 2)
        vx_error = u[1, :, ny2] / self.u_lbm
        uy_error = u[0, nx2, :] / self.u_lbm
        with open(lattice.output_dir + "cavity_vx", "w") as f:
            for i in range(self.nx):
                f.write("{} {}\n".format(i * self.dx, vx_error[i]))
        with open(lattice.output_dir + "cavity_uy", "w") as f:
            for j in range(self.ny):
                f.write("{} {}\n".format(j * self.dx, uy_error[j]))
        return vx_error, uy_error
