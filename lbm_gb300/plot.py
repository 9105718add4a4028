"""Headless field output.

The reference writes a PNG of |u| with matplotlib (lbm/src/plot/plot.py:9-32).
There is no graphics stack here, so ``plot_norm`` writes the same masked
field (|u|, obstacles set to -1, rotated by 90 degrees like the image) as a
``.npy`` array next to where the PNG would go.
"""
import os

import numpy as np


def norm_field(lattice):
    u = lattice.u
    v = np.sqrt(u[0, :, :] ** 2 + u[1, :, :] ** 2)
    v[np.where(np.asarray(lattice.lattice) > 0.0)] = -1.0
    return np.rot90(v)


def plot_norm(lattice, val_min, val_max, output_it, dpi):
    v = norm_field(lattice)
    png_dir = getattr(lattice, "png_dir", None)
    if png_dir:
        os.makedirs(png_dir, exist_ok=True)
        np.save(os.path.join(png_dir, "u_norm_%d.npy" % output_it), v)
    return v
