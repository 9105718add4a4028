"""Headless output: plot_norm writes the field the reference's plot_norm
draws (lbm/src/plot/plot.py:9-32: |u|, obstacle cells at -1, rotated by 90
degrees) as u_norm_<it>.npy in the lattice's png directory.  No GPU."""
import os
import tempfile
import types

import numpy as np

from lbm_gb300.plot import plot_norm


def test_plot_norm_writes_the_masked_rotated_norm():
    rng = np.random.default_rng(4)
    nx, ny = 9, 6
    u = rng.standard_normal((2, nx, ny))
    mask = np.zeros((nx, ny))
    mask[3:5, 2:4] = 1.0
    with tempfile.TemporaryDirectory() as d:
        lat = types.SimpleNamespace(u=u, lattice=mask, png_dir=os.path.join(d, "png"),
                                    u_lbm=0.1)
        v = plot_norm(lat, 0.0, 1.5, 12, 100)
        saved = np.load(os.path.join(d, "png", "u_norm_12.npy"))
    want = np.sqrt(u[0] ** 2 + u[1] ** 2)
    want[mask > 0.0] = -1.0
    want = np.rot90(want)
    assert np.array_equal(saved, want)
    assert np.array_equal(v, want)
    assert saved.shape == (ny, nx)
