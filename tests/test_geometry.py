"""Vectorised geometry (polygons, masks, links, IBB distances) against the
reference's own outputs and against the cell-by-cell oracle restatement."""
import types

import numpy as np
import pytest

from _cases import golden
from lbm_gb300 import geometry
from lbm_gb300.apps import turek
from oracle import oracle as O


def _lat(app):
    lat = types.SimpleNamespace(nx=app.nx, ny=app.ny, x_min=app.x_min, x_max=app.x_max,
                                y_min=app.y_min, y_max=app.y_max, dx=app.dx,
                                lattice=np.zeros((app.nx, app.ny)))
    return lat


@pytest.mark.parametrize("L,count", [(24, None), (100, 234), (200, 468)])
def test_turek_links_match_reference(L, count):
    """lbm/tst/lattice/test_lattice.py: 234 links at L=100, 468 at L=200."""
    d = golden("geometry.npz")
    app = turek()
    app.L_lbm = L
    app.compute_lbm_parameters()
    obs = app.obstacles[0]
    shape = geometry.generate_shape(obs.n_pts, obs.pos, obs.type, obs.size, obs.name, obs.n_spts)
    assert np.array_equal(shape.curve_pts, d["turek%d_poly" % L])
    lat = _lat(app)
    area, bnd, ibb = geometry.add_obstacle(lat, shape.curve_pts, 1, True)
    assert np.array_equal(bnd, d["turek%d_bnd" % L])
    assert np.array_equal(ibb, d["turek%d_ibb" % L])
    assert area == float(d["turek%d_area" % L])
    assert np.array_equal(lat.lattice.astype(np.int8), d["turek%d_mask" % L])
    if count is not None:
        assert bnd.shape[0] == count


def test_square_polygon_matches_reference():
    d = golden("geometry.npz")
    s = geometry.generate_shape(4, [0.3, -0.2], "square", 0.37, "sq", 100)
    assert np.array_equal(s.curve_pts, d["square_poly"])


@pytest.mark.parametrize("seed", range(6))
def test_vectorised_matches_cell_loops(seed):
    """Random polygons, including ones touching the walls (negative wrap)."""
    rng = np.random.default_rng(seed)
    nx, ny = int(rng.integers(20, 40)), int(rng.integers(12, 30))
    lat_a = types.SimpleNamespace(nx=nx, ny=ny, x_min=-0.3, x_max=1.7, y_min=-0.2, y_max=0.6,
                                  dx=0.8 / ny, lattice=np.zeros((nx, ny)))
    lat_b = types.SimpleNamespace(**{k: (v.copy() if isinstance(v, np.ndarray) else v)
                                     for k, v in vars(lat_a).items()})
    for tag in (1, 2):
        kind = ["cylinder", "square", "random"][int(rng.integers(0, 3))]
        n_pts = 4 if kind == "square" else int(rng.integers(5, 9))
        pos = [float(rng.uniform(-0.3, 1.5)), float(rng.uniform(-0.2, 0.6))]
        np.random.seed(seed * 10 + tag)
        s = geometry.generate_shape(n_pts, pos, kind, float(rng.uniform(0.1, 0.5)), "s", 6)
        ra = geometry.add_obstacle(lat_a, s.curve_pts, tag, True)
        rb = O.add_obstacle_loops(lat_b, s.curve_pts, tag, True)
        assert np.array_equal(ra[1], rb[1])
        assert np.array_equal(ra[2], rb[2])
        assert ra[0] == rb[0]
        assert np.array_equal(lat_a.lattice, lat_b.lattice)


@pytest.mark.parametrize("k", [0, 137, 399])
def test_obstacle_array_squares_match_cell_loops(k):
    """Squares of the obstacle-array workload (ny 128: 2-cell squares; the
    parity tests use the vectorised links at ny 256 and 2048)."""
    from lbm_gb300.apps import obstacle_array
    app = obstacle_array(L_lbm=128)
    obs = app.obstacles[k]
    s = geometry.generate_shape(obs.n_pts, obs.pos, obs.type, obs.size, obs.name, obs.n_spts)
    lat_a, lat_b = _lat(app), _lat(app)
    ra = geometry.add_obstacle(lat_a, s.curve_pts, k + 1, True)
    rb = O.add_obstacle_loops(lat_b, s.curve_pts, k + 1, True)
    assert len(rb[1]) > 0
    assert np.array_equal(ra[1], rb[1])
    assert np.array_equal(ra[2], rb[2])
    assert ra[0] == rb[0]
    assert np.array_equal(lat_a.lattice, lat_b.lattice)
