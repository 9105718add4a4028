"""Host tables of the fused engine (engine.build_tables, ibb_coefficients),
checked against their definitions on the turek cylinder, on random squares
and on squares across the walls (links on wall cells, wrapped indices).  No
GPU."""
import types

import numpy as np
import pytest

from lbm_gb300 import _lib, geometry
from lbm_gb300.apps import turek
from lbm_gb300.engine import build_tables, ibb_coefficients

CX = np.array([0, 1, -1, 0, 0, 1, -1, -1, 1])
CY = np.array([0, 0, 0, 1, -1, 1, -1, 1, -1])
NS = np.array([0, 2, 1, 4, 3, 6, 5, 8, 7])


def _obstacles(nx, ny, shapes, x_min=0.0, x_max=None, y_min=0.0, y_max=1.0):
    x_max = x_max if x_max is not None else nx / ny
    lat = types.SimpleNamespace(nx=nx, ny=ny, x_min=x_min, x_max=x_max, y_min=y_min,
                                y_max=y_max, dx=(y_max - y_min) / ny, lattice=np.zeros((nx, ny)))
    out = []
    for tag, (kind, pos, size) in enumerate(shapes, start=1):
        n_pts = 4 if kind == "square" else 6
        s = geometry.generate_shape(n_pts, pos, kind, size, "o%d" % tag, 50)
        _, bnd, ibb = geometry.add_obstacle(lat, s.curve_pts, tag, True)
        out.append(types.SimpleNamespace(name="o%d" % tag, boundary=bnd, ibb=ibb))
    return out


def _cases():
    app = turek()
    app.L_lbm = 40
    app.compute_lbm_parameters()
    o = app.obstacles[0]
    s = geometry.generate_shape(o.n_pts, o.pos, o.type, o.size, o.name, o.n_spts)
    lat = types.SimpleNamespace(nx=app.nx, ny=app.ny, x_min=app.x_min, x_max=app.x_max,
                                y_min=app.y_min, y_max=app.y_max, dx=app.dx,
                                lattice=np.zeros((app.nx, app.ny)))
    _, bnd, ibb = geometry.add_obstacle(lat, s.curve_pts, 1, True)
    yield "turek40", app.nx, app.ny, [types.SimpleNamespace(name="cyl", boundary=bnd, ibb=ibb)], True
    rng = np.random.default_rng(11)
    for k in range(3):
        nx, ny = int(rng.integers(40, 80)), int(rng.integers(24, 48))
        shapes = [("square", [float(rng.uniform(0.3, nx / ny - 0.3)), float(rng.uniform(0.25, 0.75))],
                   float(rng.uniform(0.1, 0.25))) for _ in range(3)]
        yield "squares%d" % k, nx, ny, _obstacles(nx, ny, shapes), True
    # squares across the bottom and top walls with halfway bounce-back (as
    # in the reference's step app): links on wall cells, wrapped (negative)
    # indices
    nx, ny = 60, 30
    yield "wall_squares", nx, ny, _obstacles(nx, ny, [("square", [0.6, 0.05], 0.2),
                                                      ("square", [1.3, 0.97], 0.15)]), False


@pytest.mark.parametrize("case", list(_cases()), ids=lambda c: c[0])
def test_special_and_link_tables(case):
    _, nx, ny, obstacles, ibb = case
    tb = build_tables(nx, ny, obstacles, ibb)
    special, ls, ids = tb["special"], tb["link_start"], tb["link_ids"]
    n_links = sum(len(o.boundary) for o in obstacles)
    assert tb["n_links"] == n_links and n_links > 0
    # every wall cell and every link cell, each once, sorted
    I, J = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    wall = ((I == 0) | (I == nx - 1) | (J == 0) | (J == ny - 1)).ravel()
    expect = np.union1d(np.flatnonzero(wall), tb["link_cell"])
    assert np.array_equal(special, expect)
    if case[0] == "wall_squares":
        assert np.any(wall[tb["link_cell"]])  # a wall cell that owns links
        assert np.any(np.concatenate([np.asarray(o.boundary)[:, 1] for o in obstacles]) < 0)
    # CSR: the links of special cell s are the links whose cell it is, in
    # their set_bc order (so the last one wins as in the reference loop)
    assert ls[0] == 0 and ls[-1] == n_links and np.all(np.diff(ls) >= 0)
    assert np.array_equal(np.sort(ids), np.arange(n_links))
    for s in range(len(special)):
        k = ids[ls[s]:ls[s + 1]]
        assert np.all(tb["link_cell"][k] == special[s])
        assert np.all(np.diff(k) > 0)
    # IBB neighbours x + c_qb and x + 2 c_qb (wrapped), as the reference indexes
    bnd = np.concatenate([np.asarray(o.boundary).reshape(-1, 3) for o in obstacles])
    qb = NS[bnd[:, 2]]
    for mult, key in ((1, "nb1"), (2, "nb2")) if ibb else ():
        ii = (bnd[:, 0] + mult * CX[qb]) % nx
        jj = (bnd[:, 1] + mult * CY[qb]) % ny
        need = np.ones(n_links, bool) if mult == 1 else tb["p"] < 0.5
        assert np.array_equal(tb[key][need], (ii * ny + jj)[need])
    # obstacle ranges over the concatenated links
    assert np.array_equal(tb["obs_start"], np.cumsum([0] + [len(o.boundary) for o in obstacles]))
    # corners and their x-neighbours
    for c, (i, j) in {_lib.CORNER_BOTTOM_LEFT: (0, 0), _lib.CORNER_TOP_LEFT: (0, ny - 1),
                      _lib.CORNER_TOP_RIGHT: (nx - 1, ny - 1),
                      _lib.CORNER_BOTTOM_RIGHT: (nx - 1, 0)}.items():
        assert special[tb["corner_special"][c]] == i * ny + j
        assert special[tb["corner_nb_special"][c]] == (1 if i == 0 else nx - 2) * ny + j


def test_ibb_coefficients_follow_the_reference_expressions():
    """The three factors of nb.py:98-104 in the reference's evaluation order."""
    rng = np.random.default_rng(3)
    p = np.concatenate([rng.uniform(0.0, 1.0, 200), [0.0, 0.25, 0.5, 0.75, 1.0]])
    c = ibb_coefficients(p)
    for k, pk in enumerate(p):
        pp = 2.0 * pk
        if pk < 0.5:
            want = (pk * (pp + 1.0), (1.0 + pp) * (1.0 - pp), pk * (1.0 - pp))
        else:
            want = (1.0 / (pk * (pp + 1.0)), (pp - 1.0) / pk, (1.0 - pp) / (1.0 + pp))
        assert tuple(c[:, k]) == want, pk


def test_links_leaving_the_lattice_are_refused():
    ob = types.SimpleNamespace(name="bad", boundary=np.array([[5, 3, 9]]), ibb=np.array([0.3]))
    with pytest.raises(ValueError):
        build_tables(10, 8, [ob], True)
    ob = types.SimpleNamespace(name="bad", boundary=np.array([[12, 3, 1]]), ibb=np.array([0.3]))
    with pytest.raises(IndexError):
        build_tables(10, 8, [ob], True)
