"""Host tables of the fused engine (engine.build_tables, ibb_coefficients),
checked against their definitions on the turek cylinder, on random squares
and on squares across the walls (links on wall cells, wrapped indices).  No
GPU."""
import types

import numpy as np
import pytest

from lbm_gb300 import _lib, geometry
from lbm_gb300.apps import turek
from lbm_gb300.engine import build_tables, ibb_coefficients, link_groups

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


@pytest.mark.parametrize("case", list(_cases()), ids=lambda c: c[0])
@pytest.mark.parametrize("pitch", [0, 8])
def test_link_group_tables(case, pitch):
    """Link groups (engine.link_groups): the reordered table holds every
    special cell once, the per-cell kernel's cells first in their original
    order; group cells are off the walls with all links to one obstacle;
    every pull slot and IBB stencil slot names the storage cell it stands
    for; the CSR lists and the corner indices follow the new order."""
    _, nx, ny, obstacles, ibb = case
    tb = build_tables(nx, ny, obstacles, ibb)
    sy = ny if pitch == 0 else -(-ny // pitch) * pitch
    gr = link_groups(tb, nx, ny, sy, ibb, 8, smem_cap=9 * 8 * 64)  # small cap: splits
    sp = gr["special"]
    assert np.array_equal(np.sort(sp), tb["special"])
    nm = gr["n_main"]
    assert np.all(np.diff(sp[:nm]) > 0)
    gc, gs, slot_cell = gr["group_cell_start"], gr["group_slot_start"], gr["slot_cell"]
    assert gc[0] == nm and gc[-1] == len(sp)
    if case[0] != "wall_squares":
        assert len(gc) > 2  # several groups (the small cap splits them)
    assert np.all(np.diff(gs) * 9 * 8 <= 9 * 8 * 64)
    obs_of = np.searchsorted(tb["obs_start"], np.arange(tb["n_links"]), side="right") - 1
    ls, ids = gr["link_start"], gr["link_ids"]
    for s in range(len(sp)):
        k = ids[ls[s]:ls[s + 1]]
        assert np.all(tb["link_cell"][k] == sp[s]) and np.all(np.diff(k) > 0)
    for g in range(len(gc) - 1):
        base = gs[g]
        for s in range(gc[g], gc[g + 1]):
            i, j = sp[s] // ny, sp[s] % ny
            assert 1 <= i <= nx - 2 and 1 <= j <= ny - 2
            k = ids[ls[s]:ls[s + 1]]
            assert len(k) > 0 and len(np.unique(obs_of[k])) == 1
            for q in range(9):
                assert slot_cell[base + gr["pull_slot"][s - nm, q]] == (i - CX[q]) * sy + (j - CY[q])
            if ibb:
                for kk in k:
                    qb = NS[tb["link_q"][kk]]
                    st = lambda r: (r // ny) * sy + r % ny
                    near = tb["p"][kk] < 0.5
                    y1 = st(tb["nb1"][kk]) if near else st(tb["link_cell"][kk])
                    y2 = st(tb["nb2"][kk]) if near else st(tb["nb1"][kk])
                    assert slot_cell[base + gr["link_slot"][kk, 0]] == y1
                    assert slot_cell[base + gr["link_slot"][kk, 1]] == y2
    for c in range(4):
        assert sp[gr["corner_special"][c]] == tb["special"][tb["corner_special"][c]]
        assert sp[gr["corner_nb_special"][c]] == tb["special"][tb["corner_nb_special"][c]]
