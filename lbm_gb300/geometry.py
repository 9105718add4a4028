"""Obstacle geometry: polygons and obstacle link lists (host side, NumPy).

Two inputs of the lattice update are prepared here:

* ``generate_shape`` -- the Bezier-sampled polygon of a cylinder, square or
  random shape (lbm/src/utils/shapes.py:253-466).  It is headless: no PNG and
  no CSV are written.  The floating-point operations are kept in the same
  order as the reference so that the polygon, and hence the link list, is
  identical bit for bit.
* ``add_obstacle`` -- the solid mask, the link list ``bnd`` and the IBB
  distances ``ibb`` of one obstacle (lbm/src/core/lattice.py:290-414),
  vectorised over cells and links.  Same crossing-number test, same
  coordinates (``get_coords`` uses (x_max-x_min)/(nx-1) while the IBB
  distance divides by ``dx = (y_max-y_min)/ny``), same negative-index wrap of
  the neighbour test, same ``np.unique`` ordering.
"""
import math
import warnings

import numpy as np
import scipy.special

C = np.array([[0, 0], [1, 0], [-1, 0], [0, 1], [0, -1],
              [1, 1], [-1, -1], [-1, 1], [1, -1]])
NS = np.array([0, 2, 1, 4, 3, 6, 5, 8, 7])


# ---------------------------------------------------------------------------
# Shapes (lbm/src/utils/shapes.py)
# ---------------------------------------------------------------------------
class Shape:
    """Result of ``generate_shape``: control points and the sampled curve."""

    def __init__(self, name, control_pts, curve_pts, radius, edgy, n_sampling_pts):
        self.name = name
        self.control_pts = control_pts
        self.curve_pts = curve_pts
        self.radius = radius
        self.edgy = edgy
        self.n_control_pts = len(control_pts)
        self.n_sampling_pts = n_sampling_pts


def _distance(p1, p2):
    return np.sqrt((p1[0] - p2[0]) ** 2 + (p1[1] - p2[1]) ** 2)


def _cylinder_control_points(n_pts):
    if n_pts < 4:
        raise ValueError("a cylinder needs at least 4 control points")
    ang = 2.0 * math.pi / n_pts
    pts = np.zeros([n_pts, 2])
    for i in range(n_pts):
        pts[i, :] = [0.5 * math.cos(float(i) * ang), 0.5 * math.sin(float(i) * ang)]
    return pts


def _square_control_points(n_pts):
    if n_pts != 4:
        raise ValueError("a square needs exactly 4 control points")
    pts = np.array([[1.0, 1.0], [-1.0, 1.0], [-1.0, -1.0], [1.0, -1.0]])
    pts[:, :] *= 0.5
    return pts


def _ccw_order(pts):
    """Indices sorting points by angle around their mean (shapes.py:329-338)."""
    rel = pts - np.mean(pts, axis=0)
    return np.arctan2(rel[:, 1], rel[:, 0]).argsort()


def _bernstein(n, k, t):
    return scipy.special.binom(n, k) * (t ** k) * ((1.0 - t) ** (n - k))


def _cubic_bezier(p1, p2, d1, d2, db1, db2, r1, r2, e1, e2, n_samples):
    """Cubic Bezier between two control points (shapes.py:366-403)."""
    if n_samples == 0:
        return np.vstack([p1, p2])
    ctrl = np.zeros((4, 2))
    ctrl[0, :] = p1[:]
    ctrl[3, :] = p2[:]
    ctrl[1, :] = p1 + e1 * (r1 * d1) + (1.0 - e1) * (r1 * db1)
    ctrl[2, :] = p2 + e2 * (-r2 * d2) + (1.0 - e2) * (r2 * db2)
    t = np.linspace(0, 1, n_samples)
    curve = np.zeros((n_samples, 2))
    for k in range(4):
        curve += np.outer(_bernstein(3, k, t), ctrl[k])
    return curve


def _drop_duplicates(pts, tol=1.0e-8):
    """Remove points closer than tol to an earlier kept point (shapes.py:292-321)."""
    n = len(pts)
    removed = np.zeros(n, dtype=bool)
    for i in range(n):
        if removed[i]:
            continue
        d = np.sqrt((pts[i, 0] - pts[:, 0]) ** 2 + (pts[i, 1] - pts[:, 1]) ** 2)
        close = (d < tol) & ~removed
        close[i] = False
        removed |= close
    return np.delete(pts, np.nonzero(removed)[0], 0)


def generate_shape(n_pts, position, shape_type, shape_size, shape_name, n_sampling_pts,
                   output_dir=None):
    """Polygon of an obstacle (shapes.py:417-466), without image or CSV output."""
    if shape_type == "cylinder":
        radius = 0.5 * np.ones((n_pts))
        edgy = 1.0 * np.ones((n_pts))
        ctrl = _cylinder_control_points(n_pts)
        ctrl[:, :] *= shape_size
    elif shape_type == "square":
        radius = np.zeros((n_pts))
        edgy = np.ones((n_pts))
        ctrl = _square_control_points(n_pts)
        ctrl[:, :] *= shape_size
    elif shape_type == "random":
        radius = np.random.uniform(low=0.8, high=1.0, size=n_pts)
        edgy = np.random.uniform(low=0.45, high=0.55, size=n_pts)
        ctrl = np.random.rand(n_pts, 2)
        ctrl[:, :] *= shape_size
    else:
        raise ValueError('shape_type must be "cylinder", "square" or "random"')

    ctrl = ctrl - np.mean(ctrl, axis=0)
    order = _ccw_order(ctrl)
    pts = np.array(ctrl)[order, :]
    radius = np.array(radius)[order]
    edgy = np.array(edgy)[order]

    n = n_pts
    delta = np.zeros([n, 2])
    radii = np.zeros([n, 2])
    delta_b = np.zeros([n, 2])
    for i in range(n):
        pm, pc, pn = pts[i - 1, :], pts[i, :], pts[(i + 1) % n, :]
        diff = pn - pm
        delta[i, :] = diff / np.linalg.norm(diff)
        delta_b[i, :] = 0.5 * (pm + pn) - pc
        radii[i, 0] = 0.5 * _distance(pm, pc) * radius[i]
        radii[i, 1] = 0.5 * _distance(pc, pn) * radius[i]

    pieces = []
    for i in range(n):
        nx_ = (i + 1) % n
        pc, pn = pts[i, :], pts[nx_, :]
        smpl = math.ceil(n_sampling_pts * math.sqrt(_distance(pc, pn)))
        pieces.append(_cubic_bezier(pc, pn, delta[i, :], delta[nx_, :], delta_b[i, :],
                                    delta_b[nx_, :], radii[i, 1], radii[nx_, 0], edgy[i],
                                    edgy[nx_], smpl))
    curve = np.concatenate(pieces)
    curve_pts = np.column_stack((curve[:, 0], curve[:, 1], np.zeros(curve.shape[0])))
    curve_pts = _drop_duplicates(curve_pts)

    center = np.mean(curve_pts, axis=0)
    curve_pts -= center
    ctrl_out = ctrl.copy()
    ctrl_out[:, 0:2] -= center[0:2]
    ctrl_out[:, 0:2] += position[0:2]
    curve_pts[:, 0:2] += position[0:2]
    return Shape(shape_name, ctrl_out, curve_pts, radius, edgy, n_sampling_pts)


# ---------------------------------------------------------------------------
# Lattice geometry (lbm/src/core/lattice.py:290-414)
# ---------------------------------------------------------------------------
def cell_coords(x_min, x_max, y_min, y_max, nx, ny):
    """x of every column and y of every row, as lattice.get_coords computes them."""
    dxc = (x_max - x_min) / (nx - 1)
    dyc = (y_max - y_min) / (ny - 1)
    xs = x_min + np.arange(nx, dtype=np.float64) * dxc
    ys = y_min + np.arange(ny, dtype=np.float64) * dyc
    return xs, ys, dxc, dyc


def points_inside(poly, x, y):
    """Crossing-number test of lattice.is_inside, vectorised over points."""
    poly = np.asarray(poly, dtype=np.float64)
    odd = np.zeros(x.shape, dtype=bool)
    n = len(poly)
    j = n - 1
    with np.errstate(divide="ignore", invalid="ignore"):
        for i in range(n):
            xi, yi, xj, yj = poly[i, 0], poly[i, 1], poly[j, 0], poly[j, 1]
            cond = (((yi < y) & (yj >= y)) | ((yj < y) & (yi >= y))) & ((xi < x) | (xj < x))
            if cond.any():
                slope = (xj - xi) / (yj - yi)
                cross = (xi + (y - yi) * slope) < x
                odd ^= cond & cross
            j = i
    return odd


def add_obstacle(lat, polygon, tag, ibb_on):
    """Rasterise one obstacle into ``lat.lattice`` and build its links.

    Returns ``(area, bnd, ibb)``: area in physical units, links ``bnd`` as an
    (n, 3) int64 array of (i, j, q) -- the fluid cell and the direction that
    points into the solid, i/j possibly -1 where the reference's NumPy index
    wraps -- sorted by ``np.unique``, and the IBB distances.
    """
    polygon = np.asarray(polygon, dtype=np.float64)
    nx, ny = lat.nx, lat.ny
    b0, b1 = np.amin(polygon[:, 0]), np.amax(polygon[:, 0])
    b2, b3 = np.amin(polygon[:, 1]), np.amax(polygon[:, 1])
    xs, ys, _, _ = cell_coords(lat.x_min, lat.x_max, lat.y_min, lat.y_max, nx, ny)
    ii = np.nonzero((xs > b0) & (xs < b1))[0]
    jj = np.nonzero((ys > b2) & (ys < b3))[0]
    mask = lat.lattice
    if len(ii) and len(jj):
        I, J = np.meshgrid(ii, jj, indexing="ij")
        inside = points_inside(polygon, xs[I], ys[J])
        si, sj = I[inside], J[inside]
    else:
        si = sj = np.empty(0, dtype=np.int64)
    mask[si, sj] = tag

    links = []
    for q in range(1, 9):
        ni = si + C[q, 0]
        nj = sj + C[q, 1]
        ok = (ni <= nx - 1) & (nj <= ny - 1)
        ni, nj = ni[ok], nj[ok]
        fluid = mask[ni, nj] == 0
        if fluid.any():
            links.append(np.stack([ni[fluid], nj[fluid], np.full(int(fluid.sum()), NS[q])], axis=1))
    if links:
        bnd = np.unique(np.concatenate(links).astype(np.int64), axis=0)
    else:
        bnd = np.empty((0, 3), dtype=np.int64)

    ibb = np.empty(0, dtype=np.float64)
    if ibb_on and len(bnd):
        dxc = (lat.x_max - lat.x_min) / (nx - 1)
        dyc = (lat.y_max - lat.y_min) / (ny - 1)
        px = lat.x_min + bnd[:, 0].astype(np.float64) * dxc
        py = lat.y_min + bnd[:, 1].astype(np.float64) * dyc
        out = np.empty(len(bnd))
        norms = np.array([np.linalg.norm(C[q]) for q in range(9)])
        step = max(1, 4_000_000 // max(1, len(polygon)))
        for s in range(0, len(bnd), step):
            x = polygon[None, :, 0] - px[s:s + step, None]
            y = polygon[None, :, 1] - py[s:s + step, None]
            dist = np.sqrt(np.square(x) + np.square(y))
            out[s:s + step] = np.min(dist, axis=1) / (lat.dx * norms[bnd[s:s + step, 2]])
        ibb = out
        if np.any(ibb > 1.5):
            warnings.warn("obstacle %s: %d IBB distances exceed 1.5 links (max %.2f); the polygon "
                          "is sampled coarser than the lattice and the interpolated bounce-back "
                          "extrapolates" % (tag, int(np.sum(ibb > 1.5)), float(ibb.max())))

    count = int(np.count_nonzero(mask == tag))
    area = float(np.cumsum(np.full(count, lat.dx ** 2))[-1]) if count else 0.0
    return area, bnd, ibb
