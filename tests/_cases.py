"""Shared test cases: the golden runs and helpers to run them on the oracle
(CPU) or on the GPU lattice."""
import contextlib
import io
import os
import tempfile

import numpy as np

from lbm_gb300.apps import cavity, turek, poiseuille, step, array

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden(name):
    return np.load(os.path.join(GOLDEN, name))


def make_case(name):
    """App configured exactly as tests/golden/make_golden.py configures it."""
    if name == "cavity32":
        a = cavity()
        a.L_lbm, a.u_lbm = 32, 0.1
        a.compute_lbm_parameters()
        a.sigma, n = 100.0, 1000
    elif name == "poiseuille20":
        a = poiseuille()
        a.L_lbm = 20
        a.compute_lbm_parameters()
        a.sigma, n = 60.0, 600
    elif name == "turek24":
        a = turek()
        a.L_lbm = 24
        a.Re_lbm = 20.0
        a.compute_lbm_parameters()
        a.sigma, n = 40.0, 400
    elif name == "step20":
        a = step()
        a.L_lbm = 20
        a.compute_lbm_parameters()
        a.sigma, n = 40.0, 300
    elif name == "array32":
        a = array()
        a.L_lbm = 32
        a.compute_lbm_parameters()
        a.sigma, n = 40.0, 300
    else:
        raise KeyError(name)
    a.stop = "it"
    a.it_max = n - 1
    a.output_freq = 10 ** 12
    return a, n


CASES = ["cavity32", "poiseuille20", "turek24", "step20", "array32"]


def _record_drag(lat):
    hist = []
    orig = lat.drag_lift

    def wrapped(obs, R, U, L):
        r = orig(obs, R, U, L)
        hist.append(r)
        return r

    lat.drag_lift = wrapped
    return hist


def run_oracle(app, quiet=True):
    from oracle import oracle as O
    with tempfile.TemporaryDirectory() as td, contextlib.redirect_stdout(
            io.StringIO() if quiet else None):
        lat = O.OracleLattice(app, output_dir=os.path.join(td, ""))
        hist = _record_drag(lat)
        O.run(lat, app)
    return lat, np.array(hist, dtype=np.float64).reshape(-1, 2)


def run_gpu(app, fused=None, precision=None, chunk=1000, graph=True, quiet=True, record=True):
    """Run an app on the GPU lattice.  record: return the drag/lift series of
    every lattice.drag_lift call (the app's per-iteration observables; an
    app's chunked observables are turned off for that)."""
    import lbm_gb300
    if record and getattr(app, "observables_chunk", None) is not None:
        app.observables_chunk = None
    # The directory outlives the run: apps write their final files there.
    td = tempfile.mkdtemp(prefix="lbm_test_")
    with contextlib.redirect_stdout(io.StringIO() if quiet else None):
        lat = lbm_gb300.lattice(app, precision=precision, output_dir=td, verbose=False)
        hist = _record_drag(lat)
        lbm_gb300.run(lat, app, fused=fused, chunk=chunk, graph=graph)
        out = {k: getattr(lat, k).copy() for k in ("g", "g_up", "g_eq", "rho", "u")}
    return out, np.array(hist, dtype=np.float64).reshape(-1, 2), lat


def max_rel(a, b):
    """max |a - b| / |b| (elementwise, exact zeros must match)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    d = np.abs(a - b)
    den = np.abs(b)
    zero = den == 0
    if np.any(d[zero] > 0):
        return np.inf
    return float(np.max(d[~zero] / den[~zero])) if np.any(~zero) else 0.0


def perturb_initial_state(app, eps, seed):
    """Wrap app.initialize so that g(0) = g_eq(0) * (1 + eps * U(-1, 1)),
    seeded: the same start for the oracle and the GPU lattice, with
    non-equilibrium populations in every cell from the first iteration."""
    orig = app.initialize

    def init(lat):
        orig(lat)
        if eps:
            rng = np.random.default_rng(seed)
            g = lat.g
            lat.g = g * (1.0 + eps * (2.0 * rng.random(g.shape) - 1.0))

    app.initialize = init
    return app


def run_oracle_program(app, n):
    """Iterations 0 .. n-1 of the app on the oracle in one C call
    (oracle.run_program), links from the vectorised builder (pinned to the
    cell loops by test_geometry).  Returns the oracle lattice and the raw
    per-obstacle drag/lift sums, shape (n, n_obstacles, 2)."""
    from lbm_gb300 import geometry
    from oracle import oracle as O

    class _Lat(O.OracleLattice):
        def add_obstacle(self, obstacle):
            return geometry.add_obstacle(self, obstacle.polygon, obstacle.tag, self.IBB)

    with tempfile.TemporaryDirectory() as td, contextlib.redirect_stdout(io.StringIO()):
        lat = _Lat(app, output_dir=os.path.join(td, ""))
        base, vec, scale = app.bc_schedule(lat)
        drag = O.run_program(lat, app, n, (base, vec, scale(np.arange(n))))
    return lat, drag
