"""Generate the golden fixtures under tests/golden/ from the reference itself.

This script imports the reference package ``lbm`` (jviquerat/lbm) read-only
from a checkout given by ``--reference`` (default: the ``LBM_REFERENCE``
environment variable) and runs its own source.  numba, matplotlib and PIL are
absent from the fixture container, so the stand-ins in ``ref_stubs/`` are put
first on ``sys.path``: ``njit`` becomes an identity decorator, ``prange``
becomes ``range`` and plotting is a no-op.  The reference kernels in
``lbm/src/core/nb.py`` therefore run as plain NumPy with IEEE arithmetic.

Outputs (``*.npz``, float64 / int64):

* ``fn_kernels.npz`` -- one known-answer vector per reference kernel
  (``lattice.macro``, ``nb_equilibrium``, ``nb_col_str``, the five Zou-He
  walls, the four corners, ``nb_bounce_back_obstacle`` with IBB on and off,
  ``nb_drag_lift``) on seeded random inputs of a 13x11 lattice.
* ``run_<case>.npz`` -- the reference ``run()`` loop for a few small apps
  (cavity, poiseuille, turek with IBB, step with plain bounce-back touching
  the walls, array with 8 IBB squares; ``g_up`` kept for cavity and turek): final ``g``, ``g_up``, ``rho``, ``u``,
  per-step drag/lift, and for obstacle apps the link list and IBB distances.
* ``geometry.npz`` -- polygons from ``generate_shape`` and link lists from
  ``lattice.add_obstacle`` (turek at L=24/100/200, squares).
* ``buff.npz`` -- the reference observable buffer (``lbm/src/utils/buff.py``)
  fed a seeded decaying oscillation: ``mv_avg`` output and the convergence
  flag at every iteration, and the final history arrays.

The GPU machine does not hold the reference; only these files travel.
Run: ``python tests/golden/make_golden.py --reference <path-to-lbm-checkout>``.
"""
import argparse
import contextlib
import io
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _import_reference(ref_root):
    sys.path.insert(0, ref_root)
    sys.path.insert(0, os.path.join(HERE, "ref_stubs"))
    import lbm.src.core.nb as nb  # noqa: E402
    from lbm.src.core import lattice as lat_mod  # noqa: E402
    from lbm.src.core import run as run_mod  # noqa: E402
    from lbm.src.app import cavity, turek, poiseuille, array, step  # noqa: E402
    from lbm.src.utils import shapes  # noqa: E402
    return dict(nb=nb, lattice=lat_mod.lattice, run=run_mod.run,
                cavity=cavity.cavity, turek=turek.turek,
                poiseuille=poiseuille.poiseuille, array=array.array,
                step=step.step, shapes=shapes)


@contextlib.contextmanager
def _in_tmpdir():
    old = os.getcwd()
    with tempfile.TemporaryDirectory() as d:
        os.chdir(d)
        try:
            yield d
        finally:
            os.chdir(old)


def _quiet():
    return contextlib.redirect_stdout(io.StringIO())


def _d2q9():
    c = np.array([[0, 0], [1, 0], [-1, 0], [0, 1], [0, -1],
                  [1, 1], [-1, -1], [-1, 1], [1, -1]])
    w = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4)
    ns = np.array([0, 2, 1, 4, 3, 6, 5, 8, 7])
    return c, w, ns


def make_fn_kernels(R, out):
    """Known-answer vectors for every reference kernel on one random state."""
    nb = R["nb"]
    rng = np.random.default_rng(20240611)
    nx, ny = 13, 11
    lx, ly = nx - 1, ny - 1
    c, w, ns = _d2q9()
    g = w[:, None, None] * (1.0 + 0.2 * rng.random((9, nx, ny)))
    g_up = w[:, None, None] * (1.0 + 0.2 * rng.random((9, nx, ny)))
    u = 0.05 * (rng.random((2, nx, ny)) - 0.5)
    rho = 1.0 + 0.02 * (rng.random((nx, ny)) - 0.5)
    u_left = 0.05 * rng.random((2, ny))
    u_right = 0.05 * rng.random((2, ny))
    u_top = 0.05 * rng.random((2, nx))
    u_bot = 0.05 * rng.random((2, nx))
    rho_right = 1.0 + 0.01 * rng.random(ny)
    om_p, om_m = 1.0 / 0.548, 1.0 / (0.25 / (0.548 - 0.5) + 0.5)
    res = dict(g=g, g_up=g_up, u=u, rho=rho, u_left=u_left, u_right=u_right,
               u_top=u_top, u_bot=u_bot, rho_right=rho_right,
               om_p=np.float64(om_p), om_m=np.float64(om_m))

    # lattice.macro (numpy sum + tensordot)
    m_rho = np.sum(g, axis=0)
    m_u = np.zeros((2, nx, ny))
    m_u[0] = np.tensordot(c[:, 0], g, axes=(0, 0)) / m_rho
    m_u[1] = np.tensordot(c[:, 1], g, axes=(0, 0)) / m_rho
    res["macro_rho"], res["macro_u"] = m_rho, m_u

    g_eq = np.zeros((9, nx, ny))
    nb.nb_equilibrium(u, c, w, rho, g_eq)
    res["eq_g_eq"] = g_eq.copy()

    gg, gup = g.copy(), np.zeros((9, nx, ny))
    nb.nb_col_str(gg, g_eq, gup, om_p, om_m, c, ns, nx, ny, lx, ly)
    res["colstr_g"], res["colstr_g_up"] = gg, gup

    walls = {
        "zh_left": lambda uu, rr, g2: nb.nb_zou_he_left_wall_velocity(lx, ly, uu, u_left, rr, g2),
        "zh_right": lambda uu, rr, g2: nb.nb_zou_he_right_wall_velocity(lx, ly, uu, u_right, rr, g2),
        "zh_right_p": lambda uu, rr, g2: nb.nb_zou_he_right_wall_pressure(lx, ly, uu, rho_right, u_right, rr, g2),
        "zh_top": lambda uu, rr, g2: nb.nb_zou_he_top_wall_velocity(lx, ly, uu, u_top, rr, g2),
        "zh_bot": lambda uu, rr, g2: nb.nb_zou_he_bottom_wall_velocity(lx, ly, uu, u_bot, rr, g2),
        "corner_bl": lambda uu, rr, g2: nb.nb_zou_he_bottom_left_corner_velocity(lx, ly, uu, rr, g2),
        "corner_tl": lambda uu, rr, g2: nb.nb_zou_he_top_left_corner_velocity(lx, ly, uu, rr, g2),
        "corner_tr": lambda uu, rr, g2: nb.nb_zou_he_top_right_corner_velocity(lx, ly, uu, rr, g2),
        "corner_br": lambda uu, rr, g2: nb.nb_zou_he_bottom_right_corner_velocity(lx, ly, uu, rr, g2),
    }
    for name, fn in walls.items():
        uu, rr, g2 = u.copy(), rho.copy(), g.copy()
        fn(uu, rr, g2)
        res[name + "_u"], res[name + "_rho"], res[name + "_g"] = uu, rr, g2

    # Links away from the edges so that x + 2*c_qb stays inside.
    n_links = 40
    li = rng.integers(2, nx - 2, n_links)
    lj = rng.integers(2, ny - 2, n_links)
    lq = rng.integers(1, 9, n_links)
    links = np.stack([li, lj, lq], axis=1).astype(np.int64)
    p = rng.random(n_links)
    p[:5] = [0.0 + 1e-3, 0.25, 0.5, 0.75, 0.999]
    res["links"], res["links_p"] = links, p
    for ibb in (True, False):
        g2 = g.copy()
        nb.nb_bounce_back_obstacle(ibb, links, ns, c, p, g_up, g2, u, np.zeros((nx, ny)))
        res["bb_ibb%d_g" % int(ibb)] = g2
    cx, cy = nb.nb_drag_lift(links, ns, c, g_up, g, 1.0, 0.05, 10.0)
    res["drag_lift"] = np.array([cx, cy])
    np.savez_compressed(out, **res)


def _record_drag(ltc):
    hist = []
    orig = ltc.drag_lift

    def wrapped(obs, R_ref, U_ref, L_ref):
        cx, cy = orig(obs, R_ref, U_ref, L_ref)
        hist.append((cx, cy))
        return cx, cy

    ltc.drag_lift = wrapped
    return hist


def run_case(R, name, app, n_iter, out, keep_g_up=True):
    """Run the reference run() for exactly ``n_iter`` iterations."""
    app.stop = "it"
    app.it_max = n_iter - 1
    app.output_freq = 10 ** 12
    with _in_tmpdir(), _quiet():
        ltc = R["lattice"](app)
        hist = _record_drag(ltc)
        R["run"](ltc, app)
    res = dict(g=ltc.g, rho=ltc.rho, u=ltc.u,
               nx=np.int64(ltc.nx), ny=np.int64(ltc.ny),
               tau=np.float64(ltc.tau_lbm), n_iter=np.int64(n_iter),
               sigma=np.float64(app.sigma), u_lbm=np.float64(app.u_lbm),
               drag_lift=np.array(hist, dtype=np.float64).reshape(-1, 2))
    if keep_g_up:
        res["g_up"] = ltc.g_up
    for k, obs in enumerate(getattr(app, "obstacles", [])):
        res["bnd%d" % k] = np.asarray(obs.boundary, dtype=np.int64)
        res["ibb%d" % k] = np.asarray(obs.ibb, dtype=np.float64)
        res["poly%d" % k] = np.asarray(obs.polygon, dtype=np.float64)
    if getattr(app, "obstacles", None):
        res["mask"] = ltc.lattice.copy()
    np.savez_compressed(out, **res)
    print("  %-12s nx=%d ny=%d iters=%d" % (name, ltc.nx, ltc.ny, n_iter))


def make_runs(R):
    app = R["cavity"]()
    app.L_lbm, app.u_lbm = 32, 0.1
    app.compute_lbm_parameters()
    app.sigma = 100.0
    run_case(R, "cavity32", app, 1000, os.path.join(HERE, "run_cavity32.npz"))

    app = R["poiseuille"]()
    app.L_lbm = 20
    app.compute_lbm_parameters()
    app.sigma = 60.0
    run_case(R, "poiseuille20", app, 600, os.path.join(HERE, "run_poiseuille20.npz"))

    # Turek 2D-1 (Re = 20): tau = 0.525 at this resolution.
    app = R["turek"]()
    app.L_lbm = 24
    app.Re_lbm = 20.0
    app.compute_lbm_parameters()
    app.sigma = 40.0
    run_case(R, "turek24", app, 400, os.path.join(HERE, "run_turek24.npz"))

    app = R["step"]()
    app.L_lbm = 20
    app.compute_lbm_parameters()
    app.sigma = 40.0
    run_case(R, "step20", app, 300, os.path.join(HERE, "run_step20.npz"),
             keep_g_up=False)

    app = R["array"]()
    app.L_lbm = 32
    app.compute_lbm_parameters()
    app.sigma = 40.0
    run_case(R, "array32", app, 300, os.path.join(HERE, "run_array32.npz"),
             keep_g_up=False)


def make_geometry(R, out):
    res = {}
    with _in_tmpdir(), _quiet():
        for L in (24, 100, 200):
            app = R["turek"]()
            app.L_lbm = L
            app.compute_lbm_parameters()
            ltc = R["lattice"](app)
            app.add_obstacles(ltc, app.obstacles)
            obs = app.obstacles[0]
            res["turek%d_poly" % L] = obs.polygon
            res["turek%d_bnd" % L] = np.asarray(obs.boundary, dtype=np.int64)
            res["turek%d_ibb" % L] = obs.ibb
            res["turek%d_area" % L] = np.float64(obs.area)
            res["turek%d_mask" % L] = ltc.lattice.astype(np.int8)
        sq = R["shapes"].generate_shape(4, [0.3, -0.2], "square", 0.37, "sq", 100, "./")
        res["square_poly"] = sq.curve_pts
    np.savez_compressed(out, **res)


def buff_series(n=3000, seed=5):
    """Seeded observable history fed to the buffer (also used by the test)."""
    rng = np.random.default_rng(seed)
    it = np.arange(n)
    return 3.0 + 0.5 * np.exp(-it / 400.0) * np.sin(it / 15.0) + 1e-3 * rng.standard_normal(n)


BUFF_ARGS = dict(dt=0.01, obs_cv_ct=1e-2, obs_cv_nb=100)


def make_buff(out):
    from lbm.src.utils.buff import buff
    b = buff("drag", BUFF_ARGS["dt"], BUFF_ARGS["obs_cv_ct"], BUFF_ARGS["obs_cv_nb"], ".")
    obs, growth, cv = [], [], []
    for v in buff_series():
        b.add(v)
        o, g = b.mv_avg()
        obs.append(o)
        growth.append(g)
        cv.append(int(b.obs_cv))
    np.savez_compressed(out, obs=np.array(obs), growth=np.array(growth), cv=np.array(cv),
                        buff=b.buff, avg1=b.avg1_buff, avg2=b.avg2_buff, avg3=b.avg3_buff,
                        f_avg=b.f_avg())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("LBM_REFERENCE"))
    ap.add_argument("--only", choices=["kernels", "geometry", "runs", "buff"], default=None)
    args = ap.parse_args()
    if not args.reference or not os.path.isdir(args.reference):
        sys.exit("pass --reference <path to the jviquerat/lbm checkout>")
    R = _import_reference(os.path.abspath(args.reference))
    if args.only in (None, "kernels"):
        make_fn_kernels(R, os.path.join(HERE, "fn_kernels.npz"))
        print("fn_kernels.npz written")
    if args.only in (None, "geometry"):
        make_geometry(R, os.path.join(HERE, "geometry.npz"))
        print("geometry.npz written")
    if args.only in (None, "runs"):
        make_runs(R)
    if args.only in (None, "buff"):
        make_buff(os.path.join(HERE, "buff.npz"))
        print("buff.npz written")


if __name__ == "__main__":
    main()
