"""The CPU oracle against vectors produced by the reference source itself.

tests/golden/*.npz come from tests/golden/make_golden.py, which runs the
reference's own nb.py/lattice.py/run.py/apps (NumPy execution).  Kernel-level
vectors must match bit for bit (lattice.macro's velocity uses BLAS tensordot
in the reference, so u is compared to 1e-13); whole runs of our app
restatements on the oracle lattice must match to the tolerances below, and
the obstacle geometry exactly.
"""
import numpy as np
import pytest

from _cases import CASES, golden, make_case, max_rel, run_oracle
from oracle import oracle as O


@pytest.fixture(scope="module")
def fn():
    return golden("fn_kernels.npz")


def test_macro(fn):
    g = fn["g"].copy()
    rho, u = np.zeros_like(fn["rho"]), np.zeros_like(fn["u"])
    O.macro(g, rho, u)
    assert np.array_equal(rho, fn["macro_rho"])
    assert np.max(np.abs(u - fn["macro_u"])) <= 1e-13 * np.max(np.abs(fn["macro_u"]))


def test_equilibrium(fn):
    g_eq = np.zeros_like(fn["g"])
    O.equilibrium(fn["u"].copy(), fn["rho"].copy(), g_eq)
    assert np.array_equal(g_eq, fn["eq_g_eq"])


def test_collision_stream(fn):
    g, g_up = fn["g"].copy(), np.zeros_like(fn["g"])
    O.col_str(g, fn["eq_g_eq"].copy(), g_up, float(fn["om_p"]), float(fn["om_m"]))
    assert np.array_equal(g, fn["colstr_g"])
    assert np.array_equal(g_up, fn["colstr_g_up"])


@pytest.mark.parametrize("key,kind,vec", [("zh_left", "left", "u_left"),
                                          ("zh_right", "right", "u_right"),
                                          ("zh_top", "top", "u_top"),
                                          ("zh_bot", "bottom", "u_bot"),
                                          ("zh_right_p", "right_pressure", "u_right")])
def test_zou_he_walls(fn, key, kind, vec):
    u, rho, g = fn["u"].copy(), fn["rho"].copy(), fn["g"].copy()
    O.zou_he(kind, u, rho, g, vec=fn[vec].copy(), rho_right=fn["rho_right"].copy())
    for name, arr in (("g", g), ("u", u), ("rho", rho)):
        assert np.array_equal(arr, fn[key + "_" + name]), name


@pytest.mark.parametrize("key,name", [("corner_bl", "bottom_left"), ("corner_tl", "top_left"),
                                      ("corner_tr", "top_right"), ("corner_br", "bottom_right")])
def test_corners(fn, key, name):
    u, rho, g = fn["u"].copy(), fn["rho"].copy(), fn["g"].copy()
    O.corner(name, u, rho, g)
    for nm, arr in (("g", g), ("u", u), ("rho", rho)):
        assert np.array_equal(arr, fn[key + "_" + nm]), nm


@pytest.mark.parametrize("ibb", [1, 0])
def test_bounce_back(fn, ibb):
    g = fn["g"].copy()
    O.bounce_back(ibb, fn["links"], fn["links_p"], fn["g_up"].copy(), g)
    assert np.array_equal(g, fn["bb_ibb%d_g" % ibb])


def test_drag_lift(fn):
    cx, cy = O.drag_lift(fn["links"], fn["g_up"].copy(), fn["g"].copy(), 1.0, 0.05, 10.0)
    assert np.array_equal(np.array([cx, cy]), fn["drag_lift"])


def test_bounce_back_rejects_out_of_range():
    g = np.zeros((9, 6, 6))
    with pytest.raises(IndexError):
        O.bounce_back(1, np.array([[5, 2, 2]]), np.array([0.2]), g.copy(), g)


# Whole runs: oracle lattice + our app restatements vs the reference run().
RUN_TOL = {"cavity32": 1e-12, "poiseuille20": 1e-12, "turek24": 1e-12, "step20": 1e-12,
           "array32": 1e-12}


@pytest.mark.parametrize("case", CASES)
def test_oracle_runs_match_reference(case):
    app, n = make_case(case)
    lat, hist = run_oracle(app)
    d = golden("run_%s.npz" % case)
    assert max_rel(lat.g, d["g"]) <= RUN_TOL[case]
    assert max_rel(lat.rho, d["rho"]) <= RUN_TOL[case]
    assert np.max(np.abs(lat.u - d["u"])) <= RUN_TOL[case] * np.max(np.abs(d["u"]))
    if "g_up" in d.files:
        assert max_rel(lat.g_up, d["g_up"]) <= RUN_TOL[case]
    if len(d["drag_lift"]):
        ref = d["drag_lift"]
        assert np.max(np.abs(hist - ref)) <= RUN_TOL[case] * np.max(np.abs(ref))
    for k in range(len(getattr(app, "obstacles", []))):
        obs = app.obstacles[k]
        assert np.array_equal(obs.polygon, d["poly%d" % k])
        assert np.array_equal(obs.boundary, d["bnd%d" % k])
        assert np.array_equal(obs.ibb, d["ibb%d" % k])
    if "mask" in d.files:
        assert np.array_equal(lat.lattice, d["mask"])
