"""The boundary program the fused engine derives from an app's set_bc
(engine.trace_bc_program): obstacle links first, then the Zou-He walls and
corners in the app's call order, e.g. cavity.py:79-89 (bottom, left, right,
top, then the four corners) and turek.py:112-125 (the cylinder, then bottom,
left, top, right pressure, corners).  Orders the fused kernels cannot
reproduce are refused.  No GPU."""
import pytest

from _cases import make_case
from lbm_gb300 import _lib
from lbm_gb300.engine import Unfusable, trace_bc_program

W = _lib
CORNERS = [W.CORNER_BOTTOM_LEFT, W.CORNER_TOP_LEFT, W.CORNER_TOP_RIGHT, W.CORNER_BOTTOM_RIGHT]
CHANNEL = [W.WALL_BOTTOM_VELOCITY, W.WALL_LEFT_VELOCITY, W.WALL_TOP_VELOCITY,
           W.WALL_RIGHT_PRESSURE]


@pytest.mark.parametrize("case,n_obs,walls", [
    ("cavity32", 0, [W.WALL_BOTTOM_VELOCITY, W.WALL_LEFT_VELOCITY, W.WALL_RIGHT_VELOCITY,
                     W.WALL_TOP_VELOCITY]),
    ("poiseuille20", 0, CHANNEL),
    ("turek24", 1, CHANNEL),
    ("step20", 2, CHANNEL),
    ("array32", 8, CHANNEL),
])
def test_programs_of_the_apps(case, n_obs, walls):
    app, _ = make_case(case)
    obstacles, w, c = trace_bc_program(app)
    assert len(obstacles) == n_obs
    assert obstacles == list(getattr(app, "obstacles", []))[:n_obs]
    assert w == walls
    assert c == CORNERS


class _App:
    def __init__(self, calls):
        self.calls = calls

    def set_bc(self, lattice):
        for name, arg in self.calls:
            getattr(lattice, name)(*arg)


@pytest.mark.parametrize("calls,why", [
    ([("zou_he_left_wall_velocity", ()), ("bounce_back_obstacle", ("o",))], "bounce-back after"),
    ([("zou_he_bottom_left_corner", ()), ("zou_he_left_wall_velocity", ())], "after a corner"),
    ([("zou_he_left_wall_velocity", ())] * 6, "more than five"),
    ([("periodic_x", ())], "periodic_x"),
])
def test_programs_the_fused_kernels_cannot_run(calls, why):
    with pytest.raises(Unfusable, match=why):
        trace_bc_program(_App(calls))


def test_repeated_corner_counted_once():
    app = _App([("zou_he_bottom_left_corner", ()), ("zou_he_bottom_left_corner", ())])
    assert trace_bc_program(app) == ([], [], [W.CORNER_BOTTOM_LEFT])
