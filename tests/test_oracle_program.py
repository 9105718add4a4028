"""The oracle's one-call driver loop (oracle.run_program / oracle_run in C)
against the oracle driven by the reference's run() loop from Python
(oracle.run): same kernels in the same order, so every array and every
drag/lift value must be identical, bit for bit, on the golden runs."""
import contextlib
import io
import os
import tempfile

import numpy as np
import pytest

from _cases import CASES, make_case
from oracle import oracle as O


def _run_python(case):
    app, n = make_case(case)
    calls = []
    with tempfile.TemporaryDirectory() as td, contextlib.redirect_stdout(io.StringIO()):
        lat = O.OracleLattice(app, output_dir=os.path.join(td, ""))
        orig = lat.drag_lift

        def rec(obs, R, U, L):
            r = orig(obs, R, U, L)
            calls.append((obs, R, U, L, r))
            return r

        lat.drag_lift = rec
        O.run(lat, app)
    return lat, app, calls, n


def _run_program(case):
    app, n = make_case(case)
    with tempfile.TemporaryDirectory() as td, contextlib.redirect_stdout(io.StringIO()):
        lat = O.OracleLattice(app, output_dir=os.path.join(td, ""))
        base, vec, scale = app.bc_schedule(lat)
        drag = O.run_program(lat, app, n, (base, vec, scale(np.arange(n))))
    return lat, app, drag


@pytest.mark.parametrize("case", CASES)
def test_program_loop_equals_python_loop(case):
    ref, app_r, calls, n = _run_python(case)
    got, app_g, drag = _run_program(case)
    for k in ("g", "g_up", "g_eq", "rho", "u"):
        assert np.array_equal(getattr(got, k), getattr(ref, k)), k
    # every drag_lift call of the app's observables, from the raw sums
    per_it = len(calls) // n
    assert per_it * n == len(calls)
    for t, (obs, R, U, L, r) in enumerate(calls):
        o = next(k for k, x in enumerate(app_r.obstacles) if x is obs)
        fx, fy = drag[t // per_it, o]
        assert -2.0 * fx / (R * L * (U * U)) == r[0]
        assert -2.0 * fy / (R * L * (U * U)) == r[1]


def test_program_refuses_out_of_range_links():
    app, n = make_case("turek24")
    with tempfile.TemporaryDirectory() as td, contextlib.redirect_stdout(io.StringIO()):
        lat = O.OracleLattice(app, output_dir=os.path.join(td, ""))
        base, vec, scale = app.bc_schedule(lat)
        orig = app.initialize

        def bad_init(lattice):
            orig(lattice)
            b = np.array(app.obstacles[0].boundary)
            b[0, 0] = lattice.nx + 5
            app.obstacles[0].boundary = b

        app.initialize = bad_init
        with pytest.raises(IndexError):
            O.run_program(lat, app, 3, (base, vec, scale(np.arange(3))))
