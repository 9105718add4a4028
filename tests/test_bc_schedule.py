"""The device BC schedule of every app: BC(it) = base + scale(it) vec must
give, iteration by iteration, the same packed BC vectors as the app's own
set_inlets (the reference's per-iteration host update, e.g. turek.py:94-109,
cavity.py:65-76) applied to the CPU restatement of the lattice.  No GPU."""
import contextlib
import io
import tempfile

import numpy as np
import pytest

from _cases import CASES, make_case
from lbm_gb300.engine import pack_bc
from oracle import oracle as O

KEYS = ("u_left", "u_right", "u_top", "u_bot", "rho_right")


@pytest.mark.parametrize("case", CASES)
def test_schedule_reproduces_set_inlets(case):
    app, n = make_case(case)
    with contextlib.redirect_stdout(io.StringIO()), tempfile.TemporaryDirectory() as td:
        lat = O.OracleLattice(app, output_dir=td + "/")
        sched = app.bc_schedule(lat)
        if sched is None:
            pytest.skip("app without inlet ramp")
        base, vec, scale = sched
        its = sorted({0, 1, 2, 7, n // 3, n // 2, n - 1, 10 * n})
        s = scale(its)
        for it, sk in zip(its, s):
            app.set_inlets(lat, it)
            want = pack_bc({k: getattr(lat, k) for k in KEYS}, lat.nx, lat.ny)
            got = base + sk * vec
            assert np.array_equal(got, want), (case, it, float(np.max(np.abs(got - want))))
