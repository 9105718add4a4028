"""The two bulk kernels of the 16-bit forms give the same bits.

The default TMA-staged kernel (cp.async.bulk copies of each tile's pull
sources into shared-memory stages, mbarrier pipeline) and the
register-pipelined kernel (16-byte global loads, warp-shuffle halos) run the
same per-group update; their states and drag/lift series must be
bit-identical after many iterations, on lattices whose tiles lie inside one
column (ny = 512), span several columns (ny = 64 and 200) and include padded
rows (ny = 70, rows of 72).
"""
import contextlib
import io
import tempfile

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FORMS = ["f16s", "f16sr", "bf16s", "bf16sr"]


def _obstacle_array():
    from lbm_gb300.apps import obstacle_array
    a = obstacle_array(L_lbm=512)
    a.sigma = 500.0
    return a


def _cavity(n):
    from lbm_gb300.apps import cavity
    a = cavity()
    a.L_lbm, a.u_lbm = n, 0.1
    a.compute_lbm_parameters()
    a.sigma = 100.0
    return a


def _turek():
    from lbm_gb300.apps import turek
    a = turek()
    a.L_lbm = 200
    a.compute_lbm_parameters()
    a.sigma = 500.0
    return a


CASES = {"obstacle_array_2048x512": _obstacle_array, "cavity64": lambda: _cavity(64),
         "cavity70_padded": lambda: _cavity(70), "turek_1100x200": _turek}


def _engine(make, precision, kernel, steps):
    import lbm_gb300
    from lbm_gb300.engine import FusedEngine, trace_bc_program
    app = make()
    app.output_freq = 10 ** 12
    with contextlib.redirect_stdout(io.StringIO()):
        lat = lbm_gb300.lattice(app, precision=precision, output_dir=tempfile.mkdtemp(),
                                verbose=False)
        lat.generate_image = lambda obstacles: None
        app.initialize(lat)
    obstacles, walls, corners = trace_bc_program(app)
    eng = FusedEngine(lat, obstacles, walls, corners, precision=precision, drag_cap=steps + 8)
    eng.bulk_kernel = kernel
    base, vec, scale = app.bc_schedule(lat)
    eng.set_bc_schedule(base, vec, scale(np.arange(steps + 8)), it0=0)
    eng.collide_from_g(0, macro=False)
    return eng


def _run(make, precision, kernel, steps):
    import torch
    eng = _engine(make, precision, kernel, steps)
    eng.steps(1, steps // 2, graph=False)
    eng.steps(1 + steps // 2, steps - steps // 2, graph=True)
    eng.check_status()
    f = eng.f[eng.cur]
    assert bool(torch.isfinite(f.float()).all())
    return f.view(torch.int16).cpu().numpy(), eng.drag_rows(1, steps - 1)


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("precision", FORMS)
def test_tma_equals_register_kernel(cuda, case, precision):
    steps = 400
    f_t, d_t = _run(CASES[case], precision, "tma", steps)
    f_r, d_r = _run(CASES[case], precision, "registers", steps)
    assert np.array_equal(f_t, f_r)
    assert np.array_equal(d_t, d_r)


def test_stage_wait_timeout_reports_status(cuda):
    """The failure path of the bounded waits: with LBM_FLAG_TEST_STALL the
    producer withholds each block's first tile, the consumers' wait on it runs
    out (0.5 s), the kernel sets status bit 3 and returns; the host raises on
    it, and the context keeps working (a fresh start then steps normally)."""
    import torch
    eng = _engine(CASES["cavity64"], "f16s", "tma", 20)
    eng.test_stall = True
    eng.steps(1, 1, graph=False)
    torch.cuda.synchronize()
    with pytest.raises(RuntimeError, match="stage wait timed out"):
        eng.check_status()
    eng.test_stall = False
    eng.status.zero_()
    eng.collide_from_g(0, macro=False)
    eng.steps(1, 10, graph=False)
    eng.check_status()
    assert bool(torch.isfinite(eng.f[eng.cur].float()).all())
