"""Per-step precision of the plain path's two forms against exact arithmetic.

One fused step (pull + macro + equilibrium + TRT collision, nb.py:7-45) is
applied to the same developed cavity state by the FP64 form ("f64") and by
the 64-bit fixed-point form ("q60"), and the interior cells are compared
with the reference update evaluated in exact rational arithmetic
(fractions.Fraction) from the same input values and the same FP64 rates.
The fixed-point form's error must not exceed the FP64 form's: that is what
makes it a drop-in for the FP64 path rather than a reduced-precision form.
"""
import ctypes
from fractions import Fraction

import numpy as np
import pytest
import torch

from _cases import run_gpu

pytestmark = pytest.mark.gpu

CX = [0, 1, -1, 0, 0, 1, -1, -1, 1]
CY = [0, 0, 0, 1, -1, 1, -1, 1, -1]
W = [Fraction(4, 9)] + [Fraction(1, 9)] * 4 + [Fraction(1, 36)] * 4
NS = [0, 2, 1, 4, 3, 6, 5, 8, 7]


def _cavity(n_it):
    from lbm_gb300.apps import cavity
    a = cavity()
    a.L_lbm, a.u_lbm, a.Re_lbm = 40, 0.1, 100.0
    a.compute_lbm_parameters()
    a.sigma = 100.0
    a.stop, a.it_max, a.output_freq = "it", n_it - 1, 10 ** 12
    return a


def exact_update(f_in, i, j, om_p, om_m):
    """g_up of cell (i, j) from the pulled values, exact (nb.py:7-45)."""
    g = [Fraction(float(f_in[q, i - CX[q], j - CY[q]])) for q in range(9)]
    rho = sum(g)
    jx = sum(CX[q] * g[q] for q in range(9))
    jy = sum(CY[q] * g[q] for q in range(9))
    ux, uy = jx / rho, jy / rho
    v = Fraction(3, 2) * (ux * ux + uy * uy)
    eq = []
    for q in range(9):
        t = 3 * (CX[q] * ux + CY[q] * uy)
        eq.append((1 + t + t * t / 2 - v) * rho * W[q])
    out = []
    for q in range(9):
        qb = NS[q]
        gp, gm = (g[q] + g[qb]) / 2, (g[q] - g[qb]) / 2
        ep, em = (eq[q] + eq[qb]) / 2, (eq[q] - eq[qb]) / 2
        out.append(g[q] - om_p * (gp - ep) - om_m * (gm - em))
    return out


def _state(lat):
    """The lattice's fused engine and its current state g_up in FP64."""
    eng = lat._engine
    f_in = torch.empty((9, lat.nx, lat.ny), dtype=torch.float64, device=lat.device)
    eng.g_up_into(f_in)
    return eng, f_in


def test_q60_step_error_not_above_fp64(cuda):
    from lbm_gb300 import _lib
    n_it = 400
    _, _, lat64 = run_gpu(_cavity(n_it), fused=True, precision="f64")
    _, _, latq = run_gpu(_cavity(n_it), fused=True, precision="q60")
    eng64, f_in = _state(lat64)
    engq = latq._engine
    # the same input state in both forms (exact: every population is >= 2^-8)
    f_np = f_in.cpu().numpy()
    assert f_np.min() > 2.0 ** -8
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.call("lbm_pack_f64", _lib.PREC_Q60, ctypes.c_void_p(f_in.data_ptr()),
              ctypes.c_void_p(engq.f[engq.cur].data_ptr()), lat64.nx, lat64.ny, 0, 1.0, st)
    for eng in (eng64, engq):
        eng.steps(n_it, 1, graph=False)
        eng.check_status()
    out64 = eng64.f[eng64.cur].cpu().numpy()
    outq = engq.f[engq.cur].cpu().numpy()  # int64, value * 2^60

    om_p, om_m = Fraction(lat64.om_p_lbm), Fraction(lat64.om_m_lbm)
    rng = np.random.default_rng(7)
    cells = [(int(i), int(j)) for i, j in zip(rng.integers(1, lat64.nx - 1, 150),
                                              rng.integers(1, lat64.ny - 1, 150))]
    err64 = errq = 0.0
    for i, j in cells:
        ex = exact_update(f_np, i, j, om_p, om_m)
        for q in range(9):
            err64 = max(err64, abs(float(Fraction(float(out64[q, i, j])) - ex[q])))
            errq = max(errq, abs(float(Fraction(int(outq[q, i, j]), 2 ** 60) - ex[q])))
    # FP64: a few ulps of populations up to ~0.5; Q3.60: a few units of 2^-60.
    assert err64 < 1e-15
    assert errq <= 8 * 2.0 ** -60
    assert errq <= err64
