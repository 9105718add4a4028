"""Kernel-level parity: each C-ABI kernel against the C oracle, bit for bit.

The per-method kernels are compiled with -fmad=false and evaluate the
reference expressions in the same order as the oracle, so outputs must be
identical (the oracle itself is pinned to the reference by
test_oracle_golden.py).
"""
import ctypes

import numpy as np
import pytest
import torch

from _cases import golden
from lbm_gb300 import _lib
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def dev(a, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device="cuda", dtype=dtype)


def p(t):
    return ctypes.c_void_p(t.data_ptr())


def S():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def random_state(nx, ny, seed):
    rng = np.random.default_rng(seed)
    w = O.W
    g = w[:, None, None] * (1.0 + 0.2 * rng.random((9, nx, ny)))
    g_up = w[:, None, None] * (1.0 + 0.2 * rng.random((9, nx, ny)))
    u = 0.05 * (rng.random((2, nx, ny)) - 0.5)
    rho = 1.0 + 0.02 * (rng.random((nx, ny)) - 0.5)
    return g, g_up, u, rho, rng


SIZES = [(13, 11), (64, 48), (257, 130)]


@pytest.mark.parametrize("nx,ny", SIZES)
def test_macro_equilibrium_collision(cuda, nx, ny):
    g, _, u, rho, _ = random_state(nx, ny, nx)
    # macro
    r_ref, u_ref = np.zeros((nx, ny)), np.zeros((2, nx, ny))
    O.macro(g.copy(), r_ref, u_ref)
    G, R, U = dev(g), torch.zeros((nx, ny), dtype=torch.float64, device="cuda"), \
        torch.zeros((2, nx, ny), dtype=torch.float64, device="cuda")
    _lib.call("lbm_macro_f64", p(G), p(R), p(U), nx, ny, S())
    assert np.array_equal(R.cpu().numpy(), r_ref)
    assert np.array_equal(U.cpu().numpy(), u_ref)
    # equilibrium
    geq_ref = np.zeros((9, nx, ny))
    O.equilibrium(u.copy(), rho.copy(), geq_ref)
    GEQ = torch.zeros((9, nx, ny), dtype=torch.float64, device="cuda")
    Ud, Rd = dev(u), dev(rho)  # keep the tensors alive until the kernel has run
    _lib.call("lbm_equilibrium_f64", p(Ud), p(Rd), p(GEQ), nx, ny, S())
    assert np.array_equal(GEQ.cpu().numpy(), geq_ref)
    # collision + stream
    om_p, om_m = 1.0 / 0.548, 1.0 / (0.25 / 0.048 + 0.5)
    g_ref, gup_ref = g.copy(), np.zeros((9, nx, ny))
    O.col_str(g_ref, geq_ref, gup_ref, om_p, om_m)
    G2, GUP = dev(g), torch.zeros((9, nx, ny), dtype=torch.float64, device="cuda")
    _lib.call("lbm_collision_stream_f64", p(G2), p(GEQ), p(GUP), om_p, om_m, nx, ny, S())
    assert np.array_equal(GUP.cpu().numpy(), gup_ref)
    assert np.array_equal(G2.cpu().numpy(), g_ref)


WALLS = [(_lib.WALL_LEFT_VELOCITY, "left", "ny"), (_lib.WALL_RIGHT_VELOCITY, "right", "ny"),
         (_lib.WALL_RIGHT_PRESSURE, "right_pressure", "ny"), (_lib.WALL_TOP_VELOCITY, "top", "nx"),
         (_lib.WALL_BOTTOM_VELOCITY, "bottom", "nx")]


@pytest.mark.parametrize("nx,ny", SIZES)
@pytest.mark.parametrize("wall,kind,axis", WALLS)
def test_zou_he_walls(cuda, nx, ny, wall, kind, axis):
    g, _, u, rho, rng = random_state(nx, ny, 3 * nx + wall)
    n = ny if axis == "ny" else nx
    vec = 0.05 * rng.random((2, n))
    rr = 1.0 + 0.01 * rng.random(ny)
    uo, ro, go = u.copy(), rho.copy(), g.copy()
    O.zou_he(kind, uo, ro, go, vec=vec.copy(), rho_right=rr.copy())
    U, R, G = dev(u), dev(rho), dev(g)
    V, RR = dev(vec), dev(rr)
    _lib.call("lbm_zou_he_f64", wall, p(U), p(R), p(G), p(V), p(RR), nx, ny, S())
    assert np.array_equal(G.cpu().numpy(), go)
    assert np.array_equal(R.cpu().numpy(), ro)
    assert np.array_equal(U.cpu().numpy(), uo)


@pytest.mark.parametrize("corner,name", [(0, "bottom_left"), (1, "top_left"), (2, "top_right"),
                                         (3, "bottom_right")])
def test_corners(cuda, corner, name):
    g, _, u, rho, _ = random_state(13, 11, 50 + corner)
    uo, ro, go = u.copy(), rho.copy(), g.copy()
    O.corner(name, uo, ro, go)
    U, R, G = dev(u), dev(rho), dev(g)
    _lib.call("lbm_zou_he_corner_f64", corner, p(U), p(R), p(G), 13, 11, S())
    assert np.array_equal(G.cpu().numpy(), go)
    assert np.array_equal(R.cpu().numpy(), ro)
    assert np.array_equal(U.cpu().numpy(), uo)


@pytest.mark.parametrize("ibb", [1, 0])
def test_bounce_back_and_drag_golden(cuda, ibb):
    d = golden("fn_kernels.npz")
    nx, ny = d["g"].shape[1:]
    links = d["links"]
    G, GUP = dev(d["g"]), dev(d["g_up"])
    LK, PP = dev(links, torch.int32), dev(d["links_p"])
    _lib.call("lbm_bounce_back_f64", ibb, p(LK), len(links), p(PP), p(GUP), p(G), nx, ny, S())
    assert np.array_equal(G.cpu().numpy(), d["bb_ibb%d_g" % ibb])


def test_drag_lift_golden(cuda):
    d = golden("fn_kernels.npz")
    nx, ny = d["g"].shape[1:]
    links = d["links"]
    L = _lib.load()
    scratch = torch.zeros(L.lbm_drag_lift_scratch_bytes(len(links)), dtype=torch.uint8,
                          device="cuda")
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    LK, GUP, G = dev(links, torch.int32), dev(d["g_up"]), dev(d["g"])
    _lib.call("lbm_drag_lift_f64", p(LK), len(links), p(GUP), p(G), nx, ny, p(out), p(scratch),
              S())
    fx, fy = out.cpu().numpy()
    cx, cy = -2.0 * fx / (1.0 * 10.0 * 0.05 ** 2), -2.0 * fy / (1.0 * 10.0 * 0.05 ** 2)
    ref = d["drag_lift"]
    # tree order differs from the serial sum: a few ulps of the largest term
    assert abs(cx - ref[0]) <= 1e-13 * abs(ref[0]) + 1e-12
    assert abs(cy - ref[1]) <= 1e-13 * abs(ref[1]) + 1e-12
