"""Pure-tensor reference of one lattice iteration -- TEST INFRASTRUCTURE ONLY.

A differentiable PyTorch restatement (FP64, any device) of the reference
iteration of a channel with obstacles (lbm/src/core/run.py:24-54 with the
turek set_bc order, turek.py:112-125): macro, equilibrium, TRT
collision-stream (nb.py:7-45), interpolated bounce-back (nb.py:77-104),
Zou-He bottom / left velocity / top / right pressure and the four corners
(nb.py:121-344), drag/lift (nb.py:49-73).  torch.autograd through it gives the
gradient the hand-written CUDA adjoint must reproduce.  Only tests import it.
"""
import torch

C = [(0, 0), (1, 0), (-1, 0), (0, 1), (0, -1), (1, 1), (-1, -1), (-1, 1), (1, -1)]
NS = [0, 2, 1, 4, 3, 6, 5, 8, 7]
W = [4.0 / 9.0] + [1.0 / 9.0] * 4 + [1.0 / 36.0] * 4


def om_minus(om_p, lam=0.25):
    """TRT: tau- = lambda / (tau+ - 1/2) + 1/2 (lattice.py:127-131)."""
    tau_p = 1.0 / om_p
    return 1.0 / (lam / (tau_p - 0.5) + 0.5)


def macro(g):
    rho = g[0]
    for q in range(1, 9):
        rho = rho + g[q]
    jx = g[1] - g[2] + g[5] - g[6] - g[7] + g[8]
    jy = g[3] - g[4] + g[5] - g[6] + g[7] - g[8]
    return rho, jx / rho, jy / rho


def equilibrium(rho, ux, uy):
    v = 1.5 * (ux * ux + uy * uy)
    out = []
    for q in range(9):
        t = 3.0 * (ux * C[q][0] + uy * C[q][1])
        out.append((1.0 + t + 0.5 * t * t - v) * (rho * W[q]))
    return out


def collide(g, om_p):
    om_m = om_minus(om_p)
    rho, ux, uy = macro(g)
    geq = equilibrium(rho, ux, uy)
    a = 1.0 - 0.5 * (om_p + om_m)
    b = 0.5 * (om_p - om_m)
    cc = 0.5 * (om_p + om_m)
    up = [(1.0 - om_p) * g[0] + om_p * geq[0]]
    for q in range(1, 9):
        qb = NS[q]
        up.append(a * g[q] - b * g[qb] + cc * geq[q] + b * geq[qb])
    return up


def stream(g, up):
    """Shift-copy on interior slices; edge entries keep g (nb.py:37-45)."""
    nx, ny = g[0].shape
    out = [up[0]]
    for q in range(1, 9):
        cx, cy = C[q]
        new = g[q].clone()
        dst_i = slice(max(cx, 0), nx + min(cx, 0))
        src_i = slice(max(-cx, 0), nx + min(-cx, 0))
        dst_j = slice(max(cy, 0), ny + min(cy, 0))
        src_j = slice(max(-cy, 0), ny + min(-cy, 0))
        new[dst_i, dst_j] = up[q][src_i, src_j]
        out.append(new)
    return out


def ibb(g, up, links, p):
    """Quadratic interpolated bounce-back; links (n, 3) without duplicates."""
    g = list(g)
    for k in range(links.shape[0]):
        i, j, q = (int(v) for v in links[k])
        qb = NS[q]
        cb = C[qb]
        im, jm = i + cb[0], j + cb[1]
        imm, jmm = i + 2 * cb[0], j + 2 * cb[1]
        pk = float(p[k])
        pp = 2.0 * pk
        if pk < 0.5:
            val = (pk * (pp + 1.0) * up[q][i, j] + (1.0 + pp) * (1.0 - pp) * up[q][im, jm]
                   - pk * (1.0 - pp) * up[q][imm, jmm])
        else:
            val = ((1.0 / (pk * (pp + 1.0))) * up[q][i, j] + ((pp - 1.0) / pk) * up[qb][i, j]
                   + ((1.0 - pp) / (1.0 + pp)) * up[qb][im, jm])
        new = g[qb].clone()
        new[i, j] = val
        g[qb] = new
    return g


def _set(g, q, idx, val):
    new = g[q].clone()
    new[idx] = val
    g[q] = new


def zou_he_channel(g, u_left_x, rho_right):
    """Bottom, left (velocity), top, right (pressure) walls, then the corners.

    Returns g and the rho/u values the corners read (nb.py:121-344)."""
    g = list(g)
    nx, ny = g[0].shape
    lx, ly = nx - 1, ny - 1
    C1, C2, C3 = 2.0 / 3.0, 1.0 / 6.0, 0.5
    rho = {}
    ux = {}
    uy = {}
    # bottom (u_bot = 0)
    r = (g[0][:, 0] + g[1][:, 0] + g[2][:, 0] + 2.0 * g[4][:, 0] + 2.0 * g[6][:, 0]
         + 2.0 * g[8][:, 0]) / (1.0 - 0.0)
    rb = r
    _set(g, 3, (slice(None), 0), g[4][:, 0] + C1 * r * 0.0)
    _set(g, 5, (slice(None), 0), g[6][:, 0] - C3 * (g[1][:, 0] - g[2][:, 0]) + C3 * r * 0.0 + C2 * r * 0.0)
    _set(g, 7, (slice(None), 0), g[8][:, 0] + C3 * (g[1][:, 0] - g[2][:, 0]) - C3 * r * 0.0 + C2 * r * 0.0)
    # left velocity (u_left = (u_left_x, 0))
    u0 = u_left_x
    r = (g[0][0, :] + g[3][0, :] + g[4][0, :] + 2.0 * g[2][0, :] + 2.0 * g[6][0, :]
         + 2.0 * g[7][0, :]) / (1.0 - u0)
    _set(g, 1, (0, slice(None)), g[2][0, :] + C1 * r * u0)
    _set(g, 5, (0, slice(None)), g[6][0, :] - C3 * (g[3][0, :] - g[4][0, :]) + C2 * r * u0 + C3 * r * 0.0)
    _set(g, 8, (0, slice(None)), g[7][0, :] + C3 * (g[3][0, :] - g[4][0, :]) + C2 * r * u0 - C3 * r * 0.0)
    # top (u_top = 0)
    r = (g[0][:, ly] + g[1][:, ly] + g[2][:, ly] + 2.0 * g[3][:, ly] + 2.0 * g[5][:, ly]
         + 2.0 * g[7][:, ly]) / (1.0 + 0.0)
    rt = r
    _set(g, 4, (slice(None), ly), g[3][:, ly] - C1 * r * 0.0)
    _set(g, 8, (slice(None), ly), g[7][:, ly] - C3 * (g[1][:, ly] - g[2][:, ly]) + C3 * r * 0.0 - C2 * r * 0.0)
    _set(g, 6, (slice(None), ly), g[5][:, ly] + C3 * (g[1][:, ly] - g[2][:, ly]) - C3 * r * 0.0 - C2 * r * 0.0)
    # right pressure (u_right_y = 0)
    r = rho_right
    uxr = (g[0][lx, :] + g[3][lx, :] + g[4][lx, :] + 2.0 * g[1][lx, :] + 2.0 * g[5][lx, :]
           + 2.0 * g[8][lx, :]) / r - 1.0
    _set(g, 2, (lx, slice(None)), g[1][lx, :] - C1 * r * uxr)
    _set(g, 6, (lx, slice(None)), g[5][lx, :] + C3 * (g[3][lx, :] - g[4][lx, :]) - C2 * r * uxr - C3 * r * 0.0)
    _set(g, 7, (lx, slice(None)), g[8][lx, :] - C3 * (g[3][lx, :] - g[4][lx, :]) - C2 * r * uxr + C3 * r * 0.0)
    # corners: rho from the x-neighbour on the bottom/top wall, u = 0 there
    for (i, j, in_, rr) in ((0, 0, 1, rb), (0, ly, 1, rt), (lx, ly, lx - 1, rt), (lx, 0, lx - 1, rb)):
        r = rr[in_]
        vx = vy = 0.0
        if (i, j) == (0, 0):
            _set(g, 1, (i, j), g[2][i, j] + (2.0 / 3.0) * r * vx)
            _set(g, 3, (i, j), g[4][i, j] + (2.0 / 3.0) * r * vy)
            _set(g, 5, (i, j), g[6][i, j] + (1.0 / 6.0) * r * vx + (1.0 / 6.0) * r * vy)
            z1, z2 = 7, 8
        elif (i, j) == (0, ly):
            _set(g, 1, (i, j), g[2][i, j] + (2.0 / 3.0) * r * vx)
            _set(g, 4, (i, j), g[3][i, j] - (2.0 / 3.0) * r * vy)
            _set(g, 8, (i, j), g[7][i, j] + (1.0 / 6.0) * r * vx - (1.0 / 6.0) * r * vy)
            z1, z2 = 5, 6
        elif (i, j) == (lx, ly):
            _set(g, 2, (i, j), g[1][i, j] - (2.0 / 3.0) * r * vx)
            _set(g, 4, (i, j), g[3][i, j] - (2.0 / 3.0) * r * vy)
            _set(g, 6, (i, j), g[5][i, j] - (1.0 / 6.0) * r * vx - (1.0 / 6.0) * r * vy)
            z1, z2 = 7, 8
        else:
            _set(g, 2, (i, j), g[1][i, j] - (2.0 / 3.0) * r * vx)
            _set(g, 3, (i, j), g[4][i, j] + (2.0 / 3.0) * r * vy)
            _set(g, 7, (i, j), g[8][i, j] - (1.0 / 6.0) * r * vx + (1.0 / 6.0) * r * vy)
            z1, z2 = 5, 6
        _set(g, z1, (i, j), torch.zeros((), dtype=g[0].dtype, device=g[0].device))
        _set(g, z2, (i, j), torch.zeros((), dtype=g[0].dtype, device=g[0].device))
        tot = g[1][i, j]
        for q in range(2, 9):
            tot = tot + g[q][i, j]
        _set(g, 0, (i, j), r - tot)
    return g


def drag_lift(up, g, links):
    fx = torch.zeros((), dtype=g[0].dtype, device=g[0].device)
    fy = torch.zeros((), dtype=g[0].dtype, device=g[0].device)
    for k in range(links.shape[0]):
        i, j, q = (int(v) for v in links[k])
        g0 = up[q][i, j] + g[NS[q]][i, j]
        fx = fx + g0 * C[q][0]
        fy = fy + g0 * C[q][1]
    return fx, fy


def run_channel(g0, om_p, profile, ramp, links, p, n_iter, window, rho_right=1.0):
    """Reference iterations 0..n_iter-1 of a channel with IBB obstacle links.

    g0: list of 9 (nx, ny) tensors (initial g); profile: (ny,) inlet u_x;
    ramp[it]: scale of the inlet at iteration it; window: iterations whose
    drag fx enters the objective.  Returns (sum of fx over the window, fx list).
    """
    g = list(g0)
    J = torch.zeros((), dtype=g[0].dtype, device=g[0].device)
    fxs = []
    for it in range(n_iter):
        up = collide(g, om_p)
        g = stream(g, up)
        g = ibb(g, up, links, p)
        g = zou_he_channel(g, ramp[it] * profile, rho_right)
        fx, fy = drag_lift(up, g, links)
        fxs.append(fx)
        if it in window:
            J = J + fx
    return J, fxs
