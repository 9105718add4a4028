"""Adjoint gradient of a drag objective: CUDA adjoint vs torch autograd
through the pure-tensor reference step (oracle/torch_ref.py), and vs FP64
central finite differences of the CUDA forward."""
import contextlib
import io
import tempfile

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

T, WIN = 60, (30, 59)


def _turek(L=32):
    from lbm_gb300.apps import turek
    a = turek()
    a.L_lbm = L
    a.compute_lbm_parameters()
    a.sigma = 20.0
    a.stop, a.it_max, a.output_freq = "it", T - 1, 10 ** 12
    return a


def _adjoint():
    import lbm_gb300
    from lbm_gb300.adjoint import DragAdjoint
    app = _turek()
    with contextlib.redirect_stdout(io.StringIO()):
        lat = lbm_gb300.lattice(app, precision="f64", output_dir=tempfile.mkdtemp(), verbose=False)
        app.initialize(lat)
    return app, lat, DragAdjoint(lat, app)


@pytest.fixture(scope="module")
def run(cuda):
    app, lat, adj = _adjoint()
    w = np.zeros(2 * len(adj.eng.obstacles))
    w[0] = 1.0  # J = sum of the raw drag sum fx over the window
    J = adj.forward(T, WIN, w)
    grad = adj.gradient()
    return app, lat, adj, J, grad, w


def test_adjoint_matches_torch_autograd(run):
    from oracle import torch_ref
    app, lat, adj, J, grad, _ = run
    ny = lat.ny
    g0 = [torch.from_numpy(adj.g0[q].cpu().numpy().copy()) for q in range(9)]
    obs = adj.eng.obstacles[0]
    links = np.asarray(obs.boundary)
    p = np.asarray(obs.ibb)
    base, vec, scale = adj.sched
    prof = torch.tensor(vec[:ny], dtype=torch.float64, requires_grad=True)
    om = torch.tensor(lat.om_p_lbm, dtype=torch.float64, requires_grad=True)
    ramp = [float(s) for s in scale(np.arange(T))]
    Jt, _ = torch_ref.run_channel(g0, om, prof, ramp, links, p, T, set(range(WIN[0], WIN[1] + 1)))
    Jt.backward()
    assert abs(J - Jt.item()) <= 1e-10 * abs(Jt.item())
    g_prof = prof.grad.numpy()
    assert np.max(np.abs(grad["bc_vec"][:ny] - g_prof)) <= 1e-7 * np.max(np.abs(g_prof))
    assert abs(grad["omega"] - om.grad.item()) <= 1e-7 * abs(om.grad.item())


def test_adjoint_matches_central_differences(run):
    app, lat, adj, J, grad, w = run
    h = 1e-6
    om0 = lat.om_p_lbm
    vec0 = adj.vec.copy()
    ny = lat.ny

    def J_at(om=None, vec=None):
        adj.set_omega(om if om is not None else om0)
        adj.set_bc_vec(vec if vec is not None else vec0)
        return adj.forward(T, WIN, w, checkpoint=False)

    fd_om = (J_at(om=om0 + h) - J_at(om=om0 - h)) / (2 * h)
    assert abs(fd_om - grad["omega"]) <= 1e-5 * abs(grad["omega"])
    for j in (ny // 4, ny // 2):
        vp, vm = vec0.copy(), vec0.copy()
        vp[j] += h
        vm[j] -= h
        fd = (J_at(vec=vp) - J_at(vec=vm)) / (2 * h)
        assert abs(fd - grad["bc_vec"][j]) <= 1e-5 * abs(grad["bc_vec"][j]) + 1e-9
    J_at()


def test_autograd_function_gives_the_adjoint_gradient(run):
    from lbm_gb300.adjoint import DragObjective
    app, lat, adj, J, grad, w = run
    ny = lat.ny
    base, vec, _ = adj.sched
    om = torch.tensor(lat.om_p_lbm, dtype=torch.float64, requires_grad=True)
    inlet = torch.tensor(vec[:ny], dtype=torch.float64, requires_grad=True)
    Jt = DragObjective.apply(om, inlet, adj, T, WIN, w)
    (2.0 * Jt).backward()
    assert abs(Jt.item() - J) <= 1e-13 * abs(J)
    assert abs(om.grad.item() - 2.0 * grad["omega"]) <= 1e-12 * abs(grad["omega"])
    ref = 2.0 * grad["bc_vec"][:ny]
    assert np.max(np.abs(inlet.grad.numpy() - ref)) <= 1e-12 * np.max(np.abs(ref))
