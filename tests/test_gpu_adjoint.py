"""GPU: the differentiable time loop (gbf_adj_*) against the pure-torch restatement of the same
model (tests/adjoint_reference.py, fp64 on the CPU): forward traces, and the checkpointed
discrete-adjoint gradient with respect to per-cell eps_r and sigma against torch's autograd
gradient; the gradient must not depend on the checkpoint interval."""
import numpy as np
import pytest

torch = pytest.importorskip('torch')

import adjoint_reference as ar  # noqa: E402
from adjoint_models import SMALL, materials  # noqa: E402

pytestmark = pytest.mark.gpu


def _setup(interval=0):
    from gprmax_gb300.adjoint import AdjointModel, AdjointSolver
    m = AdjointModel(SMALL.splitlines(True))
    return m, AdjointSolver(m, checkpoint_interval=interval)


def test_forward_traces_match_torch_reference(native):
    m, solver = _setup()
    eps, sig = materials(m, 2, torch.float64)
    ref = ar.forward(m, *m.edge_coefficients(eps, sig)).numpy()
    CA, CB = m.edge_coefficients(eps.cuda(), sig.cuda())
    tr = solver.forward(CA.float().contiguous(), CB.float().contiguous()).cpu().numpy()
    solver.close()
    for r in range(len(m.receivers)):
        assert np.abs(tr[r] - ref[r]).max() <= 2e-5 * np.abs(ref[r]).max()


def _gpu_gradient(m, solver, eps, sig, obs):
    from gprmax_gb300.adjoint import misfit
    e = eps.cuda().clone().requires_grad_(True)
    s = sig.cuda().clone().requires_grad_(True)
    loss, _ = misfit(m, solver, e, s, obs.cuda())
    loss.backward()
    return float(loss.detach()), e.grad.cpu(), s.grad.cpu()


def test_adjoint_gradient_matches_torch_autograd(native):
    m, solver = _setup()
    eps, sig = materials(m, 4, torch.float64)
    obs = ar.forward(m, *m.edge_coefficients(eps * 1.05, sig)).detach()
    e = eps.clone().requires_grad_(True)
    s = sig.clone().requires_grad_(True)
    loss = 0.5 * ((ar.forward(m, *m.edge_coefficients(e, s)) - obs) ** 2).sum()
    loss.backward()
    gl, ge, gs = _gpu_gradient(m, solver, eps, sig, obs)
    solver.close()
    assert abs(gl - float(loss)) <= 1e-4 * float(loss)
    for got, want in ((ge, e.grad), (gs, s.grad)):
        err = float((got - want).norm() / want.norm())
        assert err <= 1e-3, err
        assert float((got - want).abs().max()) <= 5e-3 * float(want.abs().max())


def test_gradient_independent_of_checkpoint_interval(native):
    grads = []
    for interval in (1, 9, 0, 70):
        m, solver = _setup(interval)
        eps, sig = materials(m, 6, torch.float64)
        obs = torch.zeros((len(m.receivers), m.iterations), dtype=torch.float64)
        grads.append(_gpu_gradient(m, solver, eps, sig, obs))
        solver.close()
    for g in grads[1:]:
        assert g[0] == grads[0][0]
        assert torch.equal(g[1], grads[0][1]) and torch.equal(g[2], grads[0][2])
