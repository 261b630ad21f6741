"""GPU: the differentiable time loop (gbf_adj_*) against the pure-torch restatement of the same
model (tests/adjoint_reference.py, fp64 on the CPU): forward traces, and the checkpointed
discrete-adjoint gradient with respect to per-cell eps_r and sigma against torch's autograd
gradient; the gradient must not depend on the checkpoint interval beyond the rounding of its sums."""
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
    assert abs(gl - float(loss.detach())) <= 1e-4 * float(loss.detach())
    for got, want in ((ge, e.grad), (gs, s.grad)):
        err = float((got - want).norm() / want.norm())
        assert err <= 1e-3, err
        assert float((got - want).abs().max()) <= 5e-3 * float(want.abs().max())


def test_gradient_independent_of_checkpoint_interval(native):
    grads = []
    for interval in (1, 9, 0, 70, -1):
        m, solver = _setup(interval)
        eps, sig = materials(m, 6, torch.float64)
        obs = torch.zeros((len(m.receivers), m.iterations), dtype=torch.float64)
        grads.append(_gpu_gradient(m, solver, eps, sig, obs))
        solver.close()
    # the forward is the same; the gradient partials are summed in fp32 within a segment and in
    # fp64 across segments, so the interval changes only the rounding of the sums
    for g in grads[1:]:
        assert g[0] == grads[0][0]
        for a, b in ((g[1], grads[0][1]), (g[2], grads[0][2])):
            assert float((a - b).abs().max()) <= 1e-5 * float(b.abs().max())


CROP = """#domain: 0.064 0.064 0.064
#dx_dy_dz: 0.002 0.002 0.002
#time_window: 240
#pml_cells: 6
#waveform: ricker 1 3e9 w
#hertzian_dipole: z 0.032 0.032 0.044 w
#rx: 0.020 0.032 0.044
#rx: 0.044 0.032 0.044
"""


@pytest.mark.parametrize('window', ['240', '8e-9'])
def test_adjoint_on_a_crop_of_the_gradient_workload(native, window):
    """A 32^3 crop of the 200x200x100 Gaussian-random-field model, over 240 iterations and over
    the gradient workload's full 8 ns (2079 iterations, where the default checkpointing makes the
    last segment most of the run: the fp32 partial sums go into fp64 every ceil(sqrt(T)) steps).
    The misfit's residual r (GPU traces minus data from the crop of the 'true' model) is small
    here, so fp32 rounding in the forward moves it; the adjoint is therefore checked on the
    residual it was given: the GPU gradient J^T r against torch's fp64 autograd of
    sum(traces * r) of the pure-torch model (relative L2 <= 1e-3), and, over 240 iterations,
    against fp64 central finite differences of that sum on 20 seeded cells."""
    from gprmax_gb300 import workloads
    from gprmax_gb300.adjoint import AdjointModel, AdjointSolver
    _, eps, sig, true = workloads.adjoint_problem()
    crop = (slice(84, 116), slice(84, 116), slice(34, 66))
    dev = torch.device('cuda')
    e0 = torch.tensor(eps[crop], dtype=torch.float64, device=dev)
    s0 = torch.tensor(sig[crop], dtype=torch.float64, device=dev)
    et = torch.tensor(true[crop], dtype=torch.float64, device=dev)
    m = AdjointModel(CROP.replace('#time_window: 240', '#time_window: ' + window).splitlines(True))
    solver = AdjointSolver(m)
    obs = ar.forward(m, *m.edge_coefficients(et, s0)).detach()
    _, ge, _ = _gpu_gradient(m, solver, e0.cpu(), s0.cpu(), obs.cpu())
    CA, CB = m.edge_coefficients(e0, s0)
    r = (solver.forward(CA.float().contiguous(), CB.float().contiguous()).double() - obs).detach()
    solver.close()
    e = e0.clone().requires_grad_(True)
    (ar.forward(m, *m.edge_coefficients(e, s0)) * r).sum().backward()
    want = e.grad.cpu()
    err = float((ge - want).norm() / want.norm())
    print('\n{} iterations: GPU gradient against fp64 autograd, relative L2 {:.2e}'.format(
        m.iterations, err))
    assert err <= 1e-3
    if m.iterations > 1000:
        return

    def L(ee):
        return float((ar.forward(m, *m.edge_coefficients(ee, s0)) * r).sum())
    flat = want.abs().flatten()
    top = torch.topk(flat, flat.numel() // 10).indices.numpy()
    cells = np.random.default_rng(9).choice(top, 20, replace=False)
    for c in cells:
        idx = np.unravel_index(int(c), want.shape)
        h = 1e-4 * float(e0[idx])
        p = e0.clone()
        p[idx] += h
        up = L(p)
        p[idx] -= 2 * h
        fd = (up - L(p)) / (2 * h)
        assert abs(float(ge[idx]) - fd) <= 1e-3 * abs(fd), (idx, float(ge[idx]), fd)
