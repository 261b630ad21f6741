"""CPU checks of the pure-torch restatement of the differentiable model (the reference the GPU
adjoint is tested against): its traces agree with the oracle (the reference's time loop) in
free space, and its autograd gradient agrees with central finite differences in fp64."""
import numpy as np
import pytest

torch = pytest.importorskip('torch')

import adjoint_reference as ar  # noqa: E402
from adjoint_models import SMALL, TINY, materials  # noqa: E402


def test_reference_traces_match_the_oracle_in_free_space():
    import oracle
    from gprmax_gb300.adjoint import AdjointModel
    from gprmax_gb300.model import build_grid
    m = AdjointModel(SMALL.splitlines(True))
    eps = torch.ones((m.nx, m.ny, m.nz), dtype=torch.float64)
    CA, CB = m.edge_coefficients(eps, torch.zeros_like(eps))
    tr = ar.forward(m, CA, CB).numpy()
    G = build_grid(SMALL.splitlines(True), messages=False)
    rx = oracle.OracleSolver(G).run().receivers()
    for r in range(len(m.receivers)):
        ref = rx[2, :, r]
        assert np.abs(tr[r] - ref).max() <= 1e-5 * np.abs(ref).max()


def test_reference_gradient_matches_finite_differences():
    from gprmax_gb300.adjoint import AdjointModel
    m = AdjointModel(TINY.splitlines(True))
    eps, sig = materials(m, 5, torch.float64)
    obs = ar.forward(m, *m.edge_coefficients(eps * 1.05, sig)).detach()
    e = eps.clone().requires_grad_(True)
    s = sig.clone().requires_grad_(True)
    loss = 0.5 * ((ar.forward(m, *m.edge_coefficients(e, s)) - obs) ** 2).sum()
    loss.backward()

    def L(ee, ss):
        return float(0.5 * ((ar.forward(m, *m.edge_coefficients(ee, ss)) - obs) ** 2).sum())
    rng = np.random.default_rng(1)
    for _ in range(4):
        c = tuple(int(rng.integers(2, n - 2)) for n in (m.nx, m.ny, m.nz))
        for which, grad, h in ((0, e.grad, 1e-4), (1, s.grad, 1e-6)):
            p, q = eps.clone(), sig.clone()
            (p if which == 0 else q)[c] += h
            up = L(p, q)
            (p if which == 0 else q)[c] -= 2 * h
            dn = L(p, q)
            fd = (up - dn) / (2 * h)
            assert abs(fd - float(grad[c])) <= 1e-5 * max(abs(fd), 1e-30) + 1e-12
