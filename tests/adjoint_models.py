"""Small differentiable models for the adjoint tests (shared by the CPU and GPU tests)."""
import numpy as np

SMALL = """#domain: 0.016 0.015 0.014
#dx_dy_dz: 0.001 0.001 0.001
#time_window: 70
#pml_cells: 4 3 4 3 4 3
#waveform: ricker 1 3e9 w
#waveform: gaussiandot 1 4e9 w2
#hertzian_dipole: z 0.008 0.007 0.009 w
#hertzian_dipole: x 0.006 0.009 0.006 w2
#rx: 0.010 0.008 0.008
#rx: 0.005 0.006 0.009
#rx: 0.011 0.010 0.005
"""

TINY = """#domain: 0.010 0.009 0.008
#dx_dy_dz: 0.001 0.001 0.001
#time_window: 30
#pml_cells: 2
#waveform: ricker 1 5e9 w
#hertzian_dipole: z 0.005 0.004 0.004 w
#rx: 0.007 0.005 0.004
"""


def materials(model, seed, dtype):
    """Seeded heterogeneous eps_r in [1, 9] and sigma in [0, 0.02] S/m per cell."""
    import torch
    rng = np.random.default_rng(seed)
    shape = (model.nx, model.ny, model.nz)
    eps = torch.tensor(1 + 8 * rng.random(shape), dtype=dtype)
    sig = torch.tensor(0.02 * rng.random(shape), dtype=dtype)
    return eps, sig
