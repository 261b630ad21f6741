"""GPU: gbf_adj_backward_static, the adjoint backward whose fp32 segment partials live in a
fixed device array of the library (for callers that may not allocate device memory during the
call), gives the same gradients as gbf_adj_backward, bit for bit, on two consecutive calls, and
after its first call takes no device memory; grids too large for that array are rejected with
GBF_EINVAL."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip('torch')

from adjoint_models import SMALL, materials  # noqa: E402

pytestmark = pytest.mark.gpu

GBF_EINVAL = -1


def _call(solver, fn, CA, CB, gtr, free=None):
    """One backward call into fresh NaN-filled outputs; with `free`, the device's free bytes
    (cudaMemGetInfo) just before and after the call are appended to it."""
    gCA = torch.full((3,) + solver.model.shape, float('nan'), dtype=torch.float64, device='cuda')
    gCB = torch.full_like(gCA, float('nan'))
    torch.cuda.synchronize()
    before = torch.cuda.mem_get_info()[0]
    rc = fn(solver.h, CA.data_ptr(), CB.data_ptr(), gtr.data_ptr(), gCA.data_ptr(), gCB.data_ptr())
    torch.cuda.synchronize()
    if free is not None:
        free.append((before, torch.cuda.mem_get_info()[0]))
    solver._check(rc)
    return gCA.cpu(), gCB.cpu()


def test_static_scratch_backward_matches_backward(native):
    from gprmax_gb300.adjoint import AdjointModel, AdjointSolver
    m = AdjointModel(SMALL.splitlines(True))
    solver = AdjointSolver(m, checkpoint_interval=9)
    try:
        eps, sig = materials(m, 3, torch.float64)
        CA, CB = m.edge_coefficients(eps.cuda(), sig.cuda())
        CA = CA.float().contiguous()
        CB = CB.float().contiguous()
        tr = solver.forward(CA, CB)
        gtr = (0.25 * tr).contiguous()
        want = _call(solver, native.gbf_adj_backward, CA, CB, gtr)
        assert float(want[0].abs().max()) > 0
        free = []
        for _ in range(2):
            got = _call(solver, native.gbf_adj_backward_static, CA, CB, gtr, free)
            for g, w in zip(got, want):
                np.testing.assert_array_equal(g.numpy(), w.numpy())
        # after the first call (which looks the array up) the call takes no device memory
        assert free[1][0] == free[1][1], 'the second call changed free device memory'
        assert free[0][1] == free[1][1]
        # the context's own buffers are untouched: the plain call still agrees afterwards
        again = _call(solver, native.gbf_adj_backward, CA, CB, gtr)
        for g, w in zip(again, want):
            np.testing.assert_array_equal(g.numpy(), w.numpy())
    finally:
        solver.close()


BIG = """#domain: 0.090 0.090 0.090
#dx_dy_dz: 0.001 0.001 0.001
#time_window: 4
#pml_cells: 4
#waveform: ricker 1 3e9 w
#hertzian_dipole: z 0.045 0.045 0.045 w
#rx: 0.050 0.045 0.045
"""


def test_static_scratch_rejects_large_grids(native):
    from gprmax_gb300.adjoint import AdjointModel, AdjointSolver
    m = AdjointModel(BIG.splitlines(True))
    assert (m.nx + 1) * (m.ny + 1) * (m.nz + 1) > 699050
    solver = AdjointSolver(m)
    try:
        z = torch.zeros((3,) + m.shape, dtype=torch.float32, device='cuda')
        g = torch.zeros((3,) + m.shape, dtype=torch.float64, device='cuda')
        tr = torch.zeros((len(m.receivers), m.iterations), dtype=torch.float32, device='cuda')
        rc = native.gbf_adj_backward_static(solver.h, z.data_ptr(), z.data_ptr(), tr.data_ptr(),
                                            g.data_ptr(), g.data_ptr())
        assert rc == GBF_EINVAL
        buf = ctypes.create_string_buffer(1024)
        native.gbf_adj_last_error(solver.h, buf, 1024)
        assert b'699050' in buf.value
    finally:
        solver.close()
