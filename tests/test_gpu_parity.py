"""GPU parity: the fused sm_103a kernels against the oracle (the reference's CPU time loop,
restated in C and pinned bit for bit to the reference's own Cython kernels by tests/golden).

The library is built without floating-point contraction, like the oracle, so receiver traces,
final fields, dispersive state and snapshots must be bit-identical. The 1e-5-of-peak bound
(peak of the field type, E or H, at that receiver / over the grid) is checked as well.
"""
import numpy as np
import pytest

from models import MODELS

TOL = 1e-5

pytestmark = pytest.mark.gpu


def _build(name):
    from gprmax_gb300.model import build_grid
    return build_grid(MODELS[name].splitlines(True), messages=False)


def _peak(a, c):
    g = 3 * (c // 3) if c < 6 else 6
    return max(np.abs(a[g:g + 3]).max(), 1e-30)


def compare(G, graph=True):
    from gprmax_gb300.solver import DeviceModel
    import oracle
    dm = DeviceModel(G)
    dm.run(graph=graph)
    rx, f = dm.receivers(), dm.fields()
    T = dm.dispersive() if G.maxpoles else None
    snaps = [dm.snapshot(s) for s in range(len(G.snapshots))]
    dm.close()
    ref = oracle.OracleSolver(G).run()
    rrx, rf = ref.receivers(), ref.fields()
    worst = 0.0
    for n in range(len(G.rxs)):
        for c in range(9):
            err = np.abs(rx[c, :, n] - rrx[c, :, n]).max() / _peak(rrx[:, :, n], c)
            worst = max(worst, err)
            assert err <= TOL, 'rx{} output {} differs by {:.3e} of peak'.format(n, c, err)
    np.testing.assert_array_equal(rx, rrx)
    for c in range(6):
        err = np.abs(f[c] - rf[c]).max() / _peak(rf, c)
        worst = max(worst, err)
        assert err <= TOL, 'field {} differs by {:.3e} of peak'.format(c, err)
    np.testing.assert_array_equal(f, rf)
    if T is not None:
        for c in range(3):
            Tr = ref.T[c]
            err = np.abs(T[c] - Tr).max() / max(np.abs(Tr).max(), 1e-30)
            assert err <= TOL, 'dispersive state {} differs by {:.3e}'.format(c, err)
            np.testing.assert_array_equal(T[c], Tr)
    for s in range(len(G.snapshots)):
        rs = ref.snaps[s]
        err = np.abs(snaps[s] - rs).max() / max(np.abs(rs).max(), 1e-30)
        assert err <= TOL, 'snapshot {} differs by {:.3e}'.format(s, err)
        np.testing.assert_array_equal(snaps[s], rs)
    return worst


@pytest.mark.parametrize('name', sorted(MODELS))
def test_model_matches_oracle(native, name):
    G = _build(name)
    compare(G)


def test_graph_and_stream_paths_agree(native):
    from gprmax_gb300.solver import DeviceModel
    G = _build('debye1')
    outs = []
    for graph in (True, False):
        dm = DeviceModel(G)
        dm.run(graph=graph)
        outs.append((dm.receivers(), dm.fields()))
        dm.close()
    assert np.array_equal(outs[0][0], outs[1][0])
    assert np.array_equal(outs[0][1], outs[1][1])


def test_split_runs_equal_one_run(native):
    """Advancing in pieces (with resets in between models) gives the same result."""
    from gprmax_gb300.solver import DeviceModel
    G = _build('hori2')
    dm = DeviceModel(G)
    dm.run()
    a = dm.receivers()
    dm.reset()
    for n in (1, 17, 40, G.iterations - 58):
        dm.run(n)
    b = dm.receivers()
    dm.close()
    assert np.array_equal(a, b)
