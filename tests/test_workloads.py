"""The B-scan workload inputs (CPU only, no model build): every antenna pair sits inside the
PML-free part of its domain, the reference-sized shapes keep one position per model, and small
shapes wrap the positions instead of leaving the domain."""
import pytest

from gprmax_gb300 import workloads


def _coords(lines, cmd):
    for line in lines:
        if line.startswith(cmd):
            return [float(v) for v in line.split(':', 1)[1].split()[-4:-1]] \
                if cmd == '#hertzian_dipole' else [float(v) for v in line.split(':', 1)[1].split()]
    raise AssertionError(cmd)


@pytest.mark.parametrize('shape', [(200, 200, 100), (300, 300, 150), (64, 64, 64), (96, 96, 64)])
def test_antenna_pair_inside_the_pml_free_region(shape):
    dx, pml = 0.002, 10
    xs = set()
    for m in range(64):
        lines = workloads.bscan_input(shape, 11 + m, m)
        src = _coords(lines, '#hertzian_dipole')
        rx = _coords(lines, '#rx')
        for p in (src, rx):
            for v, n in zip(p, shape):
                assert pml * dx <= v <= (n - pml) * dx, (shape, m, p)
        xs.add(round(src[0], 6))
    if shape[0] >= 200:
        assert len(xs) == 64
        assert min(xs) == pytest.approx(0.06) and max(xs) == pytest.approx(0.06 + 0.004 * 63)
    else:
        assert 1 <= len(xs) < 64


def test_2d_bscan_models_step_the_antenna_pair():
    grids = workloads.bscan_2d_models(4)
    for n, G in enumerate(grids):
        assert G.mode == '2D TMz' and G.nz == 1
        assert G.pmlthickness['z0'] == 0 and G.pmlthickness['x0'] == 10
        assert G.hertziandipoles[0].xcoord == grids[0].hertziandipoles[0].xcoord + n
        assert G.rxs[0].xcoord == grids[0].rxs[0].xcoord + n
        assert G.rxs[0].xcoord - G.hertziandipoles[0].xcoord == 20
