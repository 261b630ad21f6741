"""Geometry commands on the CPU: the cases #triangle and #cylindrical_sector refuse. A
zero-thickness face whose far rigid edge flags would fall outside the grid (last cell row, upper
boundary plane; the reference writes past the end of its array there), and a zero-thickness
shape given three materials (the reference passes its builder no material number and the call
fails). Everything they do build is pinned to the reference by the ``triangles`` and
``sectors`` golden fixtures."""
import pytest

from gprmax_gb300.exceptions import CmdInputError
from gprmax_gb300.model import build_grid

BASE = """#domain: 0.030 0.030 0.030
#dx_dy_dz: 0.001 0.001 0.001
#time_window: 10
#pml_cells: 5
#material: 4 0 1 0 a
#material: 5 0 1 0 b
#material: 6 0 1 0 c
#waveform: ricker 1 1e9 w
#hertzian_dipole: z 0.015 0.015 0.015 w
#rx: 0.017 0.015 0.015
"""


def _build(extra):
    return build_grid((BASE + extra + '\n').splitlines(True), messages=False)


@pytest.mark.parametrize('cmd', [
    '#cylindrical_sector: x 0.028 0.010 0.012 0.012 0.004 0 90 pec',
    '#triangle: 0.010 0.010 0.030 0.020 0.010 0.030 0.012 0.020 0.030 0 pec',
    '#triangle: 0.010 0.010 0.020 0.020 0.010 0.020 0.012 0.020 0.020 0 a b c',
    '#cylindrical_sector: z 0.015 0.015 0.010 0.010 0.004 0 90 a b c',
])
def test_refused(cmd):
    with pytest.raises(CmdInputError):
        _build(cmd)


@pytest.mark.parametrize('cmd', [
    '#triangle: 0.010 0.010 0.020 0.020 0.010 0.020 0.012 0.020 0.020 0 pec',
    '#triangle: 0.010 0.010 0.020 0.020 0.010 0.020 0.012 0.020 0.020 0.002 a b c',
    '#cylindrical_sector: x 0.028 0.010 0.012 0.016 0.004 0 90 a',
])
def test_built(cmd):
    G = _build(cmd)
    assert G.rigidE.any() or (G.solid > 1).any()
