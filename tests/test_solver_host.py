"""Host-side helpers of the solver that need no GPU: whether two grids may share one device
copy of their geometry (``solver.same_geometry``, used by ``BatchModel``), and whether a model's
H half-step can run without material IDs (``solver.uniform_h``)."""
import numpy as np

from gprmax_gb300.model import build_grid
from gprmax_gb300.solver import same_geometry, uniform_h
from gprmax_gb300 import workloads
from models import MODELS


def _grid(text):
    return build_grid(text.splitlines(True), messages=False)


def test_grids_built_from_the_same_lines_share_their_geometry():
    a, b = _grid(MODELS['debye1']), _grid(MODELS['debye1'])
    assert a.ID is not b.ID and same_geometry(a, b) and same_geometry(a, a)


def test_the_traces_of_a_bscan_share_their_geometry():
    """The 2D B-scan's traces differ in their source and receiver positions only."""
    grids = workloads.bscan_2d_models(3)
    assert all(same_geometry(grids[0], G) for G in grids[1:])
    assert [G.hertziandipoles[0].xcoord for G in grids] == sorted(
        set(G.hertziandipoles[0].xcoord for G in grids))


def test_different_geometry_is_told_apart():
    """A different material table, a different grid size, or the same tables with one cell of
    another material: no sharing."""
    base = MODELS['fs_hori1']
    a = _grid(base + '#material: 4 0 1 0 block\n#box: 0.010 0.010 0.010 0.014 0.014 0.014 block\n')
    other_eps = _grid(base + '#material: 5 0 1 0 block\n#box: 0.010 0.010 0.010 0.014 0.014 0.014 block\n')
    moved = _grid(base + '#material: 4 0 1 0 block\n#box: 0.011 0.010 0.010 0.015 0.014 0.014 block\n')
    assert not same_geometry(a, other_eps)
    assert np.array_equal(a.updatecoeffsE, moved.updatecoeffsE)
    assert not same_geometry(a, moved)
    assert not same_geometry(a, _grid(MODELS['pml_off']))


def test_uniform_h_rows():
    """Dielectrics, conductors and dispersive materials leave every H row equal to free
    space's; a magnetic material does not."""
    assert uniform_h(_grid(MODELS['fs_hori1']))
    assert uniform_h(_grid(MODELS['debye1']))
    assert not uniform_h(_grid(MODELS['fs_hori1'] +
                               '#material: 1 0 2 0 mag\n#box: 0.010 0.010 0.010 0.014 0.014 0.014 mag\n'))
