"""Device geometry build, host side (CPU only): with the ``gbf_geom_*`` entry points replaced by
their numpy restatement (``fake_geom.py``), ``build_grid(..., device_build=True)`` must give the
same materials (names, numbers, coefficients), ID array, solid and rigid arrays as the host
build, for every test model. The GPU tests run the same comparison on the real kernels."""
import numpy as np
import pytest

from fake_geom import FakeGeomLib
from models import MODELS

import gprmax_gb300.devgeom as devgeom
from gprmax_gb300.model import build_grid

NAMES = sorted(MODELS)


@pytest.fixture
def fake_lib(monkeypatch):
    lib = FakeGeomLib()
    monkeypatch.setattr(devgeom._native, 'lib', lambda: lib)
    return lib


def _same_build(G, D):
    assert [m.ID for m in G.materials] == [m.ID for m in D.materials]
    assert [m.numID for m in G.materials] == [m.numID for m in D.materials]
    np.testing.assert_array_equal(G.updatecoeffsE, D.updatecoeffsE)
    np.testing.assert_array_equal(G.updatecoeffsH, D.updatecoeffsH)
    if G.maxpoles:
        np.testing.assert_array_equal(G.updatecoeffsdispersive, D.updatecoeffsdispersive)
    np.testing.assert_array_equal(G.ID, D.geom.ids())
    np.testing.assert_array_equal(G.solid, D.geom.solid())
    rE, rH = D.geom.rigid()
    np.testing.assert_array_equal(G.rigidE, rE)
    np.testing.assert_array_equal(G.rigidH, rH)
    for p, q in zip(G.pmls, D.pmls):
        for n in ('ERA', 'ERB', 'ERE', 'ERF', 'HRA', 'HRB', 'HRE', 'HRF'):
            np.testing.assert_array_equal(getattr(p, n), getattr(q, n))


@pytest.mark.parametrize('name', NAMES)
def test_device_build_matches_host_build(fake_lib, name):
    lines = MODELS[name].splitlines(True)
    G = build_grid(lines, messages=False)
    D = build_grid(lines, messages=False, device_build=True)
    assert D.ID is None and D.solid is None
    _same_build(G, D)
    D.geom.close()


def test_averaged_keys_resolve_in_first_occurrence_order(fake_lib):
    """Averaged materials are numbered in the order the reference's loops first meet them."""
    lines = MODELS['smoothed'].splitlines(True)
    D = build_grid(lines, messages=False, device_build=True)
    names = [m.ID for m in D.materials]
    first = [n for n in names if n.count('+') == 3]
    assert first, names
    G = build_grid(lines, messages=False)
    assert [m.ID for m in G.materials if m.ID.count('+') == 3] == first


def test_real_dispersive_state_rule():
    """The models whose pole state the C ABI keeps as real parts (every pole Debye-like)."""
    from gprmax_gb300.solver import real_dispersive_state
    got = {n for n in MODELS
           if real_dispersive_state(build_grid(MODELS[n].splitlines(True), messages=False))}
    assert got == {'debye1', 'fractal', 'rough', 'tline', 'tmz'}
