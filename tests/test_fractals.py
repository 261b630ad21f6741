"""``#fractal_box`` / ``#soil_peplinski`` (CPU only): the fractal volume, the mixing-model
materials and the command checks against the reference (``gprMax/fractals.py:141-194``,
``gprMax/materials.py:268-330``, ``input_cmds_geometry.py:808-888``,
``input_cmds_multiuse.py:694-722``). Whole-model agreement (ID array and coefficients) is
covered by the ``fractal`` golden fixture."""
import glob
import os
import subprocess
import sys
import tempfile

import numpy as np
import pytest

from gprmax_gb300.exceptions import CmdInputError
from gprmax_gb300.fractals import FractalVolume
from gprmax_gb300.model import build_model_file

import build_ref  # noqa: E402  (oracle/ is on sys.path via conftest)

SRC = build_ref.SOURCE
HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.join(os.path.dirname(HERE), 'oracle')
REF_BUILD = os.path.join(ORACLE, '_ref', 'nofma', 'gprMax')

HEAD = """#domain: 0.020 0.020 0.020
#dx_dy_dz: 0.001 0.001 0.001
#time_window: 10
#pml_cells: 4
#soil_peplinski: 0.5 0.5 2.0 2.66 0.001 0.3 soil
#material: 4 0 1 0 rock
"""


def _build(text):
    with tempfile.TemporaryDirectory() as tmp:
        f = os.path.join(tmp, 'm.in')
        with open(f, 'w') as fh:
            fh.write(text)
        return build_model_file(f, messages=False)


def test_mixing_model_materials_are_named_and_numbered_like_the_reference():
    G = _build(HEAD + '#fractal_box: 0 0 0 0.020 0.020 0.010 1.5 1 1 1 12 soil box 5\n')
    names = [m.ID for m in G.materials]
    assert names[3:15] == ['|box_{:02d}|'.format(n) for n in range(1, 13)]
    soil = names.index('|box_01|')
    assert G.solid[:, :, :10].min() >= soil and G.solid[:, :, :10].max() < soil + 12
    assert (G.solid[:, :, 10:] == 1).all()
    assert G.maxpoles == 1
    assert len(G.fractalvolumes) == 1


@pytest.mark.parametrize('line, msg', [
    ('#fractal_box: 0 0 0 0.020 0.020 0.010 1.5 1 1 1 1 soil box 5', 'more than one material'),
    ('#fractal_box: 0 0 0 0.020 0.020 0.010 1.5 1 1 1 1 rock box 5', 'please use a #box'),
    ('#fractal_box: 0 0 0 0.020 0.020 0.010 1.5 1 1 1 6 clay box 5', 'does not exist'),
    ('#fractal_box: 0 0 0 0.020 0.020 0.010 1.5 1 1 1 6 soil box 5 x', 'either y or n'),
    ('#fractal_box: 0 0 0 0.020 0.020 0.010 1.5 1 1 1 6 soil', 'thirteen parameters'),
    ('#fractal_box: 0 0 0.012 0.020 0.020 0.010 1.5 1 1 1 6 soil box', 'lower coordinates'),
    ('#fractal_box: 0 0 0 0.020 0.020 0.030 1.5 1 1 1 6 soil box', 'not within the model domain'),
    ('#fractal_box: 0 0 0 0.020 0.020 0.010 -1 1 1 1 6 soil box', 'fractal dimension'),
    ('#fractal_box: 0 0 0 0.020 0.020 0.010 1.5 1 -1 1 6 soil box', 'y direction'),
    ('#fractal_box: 0 0 0 0.020 0.020 0.010 1.5 1 1 1 6 soil box 5\n'
     '#add_surface_water: 0 0 0.010 0.020 0.020 0.010 0.008 box', 'add_surface_water'),
])
def test_fractal_box_errors(line, msg):
    with pytest.raises(CmdInputError, match=msg):
        _build(HEAD + line + '\n')


@pytest.mark.parametrize('line, msg', [
    ('#soil_peplinski: 0.5 0.5 2.0 2.66 0.001 soil2', 'exactly seven'),
    ('#soil_peplinski: 0.5 -0.5 2.0 2.66 0.001 0.3 soil2', 'clay fraction'),
    ('#soil_peplinski: 0.5 0.5 2.0 2.66 0.001 0.3 soil', 'already exists'),
])
def test_soil_peplinski_errors(line, msg):
    with pytest.raises(CmdInputError, match=msg):
        _build(HEAD + line + '\n')


def test_volume_bins_cover_all_materials_and_are_seeded():
    a = FractalVolume(0, 24, 0, 20, 0, 16, 1.5, 42)
    a.nbins = 10
    va = a.generate_fractal_volume()
    b = FractalVolume(0, 24, 0, 20, 0, 16, 1.5, 42)
    b.nbins = 10
    assert np.array_equal(va, b.generate_fractal_volume())
    assert va.dtype == np.float32 and va.shape == (24, 20, 16)
    assert va.min() == 0 and va.max() == 9
    c = FractalVolume(0, 24, 0, 20, 0, 16, 1.5, 43)
    c.nbins = 10
    assert not np.array_equal(va, c.generate_fractal_volume())


CASES = [((40, 30, 20), 1.5, (1, 1, 1), 5, 7), ((33, 17, 25), 2.2, (1.0, 0.5, 2.0), 20, 3),
         ((50, 1, 40), 1.8, (1, 1, 1), 4, 11), ((1, 30, 26), 2.6, (1, 1, 0.5), 9, 2)]

CHILD = r'''
import sys, numpy as np
sys.path.insert(0, {oracle!r})
import ref_harness as rh
rh.load({src!r}, 'nofma')
import gprMax.fractals as F
class G: nthreads = 4
out = {{}}
for n, (shape, D, wt, nb, seed) in enumerate({cases!r}):
    v = F.FractalVolume(0, shape[0], 0, shape[1], 0, shape[2], D, seed)
    v.weighting = np.array(wt, dtype=np.float64)
    v.nbins = nb
    v.generate_fractal_volume(G)
    out['v%d' % n] = v.fractalvolume
np.savez({dest!r}, **out)
'''


@pytest.mark.skipif(not (os.path.isdir(os.path.join(SRC, 'gprMax')) and
                         bool(glob.glob(os.path.join(REF_BUILD, 'fractals_generate_ext.*.so')))),
                    reason='reference sources or compiled reference kernels absent')
def test_fractal_volume_matches_reference_bit_for_bit():
    with tempfile.TemporaryDirectory() as tmp:
        dest = os.path.join(tmp, 'v.npz')
        code = CHILD.format(oracle=ORACLE, src=SRC, cases=CASES, dest=dest)
        subprocess.run([sys.executable, '-c', code], check=True)
        ref = dict(np.load(dest))
    for n, (shape, D, wt, nb, seed) in enumerate(CASES):
        v = FractalVolume(0, shape[0], 0, shape[1], 0, shape[2], D, seed)
        v.weighting = np.array(wt, dtype=np.float64)
        v.nbins = nb
        np.testing.assert_array_equal(v.generate_fractal_volume(), ref['v%d' % n])


ROUGH = HEAD + '#fractal_box: 0 0 0 0.020 0.020 0.010 1.5 1 1 1 6 soil box 5\n'


@pytest.mark.parametrize('lines, msg', [
    ('#add_surface_water: 0 0 0.010 0.020 0.020 0.010 0.012 box', 'does not have a rough surface'),
    ('#add_surface_roughness: 0 0 0.010 0.020 0.020 0.010 1.5 1 1 0.008 0.014 box 3\n'
     '#add_surface_water: 0 0 0.010 0.020 0.020 0.010 0.016 box', 'lies with the range'),
    ('#add_surface_roughness: 0 0 0.006 0.020 0.020 0.006 1.5 1 1 0.004 0.012 box 3',
     'external surfaces'),
    ('#add_surface_roughness: 0 0 0.010 0.020 0.020 0.010 1.5 1 1 0.008 0.014 box 3\n'
     '#add_surface_roughness: 0 0 0.010 0.020 0.020 0.010 1.5 1 1 0.008 0.014 box 4',
     'already been used'),
    ('#add_surface_roughness: 0 0 0.010 0.020 0.020 0.010 1.5 1 1 0.008 0.030 box 3',
     'exceed either the lower coordinates'),
    ('#add_surface_roughness: 0 0 0.010 0.020 0.020 0.010 1.5 1 1 0.008 0.014 box 3 9',
     'too many parameters'),
    ('#add_grass: 0 0 0.010 0.020 0.020 0.010 1.5 0.010 0.015 10 box 3', 'add_grass'),
])
def test_surface_modifier_errors(lines, msg):
    with pytest.raises(CmdInputError, match=msg):
        _build(ROUGH + lines + '\n')


def test_rough_top_surface_extends_the_box_and_adds_water():
    G = _build(ROUGH + '#add_surface_roughness: 0 0 0.010 0.020 0.020 0.010 1.5 1 1 0.008 '
               '0.014 box 3\n#add_surface_water: 0 0 0.010 0.020 0.020 0.010 0.012 box\n')
    water = next(m for m in G.materials if m.ID == 'water')
    soil = [m.numID for m in G.materials if m.ID.startswith('|box_')]
    top = G.solid[:, :, 10:14]
    assert (G.solid[:, :, 14:] == 1).all()
    assert np.isin(top, soil + [water.numID, 1]).all()
    assert (top == water.numID).any() and np.isin(top, soil).any()
    assert np.isin(G.solid[:, :, :8], soil).all()


SURFACES = [((30, 24), 1.5, (1.0, 1.0), (3, 12), 7), ((17, 40), 2.2, (0.5, 2.0), (10, 20), 3)]

SURF_CHILD = r'''
import sys, numpy as np
sys.path.insert(0, {oracle!r})
import ref_harness as rh
rh.load({src!r}, 'nofma')
import gprMax.fractals as F
class G: nthreads = 4
out = {{}}
for n, (dims, D, wt, rng, seed) in enumerate({cases!r}):
    s = F.FractalSurface(0, 0, 0, dims[0], 0, dims[1], D, seed)
    s.weighting = np.array(wt, dtype=np.float64)
    s.fractalrange = rng
    s.generate_fractal_surface(G)
    out['s%d' % n] = s.fractalsurface
np.savez({dest!r}, **out)
'''


@pytest.mark.skipif(not (os.path.isdir(os.path.join(SRC, 'gprMax')) and
                         bool(glob.glob(os.path.join(REF_BUILD, 'fractals_generate_ext.*.so')))),
                    reason='reference sources or compiled reference kernels absent')
def test_fractal_surface_matches_reference_bit_for_bit():
    from gprmax_gb300.fractals import FractalSurface
    with tempfile.TemporaryDirectory() as tmp:
        dest = os.path.join(tmp, 's.npz')
        code = SURF_CHILD.format(oracle=ORACLE, src=SRC, cases=SURFACES, dest=dest)
        subprocess.run([sys.executable, '-c', code], check=True)
        ref = dict(np.load(dest))
    for n, (dims, D, wt, rng, seed) in enumerate(SURFACES):
        s = FractalSurface(0, 0, 0, dims[0], 0, dims[1], D, seed)
        s.weighting = np.array(wt, dtype=np.float64)
        s.fractalrange = rng
        got = s.generate_fractal_surface()
        assert got.dtype == ref['s%d' % n].dtype
        np.testing.assert_array_equal(got, ref['s%d' % n])
