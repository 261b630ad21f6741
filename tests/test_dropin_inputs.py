"""Drop-in contract (CPU only): the grid object that the reference's own ``run_model`` builds
yields, through ``gprmax_gb300.solver.model_inputs``, exactly the descriptor and host arrays
that our front-end's grid yields for the same input file. ``solve_gb300`` hands those to the C
ABI, so the reference can call it in place of ``solve_cpu`` (``model_build_run.py:369-373``).

Needs the reference checkout and its kernels compiled by ``oracle/build_ref.py``; skipped
where they are absent.
"""
import os
import tempfile

import numpy as np
import pytest

from models import MODELS

import build_ref  # noqa: E402  (oracle/ is on sys.path via conftest)

SRC = build_ref.SOURCE
HERE = os.path.dirname(os.path.abspath(__file__))
REF_BUILD = os.path.join(os.path.dirname(HERE), 'oracle', '_ref', 'nofma', 'gprMax')


def _reference_available():
    """The checkout and the no-contraction build of every reference module ``run_model``
    imports (``oracle/build_ref.py --variant nofma``; the kernels alone are not enough)."""
    import glob
    return (os.path.isdir(os.path.join(SRC, 'gprMax')) and
            bool(glob.glob(os.path.join(REF_BUILD, 'geometry_outputs_ext.*.so'))))


pytestmark = pytest.mark.skipif(not _reference_available(),
                                reason='reference sources or compiled reference kernels absent')

DESC_FIELDS = ('nx', 'ny', 'nz', 'iterations', 'nmat', 'maxpoles', 'pml_formulation',
               'pml_order', 'dx', 'dy', 'dz', 'nsrc', 'nrx', 'nsnap', 'options')


def _reference_grid(name, tmp):
    import subprocess
    import sys
    import pickle
    inputfile = os.path.join(tmp, name + '.in')
    with open(inputfile, 'w') as f:
        f.write(MODELS[name])
    out = os.path.join(tmp, name + '.pkl')
    # a child process: the reference's modules keep class-level state between models
    code = '''
import sys, pickle
sys.path.insert(0, {root!r}); sys.path.insert(0, {oracle!r})
import ref_harness as rh
G = rh.run_reference({inputfile!r}, src={src!r}, nthreads=2, variant='nofma')
from gprmax_gb300.solver import model_inputs
inp = model_inputs(G)
d = inp.pop('desc')
inp['desc'] = {{f: getattr(d, f) for f in {fields!r}}}
inp['desc']['pml_thickness'] = list(d.pml_thickness)
pickle.dump(inp, open({out!r}, 'wb'))
'''.format(root=os.path.dirname(HERE), oracle=os.path.join(os.path.dirname(HERE), 'oracle'),
           inputfile=inputfile, src=SRC, fields=DESC_FIELDS, out=out)
    subprocess.run([sys.executable, '-c', code], check=True, cwd=os.path.dirname(HERE))
    with open(out, 'rb') as f:
        return pickle.load(f)


@pytest.mark.parametrize('name', ['mixed', 'debye1', 'hori2', 'fractal'])
def test_reference_grid_gives_the_same_solver_inputs(name):
    from gprmax_gb300.model import build_grid
    from gprmax_gb300.solver import model_inputs
    with tempfile.TemporaryDirectory() as tmp:
        ref = _reference_grid(name, tmp)
    ours = model_inputs(build_grid(MODELS[name].splitlines(True), messages=False))
    d = ours.pop('desc')
    for f in DESC_FIELDS:
        assert getattr(d, f) == ref['desc'][f], f
    assert list(d.pml_thickness) == ref['desc']['pml_thickness']
    for key in ('ID', 'coeffE', 'coeffH', 'coeffD', 'rx', 'snapshots'):
        a, b = ours[key], ref[key]
        assert (a is None) == (b is None), key
        if a is not None:
            np.testing.assert_array_equal(a, b, err_msg=key)
    assert [s for s, _ in ours['pml']] == [s for s, _ in ref['pml']]
    for (_, ra), (_, rb) in zip(ours['pml'], ref['pml']):
        for x, y in zip(ra, rb):
            np.testing.assert_array_equal(x, y)
    assert (ours['sources'] is None) == (ref['sources'] is None)
    if ours['sources'] is not None:
        for x, y in zip(ours['sources'], ref['sources']):
            np.testing.assert_array_equal(x, y)
