"""GPU: the staged half-steps (gprmax_gb300/csrc/staged.cuh) against the plain half-step kernels
(options bit 4), bit for bit.

The staged sweeps copy each chunk's fields, neighbour rows, packed material words and pole state
into shared memory with bulk copies and update the nodes from there, with h_node's and e_node's
arithmetic; so receivers, all six fields and the dispersive state must equal the plain kernels'
exactly. The models cover every PML kind, no poles and one real pole, magnetic materials (the
H sweep reading packed IDs), complex poles (Lorentz, Drude, their state staged as pairs),
sources on the domain's upper
faces, a transmission line, receiver arrays, fractal soil and rough surfaces; grids from
20 x 18 x 16 cells (copies clamped at both ends of the arrays) up. Both runs use the two
half-step kernels (options bit 3), so the staged sweeps run every step.
"""
import numpy as np
import pytest

from models import MODELS

pytestmark = pytest.mark.gpu

STAGED_MODELS = ['fs_hori1', 'pml_off', 'hori2', 'mri1', 'mri2', 'debye1', 'faces', 'smoothed',
                 'fractal', 'rough', 'rxarray', 'tline', 'triangles', 'mixed']


def _run(G, options, nsteps=None, forms=None):
    from gprmax_gb300.solver import DeviceModel
    dm = DeviceModel(G, options)
    try:
        if forms is not None:
            dm.set_step_forms(*forms)
        dm.run(nsteps)
        out = {'rx': dm.receivers(), 'f': dm.fields(), 'info': dm.step_info()}
        if G.maxpoles:
            out['T'] = dm.dispersive()
    finally:
        dm.close()
    return out


def _equal(a, b):
    np.testing.assert_array_equal(a['rx'], b['rx'])
    np.testing.assert_array_equal(a['f'], b['f'])
    if 'T' in a:
        np.testing.assert_array_equal(a['T'], b['T'])


@pytest.mark.parametrize('name', STAGED_MODELS)
def test_staged_e_half_step_equals_plain(native, name):
    from gprmax_gb300.model import build_grid
    G = build_grid(MODELS[name].splitlines(True), messages=False)
    got = _run(G, 8, forms=(True, True))
    ref = _run(G, 8 | 16)
    assert got['info']['staged_h'], 'model {} should take the staged H half-step'.format(name)
    assert got['info']['staged'], 'model {} should take the staged E half-step'.format(name)
    assert not ref['info']['staged'] and not ref['info']['staged_h']
    _equal(got, ref)
    # each staged sweep alone, and the forms the tuner keeps
    _equal(_run(G, 8, forms=(False, True)), ref)
    _equal(_run(G, 8, forms=(True, False)), ref)
    tuned = _run(G, 8)
    assert tuned['info']['forms_tuned']
    _equal(tuned, ref)


def test_staged_against_oracle(native):
    import oracle
    from gprmax_gb300.model import build_grid
    G = build_grid(MODELS['debye1'].splitlines(True), messages=False)
    got = _run(G, 8, forms=(True, True))
    assert got['info']['staged'] and got['info']['staged_h']
    ref = oracle.OracleSolver(G).run()
    np.testing.assert_array_equal(got['rx'], ref.receivers())
    np.testing.assert_array_equal(got['f'], ref.fields())


def test_complex_pole_state_staged(native):
    """A Debye model with its pole state kept complex (option bit 2) takes the staged E sweep
    with the (re, im) pairs staged; its results equal the real-state staged run's and the plain
    kernel's."""
    from gprmax_gb300.model import build_grid
    G = build_grid(MODELS['debye1'].splitlines(True), messages=False)
    cplx = _run(G, 8 | 4, forms=(True, True))
    assert cplx['info']['staged'] and cplx['info']['staged_available']
    plain = _run(G, 8 | 4 | 16)
    assert not plain['info']['staged']
    _equal(cplx, plain)
    real = _run(G, 8, forms=(True, True))
    np.testing.assert_array_equal(cplx['rx'], real['rx'])
    np.testing.assert_array_equal(cplx['f'], real['f'])


def test_staged_soil(native):
    """A 160 x 160 x 80 cut of the benchmark soil (50 Debye materials, 10-cell PML, dipole and
    receiver), 300 iterations, staged against plain; the default run (whatever step the tuner
    keeps) equals both."""
    from gprmax_gb300 import workloads
    G = workloads.dispersive_soil(nx=160, ny=160, nz=80, surface=60, timewindow='3e-9')
    got = _run(G, 8, 300, forms=(True, True))
    ref = _run(G, 8 | 16, 300)
    assert got['info']['staged'] and got['info']['staged_h']
    _equal(got, ref)
    dflt = _run(G, 0, 300)
    _equal(dflt, ref)


@pytest.mark.parametrize('formulation,order', [('HORIPML', 2), ('MRIPML', 1), ('MRIPML', 2)])
def test_staged_soil_other_pml_kinds(native, formulation, order):
    """A 120 x 110 x 150 cut of the soil (chunks spanning several rows, z slabs on every row)
    with second-order HORIPML and first- and second-order MRIPML (the CFS parameters of the
    PML fixtures), 200 iterations: the staged sweeps equal the plain kernels."""
    from gprmax_gb300 import workloads
    cfs = ['#pml_cfs: constant forward 0 0 constant forward 1 1 sextic forward 0 0.5836',
           '#pml_cfs: constant forward 0.05 0.05 cubic forward 1 8 quadratic forward 0 5.8357']
    extra = ['#pml_formulation: {}'.format(formulation)] + cfs[2 - order:]
    G = workloads.dispersive_soil(nx=120, ny=110, nz=150, surface=110, timewindow='1.5e-9',
                                  pml=8, extra_lines=extra)
    assert len(G.cfs) == order and G.pmlformulation == formulation
    got = _run(G, 8, 200, forms=(True, True))
    ref = _run(G, 8 | 16, 200)
    assert got['info']['staged'] and got['info']['staged_h']
    _equal(got, ref)


def test_staged_two_debye_poles(native):
    """Two Debye poles per material (the real pole state with two poles, 17 streams a chunk):
    a 60 x 50 x 70 soil with a two-pole box, staged against plain and against the oracle."""
    import oracle
    from gprmax_gb300 import workloads
    extra = ['#material: 4 0.001 1 0 twopole',
             '#add_dispersion_debye: 2 3 1e-9 2 1e-10 twopole',
             '#box: 0.02 0.02 0.02 0.08 0.07 0.06 twopole']
    G = workloads.dispersive_soil(nx=60, ny=50, nz=70, surface=40, timewindow='3e-10', pml=6,
                                  extra_lines=extra)
    assert G.maxpoles == 2
    got = _run(G, 8, forms=(True, True))
    assert got['info']['staged'] and got['info']['staged_h']
    _equal(got, _run(G, 8 | 16))
    ref = oracle.OracleSolver(G).run()
    np.testing.assert_array_equal(got['rx'], ref.receivers())
    np.testing.assert_array_equal(got['f'], ref.fields())
