"""GPU: the fused step (one kernel per iteration, gprmax_gb300/csrc/fused_step.cuh) against the
two half-step kernels (options bit 3) and the oracle, bit for bit.

The fused kernel recomputes H on its tiles' halo rows, columns and first planes, double-buffers
E, H and the H-side PML state, and writes E outside the half-step's range only through the
end-of-step sources. So every tiling must give the two-kernel results exactly: receivers, all
six fields, the dispersive state and snapshots; and the models cover every PML kind, real and
complex dispersive state with one and two poles, magnetic materials (H read through IDs),
sources on the domain's upper faces and several sources in one column.
"""
import numpy as np
import pytest

from models import MODELS

pytestmark = pytest.mark.gpu

FUSED_MODELS = ['fs_hori1', 'pml_off', 'hori2', 'mri1', 'mri2', 'debye1', 'mixed', 'faces',
                'smoothed', 'fractal', 'rxarray']
TILINGS = [(7, 1), (7, 3), (15, 2), (15, 1000), (7, 0)]


def _build(name):
    from gprmax_gb300.model import build_grid
    return build_grid(MODELS[name].splitlines(True), messages=False)


def _run(G, options=0, tiles=None, nsteps=None, graph=True):
    from gprmax_gb300.solver import DeviceModel
    # option bit 5: the fused step's buffers for models with PML slabs too
    dm = DeviceModel(G, options | (32 if tiles is not None else 0))
    try:
        info = dm.step_info()
        if tiles is not None:
            dm.set_fused_tiles(*tiles)
        dm.run(nsteps, graph=graph)
        out = {'rx': dm.receivers(), 'f': dm.fields(), 'info': info}
        if G.maxpoles:
            out['T'] = dm.dispersive()
        out['snaps'] = [dm.snapshot(s) for s in range(len(G.snapshots))]
        out['info_after'] = dm.step_info()
    finally:
        dm.close()
    return out


def _equal(a, b):
    np.testing.assert_array_equal(a['rx'], b['rx'])
    np.testing.assert_array_equal(a['f'], b['f'])
    if 'T' in a:
        np.testing.assert_array_equal(a['T'], b['T'])
    for x, y in zip(a['snaps'], b['snaps']):
        np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize('name', FUSED_MODELS)
def test_fused_step_equals_half_steps(native, name):
    G = _build(name)
    ref = _run(G, options=8)
    assert not ref['info']['fused']
    for tiles in TILINGS:
        got = _run(G, tiles=tiles)
        assert got['info']['fused_available'], 'model {} should allow the fused step'.format(name)
        assert got['info_after']['fused']
        _equal(got, ref)


@pytest.mark.parametrize('name', ['debye1', 'faces', 'mixed'])
def test_fused_step_against_oracle(native, name):
    import oracle
    G = _build(name)
    got = _run(G, tiles=(7, 0))
    ref = oracle.OracleSolver(G).run()
    np.testing.assert_array_equal(got['rx'], ref.receivers())
    np.testing.assert_array_equal(got['f'], ref.fields())


def test_odd_step_counts_and_graph_parity(native):
    """Runs of odd lengths leave the current field buffer on either side; graph replays must
    start from the buffer they were captured on. Splitting a run anywhere gives the same result
    as one run, with and without graphs."""
    from gprmax_gb300.solver import DeviceModel
    G = _build('debye1')
    whole = _run(G, tiles=(7, 3))
    for split in ([1, 33, G.iterations - 34], [17, 16, G.iterations - 33], [5, G.iterations - 5]):
        dm = DeviceModel(G, 32)
        dm.set_fused_tiles(7, 3)
        try:
            for n, graph in zip(split, [True, False, True]):
                dm.run(n, graph=graph)
            np.testing.assert_array_equal(dm.receivers(), whole['rx'])
            np.testing.assert_array_equal(dm.fields(), whole['f'])
        finally:
            dm.close()


def test_fields_round_trip_and_reset(native):
    """Uploaded fields reach both buffers; reset returns to buffer 0 and zero state."""
    from gprmax_gb300.solver import DeviceModel
    G = _build('faces')
    dm = DeviceModel(G)
    dm.set_fused_tiles(7, 0)
    try:
        dm.run(7)
        assert dm.step_info()['buffer'] == 1
        f7 = dm.fields()
        dm.run(10)
        f17 = dm.fields()
        dm.reset()
        assert dm.step_info()['buffer'] == 0
        assert not dm.fields().any()
        dm.set_fields(f7)
        # restart from the uploaded state: 10 further steps give the same fields as before
        # (the sources use the iteration counter, so advance it by running from a reset copy)
        dm2 = DeviceModel(G)
        dm2.set_fused_tiles(7, 0)
        dm2.run(7)
        dm2.set_fields(f7)
        dm2.run(10)
        np.testing.assert_array_equal(dm2.fields(), f17)
        dm2.close()
    finally:
        dm.close()


def test_step_info_reports_the_tuned_tiling(native):
    """A model without PML times its candidates (fused tilings, the half-step kernels) in the
    first steps of its run; a model with PML takes the half-step kernels from the start and has
    no second field buffer unless option bit 5 asks for one."""
    from gprmax_gb300.exceptions import SolverError
    from gprmax_gb300.solver import DeviceModel
    dm = DeviceModel(_build('fs_hori1'))
    try:
        info = dm.step_info()
        assert not info['fused_available'] and not info['two_buffers'] and not info['fused']
        with pytest.raises(SolverError):
            dm.set_fused_tiles(7, 0)
    finally:
        dm.close()
    dm = DeviceModel(_build('fs_hori1'), 32)
    try:
        info = dm.step_info()
        assert info['fused_available'] and info['tuned'] and not info['fused']
    finally:
        dm.close()
    G = _build('pml_off')
    dm = DeviceModel(G)
    try:
        info = dm.step_info()
        assert info['fused_available'] and info['two_buffers'] and not info['tuned']
        whole = _run(G, options=8)
        dm.run()   # the first steps time the candidates (fused tilings, two kernels)
        info = dm.step_info()
        assert info['tuned']
        if info['fused']:
            assert info['tj'] in (7, 15) and info['nch'] >= 1
            assert info['nch'] * info['planes'] >= G.nx + 1
        # the steps that timed the candidates are ordinary steps of the run
        np.testing.assert_array_equal(dm.receivers(), whole['rx'])
        np.testing.assert_array_equal(dm.fields(), whole['f'])
    finally:
        dm.close()


def test_models_outside_the_fused_step_keep_two_kernels(native):
    for name in ('tmz', 'tline'):
        G = _build(name)
        out = _run(G, nsteps=5)
        assert not out['info']['fused_available'] and not out['info']['two_buffers']


def test_fused_step_two_debye_poles(native):
    """The fused step with two Debye poles per material (real pole state, two poles) against the
    two half-step kernels, on a PML-free soil with a two-pole box."""
    from gprmax_gb300 import workloads
    extra = ['#material: 4 0.001 1 0 twopole',
             '#add_dispersion_debye: 2 3 1e-9 2 1e-10 twopole',
             '#box: 0.02 0.02 0.02 0.08 0.07 0.06 twopole']
    G = workloads.dispersive_soil(nx=60, ny=50, nz=70, surface=40, timewindow='3e-10', pml=0,
                                  extra_lines=extra)
    assert G.maxpoles == 2
    ref = _run(G, options=8)
    for tiles in ((7, 2), (15, 0)):
        got = _run(G, tiles=tiles)
        assert got['info_after']['fused']
        _equal(got, ref)
