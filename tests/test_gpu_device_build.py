"""GPU: the geometry built in device memory (``gbf_geom_*``). For every golden fixture the
device-built ID array must hash to the reference's, with the same materials and coefficient
tables, and the model solved from it must give the reference's traces bit for bit. For every
test model and for scaled-down benchmark workloads, the device build must equal the host build
array for array (solid, rigid flags, IDs, materials)."""
import glob
import hashlib
import os

import numpy as np
import pytest

from models import MODELS

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
FIXTURES = sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(GOLDEN, '*.npz')))


@pytest.mark.parametrize('name', FIXTURES)
def test_device_build_reproduces_reference_model(native, name):
    from models import build_fixture
    from gprmax_gb300.solver import DeviceModel
    g = dict(np.load(os.path.join(GOLDEN, name + '.npz'), allow_pickle=False))
    D = build_fixture(g, device_build=True)
    try:
        ids = np.ascontiguousarray(D.geom.ids())
        assert hashlib.sha256(ids.tobytes()).hexdigest() == str(g['ID_sha256'])
        assert len(D.materials) == int(g['nmat'])
        np.testing.assert_array_equal(D.updatecoeffsE, g['coeffE'])
        np.testing.assert_array_equal(D.updatecoeffsH, g['coeffH'])
        dm = DeviceModel(D)
        dm.run()
        rx = dm.receivers()
        dm.close()
    finally:
        D.geom.close()
    from gprmax_gb300.receivers import OUTPUT_INDEX
    checked = 0
    for n, r in enumerate(D.rxs):
        for out in r.outputs:
            key = 'rx{}_{}'.format(n + 1, out)
            if key in g:
                np.testing.assert_array_equal(rx[OUTPUT_INDEX[out], :, n], g[key], err_msg=key)
                checked += 1
    assert checked == sum(1 for k in g if k.startswith('rx'))


def _same(G, D):
    assert [m.ID for m in G.materials] == [m.ID for m in D.materials]
    np.testing.assert_array_equal(G.updatecoeffsE, D.updatecoeffsE)
    np.testing.assert_array_equal(G.updatecoeffsH, D.updatecoeffsH)
    np.testing.assert_array_equal(G.solid, D.geom.solid())
    rE, rH = D.geom.rigid()
    np.testing.assert_array_equal(G.rigidE, rE)
    np.testing.assert_array_equal(G.rigidH, rH)
    for c in range(6):
        np.testing.assert_array_equal(G.ID[c], D.geom.ids(c))


@pytest.mark.parametrize('name', sorted(MODELS))
def test_device_build_equals_host_build(native, name):
    from gprmax_gb300.model import build_grid
    lines = MODELS[name].splitlines(True)
    G = build_grid(lines, messages=False)
    D = build_grid(lines, messages=False, device_build=True)
    try:
        _same(G, D)
    finally:
        D.geom.close()


@pytest.mark.parametrize('which', ['soil', 'cube', 'bscan'])
def test_device_build_equals_host_build_on_workloads(native, which):
    from gprmax_gb300 import workloads
    from gprmax_gb300.model import build_grid
    if which == 'soil':
        kw = dict(nx=96, ny=88, nz=48, surface=36, timewindow=20)
        G = workloads.dispersive_soil(**kw)
        D = workloads.dispersive_soil(device_build=True, **kw)
    elif which == 'cube':
        G = workloads.throughput_cube(72, iterations=10)
        D = workloads.throughput_cube(72, iterations=10, device_build=True)
    else:
        lines = workloads.bscan_input((90, 80, 60), seed=5, position=3)
        G = build_grid(lines, messages=False)
        D = build_grid(lines, messages=False, device_build=True)
    try:
        _same(G, D)
    finally:
        D.geom.close()


@pytest.mark.parametrize('name', ['smoothed', 'fractal', 'debye1'])
def test_run_model_writes_the_reference_traces(native, name, tmp_path):
    """The public driver (``run_model``: device geometry build, solve, ``.out`` file) against
    the reference's traces."""
    from gprmax_gb300.model import run_model
    from gprmax_gb300.outputs import read_outputfile
    g = dict(np.load(os.path.join(GOLDEN, name + '.npz'), allow_pickle=False))
    inputfile = tmp_path / (name + '.in')
    inputfile.write_text(str(g['input']))
    G = run_model(str(inputfile), messages=False)
    rxs, attrs = read_outputfile(G.outputfile)
    checked = 0
    for n in range(len(G.rxs)):
        for out, v in rxs['rx{}'.format(n + 1)].items():
            key = 'rx{}_{}'.format(n + 1, out)
            if key in g:
                np.testing.assert_array_equal(v, g[key], err_msg=key)
                checked += 1
    assert checked == sum(1 for k in g if k.startswith('rx'))


def test_upload_rejects_an_id_beyond_the_tables(native):
    """IDs are checked on the device after the copy; one past the last material is refused."""
    from gprmax_gb300.exceptions import SolverError
    from gprmax_gb300.model import build_grid
    from gprmax_gb300.solver import DeviceModel
    G = build_grid(MODELS['fs_hori1'].splitlines(True), messages=False)
    G.ID[1, 3, 4, 5] = len(G.materials)
    with pytest.raises(SolverError, match='nmat'):
        DeviceModel(G)


@pytest.mark.parametrize('geometry_fixed', [False, True])
def test_bscan_driver_writes_the_reference_traces(native, tmp_path, geometry_fixed):
    """A 6-run 2D B-scan through the public driver (``api``: model runs, source and receiver
    stepping, device geometry build, ``.out`` files), rebuilt per run or with its geometry fixed:
    either way, runs 1 and 6 equal the reference's own runs bit for bit."""
    from gprmax_gb300.model import api
    from gprmax_gb300.outputs import read_outputfile
    g1 = dict(np.load(os.path.join(GOLDEN, 'bscan2d_run1.npz'), allow_pickle=False))
    g6 = dict(np.load(os.path.join(GOLDEN, 'bscan2d_run6.npz'), allow_pickle=False))
    inputfile = tmp_path / 'bscan.in'
    inputfile.write_text(str(g1['input']))
    api(str(inputfile), n=6, geometry_fixed=geometry_fixed)
    for run, g in ((1, g1), (6, g6)):
        rxs, _ = read_outputfile(str(tmp_path / 'bscan{}.out'.format(run)))
        keys = [k for k in g if k.startswith('rx1_')]
        assert keys
        for k in keys:
            np.testing.assert_array_equal(rxs['rx1'][k[4:]], g[k], err_msg='run {} {}'.format(run, k))


def test_set_device_takes_a_present_device_and_refuses_others(native):
    """``gbf_set_device`` (the ``-gpu`` device choice): device 0 is accepted and a model then
    runs there; an index past the device count is refused before any CUDA call uses it."""
    import ctypes
    assert native.gbf_set_device(0) == 0
    assert native.gbf_set_device(4096) != 0
    buf = ctypes.create_string_buffer(256)
    native.gbf_last_error(None, buf, 256)
    assert b'device 4096' in buf.value
    assert native.gbf_set_device(-1) != 0
