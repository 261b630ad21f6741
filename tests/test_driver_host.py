"""The public driver's host side (CPU only): ``api`` / ``run_model`` with the solve replaced by a
stub and the device geometry build by its numpy restatement (``fake_geom.py``). Output file
names follow the reference's rules (``model_build_run.py:107, 346-366``): the model number is
appended when several models run or in task and restart runs, ``#output_dir`` is taken relative
to the input file's folder and created, and each ``.out`` file holds that run's receiver
positions (``#src_steps`` / ``#rx_steps``)."""
import os

import pytest

from fake_geom import FakeGeomLib

import gprmax_gb300.devgeom as devgeom
import gprmax_gb300.solver as solver
from gprmax_gb300.model import api
from gprmax_gb300.outputs import read_outputfile

MODEL = """#title: driver
#domain: 0.024 0.020 0.020
#dx_dy_dz: 0.001 0.001 0.001
#time_window: 20
#pml_cells: 4
#messages: n
#num_threads: 4
#material: 5 0 1 0 ground
#box: 0 0 0 0.024 0.020 0.008 ground
#waveform: ricker 1 3e9 w
#hertzian_dipole: z 0.008 0.010 0.012 w
#rx: 0.012 0.010 0.012
#src_steps: 0.001 0 0
#rx_steps: 0.001 0 0
"""


@pytest.fixture
def stubbed(monkeypatch):
    monkeypatch.setattr(devgeom._native, 'lib', lambda: FakeGeomLib())
    calls = []

    def solve(currentmodelrun, modelend, G, fields=True):
        calls.append((currentmodelrun, modelend, G.rxs[0].xcoord))
        return 0.0, 0
    monkeypatch.setattr(solver, 'solve_gb300', solve)
    return calls


def _write(tmp_path, text):
    p = tmp_path / 'model.in'
    p.write_text(text)
    return str(p)


def test_one_model_writes_name_out(stubbed, tmp_path):
    api(_write(tmp_path, MODEL))
    assert sorted(os.listdir(tmp_path)) == ['model.in', 'model.out']
    assert stubbed == [(1, 1, 12)]


def test_bscan_runs_append_the_model_number_and_step_the_receivers(stubbed, tmp_path):
    grids = api(_write(tmp_path, MODEL), n=3)
    assert sorted(f for f in os.listdir(tmp_path) if f.endswith('.out')) == \
        ['model1.out', 'model2.out', 'model3.out']
    assert stubbed == [(1, 3, 12), (2, 3, 13), (3, 3, 14)]
    for n, G in enumerate(grids):
        rxs, attrs = read_outputfile(str(tmp_path / 'model{}.out'.format(n + 1)))
        assert list(rxs) == ['rx1']
        assert int(attrs['Iterations']) == G.iterations


@pytest.mark.parametrize('kw,names,runs', [
    ({'task': 2}, ['model2.out'], [(2, 2, 13)]),
    ({'restart': 2, 'n': 2}, ['model2.out', 'model3.out'], [(2, 3, 13), (3, 3, 14)]),
])
def test_task_and_restart_runs_append_the_model_number(stubbed, tmp_path, kw, names, runs):
    api(_write(tmp_path, MODEL), **kw)
    assert sorted(f for f in os.listdir(tmp_path) if f.endswith('.out')) == names
    assert stubbed == runs


def test_output_dir_is_relative_to_the_input_file(stubbed, tmp_path, monkeypatch):
    elsewhere = tmp_path / 'cwd'
    elsewhere.mkdir()
    monkeypatch.chdir(elsewhere)
    api(_write(tmp_path, MODEL + '#output_dir: results\n'))
    assert os.listdir(tmp_path / 'results') == ['model.out']
    assert os.listdir(elsewhere) == []


def test_fixed_geometry_builds_once_and_steps_the_same_grid(stubbed, tmp_path, monkeypatch):
    """``geometry_fixed``: one build for the whole B-scan; later runs step the same grid's sources
    and receivers, keep its device geometry open and close it after the last run."""
    import gprmax_gb300.model as model
    builds = []
    real = model.build_model_file

    def counting(*a, **k):
        builds.append(a[1] if len(a) > 1 else k.get('currentmodelrun'))
        return real(*a, **k)
    monkeypatch.setattr(model, 'build_model_file', counting)
    grids = api(_write(tmp_path, MODEL), n=3, geometry_fixed=True)
    assert builds == [1]
    assert grids[0] is grids[1] is grids[2]
    assert stubbed == [(1, 3, 12), (2, 3, 13), (3, 3, 14)]
    assert grids[0].hertziandipoles[0].xcoord == 10
    assert not grids[0].geom.h.value   # closed after the last run
    assert sorted(f for f in os.listdir(tmp_path) if f.endswith('.out')) == \
        ['model1.out', 'model2.out', 'model3.out']


def test_fixed_geometry_runs_equal_rebuilt_runs(stubbed, tmp_path):
    """The grid a fixed-geometry run solves has the inputs a rebuilt grid of that run has."""
    from gprmax_gb300.model import build_model_file
    from gprmax_gb300.solver import model_inputs
    path = _write(tmp_path, MODEL)
    fixed = api(path, n=3, geometry_fixed=True)[0]
    fresh = build_model_file(path, 3, 3, messages=False)
    a, b = model_inputs(fixed), model_inputs(fresh)
    for k in ('coeffE', 'coeffH', 'rx'):
        assert (a[k] == b[k]).all(), k
    for x, y in zip(a['sources'], b['sources']):
        assert (x == y).all()


class _DeviceLib(FakeGeomLib):
    def __init__(self, count=2):
        super().__init__()
        self.count = count
        self.devices = []

    def gbf_set_device(self, device):
        if device < 0 or device >= self.count:
            return -2
        self.devices.append(device)
        return 0

    def gbf_last_error(self, ctx, buf, n):
        buf.value = b'gbf_set_device: no such device'
        return 0


@pytest.mark.parametrize('gpu,device', [([1], 1), ([[1, 0]], 1), ([], 0), (0, 0)])
def test_gpu_option_selects_the_first_device(stubbed, tmp_path, monkeypatch, gpu, device):
    lib = _DeviceLib()
    monkeypatch.setattr(devgeom._native, 'lib', lambda: lib)
    api(_write(tmp_path, MODEL), gpu=gpu)
    assert lib.devices == [device]


def test_gpu_option_rejects_a_missing_device(stubbed, tmp_path, monkeypatch):
    from gprmax_gb300.exceptions import GeneralError
    lib = _DeviceLib(count=1)
    monkeypatch.setattr(devgeom._native, 'lib', lambda: lib)
    with pytest.raises(GeneralError, match='no such device'):
        api(_write(tmp_path, MODEL), gpu=[3])
