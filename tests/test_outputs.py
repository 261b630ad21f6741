"""CPU: the HDF5 .out writer/reader and the merged B-scan file."""
import os

import numpy as np

from models import MODELS


def _grids(n):
    from gprmax_gb300.model import build_grid
    grids = []
    rng = np.random.default_rng(0)
    for m in range(n):
        G = build_grid(MODELS['fs_hori1'].splitlines(True), messages=False)
        for r in G.rxs:
            for k in r.outputs:
                r.outputs[k] = rng.standard_normal(G.iterations).astype(np.float32)
        grids.append(G)
    return grids


def test_single_file_round_trip(tmp_path):
    from gprmax_gb300.outputs import read_outputfile, write_hdf5_outputfile
    G = _grids(1)[0]
    path = os.path.join(tmp_path, 'a.out')
    write_hdf5_outputfile(path, G)
    rxs, attrs = read_outputfile(path)
    assert int(attrs['Iterations']) == G.iterations
    for n, r in enumerate(G.rxs):
        for k, v in r.outputs.items():
            np.testing.assert_array_equal(rxs['rx{}'.format(n + 1)][k], v)


def test_merged_file_equals_merge_of_model_files(tmp_path):
    from gprmax_gb300.outputs import (merge_files, read_outputfile, write_hdf5_outputfile,
                                      write_merged_outputfile)
    grids = _grids(3)
    paths = []
    for m, G in enumerate(grids):
        paths.append(os.path.join(tmp_path, 'm{}.out'.format(m)))
        write_hdf5_outputfile(paths[-1], G)
    merge_files(paths, os.path.join(tmp_path, 'merged_a.out'))
    write_merged_outputfile(os.path.join(tmp_path, 'merged_b.out'), grids)
    a, _ = read_outputfile(os.path.join(tmp_path, 'merged_a.out'))
    b, attrs = read_outputfile(os.path.join(tmp_path, 'merged_b.out'))
    assert a.keys() == b.keys()
    for rx in a:
        for comp in a[rx]:
            assert b[rx][comp].shape == (grids[0].iterations, 3)
            np.testing.assert_array_equal(a[rx][comp], b[rx][comp])
    assert int(attrs['nrx']) == len(grids[0].rxs)


def test_reference_output_file_reads():
    from gprmax_gb300.outputs import read_outputfile
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden',
                        'hertzian_dipole_dispersive_ref.out')
    rxs, attrs = read_outputfile(here)
    assert 'rx1' in rxs and {'Ex', 'Ey', 'Ez', 'Hx', 'Hy', 'Hz'} <= set(rxs['rx1'])
    assert rxs['rx1']['Ez'].shape == (int(attrs['Iterations']),)


def test_snapshot_vti_file_equals_the_reference_byte_for_byte(tmp_path):
    """The ``.vti`` writer, given the snapshot arrays of the ``mixed`` fixture, writes the same
    bytes as the reference's ``Snapshot.write_vtk_imagedata`` (``snapshots.py:132-165``)."""
    from models import build_fixture
    g = dict(np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden',
                                  'mixed.npz'), allow_pickle=False))
    G = build_fixture(g)
    assert len(G.snapshots) == 1
    snap = G.snapshots[0]
    snap.electric = g['snap0_electric']
    snap.magnetic = g['snap0_magnetic']
    out = str(tmp_path / 'snap.vti')
    snap.write_vtk_imagedata(out, G)
    with open(out, 'rb') as f:
        data = f.read()
    assert data == g['snap0_vti'].tobytes()
