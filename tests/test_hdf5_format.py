"""CPU: the ``.out`` files this package writes, read by a second, independent HDF5 reader
(``tests/hdf5_check.py``, strict about the file format) and compared with a file that h5py
wrote for the reference (``tests/golden/hertzian_dipole_dispersive_ref.out``, from gprMax's own
test suite): the same groups, datasets and attributes with the same datatypes (text as
variable-length UTF-8 strings, as h5py stores a Python str), shapes and values. The layout the
reference's writer produces is ``gprMax/fields_outputs.py:111-161``; the older file names two
attributes the way gprMax 3.0 did ('nx, ny, nz', 'dx, dy, dz'), which v3.1.7 writes as
'nx_ny_nz', 'dx_dy_dz'.
"""
import os

import numpy as np
import pytest

import hdf5_check
from models import MODELS

HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(HERE, 'golden', 'hertzian_dipole_dispersive_ref.out')
RENAMED = {'nx, ny, nz': 'nx_ny_nz', 'dx, dy, dz': 'dx_dy_dz'}


def _signature(node):
    """Structure of a walked tree: per path the kind, datatypes and shapes of it and its
    attributes (values left out)."""
    out = {}

    def rec(n, path):
        entry = {'kind': n['kind'],
                 'attrs': {RENAMED.get(k, k): (a['dtype'], a['shape']) for k, a in n['attrs'].items()}}
        if n['kind'] == 'dataset':
            entry['dtype'], entry['shape'] = n['dtype'], n['shape']
        out[path] = entry
        for k, c in n.get('children', {}).items():
            rec(c, path + '/' + k)
    rec(node, '')
    return out


def _model_file(tmp_path, lines, name='a.out', traces=None):
    from gprmax_gb300.model import build_grid
    from gprmax_gb300.outputs import write_hdf5_outputfile
    G = build_grid(lines, messages=False)
    for r in G.rxs:
        for k in r.outputs:
            r.outputs[k] = (traces[k] if traces is not None else
                            np.arange(G.iterations, dtype=np.float32) * 0.5)
    for t in getattr(G, 'transmissionlines', []):
        for a in ('Vinc', 'Iinc', 'Vtotal', 'Itotal'):
            setattr(t, a, np.linspace(0, 1, G.iterations, dtype=np.float32))
    path = os.path.join(str(tmp_path), name)
    write_hdf5_outputfile(path, G)
    return G, path


def test_the_checker_reads_an_h5py_file():
    t = hdf5_check.walk(REF_OUT)
    assert t['attrs']['Title']['value'] == 'Hertzian dipole in water'
    assert t['attrs']['Title']['dtype']['class'] == 'vlstring'
    assert t['attrs']['Iterations']['value'] == 1559
    rx = t['children']['rxs']['children']['rx1']
    assert rx['attrs']['Name']['value'] == 'Rx(70,70,70)'
    assert rx['children']['Ez']['shape'] == (1559,)


def test_writer_output_matches_the_reference_file(tmp_path):
    ref = hdf5_check.walk(REF_OUT)
    d = np.load(os.path.join(HERE, 'golden', 'ref_hertzian_dipole_dispersive.npz'))
    traces = {k: d['rx1_' + k] for k in ('Ex', 'Ey', 'Ez', 'Hx', 'Hy', 'Hz')}
    G, path = _model_file(tmp_path, str(d['input']).splitlines(True), traces=traces)
    ours = hdf5_check.walk(path)
    assert _signature(ours) == _signature(ref)
    for k, a in ref['attrs'].items():
        if k == 'gprMax':     # the writing program's version
            continue
        np.testing.assert_array_equal(ours['attrs'][RENAMED.get(k, k)]['value'], a['value'])
    for grp in ('rxs', 'srcs'):
        for name, node in ref['children'][grp]['children'].items():
            mine = ours['children'][grp]['children'][name]
            for k, a in node['attrs'].items():
                np.testing.assert_array_equal(mine['attrs'][k]['value'], a['value'])
    rx = ours['children']['rxs']['children']['rx1']['children']
    for k, v in traces.items():
        np.testing.assert_array_equal(rx[k]['data'], v)


def test_writer_output_with_lines_arrays_and_merged_files(tmp_path):
    """Transmission lines (/tls with datasets), several sources and receivers, a receiver
    array, and a merged B-scan file: all well formed."""
    from gprmax_gb300.outputs import merge_files
    for name in ('tline', 'mixed', 'rxarray'):
        G, path = _model_file(tmp_path, MODELS[name].splitlines(True), name + '.out')
        t = hdf5_check.walk(path)
        assert len(t['children']['rxs']['children']) == len(G.rxs)
        if name == 'tline':
            tl = t['children']['tls']['children']['tl1']
            assert set(tl['children']) == {'Vinc', 'Iinc', 'Vtotal', 'Itotal'}
    paths = [_model_file(tmp_path, MODELS['fs_hori1'].splitlines(True), 'm{}.out'.format(m))[1]
             for m in range(3)]
    merged = os.path.join(str(tmp_path), 'merged.out')
    merge_files(paths, merged)
    t = hdf5_check.walk(merged)
    ez = t['children']['rxs']['children']['rx1']['children']['Ez']
    assert ez['shape'][1] == 3


@pytest.mark.parametrize('corrupt', ['eof', 'message_size', 'btree_signature', 'gheap_index'])
def test_the_checker_rejects_malformed_files(tmp_path, corrupt):
    import struct
    _, path = _model_file(tmp_path, MODELS['fs_hori1'].splitlines(True))
    b = bytearray(open(path, 'rb').read())
    if corrupt == 'eof':
        b[40:48] = struct.pack('<Q', len(b) + 8)
    elif corrupt == 'message_size':
        root = struct.unpack_from('<Q', b, 64)[0]
        struct.pack_into('<H', b, root + 16 + 2, 12)       # not a multiple of 8
    elif corrupt == 'btree_signature':
        b[b.index(b'TREE')] = ord('X')
    else:
        g = b.index(b'GCOL')
        struct.pack_into('<H', b, g + 16, 9)                # the first text object renumbered
    bad = os.path.join(str(tmp_path), 'bad.out')
    open(bad, 'wb').write(bytes(b))
    with pytest.raises(hdf5_check.FormatError):
        hdf5_check.walk(bad)
