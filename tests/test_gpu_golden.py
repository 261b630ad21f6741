"""GPU against the reference itself: every golden fixture (tests/golden, written by gprMax
v3.1.7's own time loop compiled without floating-point contraction) is rebuilt from its input
text by the front-end and run through the C ABI; receiver traces must equal the reference's bit
for bit (transmission-line voltages and currents too) and the final fields must hash to the
reference's."""
import glob
import hashlib
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
NAMES = sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(GOLDEN, '*.npz')))
COMPONENTS = ('Ex', 'Ey', 'Ez', 'Hx', 'Hy', 'Hz')


@pytest.mark.parametrize('name', NAMES)
def test_gpu_reproduces_reference_run(native, name):
    from models import build_fixture
    from gprmax_gb300.receivers import OUTPUT_INDEX
    from gprmax_gb300.solver import DeviceModel
    g = dict(np.load(os.path.join(GOLDEN, name + '.npz'), allow_pickle=False))
    G = build_fixture(g)
    dm = DeviceModel(G)
    dm.run()
    rx = dm.receivers()
    f = dm.fields()
    snaps = [dm.snapshot(s) for s in range(len(G.snapshots))]
    tls = dm.transmission_lines()
    dm.close()
    for n in range(len(G.transmissionlines)):
        np.testing.assert_array_equal(tls[n, 0], g['tl{}_Vtotal'.format(n + 1)])
        np.testing.assert_array_equal(tls[n, 1], g['tl{}_Itotal'.format(n + 1)])
    checked = 0
    for n, r in enumerate(G.rxs):
        for out in r.outputs:
            key = 'rx{}_{}'.format(n + 1, out)
            np.testing.assert_array_equal(rx[OUTPUT_INDEX[out], :, n], g[key], err_msg=key)
            checked += 1
    assert checked
    for c, comp in enumerate(COMPONENTS):
        sha = hashlib.sha256(np.ascontiguousarray(f[c]).tobytes()).hexdigest()
        assert sha == str(g['field_{}_sha256'.format(comp)]), 'final {} differs'.format(comp)
    for s, snap in enumerate(snaps):
        key = 'snap{}_electric'.format(s)
        if key in g:
            np.testing.assert_array_equal(np.stack(snap[:3]).reshape(-1, order='F'), g[key])
            np.testing.assert_array_equal(np.stack(snap[3:]).reshape(-1, order='F'),
                                          g['snap{}_magnetic'.format(s)])
