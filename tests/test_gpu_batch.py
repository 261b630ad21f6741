"""GPU: the batched form (one launch per half-step over many models) against the plain
solver model by model. Both run the same per-node code, so the traces and fields must be
bit-identical; the plain solver is pinned to the oracle by test_gpu_parity.py."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FREE = """#domain: {x} {y} {z}
#dx_dy_dz: 0.001 0.001 0.001
#time_window: {steps}
#pml_cells: {pml}
#waveform: ricker 1 2e9 w
#hertzian_dipole: z {sx} {sy} {sz} w
#rx: {rx} {sy} {sz}
#rx: {sx} {ry} {sz} r2 Ex Ey Ez Hx Hy Hz Ix Iy Iz
"""

SOIL = FREE + """#material: 6 0.005 1 0 soil
#add_dispersion_debye: 1 10 1e-9 soil
#box: 0 0 0 {x} {y} {surf} soil
#sphere: {bx} {by} {bz} 0.004 pec
"""


def _grids(template, n, steps, pml='6'):
    from gprmax_gb300.model import build_grid
    rng = np.random.default_rng(3)
    grids = []
    for m in range(n):
        x, y, z = (int(v) for v in rng.integers(24, 40, 3))
        sx, sy, sz = x // 2 + m % 3, y // 2, z // 2 + 2
        text = template.format(x=x / 1000, y=y / 1000, z=z / 1000, steps=steps, pml=pml,
                               sx=sx / 1000, sy=sy / 1000, sz=sz / 1000, rx=(sx + 3) / 1000,
                               ry=(sy - 4) / 1000, surf=(z // 2) / 1000, bx=x / 2000,
                               by=y / 2000, bz=z / 4000)
        grids.append(build_grid(text.splitlines(True), messages=False))
    return grids


def _plain(G):
    from gprmax_gb300.solver import DeviceModel
    dm = DeviceModel(G)
    dm.run()
    out = dm.receivers(), dm.fields()
    dm.close()
    return out


@pytest.mark.parametrize('template,pml', [(FREE, '6'), (SOIL, '6'), (FREE, '0'),
                                          (SOIL, '5 4 6 6 5 4')])
def test_batch_matches_plain_runs(native, template, pml):
    from gprmax_gb300.solver import BatchModel
    grids = _grids(template, 4, 80, pml)
    bm = BatchModel(grids)
    bm.run()
    # the first steps timed the candidate grid sizes; every later run uses the fastest
    info = bm.info()
    assert info['tuned'] and info['blocks_h'] > 0 and info['blocks_e'] > 0
    rx = bm.receivers()
    fields = [m.fields() for m in bm.models]
    bm.close()
    for n, G in enumerate(grids):
        prx, pf = _plain(G)
        np.testing.assert_array_equal(rx[n], prx, err_msg='model {} traces'.format(n))
        np.testing.assert_array_equal(fields[n], pf, err_msg='model {} fields'.format(n))


def test_batch_in_pieces_and_without_graph(native):
    from gprmax_gb300.solver import BatchModel
    grids = _grids(SOIL, 3, 60)
    outs = []
    for pieces, graph in (((60,), True), ((17, 25, 18), True), ((60,), False)):
        bm = BatchModel(grids)
        for n in pieces:
            bm.run(n, graph=graph)
        outs.append(bm.receivers())
        bm.close()
    for o in outs[1:]:
        for a, b in zip(outs[0], o):
            np.testing.assert_array_equal(a, b)


def test_batch_rejects_mixed_pml_kinds(native):
    from gprmax_gb300.exceptions import SolverError
    from gprmax_gb300.solver import BatchModel
    grids = _grids(FREE, 1, 20, '6') + _grids(FREE, 1, 20, '0')
    with pytest.raises(SolverError):
        BatchModel(grids)


LORENTZ = FREE + """#material: 4 0.002 1 0 wet
#add_dispersion_lorentz: 1 3 2e9 1e8 wet
#box: 0 0 0 {x} {y} {surf} wet
"""


def test_batch_of_debye_and_lorentz_models_keeps_complex_state(native):
    """A Debye model alone keeps only the real part of its pole state; batched with a Lorentz
    model both keep it complex (option bit 2), and the results do not change."""
    from gprmax_gb300.solver import BatchModel, real_dispersive_state
    grids = _grids(SOIL, 2, 70) + _grids(LORENTZ, 2, 70)
    assert real_dispersive_state(grids[0]) and not real_dispersive_state(grids[2])
    bm = BatchModel(grids)
    bm.run()
    rx = bm.receivers()
    fields = [m.fields() for m in bm.models]
    T = [m.dispersive() for m in bm.models]
    bm.close()
    for n, G in enumerate(grids):
        prx, pf = _plain(G)
        np.testing.assert_array_equal(rx[n], prx, err_msg='model {} traces'.format(n))
        np.testing.assert_array_equal(fields[n], pf, err_msg='model {} fields'.format(n))
    from gprmax_gb300.solver import DeviceModel
    dm = DeviceModel(grids[0])
    dm.run()
    Treal = dm.dispersive()
    dm.close()
    # the real-part layout gives back the complex state with imaginary parts +0
    np.testing.assert_array_equal(np.asarray(Treal).view(np.uint32), np.asarray(T[0]).view(np.uint32))


def test_batch_of_2d_bscan_traces(native, tmp_path):
    """A 2D (TMz) B-scan as one batch, the antenna pair stepped one cell per trace: every
    trace and final field equals the plain solver's bit for bit, the first and last traces
    equal the oracle's, and the merged ``.out`` file holds the traces in model order."""
    import oracle
    from gprmax_gb300 import workloads
    from gprmax_gb300.outputs import read_outputfile
    from gprmax_gb300.solver import BatchModel, solve_gb300_batch
    grids = workloads.bscan_2d_models(8)
    assert grids[0].nz == 1 and grids[0].mode == '2D TMz'
    assert grids[-1].rxs[0].xcoord == grids[0].rxs[0].xcoord + 7
    bm = BatchModel(grids)
    # one geometry: every trace uses the first trace's device IDs and tables
    assert all(m.shared_from is bm.models[0] for m in bm.models[1:])
    assert bm.models[1].device_bytes() < bm.models[0].device_bytes()
    bm.run()
    rx = bm.receivers()
    fields = [m.fields() for m in bm.models]
    bm.close()
    for n, G in enumerate(grids):
        prx, pf = _plain(G)
        np.testing.assert_array_equal(rx[n], prx, err_msg='trace {}'.format(n))
        np.testing.assert_array_equal(fields[n], pf, err_msg='trace {} fields'.format(n))
    for n in (0, len(grids) - 1):
        ref = oracle.OracleSolver(grids[n]).run()
        np.testing.assert_array_equal(rx[n], ref.receivers(), err_msg='trace {} oracle'.format(n))
    out = str(tmp_path / 'bscan2d_merged.out')
    solve_gb300_batch(grids, outputfile=out)
    merged, _ = read_outputfile(out)
    from gprmax_gb300.receivers import OUTPUT_INDEX
    ez = merged['rx1']['Ez']
    assert ez.shape == (grids[0].iterations, len(grids))
    for n in range(len(grids)):
        np.testing.assert_array_equal(ez[:, n], rx[n][OUTPUT_INDEX['Ez'], :, 0])


def test_shared_geometry_3d_soil(native):
    """Traces of one 3D dispersive soil with PML, the dipole and receiver moved per trace: the
    batch shares one copy of the IDs and tables and its results equal the same batch without
    sharing and the plain runs bit for bit; models sharing another's arrays keep them after
    that model is destroyed."""
    from gprmax_gb300.model import build_grid
    from gprmax_gb300.solver import BatchModel, DeviceModel
    grids = []
    for m in range(4):
        text = SOIL.format(x=0.034, y=0.030, z=0.032, steps=160, pml='6', sx=(14 + m) / 1000,
                           sy=0.015, sz=0.022, rx=(18 + m) / 1000, ry=0.011, surf=0.016,
                           bx=0.017, by=0.015, bz=0.008)
        grids.append(build_grid(text.splitlines(True), messages=False))
    runs = {}
    for share in (True, False):
        bm = BatchModel(grids, share_geometry=share)
        assert all((m.shared_from is bm.models[0]) == share for m in bm.models[1:])
        bm.run()
        runs[share] = bm.receivers()
        bm.close()
    owner = DeviceModel(grids[0])
    others = [DeviceModel(G, share=owner) for G in grids[1:]]
    owner.close()
    for n, m in enumerate(others, start=1):
        m.run()
        got = m.receivers()
        m.close()
        prx, _ = _plain(grids[n])
        np.testing.assert_array_equal(got, prx)
        np.testing.assert_array_equal(runs[True][n], prx)
        np.testing.assert_array_equal(runs[False][n], prx)


def test_share_materials_refuses_other_grids(native):
    from gprmax_gb300.exceptions import SolverError
    from gprmax_gb300.solver import DeviceModel
    a, b = _grids(FREE, 2, 20)
    assert (a.nx, a.ny, a.nz) != (b.nx, b.ny, b.nz)
    owner = DeviceModel(a)
    try:
        with pytest.raises(SolverError):
            DeviceModel(b, share=owner)
    finally:
        owner.close()


def test_large_models_step_with_their_own_kernels(native):
    """A model of 2^21 nodes or more takes its own half-step kernels (staged where they apply)
    inside the batch's graph, the small ones the batched kernels: every trace and field equals
    the plain run's."""
    from gprmax_gb300.model import build_grid
    from gprmax_gb300.solver import BatchModel
    # two large models of different sizes, their staged kernels' shared-memory rings of
    # different sizes: each launch states its own size, whichever context was set up last
    bigs = [build_grid(SOIL.format(x=x, y=0.130, z=z, steps=40, pml='6', sx=0.060, sy=0.065,
                                   sz=0.090, rx=0.070, ry=0.060, surf=0.064, bx=0.065, by=0.065,
                                   bz=0.032).splitlines(True), messages=False)
            for x, z in ((0.136, 0.140), (0.130, 0.128))]
    for big in bigs:
        assert (big.nx + 1) * (big.ny + 1) * (big.nz + 1) >= 2 ** 21
    grids = _grids(SOIL, 2, 40) + bigs
    bm = BatchModel(grids)
    assert bm.info()['own_kernels'] == 2
    bm.run()
    rx = bm.receivers()
    fields = [m.fields() for m in bm.models]
    bm.close()
    for n, G in enumerate(grids):
        prx, pf = _plain(G)
        np.testing.assert_array_equal(rx[n], prx, err_msg='model {}'.format(n))
        np.testing.assert_array_equal(fields[n], pf, err_msg='model {} fields'.format(n))
