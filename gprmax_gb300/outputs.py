"""The ``.out`` receiver file (``gprMax/fields_outputs.py:111-161``), written with the
package's own HDF5 writer. Layout: root attributes gprMax, Title, Iterations, nx_ny_nz,
dx_dy_dz, dt, nsrc, nrx, srcsteps, rxsteps; ``/srcs/srcN`` groups with Type and Position;
``/tls/tlN`` groups with Position, Resistance, dl and fp32 Vinc, Iinc, Vtotal, Itotal;
``/rxs/rxN`` groups with Name and Position and one fp32 [iterations] dataset per output.
"""
import numpy as np

from . import hdf5

VERSION = '3.1.7'


def write_hdf5_outputfile(outputfile, G):
    f = hdf5.File(outputfile, 'w')
    f.attrs['gprMax'] = VERSION
    f.attrs['Title'] = G.title
    f.attrs['Iterations'] = np.int64(G.iterations)
    f.attrs['nx_ny_nz'] = np.array((G.nx, G.ny, G.nz), dtype=np.int64)
    f.attrs['dx_dy_dz'] = np.array((G.dx, G.dy, G.dz), dtype=np.float64)
    f.attrs['dt'] = np.float64(G.dt)
    nsrc = len(G.voltagesources + G.hertziandipoles + G.magneticdipoles + G.transmissionlines)
    f.attrs['nsrc'] = np.int64(nsrc)
    f.attrs['nrx'] = np.int64(len(G.rxs))
    f.attrs['srcsteps'] = np.array(G.srcsteps, dtype=np.int64)
    f.attrs['rxsteps'] = np.array(G.rxsteps, dtype=np.int64)
    for n, src in enumerate(G.voltagesources + G.hertziandipoles + G.magneticdipoles):
        grp = f.create_group('/srcs/src' + str(n + 1))
        grp.attrs['Type'] = type(src).__name__
        grp.attrs['Position'] = np.array((src.xcoord * G.dx, src.ycoord * G.dy, src.zcoord * G.dz))
    for n, tl in enumerate(G.transmissionlines):
        grp = f.create_group('/tls/tl' + str(n + 1))
        grp.attrs['Position'] = np.array((tl.xcoord * G.dx, tl.ycoord * G.dy, tl.zcoord * G.dz))
        grp.attrs['Resistance'] = np.float64(tl.resistance)
        grp.attrs['dl'] = np.float64(tl.dl)
        for name in ('Vinc', 'Iinc', 'Vtotal', 'Itotal'):
            grp[name] = np.asarray(getattr(tl, name), dtype=np.float32)
    for n, rx in enumerate(G.rxs):
        grp = f.create_group('/rxs/rx' + str(n + 1))
        if rx.ID:
            grp.attrs['Name'] = rx.ID
        grp.attrs['Position'] = np.array((rx.xcoord * G.dx, rx.ycoord * G.dy, rx.zcoord * G.dz))
        for output, values in rx.outputs.items():
            grp[output] = np.asarray(values, dtype=np.float32)
    f.close()


def read_outputfile(path):
    """Receiver traces of an ``.out`` file: ({'rx1': {'Ex': array, ...}, ...}, root attrs)."""
    root = hdf5.read(path)
    rxs = {}
    if 'rxs' in root:
        for name in root['rxs'].keys():
            node = root['rxs'][name]
            rxs[name] = {k: node[k].data for k in node.keys()}
    return rxs, root.attrs


def merge_files(paths, outputfile):
    """Merge the ``.out`` files of a B-scan into one file whose datasets are
    [iterations][nmodels] (the layout of the reference's ``tools/outputfiles_merge.py``)."""
    first = hdf5.read(paths[0])
    f = hdf5.File(outputfile, 'w')
    for k, v in first.attrs.items():
        if v is not None:
            f.attrs[k] = v
    f.attrs['Iterations'] = first.attrs['Iterations']
    traces = [read_outputfile(p)[0] for p in paths]
    for rx in traces[0]:
        for comp in traces[0][rx]:
            f['/rxs/{}/{}'.format(rx, comp)] = np.stack([t[rx][comp] for t in traces], axis=1)
    f.close()


def write_merged_outputfile(outputfile, grids):
    """One merged ``.out`` file straight from the grids of a B-scan whose receiver outputs are
    filled (for example by ``solver.solve_gb300_batch``): root attributes of the first model,
    and per receiver and output one fp32 [iterations][nmodels] dataset, the layout that merging
    the per-model files gives (``merge_files``, the reference's ``tools/outputfiles_merge.py``).
    Every model must have the same iterations, receivers and outputs."""
    G0 = grids[0]
    for G in grids[1:]:
        if G.iterations != G0.iterations or len(G.rxs) != len(G0.rxs) or any(
                list(a.outputs) != list(b.outputs) for a, b in zip(G.rxs, G0.rxs)):
            raise ValueError('B-scan models differ in iterations, receivers or outputs')
    f = hdf5.File(outputfile, 'w')
    f.attrs['gprMax'] = VERSION
    f.attrs['Title'] = G0.title
    f.attrs['Iterations'] = np.int64(G0.iterations)
    f.attrs['nx_ny_nz'] = np.array((G0.nx, G0.ny, G0.nz), dtype=np.int64)
    f.attrs['dx_dy_dz'] = np.array((G0.dx, G0.dy, G0.dz), dtype=np.float64)
    f.attrs['dt'] = np.float64(G0.dt)
    nsrc = len(G0.voltagesources + G0.hertziandipoles + G0.magneticdipoles + G0.transmissionlines)
    f.attrs['nsrc'] = np.int64(nsrc)
    f.attrs['nrx'] = np.int64(len(G0.rxs))
    f.attrs['srcsteps'] = np.array(G0.srcsteps, dtype=np.int64)
    f.attrs['rxsteps'] = np.array(G0.rxsteps, dtype=np.int64)
    for n, rx in enumerate(G0.rxs):
        for output in rx.outputs:
            f['/rxs/rx{}/{}'.format(n + 1, output)] = np.stack(
                [np.asarray(G.rxs[n].outputs[output], dtype=np.float32) for G in grids], axis=1)
    f.close()

