"""Model build and run: the reference's ``run_model`` with the GB300 solver in place of
``solve_cpu``/``solve_gpu`` (``gprMax/model_build_run.py:84-405``) and ``api``
(``gprMax/gprMax.py:72-108, 194-236``) for standard (non-MPI) runs.
"""
import itertools
import os

import numpy as np

from .constants import c, e0, m0, z0
from .exceptions import GeneralError
from .grid import FDTDGrid
from .inputfile import check_cmd_names, process_python_include_code
from .materials import builtin_materials, process_materials
from .pml import CFS, build_pmls
from . import cmds
from .yee_build import build_electric_components, build_magnetic_components


def build_grid(lines, G=None, usernamespace=None, inputfilename='', messages=None,
               geometry_hook=None, device_build=False, device_fractals=False):
    """Build a model from input-file lines up to the coefficient tables (before solving).

    Follows the build sequence of ``run_model`` (``model_build_run.py:110-292``).
    ``geometry_hook(G)``, when given, runs before the geometry commands (used to place
    programmatic voxel blocks, as ``#fractal_box`` would). ``device_build``: the geometry
    arrays are built in GPU memory (:mod:`gprmax_gb300.devgeom`) and handed to the solver there.
    ``device_fractals``: fractal volumes and surfaces are transformed on the GPU (equal to the
    host's to rounding; cells at a bin edge can change bin), an opt-in for realisations.
    """
    G = G or FDTDGrid()
    G.device_fractals = device_fractals
    if usernamespace is None:
        usernamespace = {'c': c, 'e0': e0, 'm0': m0, 'z0': z0, 'number_model_runs': 1,
                         'inputfile': os.path.abspath(inputfilename) if inputfilename else '',
                         'current_model_run': 1}
    G.inputfilename = os.path.split(inputfilename)[1]
    G.inputdirectory = os.path.dirname(os.path.abspath(inputfilename)) if inputfilename else os.getcwd()
    processed = process_python_include_code(lines, usernamespace, inputfilename)
    singlecmds, multicmds, geometry = check_cmd_names(processed)
    G.materials = builtin_materials()
    if messages is not None:
        G.messages = messages
    cmds.process_singlecmds(singlecmds, G)
    if messages is not None:
        G.messages = messages
    cmds.process_multicmds(multicmds, G)
    G.initialise_geometry_arrays(device=device_build)
    if geometry_hook is not None:
        geometry_hook(G)
    cmds.process_geometrycmds(geometry, G)
    finish_build(G)
    return G


def finish_build(G):
    """PML slabs, edge IDs, 2D PEC planes, voltage-source materials and coefficient tables."""
    if any(v > 0 for v in G.pmlthickness.values()):
        if not G.cfs:
            G.cfs = [CFS()]
        build_pmls(G)
    else:
        G.pmls = []
    build_electric_components(G)
    build_magnetic_components(G)
    geom = getattr(G, 'geom', None)
    if geom is not None:
        # PEC planes of the 2D modes (the same writes as below, on the device)
        n1 = (G.nx + 1, G.ny + 1, G.nz + 1)
        planes = {'2D TMx': ((1, 0), (2, 0)), '2D TMy': ((0, 1), (2, 1)),
                  '2D TMz': ((0, 2), (1, 2))}
        for mode, pairs in planes.items():
            if mode in G.mode:
                for comp, axis in pairs:
                    for idx in (0, 1):
                        origin = [0, 0, 0]
                        shape = list(n1)
                        origin[axis] = idx
                        shape[axis] = 1
                        geom.fill(2 + comp, origin, shape, 0)
    elif '2D TMx' in G.mode:
        G.ID[1, 0, :, :] = 0
        G.ID[1, 1, :, :] = 0
        G.ID[2, 0, :, :] = 0
        G.ID[2, 1, :, :] = 0
    elif '2D TMy' in G.mode:
        G.ID[0, :, 0, :] = 0
        G.ID[0, :, 1, :] = 0
        G.ID[2, :, 0, :] = 0
        G.ID[2, :, 1, :] = 0
    elif '2D TMz' in G.mode:
        G.ID[0, :, :, 0] = 0
        G.ID[0, :, :, 1] = 0
        G.ID[1, :, :, 0] = 0
        G.ID[1, :, :, 1] = 0
    for vs in G.voltagesources:
        vs.create_material(G)
    process_materials(G)
    return G


def step_sources_receivers(G, currentmodelrun, modelend):
    """Shift simple sources and receivers for B-scan model runs (``model_build_run.py:308-324``)."""
    if any(G.srcsteps):
        for source in itertools.chain(G.hertziandipoles, G.magneticdipoles):
            if currentmodelrun == 1:
                for co, st, n in ((source.xcoord, G.srcsteps[0], G.nx), (source.ycoord, G.srcsteps[1], G.ny),
                                  (source.zcoord, G.srcsteps[2], G.nz)):
                    if co + st * modelend < 0 or co + st * modelend > n:
                        raise GeneralError('Source(s) will be stepped to a position outside the domain.')
            source.xcoord = source.xcoordorigin + (currentmodelrun - 1) * G.srcsteps[0]
            source.ycoord = source.ycoordorigin + (currentmodelrun - 1) * G.srcsteps[1]
            source.zcoord = source.zcoordorigin + (currentmodelrun - 1) * G.srcsteps[2]
    if any(G.rxsteps):
        for r in G.rxs:
            if currentmodelrun == 1:
                for co, st, n in ((r.xcoord, G.rxsteps[0], G.nx), (r.ycoord, G.rxsteps[1], G.ny),
                                  (r.zcoord, G.rxsteps[2], G.nz)):
                    if co + st * modelend < 0 or co + st * modelend > n:
                        raise GeneralError('Receiver(s) will be stepped to a position outside the domain.')
            r.xcoord = r.xcoordorigin + (currentmodelrun - 1) * G.rxsteps[0]
            r.ycoord = r.ycoordorigin + (currentmodelrun - 1) * G.rxsteps[1]
            r.zcoord = r.zcoordorigin + (currentmodelrun - 1) * G.rxsteps[2]


def build_model_file(inputfile, currentmodelrun=1, modelend=1, messages=None, device_build=False):
    """Build the model of an ``.in`` file for one model run of a B-scan (``device_build``: the
    geometry arrays in GPU memory)."""
    usernamespace = {'c': c, 'e0': e0, 'm0': m0, 'z0': z0, 'number_model_runs': modelend,
                     'inputfile': os.path.abspath(inputfile), 'current_model_run': currentmodelrun}
    with open(inputfile) as f:
        lines = f.readlines()
    G = build_grid(lines, usernamespace=usernamespace, inputfilename=inputfile, messages=messages,
                   device_build=device_build)
    step_sources_receivers(G, currentmodelrun, modelend)
    return G


def run_model(inputfile, currentmodelrun=1, modelend=1, numbermodelruns=1, write_output=True,
              messages=None, device_build=True, append_number=False, G=None,
              keep_geometry=False):
    """Build, solve on the GPU and write ``<name>[n].out``; returns the solved grid. The model
    number is appended to the file name when more than one model runs or ``append_number``
    (task and restart runs, ``model_build_run.py:107``). ``device_build``: build the geometry
    arrays in GPU memory, where the solver takes them.

    ``G``: the grid of an earlier run of a B-scan whose geometry is fixed (the reference's
    ``--geometry-fixed``, ``model_build_run.py:108, 286-300, 402``): it is not rebuilt, only its
    sources and receivers are stepped to this run; the solve starts from zero fields as a new
    grid's would. ``keep_geometry``: leave a device-built geometry open for a following run."""
    from .solver import solve_gb300
    from .outputs import write_hdf5_outputfile
    if G is None:
        G = build_model_file(inputfile, currentmodelrun, modelend, messages=messages,
                             device_build=device_build)
    else:
        step_sources_receivers(G, currentmodelrun, modelend)
    tsolve, mem = solve_gb300(currentmodelrun, modelend, G)
    if getattr(G, 'geom', None) is not None and not keep_geometry:
        G.geom.close()
    G.tsolve = tsolve
    G.memsolve = mem
    if write_output:
        append = '' if numbermodelruns == 1 and not append_number else str(currentmodelrun)
        outdir = G.outputdirectory or G.inputdirectory
        if not os.path.isabs(outdir):
            outdir = os.path.join(G.inputdirectory, outdir)
        os.makedirs(outdir, exist_ok=True)
        base = os.path.splitext(G.inputfilename)[0]
        G.outputfile = os.path.join(outdir, base + append + '.out')
        write_hdf5_outputfile(G.outputfile, G)
        if G.snapshots:
            snapdir = os.path.join(G.inputdirectory, base + '_snaps' + append)
            os.makedirs(snapdir, exist_ok=True)
            for snap in G.snapshots:
                snap.write_vtk_imagedata(os.path.join(snapdir, snap.basefilename + '.vti'), G)
    if G.messages:
        print('Solving time [s]: {:.3f}, GPU memory {:.3g} GB'.format(tsolve, mem / 1e9))
    return G


def select_device(gpu):
    """Run the models of this thread on one CUDA device: the first of the device IDs given (a
    list, possibly of lists, as the reference's ``-gpu`` option collects them; none: device 0),
    as the reference does for a standard run (``gprMax/gprMax.py:132-144``)."""
    import ctypes
    from . import _native
    ids = gpu if isinstance(gpu, (list, tuple)) else [gpu]
    flat = [v for x in ids for v in (x if isinstance(x, (list, tuple)) else [x])]
    device = int(flat[0]) if flat else 0
    lib = _native.lib()
    if lib.gbf_set_device(device) != 0:
        buf = ctypes.create_string_buffer(512)
        lib.gbf_last_error(None, buf, 512)
        raise GeneralError(buf.value.decode())
    return device


def api(inputfile, n=1, task=None, restart=None, gpu=None, geometry_fixed=False, **unused):
    """Run ``n`` models of an input file on the GPU (``gprMax/gprMax.py:72-108``); returns the
    solved grids. With ``geometry_fixed`` the input is built once and every later run reuses that
    grid with its sources and receivers stepped, so the returned entries are that one grid
    (holding the last run's outputs; each run's traces are in its ``.out`` file).

    MPI task farming, Taguchi optimisation and benchmark mode are not part of the solver core.
    """
    for key in ('mpi', 'mpi_no_spawn', 'benchmark', 'opt_taguchi', 'geometry_only'):
        if unused.get(key):
            raise GeneralError('{} mode is not supported by the GB300 solver core'.format(key))
    if gpu is not None:
        select_device(gpu)
    if task:
        start, end = task, task + 1
    elif restart:
        start, end = restart, restart + n
    else:
        start, end = 1, 1 + n
    results = []
    G = None
    for run in range(start, end):
        G = run_model(inputfile, run, end - 1, n, append_number=bool(task or restart),
                      G=G if geometry_fixed else None,
                      keep_geometry=bool(geometry_fixed) and run < end - 1)
        results.append(G)
    return results
