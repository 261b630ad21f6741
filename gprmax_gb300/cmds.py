"""Processing of input commands into an :class:`FDTDGrid`.

Single-use commands follow ``gprMax/input_cmds_singleuse.py:41-336``, multi-use commands
``input_cmds_multiuse.py:45-851`` and geometry commands ``input_cmds_geometry.py:51-1527`` for
the commands this solver core supports. Parameter checks raise :class:`CmdInputError` with the
reference's messages. ``#fractal_box`` is built with its materials from ``#soil_peplinski``,
with ``#add_surface_roughness`` and ``#add_surface_water``; ``#add_grass`` is rejected with an
explicit error.
"""
import decimal as d
import inspect
import os

import numpy as np
from scipy import interpolate

from .constants import c, floattype, z0
from .exceptions import CmdInputError
from .fractals import FractalSurface, FractalVolume, PeplinskiSoil
from .materials import Material
from .pml import CFS, CFSParameter, PML
from .receivers import Rx, allocate_outputs
from .snapshots import Snapshot
from .sources import HertzianDipole, MagneticDipole, TransmissionLine, VoltageSource
from .utilities import round_value
from .waveforms import Waveform
from . import geometry as geo


def _log(G, msg):
    if G.messages:
        print(msg)


def process_singlecmds(singlecmds, G):
    """Domain, discretisation, dt, iterations and PML settings (``input_cmds_singleuse.py:41-336``)."""
    cmd = '#messages'
    if singlecmds[cmd] is not None:
        tmp = singlecmds[cmd].split()
        if len(tmp) != 1:
            raise CmdInputError(cmd + ' requires exactly one parameter')
        if singlecmds[cmd].lower() == 'y':
            G.messages = True
        elif singlecmds[cmd].lower() == 'n':
            G.messages = False
        else:
            raise CmdInputError(cmd + ' requires input values of either y or n')

    cmd = '#title'
    if singlecmds[cmd] is not None:
        G.title = singlecmds[cmd]
        _log(G, 'Model title: {}'.format(G.title))

    cmd = '#num_threads'
    if singlecmds[cmd] is not None:
        tmp = tuple(int(x) for x in singlecmds[cmd].split())
        if len(tmp) != 1:
            raise CmdInputError(cmd + ' requires exactly one parameter to specify the number of threads to use')
        if tmp[0] < 1:
            raise CmdInputError(cmd + ' requires the value to be an integer not less than one')
        G.nthreads = tmp[0]

    cmd = '#dx_dy_dz'
    tmp = [float(x) for x in singlecmds[cmd].split()]
    if len(tmp) != 3:
        raise CmdInputError(cmd + ' requires exactly three parameters')
    for v, ax in zip(tmp, 'xyz'):
        if v <= 0:
            raise CmdInputError(cmd + ' requires the {}-direction spatial step to be greater than zero'.format(ax))
    G.dx, G.dy, G.dz = tmp

    cmd = '#domain'
    tmp = [float(x) for x in singlecmds[cmd].split()]
    if len(tmp) != 3:
        raise CmdInputError(cmd + ' requires exactly three parameters')
    G.nx = round_value(tmp[0] / G.dx)
    G.ny = round_value(tmp[1] / G.dy)
    G.nz = round_value(tmp[2] / G.dz)
    if G.nx == 0 or G.ny == 0 or G.nz == 0:
        raise CmdInputError(cmd + ' requires at least one cell in every dimension')

    # CFL time step (3D, or 2D with the invariant direction's PML switched off)
    if G.nx == 1:
        G.dt = 1 / (c * np.sqrt((1 / G.dy) * (1 / G.dy) + (1 / G.dz) * (1 / G.dz)))
        G.mode = '2D TMx'
        G.pmlthickness['x0'] = 0
        G.pmlthickness['xmax'] = 0
    elif G.ny == 1:
        G.dt = 1 / (c * np.sqrt((1 / G.dx) * (1 / G.dx) + (1 / G.dz) * (1 / G.dz)))
        G.mode = '2D TMy'
        G.pmlthickness['y0'] = 0
        G.pmlthickness['ymax'] = 0
    elif G.nz == 1:
        G.dt = 1 / (c * np.sqrt((1 / G.dx) * (1 / G.dx) + (1 / G.dy) * (1 / G.dy)))
        G.mode = '2D TMz'
        G.pmlthickness['z0'] = 0
        G.pmlthickness['zmax'] = 0
    else:
        G.dt = 1 / (c * np.sqrt((1 / G.dx) * (1 / G.dx) + (1 / G.dy) * (1 / G.dy)
                                + (1 / G.dz) * (1 / G.dz)))
        G.mode = '3D'
    # round down with one digit less than the decimal context precision
    G.dt = round_value(G.dt, decimalplaces=d.getcontext().prec - 1)

    cmd = '#time_step_stability_factor'
    if singlecmds[cmd] is not None:
        tmp = tuple(float(x) for x in singlecmds[cmd].split())
        if len(tmp) != 1:
            raise CmdInputError(cmd + ' requires exactly one parameter')
        if tmp[0] <= 0 or tmp[0] > 1:
            raise CmdInputError(cmd + ' requires the value of the time step stability factor to be between zero and one')
        G.dt = G.dt * tmp[0]

    cmd = '#time_window'
    tmp = singlecmds[cmd].split()
    if len(tmp) != 1:
        raise CmdInputError(cmd + ' requires exactly one parameter to specify the time window. Either in seconds or number of iterations.')
    tmp = tmp[0].lower()
    try:
        tmp = int(tmp)
        G.timewindow = (tmp - 1) * G.dt
        G.iterations = tmp
    except ValueError:
        tmp = float(tmp)
        if tmp > 0:
            G.timewindow = tmp
            G.iterations = int(np.ceil(tmp / G.dt)) + 1
        else:
            raise CmdInputError(cmd + ' must have a value greater than zero')
    _log(G, 'Time window: {:g} secs ({} iterations)'.format(G.timewindow, G.iterations))

    cmd = '#pml_cells'
    if singlecmds[cmd] is not None:
        tmp = singlecmds[cmd].split()
        if len(tmp) != 1 and len(tmp) != 6:
            raise CmdInputError(cmd + ' requires either one or six parameter(s)')
        if len(tmp) == 1:
            for key in G.pmlthickness.keys():
                G.pmlthickness[key] = int(tmp[0])
        else:
            for key, v in zip(('x0', 'y0', 'z0', 'xmax', 'ymax', 'zmax'), tmp):
                G.pmlthickness[key] = int(v)
    if (2 * G.pmlthickness['x0'] >= G.nx or 2 * G.pmlthickness['y0'] >= G.ny
            or 2 * G.pmlthickness['z0'] >= G.nz or 2 * G.pmlthickness['xmax'] >= G.nx
            or 2 * G.pmlthickness['ymax'] >= G.ny or 2 * G.pmlthickness['zmax'] >= G.nz):
        raise CmdInputError(cmd + ' has too many cells for the domain size')

    cmd = '#pml_formulation'
    if singlecmds[cmd] is not None:
        tmp = singlecmds[cmd].split()
        if len(tmp) != 1:
            raise CmdInputError(cmd + ' requires exactly one parameter')
        if singlecmds[cmd].upper() in PML.formulations:
            G.pmlformulation = singlecmds[cmd].upper()
        else:
            raise CmdInputError(cmd + ' PML formulation is not found')

    for cmd, target in (('#src_steps', G.srcsteps), ('#rx_steps', G.rxsteps)):
        if singlecmds[cmd] is not None:
            tmp = singlecmds[cmd].split()
            if len(tmp) != 3:
                raise CmdInputError(cmd + ' requires exactly three parameters')
            target[0] = round_value(float(tmp[0]) / G.dx)
            target[1] = round_value(float(tmp[1]) / G.dy)
            target[2] = round_value(float(tmp[2]) / G.dz)

    cmd = '#excitation_file'
    if singlecmds[cmd] is not None:
        _excitation_file(singlecmds[cmd], G)

    cmd = '#output_dir'
    if singlecmds[cmd] is not None:
        G.outputdirectory = singlecmds[cmd]


def _excitation_file(params, G):
    """User waveforms from a text file, interpolated with scipy (``input_cmds_singleuse.py:264-331``)."""
    tmp = params.split()
    if len(tmp) != 1 and len(tmp) != 3:
        raise CmdInputError('#excitation_file requires either one or three parameter(s)')
    excitationfile = tmp[0]
    if len(tmp) > 1:
        kwargs = {'kind': tmp[1], 'fill_value': tmp[2]}
    else:
        spec = inspect.getfullargspec(interpolate.interp1d)
        kwargs = dict(zip(reversed(spec.args), reversed(spec.defaults)))
    if not os.path.isfile(excitationfile):
        excitationfile = os.path.abspath(os.path.join(G.inputdirectory, excitationfile))
    with open(excitationfile, 'r') as f:
        waveformIDs = f.readline().split()
    waveformvalues = np.loadtxt(excitationfile, skiprows=1, dtype=floattype)
    if waveformIDs[0].lower() == 'time':
        waveformIDs = waveformIDs[1:]
        waveformtime = waveformvalues[:, 0]
        waveformvalues = waveformvalues[:, 1:]
    else:
        waveformtime = np.arange(0, G.timewindow + G.dt, G.dt)
    for n, wid in enumerate(waveformIDs):
        if any(x.ID == wid for x in G.waveforms):
            raise CmdInputError('Waveform with ID {} already exists'.format(wid))
        w = Waveform()
        w.ID = wid
        w.type = 'user'
        vals = waveformvalues[:] if len(waveformvalues.shape) == 1 else waveformvalues[:, n]
        if len(vals) > len(waveformtime):
            vals = vals[:len(waveformtime)]
        elif len(vals) < len(waveformtime):
            padded = np.zeros(len(waveformtime))
            padded[:len(vals)] = vals
            vals = padded
        w.userfunc = interpolate.interp1d(waveformtime, vals, **kwargs)
        G.waveforms.append(w)


def _err(cmdname, tmp, msg):
    return CmdInputError("'" + cmdname + ': ' + ' '.join(tmp) + "'" + msg)


def _check_coords(G, cmdname, tmp, x, y, z, name=''):
    try:
        G.within_bounds(x=x, y=y, z=z)
    except ValueError as err:
        raise CmdInputError("'{}: {} ' {} {}-coordinate is not within the model domain".format(
            cmdname, ' '.join(tmp), name, err.args[0]))


def _in_pml_warning(G, cmdname, tmp, x, y, z):
    if (x < G.pmlthickness['x0'] or x > G.nx - G.pmlthickness['xmax'] or y < G.pmlthickness['y0']
            or y > G.ny - G.pmlthickness['ymax'] or z < G.pmlthickness['z0']
            or z > G.nz - G.pmlthickness['zmax']):
        _log(G, "WARNING: '" + cmdname + ': ' + ' '.join(tmp) + "'"
             + ' sources and receivers should not normally be positioned within the PML.')


def _check_polarisation(G, cmdname, tmp, pol):
    if pol not in ('x', 'y', 'z'):
        raise _err(cmdname, tmp, ' polarisation must be x, y, or z')
    if '2D TMx' in G.mode and pol in ('y', 'z'):
        raise _err(cmdname, tmp, ' polarisation must be x in 2D TMx mode')
    if '2D TMy' in G.mode and pol in ('x', 'z'):
        raise _err(cmdname, tmp, ' polarisation must be y in 2D TMy mode')
    if '2D TMz' in G.mode and pol in ('x', 'y'):
        raise _err(cmdname, tmp, ' polarisation must be z in 2D TMz mode')


def _start_stop(G, cmdname, tmp, src, first):
    if len(tmp) > first:
        start = float(tmp[first])
        stop = float(tmp[first + 1])
        if start < 0:
            raise _err(cmdname, tmp, ' delay of the initiation of the source should not be less than zero')
        if stop < 0:
            raise _err(cmdname, tmp, ' time to remove the source should not be less than zero')
        if stop - start <= 0:
            raise _err(cmdname, tmp, ' duration of the source should not be zero or less')
        src.start = start
        src.stop = G.timewindow if stop > G.timewindow else stop
    else:
        src.start = 0
        src.stop = G.timewindow


def _simple_source(G, cmdname, cmdinstance, cls, minparams):
    tmp = cmdinstance.split()
    if len(tmp) < minparams:
        raise _err(cmdname, tmp, ' requires at least {} parameters'.format(
            {5: 'five', 6: 'six'}[minparams]))
    pol = tmp[0].lower()
    _check_polarisation(G, cmdname, tmp, pol)
    x = G.calculate_coord('x', tmp[1])
    y = G.calculate_coord('y', tmp[2])
    z = G.calculate_coord('z', tmp[3])
    _check_coords(G, cmdname, tmp, x, y, z)
    _in_pml_warning(G, cmdname, tmp, x, y, z)
    src = cls()
    src.polarisation = pol
    src.xcoord, src.ycoord, src.zcoord = x, y, z
    src.xcoordorigin, src.ycoordorigin, src.zcoordorigin = x, y, z
    src.ID = cls.__name__ + '(' + str(x) + ',' + str(y) + ',' + str(z) + ')'
    return tmp, src


def process_multicmds(multicmds, G):
    """Waveforms, sources, receivers, snapshots, materials, dispersion and CFS terms. Geometry
    views and geometry-object files are not written by this package (in the drop-in route the
    reference writes them); their commands are accepted and, with messages on, noted."""
    for cmdname in ('#geometry_view', '#geometry_objects_write'):
        if multicmds.get(cmdname) and G.messages:
            print('{} ({} given) is not written by the GB300 driver; the reference writes it '
                  'when it builds the model'.format(cmdname, len(multicmds[cmdname])))
    cmdname = '#waveform'
    for cmdinstance in multicmds[cmdname]:
        tmp = cmdinstance.split()
        if len(tmp) != 4:
            raise _err(cmdname, tmp, ' requires exactly four parameters')
        if tmp[0].lower() not in Waveform.types:
            raise _err(cmdname, tmp, ' must have one of the following types {}'.format(','.join(Waveform.types)))
        if float(tmp[2]) <= 0:
            raise _err(cmdname, tmp, ' requires an excitation frequency value of greater than zero')
        if any(x.ID == tmp[3] for x in G.waveforms):
            raise _err(cmdname, tmp, ' with ID {} already exists'.format(tmp[3]))
        w = Waveform()
        w.ID = tmp[3]
        w.type = tmp[0].lower()
        w.amp = float(tmp[1])
        w.freq = float(tmp[2])
        G.waveforms.append(w)

    cmdname = '#voltage_source'
    for cmdinstance in multicmds[cmdname]:
        tmp, v = _simple_source(G, cmdname, cmdinstance, VoltageSource, 6)
        resistance = float(tmp[4])
        if resistance < 0:
            raise _err(cmdname, tmp, ' requires a source resistance of zero or greater')
        if not any(x.ID == tmp[5] for x in G.waveforms):
            raise _err(cmdname, tmp, ' there is no waveform with the identifier {}'.format(tmp[5]))
        v.resistance = resistance
        v.waveformID = tmp[5]
        _start_stop(G, cmdname, tmp, v, 6)
        v.calculate_waveform_values(G)
        G.voltagesources.append(v)

    cmdname = '#hertzian_dipole'
    for cmdinstance in multicmds[cmdname]:
        tmp, h = _simple_source(G, cmdname, cmdinstance, HertzianDipole, 5)
        if not any(x.ID == tmp[4] for x in G.waveforms):
            raise _err(cmdname, tmp, ' there is no waveform with the identifier {}'.format(tmp[4]))
        h.dl = {'x': G.dx, 'y': G.dy, 'z': G.dz}[h.polarisation]
        h.waveformID = tmp[4]
        _start_stop(G, cmdname, tmp, h, 5)
        h.calculate_waveform_values(G)
        G.hertziandipoles.append(h)

    cmdname = '#magnetic_dipole'
    for cmdinstance in multicmds[cmdname]:
        tmp, m = _simple_source(G, cmdname, cmdinstance, MagneticDipole, 5)
        if not any(x.ID == tmp[4] for x in G.waveforms):
            raise _err(cmdname, tmp, ' there is no waveform with the identifier {}'.format(tmp[4]))
        m.waveformID = tmp[4]
        _start_stop(G, cmdname, tmp, m, 5)
        m.calculate_waveform_values(G)
        G.magneticdipoles.append(m)

    cmdname = '#transmission_line'
    for cmdinstance in multicmds[cmdname]:
        tmp, t = _simple_source(G, cmdname, cmdinstance, TransmissionLine, 6)
        resistance = float(tmp[4])
        if resistance <= 0 or resistance >= z0:
            raise _err(cmdname, tmp, ' requires a resistance greater than zero and less than the '
                                     'impedance of free space, i.e. 376.73 Ohms')
        if not any(x.ID == tmp[5] for x in G.waveforms):
            raise _err(cmdname, tmp, ' there is no waveform with the identifier {}'.format(tmp[5]))
        t.bind(G)
        t.resistance = resistance
        t.waveformID = tmp[5]
        _start_stop(G, cmdname, tmp, t, 6)
        t.calculate_waveform_values(G)
        t.calculate_incident_V_I(G)
        G.transmissionlines.append(t)

    cmdname = '#rx'
    for cmdinstance in multicmds[cmdname]:
        tmp = cmdinstance.split()
        if len(tmp) != 3 and len(tmp) < 5:
            raise _err(cmdname, tmp, ' has an incorrect number of parameters')
        x = round_value(float(tmp[0]) / G.dx)
        y = round_value(float(tmp[1]) / G.dy)
        z = round_value(float(tmp[2]) / G.dz)
        _check_coords(G, cmdname, tmp, x, y, z)
        _in_pml_warning(G, cmdname, tmp, x, y, z)
        r = Rx()
        r.xcoord, r.ycoord, r.zcoord = x, y, z
        r.xcoordorigin, r.ycoordorigin, r.zcoordorigin = x, y, z
        if len(tmp) == 3:
            r.ID = 'Rx(' + str(x) + ',' + str(y) + ',' + str(z) + ')'
            allocate_outputs(r, Rx.defaultoutputs, G.iterations)
        else:
            r.ID = tmp[3]
            for field in tmp[4:]:
                if field not in Rx.allowableoutputs:
                    raise _err(cmdname, tmp, ' contains an output type that is not allowable. '
                               'Allowable outputs in current context are {}'.format(Rx.allowableoutputs))
                allocate_outputs(r, [field], G.iterations)
        G.rxs.append(r)

    cmdname = '#rx_array'
    for cmdinstance in multicmds[cmdname]:
        tmp = cmdinstance.split()
        if len(tmp) != 9:
            raise _err(cmdname, tmp, ' requires exactly nine parameters')
        xs, ys, zs = (G.calculate_coord(a, v) for a, v in zip('xyz', tmp[0:3]))
        xf, yf, zf = (G.calculate_coord(a, v) for a, v in zip('xyz', tmp[3:6]))
        sx, sy, sz = (G.calculate_coord(a, v) for a, v in zip('xyz', tmp[6:9]))
        _check_coords(G, cmdname, tmp, xs, ys, zs, name='lower')
        _check_coords(G, cmdname, tmp, xf, yf, zf, name='upper')
        if xs > xf or ys > yf or zs > zf:
            raise _err(cmdname, tmp, ' the lower coordinates should be less than the upper coordinates')
        if sx < 0 or sy < 0 or sz < 0:
            raise _err(cmdname, tmp, ' the step size should not be less than zero')
        steps = []
        for s in (sx, sy, sz):
            if s < 1:
                if s == 0:
                    s = 1
                else:
                    raise _err(cmdname, tmp, ' the step size should not be less than the spatial discretisation')
            steps.append(s)
        for x in range(xs, xf + 1, steps[0]):
            for y in range(ys, yf + 1, steps[1]):
                for z in range(zs, zf + 1, steps[2]):
                    r = Rx()
                    r.xcoord, r.ycoord, r.zcoord = x, y, z
                    r.xcoordorigin, r.ycoordorigin, r.zcoordorigin = x, y, z
                    r.ID = 'Rx(' + str(x) + ',' + str(y) + ',' + str(z) + ')'
                    allocate_outputs(r, Rx.defaultoutputs, G.iterations)
                    G.rxs.append(r)

    cmdname = '#snapshot'
    for cmdinstance in multicmds[cmdname]:
        tmp = cmdinstance.split()
        if len(tmp) != 11:
            raise _err(cmdname, tmp, ' requires exactly eleven parameters')
        xs, ys, zs = (G.calculate_coord(a, v) for a, v in zip('xyz', tmp[0:3]))
        xf, yf, zf = (G.calculate_coord(a, v) for a, v in zip('xyz', tmp[3:6]))
        sdx, sdy, sdz = (G.calculate_coord(a, v) for a, v in zip('xyz', tmp[6:9]))
        try:
            time = int(tmp[9])
        except ValueError:
            time = float(tmp[9])
            if time > 0:
                time = round_value((time / G.dt)) + 1
            else:
                raise _err(cmdname, tmp, ' time value must be greater than zero')
        _check_coords(G, cmdname, tmp, xs, ys, zs, name='lower')
        _check_coords(G, cmdname, tmp, xf, yf, zf, name='upper')
        if xs >= xf or ys >= yf or zs >= zf:
            raise _err(cmdname, tmp, ' the lower coordinates should be less than the upper coordinates')
        if sdx < 0 or sdy < 0 or sdz < 0:
            raise _err(cmdname, tmp, ' the step size should not be less than zero')
        if sdx < 1 or sdy < 1 or sdz < 1:
            raise _err(cmdname, tmp, ' the step size should not be less than the spatial discretisation')
        if time <= 0 or time > G.iterations:
            raise _err(cmdname, tmp, ' time value is not valid')
        G.snapshots.append(Snapshot(xs, ys, zs, xf, yf, zf, sdx, sdy, sdz, time, tmp[10]))

    cmdname = '#material'
    for cmdinstance in multicmds[cmdname]:
        tmp = cmdinstance.split()
        if len(tmp) != 5:
            raise _err(cmdname, tmp, ' requires exactly five parameters')
        if float(tmp[0]) < 1:
            raise _err(cmdname, tmp, ' requires a positive value of one or greater for static (DC) permittivity')
        if tmp[1] != 'inf':
            se = float(tmp[1])
            if se < 0:
                raise _err(cmdname, tmp, ' requires a positive value for conductivity')
        else:
            se = float('inf')
        if float(tmp[2]) < 1:
            raise _err(cmdname, tmp, ' requires a positive value of one or greater for permeability')
        if float(tmp[3]) < 0:
            raise _err(cmdname, tmp, ' requires a positive value for magnetic conductivity')
        if any(x.ID == tmp[4] for x in G.materials):
            raise _err(cmdname, tmp, ' with ID {} already exists'.format(tmp[4]))
        m = Material(len(G.materials), tmp[4])
        m.er = float(tmp[0])
        m.se = se
        m.mr = float(tmp[2])
        m.sm = float(tmp[3])
        if m.se == float('inf'):
            m.averagable = False
        G.materials.append(m)

    for cmdname, kind, per in (('#add_dispersion_debye', 'debye', 2),
                               ('#add_dispersion_lorentz', 'lorentz', 3),
                               ('#add_dispersion_drude', 'drude', 2)):
        for cmdinstance in multicmds[cmdname]:
            tmp = cmdinstance.split()
            need = 4 if kind == 'debye' else 5
            if len(tmp) < need:
                raise _err(cmdname, tmp, ' requires at least {} parameters'.format(
                    'four' if need == 4 else 'five'))
            if int(tmp[0]) < 0:
                raise _err(cmdname, tmp, ' requires a positive value for number of poles')
            poles = int(tmp[0])
            span = 2 * poles if kind in ('debye', 'drude') else 3 * poles
            if kind == 'drude':
                span = 3 * poles   # the reference slices materials after 3 values per pole
            requested = tmp[span + 1:] if kind != 'debye' else tmp[(2 * poles) + 1:]
            materials = [y for x in requested for y in G.materials if y.ID == x]
            if len(materials) != len(requested):
                notfound = [x for x in requested if x not in materials]
                raise _err(cmdname, tmp, ' material(s) {} do not exist'.format(notfound))
            for material in materials:
                material.type = kind
                material.poles = poles
                material.averagable = False
                if kind == 'debye':
                    for pole in range(1, 2 * poles, 2):
                        if float(tmp[pole]) > 0:
                            material.deltaer.append(float(tmp[pole]))
                            material.tau.append(float(tmp[pole + 1]))
                        else:
                            raise _err(cmdname, tmp, ' requires positive values for the permittivity difference.')
                elif kind == 'lorentz':
                    for pole in range(1, 3 * poles, 3):
                        if float(tmp[pole]) > 0 and float(tmp[pole + 1]) > G.dt and float(tmp[pole + 2]) > G.dt:
                            material.deltaer.append(float(tmp[pole]))
                            material.tau.append(float(tmp[pole + 1]))
                            material.alpha.append(float(tmp[pole + 2]))
                        else:
                            raise _err(cmdname, tmp, ' requires positive values for the permittivity difference and frequencies, and associated times that are greater than the time step for the model.')
                else:
                    for pole in range(1, 2 * poles, 2):
                        if float(tmp[pole]) > 0 and float(tmp[pole + 1]) > G.dt:
                            material.tau.append(float(tmp[pole]))
                            material.alpha.append(float(tmp[pole + 1]))
                        else:
                            raise _err(cmdname, tmp, ' requires positive values for the frequencies, and associated times that are greater than the time step for the model.')
                if material.poles > G.maxpoles:
                    G.maxpoles = material.poles

    cmdname = '#soil_peplinski'
    for cmdinstance in multicmds[cmdname] or []:
        tmp = cmdinstance.split()
        if len(tmp) != 7:
            raise _err(cmdname, tmp, ' requires at exactly seven parameters')
        for idx, what in ((0, 'sand fraction'), (1, 'clay fraction'), (2, 'bulk density'),
                          (3, 'sand particle density'),
                          (4, 'lower limit of the water volumetric fraction'),
                          (5, 'upper limit of the water volumetric fraction')):
            if float(tmp[idx]) < 0:
                raise _err(cmdname, tmp, ' requires a positive value for the ' + what)
        if any(x.ID == tmp[6] for x in G.mixingmodels):
            raise _err(cmdname, tmp, ' with ID {} already exists'.format(tmp[6]))
        s = PeplinskiSoil(tmp[6], float(tmp[0]), float(tmp[1]), float(tmp[2]), float(tmp[3]),
                          (float(tmp[4]), float(tmp[5])))
        _log(G, 'Mixing model (Peplinski) used to create {} with sand fraction {:g}, clay '
                'fraction {:g}, bulk density {:g}g/cm3, sand particle density {:g}g/cm3, and '
                'water volumetric fraction {:g} to {:g} created.'.format(
                    s.ID, s.S, s.C, s.rb, s.rs, s.mu[0], s.mu[1]))
        G.mixingmodels.append(s)

    cmdname = '#pml_cfs'
    if multicmds[cmdname]:
        if len(multicmds[cmdname]) > 2:
            raise CmdInputError("'" + cmdname + "' can only be used up to two times, for up to a 2nd order PML")
        for cmdinstance in multicmds[cmdname]:
            tmp = cmdinstance.split()
            if len(tmp) != 12:
                raise _err(cmdname, tmp, ' requires exactly twelve parameters')
            profiles = CFSParameter.scalingprofiles.keys()
            if tmp[0] not in profiles or tmp[4] not in profiles or tmp[8] not in profiles:
                raise _err(cmdname, tmp, ' must have scaling type {}'.format(','.join(profiles)))
            dirs = CFSParameter.scalingdirections
            if tmp[1] not in dirs or tmp[5] not in dirs or tmp[9] not in dirs:
                raise _err(cmdname, tmp, ' must have scaling type {}'.format(','.join(dirs)))
            if (float(tmp[2]) < 0 or float(tmp[3]) < 0 or float(tmp[6]) < 0 or float(tmp[7]) < 0
                    or float(tmp[10]) < 0):
                raise _err(cmdname, tmp, ' minimum and maximum scaling values must be positive')
            if float(tmp[6]) < 1 and G.pmlformulation == 'HORIPML':
                raise _err(cmdname, tmp, ' minimum scaling value for kappa must be greater than or equal to one')
            cfs = CFS()
            cfs.alpha = CFSParameter(ID='alpha', scalingprofile=tmp[0], scalingdirection=tmp[1],
                                     min=float(tmp[2]), max=float(tmp[3]))
            cfs.kappa = CFSParameter(ID='kappa', scalingprofile=tmp[4], scalingdirection=tmp[5],
                                     min=float(tmp[6]), max=float(tmp[7]))
            cfs.sigma = CFSParameter(ID='sigma', scalingprofile=tmp[8], scalingdirection=tmp[9],
                                     min=float(tmp[10]),
                                     max=None if tmp[11] == 'None' else float(tmp[11]))
            G.cfs.append(cfs)


def _lookup_materials(G, tmp, requested):
    materials = [y for x in requested for y in G.materials if y.ID == x]
    if len(materials) != len(requested):
        notfound = [x for x in requested if x not in materials]
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' material(s) {} do not exist'.format(notfound))
    return materials


def _volume_material(G, tmp, materials, averageflag):
    """Material numbers and smoothing flag of a volume primitive (isotropic or uniaxial)."""
    if len(materials) == 1:
        averaging = materials[0].averagable and averageflag
        n = materials[0].numID
        return n, n, n, n, averaging
    requiredID = materials[0].ID + '+' + materials[1].ID + '+' + materials[2].ID
    found = [x for x in G.materials if x.ID == requiredID]
    if found:
        numID = found[0].numID
    else:
        numID = len(G.materials)
        m = Material(numID, requiredID)
        m.type = 'dielectric-smoothed'
        m.er = np.mean((materials[0].er, materials[1].er, materials[2].er), axis=0)
        m.se = np.mean((materials[0].se, materials[1].se, materials[2].se), axis=0)
        m.mr = np.mean((materials[0].mr, materials[1].mr, materials[2].mr), axis=0)
        m.sm = np.mean((materials[0].sm, materials[1].sm, materials[2].sm), axis=0)
        G.materials.append(m)
    return numID, materials[0].numID, materials[1].numID, materials[2].numID, False


def _average_option(G, tmp, n_iso, opt_index):
    if len(tmp) == n_iso:
        return [tmp[n_iso - 1]], G.averagevolumeobjects
    if len(tmp) == n_iso + 1:
        flag = tmp[opt_index].lower()
        if flag == 'y':
            return [tmp[n_iso - 1]], True
        if flag == 'n':
            return [tmp[n_iso - 1]], False
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' requires averaging to be either y or n')
    if len(tmp) == n_iso + 2:
        return tmp[n_iso - 1:], False
    raise CmdInputError("'" + ' '.join(tmp) + "'" + ' too many parameters have been given')


def process_geometrycmds(geometry, G):
    """Build geometry primitives in the order given (``input_cmds_geometry.py:51``)."""
    for line in geometry:
        tmp = line.split()
        name = tmp[0]
        if name == '#box:':
            if len(tmp) < 8:
                raise CmdInputError("'" + ' '.join(tmp) + "'" + ' requires at least seven parameters')
            requested, avg = _average_option(G, tmp, 8, 8)
            xs = round_value(float(tmp[1]) / G.dx)
            xf = round_value(float(tmp[4]) / G.dx)
            ys = round_value(float(tmp[2]) / G.dy)
            yf = round_value(float(tmp[5]) / G.dy)
            zs = round_value(float(tmp[3]) / G.dz)
            zf = round_value(float(tmp[6]) / G.dz)
            for v, n, ax in ((xs, G.nx, 'x'), (xf, G.nx, 'x'), (ys, G.ny, 'y'), (yf, G.ny, 'y'),
                             (zs, G.nz, 'z'), (zf, G.nz, 'z')):
                if v < 0 or v > n:
                    raise CmdInputError("'" + ' '.join(tmp) + "'" + ' the {}-coordinate is not within the model domain'.format(ax))
            if xs >= xf or ys >= yf or zs >= zf:
                raise CmdInputError("'" + ' '.join(tmp) + "'" + ' the lower coordinates should be less than the upper coordinates')
            mats = _lookup_materials(G, tmp, requested)
            numID, nx_, ny_, nz_, averaging = _volume_material(G, tmp, mats, avg)
            geo.build_box(G, xs, xf, ys, yf, zs, zf, numID, nx_, ny_, nz_, averaging)
        elif name == '#sphere:':
            if len(tmp) < 6:
                raise CmdInputError("'" + ' '.join(tmp) + "'" + ' requires at least five parameters')
            requested, avg = _average_option(G, tmp, 6, 6)
            xc = round_value(float(tmp[1]) / G.dx)
            yc = round_value(float(tmp[2]) / G.dy)
            zc = round_value(float(tmp[3]) / G.dz)
            r = float(tmp[4])
            mats = _lookup_materials(G, tmp, requested)
            numID, nx_, ny_, nz_, averaging = _volume_material(G, tmp, mats, avg)
            geo.build_sphere(G, xc, yc, zc, r, numID, nx_, ny_, nz_, averaging)
        elif name == '#cylinder:':
            if len(tmp) < 9:
                raise CmdInputError("'" + ' '.join(tmp) + "'" + ' requires at least eight parameters')
            requested, avg = _average_option(G, tmp, 9, 9)
            # face centres snap to the nearest grid node
            x1 = round_value(float(tmp[1]) / G.dx) * G.dx
            y1 = round_value(float(tmp[2]) / G.dy) * G.dy
            z1 = round_value(float(tmp[3]) / G.dz) * G.dz
            x2 = round_value(float(tmp[4]) / G.dx) * G.dx
            y2 = round_value(float(tmp[5]) / G.dy) * G.dy
            z2 = round_value(float(tmp[6]) / G.dz) * G.dz
            r = float(tmp[7])
            if r <= 0:
                raise CmdInputError("'" + ' '.join(tmp) + "'" + ' the radius {:g} should be a positive value.'.format(r))
            mats = _lookup_materials(G, tmp, requested)
            numID, nx_, ny_, nz_, averaging = _volume_material(G, tmp, mats, avg)
            geo.build_cylinder(G, x1, y1, z1, x2, y2, z2, r, numID, nx_, ny_, nz_, averaging)
        elif name == '#edge:':
            if len(tmp) != 8:
                raise CmdInputError("'" + ' '.join(tmp) + "'" + ' requires exactly seven parameters')
            xs = round_value(float(tmp[1]) / G.dx)
            xf = round_value(float(tmp[4]) / G.dx)
            ys = round_value(float(tmp[2]) / G.dy)
            yf = round_value(float(tmp[5]) / G.dy)
            zs = round_value(float(tmp[3]) / G.dz)
            zf = round_value(float(tmp[6]) / G.dz)
            mats = _lookup_materials(G, tmp, [tmp[7]])
            geo.build_edge(G, xs, ys, zs, xf, yf, zf, mats[0].numID)
        elif name == '#plate:':
            if len(tmp) < 8:
                raise CmdInputError("'" + ' '.join(tmp) + "'" + ' requires at least seven parameters')
            requested = tmp[7:]
            xs = round_value(float(tmp[1]) / G.dx)
            xf = round_value(float(tmp[4]) / G.dx)
            ys = round_value(float(tmp[2]) / G.dy)
            yf = round_value(float(tmp[5]) / G.dy)
            zs = round_value(float(tmp[3]) / G.dz)
            zf = round_value(float(tmp[6]) / G.dz)
            mats = _lookup_materials(G, tmp, requested)
            geo.build_plate(G, xs, xf, ys, yf, zs, zf, [m.numID for m in mats])
        elif name == '#triangle:':
            _triangle(G, tmp)
        elif name == '#cylindrical_sector:':
            _cylindrical_sector(G, tmp)
        elif name == '#fractal_box:':
            _fractal_box(G, tmp, geometry)
        elif name in _FRACTAL_MODIFIERS:
            # handled (and rejected) by the fractal box they name
            continue
        else:
            raise CmdInputError('{} is not supported by the GB300 solver core'.format(name.rstrip(':')))


_FRACTAL_MODIFIERS = ('#add_surface_roughness:', '#add_surface_water:', '#add_grass:')


def _cylindrical_sector(G, tmp):
    """#cylindrical_sector: normal axis, centre (two in-plane coordinates), the extent along the
    normal, radius, start and sector angles in degrees, one material (with an optional smoothing
    flag) or three (``input_cmds_geometry.py``, #cylindrical_sector)."""
    if len(tmp) < 10:
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' requires at least nine parameters')
    requested, avg = _average_option(G, tmp, 10, 10)
    normal = tmp[1].lower()
    ctr1, ctr2 = float(tmp[2]), float(tmp[3])
    extent1, extent2 = float(tmp[4]), float(tmp[5])
    thickness = extent2 - extent1
    r = float(tmp[6])
    sectorstartangle = 2 * np.pi * (float(tmp[7]) / 360)
    sectorangle = 2 * np.pi * (float(tmp[8]) / 360)
    if normal not in ('x', 'y', 'z'):
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' the normal direction must be either x, y or z.')
    if r <= 0:
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' the radius {:g} should be a positive value.'.format(r))
    if sectorstartangle < 0 or sectorangle <= 0:
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' the starting angle and sector angle should be a positive values.')
    if sectorstartangle >= 2 * np.pi or sectorangle >= 2 * np.pi:
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' the starting angle and sector angle must be less than 360 degrees.')
    mats = _lookup_materials(G, tmp, requested)
    if thickness > 0:
        numID, nx_, ny_, nz_, averaging = _volume_material(G, tmp, mats, avg)
    elif len(mats) == 1:
        numID = nx_ = ny_ = nz_ = mats[0].numID
        averaging = False
    else:
        # the reference passes no material number for a zero-thickness uniaxial sector and its
        # builder refuses the call
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' a zero-thickness cylindrical sector '
                            'takes one material')
    d1, d2, dn = {'x': (G.dy, G.dz, G.dx), 'y': (G.dx, G.dz, G.dy), 'z': (G.dx, G.dy, G.dz)}[normal]
    ctr1 = round_value(ctr1 / d1) * d1
    ctr2 = round_value(ctr2 / d2) * d2
    level = round_value(extent1 / dn)
    geo.build_cylindrical_sector(G, ctr1, ctr2, level, sectorstartangle, sectorangle, r, normal,
                                 thickness, numID, nx_, ny_, nz_, averaging)


def _triangle(G, tmp):
    """#triangle: three vertices on one grid plane, a thickness and one material (with an
    optional smoothing flag) or three (uniaxial) (``input_cmds_geometry.py``, #triangle)."""
    if len(tmp) < 12:
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' requires at least eleven parameters')
    requested, avg = _average_option(G, tmp, 12, 12)
    v = []
    for q in range(3):
        v.append((round_value(float(tmp[1 + 3 * q]) / G.dx) * G.dx,
                  round_value(float(tmp[2 + 3 * q]) / G.dy) * G.dy,
                  round_value(float(tmp[3 + 3 * q]) / G.dz) * G.dz))
    thickness = float(tmp[10])
    for ax, n, d in ((0, G.nx, G.dx), (1, G.ny, G.dy), (2, G.nz, G.dz)):
        if any(p[ax] < 0 or p[ax] > n * d for p in v):
            raise CmdInputError("'" + ' '.join(tmp) + "'" + ' the one of the {}-coordinates is '
                                'not within the model domain'.format('xyz'[ax]))
    if thickness < 0:
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' requires a positive value for thickness')
    normal = None
    for ax in range(3):
        if v[0][ax] == v[1][ax] and v[1][ax] == v[2][ax]:
            normal = 'xyz'[ax]
            break
    if normal is None:
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' the triangle is not specified correctly')
    mats = _lookup_materials(G, tmp, requested)
    if thickness > 0:
        numID, nx_, ny_, nz_, averaging = _volume_material(G, tmp, mats, avg)
    elif len(mats) == 1:
        numID = nx_ = ny_ = nz_ = mats[0].numID
        averaging = False
    else:
        # the reference passes no material number for a zero-thickness uniaxial triangle and
        # its builder refuses the call
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' a zero-thickness triangle takes one '
                            'material')
    geo.build_triangle(G, v, normal, thickness, numID, nx_, ny_, nz_, averaging)


def _fractal_box(G, tmp, geometry):
    """``#fractal_box`` without modifiers (``input_cmds_geometry.py:808-888`` and
    ``1519-1527``): a seeded fractal volume binned into the materials of a Peplinski mixing
    model and voxelised with ``build_voxels_from_array``. Rough surfaces, surface water and
    grass are not supported and raise :class:`CmdInputError`."""
    averaging = False
    if len(tmp) < 14:
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' requires at least thirteen parameters')
    elif len(tmp) == 14:
        seed = None
    elif len(tmp) == 15:
        seed = int(tmp[14])
    elif len(tmp) == 16:
        seed = int(tmp[14])
        flag = tmp[15].lower()
        if flag not in ('y', 'n'):
            raise CmdInputError("'" + ' '.join(tmp) + "'" + ' requires averaging to be either y or n')
        averaging = flag == 'y'
    else:
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' too many parameters have been given')
    xs = round_value(float(tmp[1]) / G.dx)
    xf = round_value(float(tmp[4]) / G.dx)
    ys = round_value(float(tmp[2]) / G.dy)
    yf = round_value(float(tmp[5]) / G.dy)
    zs = round_value(float(tmp[3]) / G.dz)
    zf = round_value(float(tmp[6]) / G.dz)
    for v, n, lu, ax, dl in ((xs, G.nx, 'lower', 'x', G.dx), (xf, G.nx, 'upper', 'x', G.dx),
                             (ys, G.ny, 'lower', 'y', G.dy), (yf, G.ny, 'upper', 'y', G.dy),
                             (zs, G.nz, 'lower', 'z', G.dz), (zf, G.nz, 'upper', 'z', G.dz)):
        if v < 0 or v > n:
            raise CmdInputError("'" + ' '.join(tmp) + "'" + ' the {} {}-coordinate {:g}m is not within the model domain'.format(lu, ax, v * dl))
    if xs >= xf or ys >= yf or zs >= zf:
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' the lower coordinates should be less than the upper coordinates')
    if float(tmp[7]) < 0:
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' requires a positive value for the fractal dimension')
    for idx, ax in ((8, 'x'), (9, 'y'), (10, 'z')):
        if float(tmp[idx]) < 0:
            raise CmdInputError("'" + ' '.join(tmp) + "'" + ' requires a positive value for the fractal weighting in the {} direction'.format(ax))
    if round_value(tmp[11]) < 0:
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' requires a positive value for the number of bins')

    mixingmodel = next((x for x in G.mixingmodels if x.ID == tmp[12]), None)
    material = next((x for x in G.materials if x.ID == tmp[12]), None)
    nbins = round_value(tmp[11])
    if mixingmodel:
        if nbins == 1:
            raise CmdInputError("'" + ' '.join(tmp) + "'" + ' must be used with more than one material from the mixing model.')
        mixingmodel.calculate_debye_properties(nbins, G, tmp[13])
    elif not material:
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' mixing model or material with ID {} does not exist'.format(tmp[12]))

    volume = FractalVolume(xs, xf, ys, yf, zs, zf, float(tmp[7]), seed)
    volume.ID = tmp[13]
    volume.operatingonID = tmp[12]
    volume.nbins = nbins
    volume.weighting = np.array([float(tmp[8]), float(tmp[9]), float(tmp[10])])
    volume.averaging = averaging
    _log(G, 'Fractal box {} from {:g}m, {:g}m, {:g}m, to {:g}m, {:g}m, {:g}m with {}, fractal '
            'dimension {:g}, fractal weightings {:g}, {:g}, {:g}, fractal seeding {}, with {} '
            'material(s) created, dielectric smoothing is {}.'.format(
                volume.ID, xs * G.dx, ys * G.dy, zs * G.dz, xf * G.dx, yf * G.dy, zf * G.dz,
                volume.operatingonID, volume.dimension, volume.weighting[0],
                volume.weighting[1], volume.weighting[2], volume.seed, volume.nbins,
                'on' if averaging else 'off'))
    G.fractalvolumes.append(volume)

    for other in geometry:
        m = other.split()
        if not m:
            continue
        if m[0] == '#add_surface_roughness:':
            _surface_roughness(G, m, volume)
        elif m[0] == '#add_surface_water:':
            _surface_water(G, m, volume)
        elif m[0] == '#add_grass:' and volume.ID in m[1:]:
            raise CmdInputError('#add_grass is not supported by the GB300 solver core')

    if volume.fractalsurfaces:
        # the box grows to take in its rough surfaces; the mask picks soil, water or nothing
        volume.extend_for_surfaces()
        if nbins == 1:
            vol = np.ones((volume.nx, volume.ny, volume.nz), dtype=floattype)
            vol *= next(x.numID for x in G.materials if x.ID == volume.operatingonID)
        else:
            if not mixingmodel:
                raise CmdInputError("'" + ' '.join(tmp) + "'" + ' needs a mixing model to bin {} materials from; {} is a single material'.format(nbins, tmp[12]))
            vol = volume.generate_fractal_volume(device=getattr(G, "device_fractals", False))
            vol += mixingmodel.startmaterialnum
        mask = volume.generate_volume_mask()
        waternumID = next((x.numID for x in G.materials if x.ID == 'water'), 0)
        data = vol.astype('int16', order='C')
        cells = np.where(mask == 1, data, np.where(mask == 2, np.int16(waternumID), np.int16(-1)))
        geo.build_voxels_array(G, (volume.xs, volume.ys, volume.zs), cells.astype(np.int16),
                               averaging)
        return
    if nbins == 1:
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' is being used with a single material and no modifications, therefore please use a #box command instead.')
    if not mixingmodel:
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' needs a mixing model to bin {} materials from; {} is a single material'.format(nbins, tmp[12]))
    vol = volume.generate_fractal_volume(device=getattr(G, "device_fractals", False))
    vol += mixingmodel.startmaterialnum
    geo.build_voxels_array(G, (xs, ys, zs), vol.astype('int16', order='C'), averaging)


def _surface_extent(G, tmp):
    xs = round_value(float(tmp[1]) / G.dx)
    xf = round_value(float(tmp[4]) / G.dx)
    ys = round_value(float(tmp[2]) / G.dy)
    yf = round_value(float(tmp[5]) / G.dy)
    zs = round_value(float(tmp[3]) / G.dz)
    zf = round_value(float(tmp[6]) / G.dz)
    for v, n, lu, ax, dl in ((xs, G.nx, 'lower', 'x', G.dx), (xf, G.nx, 'upper', 'x', G.dx),
                             (ys, G.ny, 'lower', 'y', G.dy), (yf, G.ny, 'upper', 'y', G.dy),
                             (zs, G.nz, 'lower', 'z', G.dz), (zf, G.nz, 'upper', 'z', G.dz)):
        if v < 0 or v > n:
            raise CmdInputError("'" + ' '.join(tmp) + "'" + ' the {} {}-coordinate {:g}m is not within the model domain'.format(lu, ax, v * dl))
    if xs > xf or ys > yf or zs > zf:
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' the lower coordinates should be less than the upper coordinates')
    return xs, xf, ys, yf, zs, zf


def _surface_face(tmp, volume, xs, xf, ys, yf, zs, zf):
    """The face of the fractal box the surface lies on: (axis, side) with side 'minus'/'plus'."""
    lo = (xs, ys, zs)
    hi = (xf, yf, zf)
    vlo = (volume.xs, volume.ys, volume.zs)
    vhi = (volume.xf, volume.yf, volume.zf)
    for axis in range(3):
        if lo[axis] == hi[axis]:
            others = [a for a in range(3) if a != axis]
            if any(lo[a] == hi[a] for a in others):
                raise CmdInputError("'" + ' '.join(tmp) + "'" + ' dimensions are not specified correctly')
            if lo[axis] != vlo[axis] and lo[axis] != vhi[axis]:
                raise CmdInputError("'" + ' '.join(tmp) + "'" + ' can only be used on the external surfaces of a fractal box')
            if lo[axis] == vlo[axis]:
                return axis, 'minus'
            if hi[axis] == vhi[axis]:
                return axis, 'plus'
            return axis, None
    raise CmdInputError("'" + ' '.join(tmp) + "'" + ' dimensions are not specified correctly')


def _surface_roughness(G, tmp, volume):
    """``#add_surface_roughness`` on a face of ``volume`` (``input_cmds_geometry.py:893-1006``)."""
    if len(tmp) < 13:
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' requires at least twelve parameters')
    elif len(tmp) == 13:
        seed = None
    elif len(tmp) == 14:
        seed = int(tmp[13])
    else:
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' too many parameters have been given')
    if tmp[12] != volume.ID:
        return
    xs, xf, ys, yf, zs, zf = _surface_extent(G, tmp)
    if float(tmp[7]) < 0:
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' requires a positive value for the fractal dimension')
    if float(tmp[8]) < 0:
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' requires a positive value for the fractal weighting in the first direction of the surface')
    if float(tmp[9]) < 0:
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' requires a positive value for the fractal weighting in the second direction of the surface')
    axis, side = _surface_face(tmp, volume, xs, xf, ys, yf, zs, zf)
    dl = (G.dx, G.dy, G.dz)[axis]
    ax = 'xyz'[axis]
    n = (G.nx, G.ny, G.nz)[axis]
    vlo = (volume.xs, volume.ys, volume.zs)[axis]
    vhi = (volume.xf, volume.yf, volume.zf)[axis]
    fractalrange = (round_value(float(tmp[10]) / dl), round_value(float(tmp[11]) / dl))
    if side == 'minus':
        # (the reference's message names the x direction for a z-minus surface too)
        if fractalrange[0] < 0 or fractalrange[1] > vhi:
            raise CmdInputError("'" + ' '.join(tmp) + "'" + ' cannot apply fractal surface to fractal box as it would exceed either the upper coordinates of the fractal box or the domain in the {} direction'.format('x' if ax == 'z' else ax))
    elif side == 'plus':
        if fractalrange[0] < vlo or fractalrange[1] > n:
            raise CmdInputError("'" + ' '.join(tmp) + "'" + ' cannot apply fractal surface to fractal box as it would exceed either the lower coordinates of the fractal box or the domain in the {} direction'.format(ax))
    surface = FractalSurface(xs, xf, ys, yf, zs, zf, float(tmp[7]), seed)
    surface.surfaceID = ax + side
    surface.fractalrange = fractalrange
    surface.operatingonID = volume.ID
    surface.weighting = np.array([float(tmp[8]), float(tmp[9])])
    if surface.surfaceID in [x.surfaceID for x in volume.fractalsurfaces]:
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' has already been used on the {} surface'.format(surface.surfaceID))
    surface.generate_fractal_surface(device=getattr(G, "device_fractals", False))
    volume.fractalsurfaces.append(surface)
    _log(G, 'Fractal surface from {:g}m, {:g}m, {:g}m, to {:g}m, {:g}m, {:g}m with fractal '
            'dimension {:g}, fractal weightings {:g}, {:g}, fractal seeding {}, and range {:g}m '
            'to {:g}m, added to {}.'.format(xs * G.dx, ys * G.dy, zs * G.dz, xf * G.dx,
                                           yf * G.dy, zf * G.dz, surface.dimension,
                                           surface.weighting[0], surface.weighting[1],
                                           surface.seed, float(tmp[10]), float(tmp[11]),
                                           surface.operatingonID))


def _surface_water(G, tmp, volume):
    """``#add_surface_water`` on a rough surface of ``volume`` (``input_cmds_geometry.py:1008-1109``):
    water (the built-in single-pole Debye material) up to a fill depth."""
    if len(tmp) != 9:
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' requires exactly eight parameters')
    if tmp[8] != volume.ID:
        return
    xs, xf, ys, yf, zs, zf = _surface_extent(G, tmp)
    depth = float(tmp[7])
    if depth <= 0:
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' requires a positive value for the depth of water')
    axis, side = _surface_face(tmp, volume, xs, xf, ys, yf, zs, zf)
    dl = (G.dx, G.dy, G.dz)[axis]
    filldepthcells = round_value(depth / dl)
    filldepth = filldepthcells * dl
    requested = 'xyz'[axis] + (side or '')
    surface = next((x for x in volume.fractalsurfaces if x.surfaceID == requested), None)
    if not surface:
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' specified surface {} does not have a rough surface applied'.format(requested))
    surface.filldepth = filldepthcells
    if surface.filldepth < surface.fractalrange[0] or surface.filldepth > surface.fractalrange[1]:
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' requires a value for the depth of water that lies with the range of the requested surface roughness')
    if not any(x.ID == 'water' for x in G.materials):
        m = Material(len(G.materials), 'water')
        m.averagable = False
        m.type = 'builtin, debye'
        m.er = Material.watereri
        m.poles = 1
        m.deltaer.append(Material.waterdeltaer)
        m.tau.append(Material.watertau)
        G.materials.append(m)
        if G.maxpoles == 0:
            G.maxpoles = 1
    water = next(x for x in G.materials if x.ID == 'water')
    if next((x for x in water.tau if x < G.dt), None):
        raise CmdInputError("'" + ' '.join(tmp) + "'" + ' requires the time step for the model to be less than the relaxation time required to model water.')
    _log(G, 'Water on surface from {:g}m, {:g}m, {:g}m, to {:g}m, {:g}m, {:g}m with depth {:g}m, '
            'added to {}.'.format(xs * G.dx, ys * G.dy, zs * G.dz, xf * G.dx, yf * G.dy,
                                  zf * G.dz, filldepth, surface.operatingonID))
