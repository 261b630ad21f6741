"""Input-file pre-processing and command classification (``gprMax/input_cmds_file.py``).

``#python:`` blocks are executed in the user namespace and their printed ``#`` lines become
commands; ``#include_file:`` inserts another file; lines starting ``##`` are comments.
"""
import os
import sys
from io import StringIO

from .exceptions import CmdInputError

ESSENTIAL = ['#domain', '#dx_dy_dz', '#time_window']
SINGLE = ['#domain', '#dx_dy_dz', '#time_window', '#title', '#messages', '#num_threads',
          '#time_step_stability_factor', '#pml_formulation', '#pml_cells', '#excitation_file',
          '#src_steps', '#rx_steps', '#taguchi', '#end_taguchi', '#output_dir']
MULTIPLE = ['#geometry_view', '#geometry_objects_write', '#material', '#soil_peplinski',
            '#add_dispersion_debye', '#add_dispersion_lorentz', '#add_dispersion_drude',
            '#waveform', '#voltage_source', '#hertzian_dipole', '#magnetic_dipole',
            '#transmission_line', '#rx', '#rx_array', '#snapshot', '#pml_cfs', '#include_file']
GEOMETRY = ['#geometry_objects_read', '#edge', '#plate', '#triangle', '#box', '#sphere',
            '#cylinder', '#cylindrical_sector', '#fractal_box', '#add_surface_roughness',
            '#add_surface_water', '#add_grass']


def process_python_include_code(lines, usernamespace, inputfilename=''):
    """Run ``#python:`` blocks and expand includes; returns the command lines."""
    inputlines = [line.rstrip() for line in lines if not line.startswith('##') and line.rstrip('\n')]
    processed = []
    x = 0
    while x < len(inputlines):
        if inputlines[x].startswith('#python:'):
            code = ''
            x += 1
            while not inputlines[x].startswith('#end_python:'):
                code += inputlines[x] + '\n'
                x += 1
                if x == len(inputlines):
                    raise CmdInputError('Cannot find the end of the Python code block, i.e. '
                                        'missing #end_python: command.')
            compiled = compile(code, '<string>', 'exec')
            old = sys.stdout
            sys.stdout = buf = StringIO()
            try:
                exec(compiled, usernamespace)
            finally:
                sys.stdout = old
            out = buf.getvalue().split('\n')
            cmds = [line + '\n' for line in out if line.startswith('#')]
            other = [line for line in out if line and not line.startswith('#')]
            processed.extend(cmds)
            if other:
                print('Python messages (from stdout/stderr): {}\n'.format(other))
        elif inputlines[x].startswith('#'):
            processed.append(inputlines[x] + '\n')
        x += 1
    return process_include_files(processed, inputfilename)


def process_include_files(hashcmds, inputfilename):
    out = []
    for cmd in hashcmds:
        if cmd.startswith('#include_file:'):
            parts = cmd.split()
            if len(parts) != 2:
                raise CmdInputError('#include_file requires exactly one parameter')
            inc = parts[1]
            if not os.path.isfile(inc):
                inc = os.path.join(os.path.dirname(inputfilename), inc)
            with open(inc, 'r') as f:
                out.extend(line.rstrip() + '\n' for line in f
                           if not line.startswith('##') and line.rstrip('\n'))
        else:
            out.append(cmd)
    return out


def check_cmd_names(processedlines, checkessential=True):
    """Split commands into single-use (dict), multi-use (dict of lists) and geometry (list)."""
    singlecmds = dict.fromkeys(SINGLE, None)
    multiplecmds = {key: [] for key in MULTIPLE}
    geometry = []
    countessential = 0
    for line in processedlines:
        cmd = line.split(':')
        cmdname = cmd[0]
        cmdparams = cmd[1]
        if ' ' not in cmdparams[0] and len(cmdparams.strip('\n')) != 0:
            raise CmdInputError('There must be a space between the command name and parameters in ' + line)
        if cmdname not in ESSENTIAL and cmdname not in singlecmds and cmdname not in multiplecmds \
                and cmdname not in GEOMETRY:
            raise CmdInputError('Your input file contains an invalid command: ' + cmdname)
        if cmdname in ESSENTIAL:
            countessential += 1
        if cmdname in singlecmds:
            if singlecmds[cmdname] is None:
                singlecmds[cmdname] = cmd[1].strip(' \t\n')
            else:
                raise CmdInputError('You can only have a single instance of ' + cmdname + ' in your model')
        elif cmdname in multiplecmds:
            multiplecmds[cmdname].append(cmd[1].strip(' \t\n'))
        elif cmdname in GEOMETRY:
            geometry.append(line.strip(' \t\n'))
    if checkessential and countessential < len(ESSENTIAL):
        raise CmdInputError('Your input file is missing essential commands required to run a '
                            'model. Essential commands are: ' + ', '.join(ESSENTIAL))
    return singlecmds, multiplecmds, geometry
