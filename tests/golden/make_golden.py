"""Generate the golden fixtures in this directory from the reference itself.

Needs a gprMax v3.1.7 checkout (``--src``, default ``build_ref.SOURCE``) and its kernels built
by ``oracle/build_ref.py`` (both the default build and ``--variant nofma``). Each model runs
through the reference's own driver (``oracle/ref_harness.py``: input parsing, grid build,
``solve_cpu``), once per build, in a child process. Writes, per model, ``<name>.npz`` with:

* ``input``: the input-file text;
* ``iterations``, ``dt``, ``nmat``, ``ID_sha256``, ``coeffE``, ``coeffH`` (and ``coeffD``):
  the reference's model build;
* ``rx<n>_<output>``: receiver traces of the no-contraction build (bit-for-bit reproducible);
* ``tl<n>_<Vinc|Iinc|Vtotal|Itotal>``: transmission-line voltages and currents of that build;
* ``field_<C>_sha256`` and ``field_stats`` (sum, sum of |.|, max |.| in float64) of the final
  fields Ex..Hz of that build;
* ``fma_rx<n>_<output>``: the same traces from the default (-march=native) build;
* ``refout_rx<n>_<output>``: for the reference's own test models, the traces stored in their
  ``_ref.out`` files (read with ``gprmax_gb300.hdf5``), which older gprMax versions wrote;
* ``snap<n>_electric``, ``snap<n>_magnetic``, ``snap<n>_vti``: each snapshot's arrays and the
  bytes of the ``.vti`` file the reference writes from them;
* ``src<n>_whole``, ``src<n>_half``: the waveform tables of every voltage source, Hertzian
  dipole and magnetic dipole, in that order (the reference's ``calculate_waveform_values``);
* ``file_<name>``: the text of a file the input reads (an ``#excitation_file``), to be written
  beside the input before it is built;
* ``model_run``, ``model_end``: for the B-scan fixtures, the model run (of ``model_end``) that
  the reference's ``-n`` loop built and solved, its sources and receivers stepped by
  ``#src_steps`` / ``#rx_steps``.

The reference's own test models come from ``tests/models_basic`` (with ``_ref.out`` files) and
``tests/models_pmls`` (the PML slab-by-slab and thin-plate models, which have none).

It also copies one of those ``_ref.out`` files here as a fixture for the HDF5 reader.

Usage: python tests/golden/make_golden.py [--src PATH_TO_GPRMAX_CHECKOUT] [--only NAME ...]
"""
import argparse
import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, 'tests'))
sys.path.insert(0, os.path.join(ROOT, 'oracle'))
import build_ref  # noqa: E402

REFERENCE_MODELS = ['hertzian_dipole_fs', 'hertzian_dipole_dispersive', 'hertzian_dipole_hs',
                    'magnetic_dipole_fs', '2D_ExHyHz', '2D_EyHxHz', '2D_EzHxHy',
                    'cylinder_Ascan_2D']
# the reference's PML test models (tests/models_pmls; no stored outputs: golden from the run)
PML_MODELS = ['pml_off.in'] + ['pml_{0}/pml_{0}.in'.format(s) for s in
                               ('x0', 'y0', 'z0', 'xmax', 'ymax', 'zmax')] + \
    ['pml_3D_pec_plate/pml_3D_pec_plate_{}.in'.format(f) for f in
     ('CFS-PML', 'HORIPML-1', 'HORIPML-2', 'MRIPML-1', 'MRIPML-2')]
HDF5_FIXTURE = 'hertzian_dipole_dispersive_ref.out'

# every waveform type of the reference, two user waveforms from an excitation file (with a time
# column), delayed and cut-off sources, a magnetic dipole and a resistive voltage source
_TYPES = ['gaussian', 'gaussiandot', 'gaussiandotnorm', 'gaussiandotdot', 'gaussiandotdotnorm',
          'gaussianprime', 'gaussiandoubleprime', 'ricker', 'sine', 'contsine', 'impulse']
WAVEFORMS = '\n'.join(
    ['#title: every waveform type', '#domain: 0.020 0.020 0.020', '#dx_dy_dz: 0.001 0.001 0.001',
     '#time_window: 300', '#pml_cells: 0', '#excitation_file: exc.txt'] +
    ['#waveform: {} 1.3 2e9 w{}'.format(t, n) for n, t in enumerate(_TYPES)] +
    ['#hertzian_dipole: z {:.3f} 0.010 0.010 w{}'.format(0.004 + 0.001 * n, n)
     for n in range(len(_TYPES))] +
    ['#hertzian_dipole: x 0.010 0.006 0.010 u1 0 4e-10',
     '#hertzian_dipole: y 0.010 0.008 0.010 u2 1e-10 4e-10',
     '#hertzian_dipole: z 0.016 0.010 0.014 w7 1e-10 3e-10',
     '#magnetic_dipole: z 0.010 0.012 0.012 w8',
     '#voltage_source: y 0.012 0.014 0.010 50 w9',
     '#rx: 0.010 0.010 0.016', '#rx: 0.015 0.015 0.005']) + '\n'


# materials and geometry from an #include_file (with ## comments and blank lines, which the
# reference drops), placed between commands of the main file
INCLUDE = """#title: include file
#domain: 0.030 0.026 0.024
#dx_dy_dz: 0.001 0.001 0.001
#time_window: 90
#pml_cells: 5
#material: 3 0 1 0 base
#box: 0 0 0 0.030 0.026 0.010 base
#include_file: parts.txt
#waveform: ricker 1 3e9 w
#hertzian_dipole: z 0.015 0.013 0.016 w
#rx: 0.019 0.013 0.016
"""
INCLUDED = """## shapes for the include-file model

#material: 7 0.002 1 0 rock
#add_dispersion_debye: 1 5 2e-10 rock
#sphere: 0.012 0.012 0.008 0.004 rock
##   a comment between commands
#cylinder: 0.020 0.006 0.004 0.020 0.020 0.004 0.002 pec

#box: 0.004 0.016 0.002 0.010 0.022 0.012 rock n
"""


# a #python block that places the source and receiver from the model run number (run 2 of 3)
PYTHON_BSCAN = """#title: python B-scan
#domain: 0.030 0.028 0.024
#dx_dy_dz: 0.001 0.001 0.001
#time_window: 80
#pml_cells: 5
#material: 5 0.001 1 0 ground
#box: 0 0 0 0.030 0.028 0.012 ground
#cylinder: 0.015 0 0.007 0.015 0.028 0.007 0.002 pec
#waveform: ricker 1 4e9 w
#python:
x = 0.008 + 0.003 * (current_model_run - 1)
print('#hertzian_dipole: z {:g} 0.014 0.015 w'.format(x))
print('#rx: {:g} 0.014 0.015'.format(x + 0.004))
#end_python:
"""


def excitation_text():
    """An excitation file with a time column and two user waveforms (101 samples over 1 ns)."""
    t = np.linspace(0, 1e-9, 101)
    u1 = np.sin(2 * np.pi * 3e9 * t) * np.exp(-((t - 2e-10) / 8e-11) ** 2)
    u2 = np.where(t < 3e-10, t / 3e-10, 0.0)
    rows = ['time u1 u2'] + ['{!r} {!r} {!r}'.format(float(a), float(b), float(c))
                             for a, b, c in zip(t, u1, u2)]
    return '\n'.join(rows) + '\n'

CHILD = r'''
import sys, hashlib, numpy as np
sys.path.insert(0, {oracle!r})
import ref_harness as rh
G = rh.run_reference({inputfile!r}, src={src!r}, currentmodelrun={run}, modelend={end},
                     nthreads=8, variant={variant!r})
out = {{'iterations': G.iterations, 'dt': G.dt, 'nmat': len(G.materials),
        'ID_sha256': hashlib.sha256(np.ascontiguousarray(G.ID).tobytes()).hexdigest(),
        'coeffE': G.updatecoeffsE, 'coeffH': G.updatecoeffsH}}
if G.maxpoles:
    out['coeffD'] = G.updatecoeffsdispersive
for n, r in enumerate(G.rxs):
    for k, v in r.outputs.items():
        out['rx{{}}_{{}}'.format(n + 1, k)] = np.asarray(v, dtype=np.float32)
for n, s in enumerate(G.voltagesources + G.hertziandipoles + G.magneticdipoles):
    out['src{{}}_whole'.format(n + 1)] = np.asarray(s.waveformvalues_wholestep, dtype=np.float32)
    out['src{{}}_half'.format(n + 1)] = np.asarray(s.waveformvalues_halfstep, dtype=np.float32)
for n, t in enumerate(G.transmissionlines):
    for k in ('Vinc', 'Iinc', 'Vtotal', 'Itotal'):
        out['tl{{}}_{{}}'.format(n + 1, k)] = np.asarray(getattr(t, k), dtype=np.float32)
stats = []
for c in ('Ex', 'Ey', 'Ez', 'Hx', 'Hy', 'Hz'):
    a = np.ascontiguousarray(getattr(G, c))
    out['field_{{}}_sha256'.format(c)] = hashlib.sha256(a.tobytes()).hexdigest()
    stats.append([float(a.astype(np.float64).sum()), float(np.abs(a.astype(np.float64)).sum()),
                  float(np.abs(a).max())])
out['field_stats'] = np.array(stats)
for s, snap in enumerate(G.snapshots):
    out['snap{{}}_electric'.format(s)] = snap.electric
    out['snap{{}}_magnetic'.format(s)] = snap.magnetic


class _Bar:
    def update(self, n=1):
        pass


import os, tempfile
for s, snap in enumerate(G.snapshots):
    fd, path = tempfile.mkstemp(suffix='.vti')
    os.close(fd)
    snap.filename = path
    snap.write_vtk_imagedata(_Bar(), G)
    out['snap{{}}_vti'.format(s)] = np.fromfile(path, dtype=np.uint8)
    os.remove(path)
np.savez({dest!r}, **out)
'''


def run_child(inputfile, src, variant, dest, run=1, end=1):
    code = CHILD.format(oracle=os.path.join(ROOT, 'oracle'), inputfile=inputfile, src=src,
                        variant=variant, dest=dest, run=run, end=end)
    subprocess.run([sys.executable, '-c', code], check=True, cwd=ROOT)
    return dict(np.load(dest, allow_pickle=False))


def make(name, text, src, refout=None, run=1, end=1, files=None):
    with tempfile.TemporaryDirectory() as tmp:
        inputfile = os.path.join(tmp, name + '.in')
        with open(inputfile, 'w') as f:
            f.write(text)
        for fname, ftext in (files or {}).items():
            with open(os.path.join(tmp, fname), 'w') as f:
                f.write(ftext)
        exact = run_child(inputfile, src, 'nofma', os.path.join(tmp, 'exact.npz'), run, end)
        fma = run_child(inputfile, src, '', os.path.join(tmp, 'fma.npz'), run, end)
    out = dict(exact)
    out['input'] = np.array(text)
    if end > 1:
        out['model_run'] = np.int64(run)
        out['model_end'] = np.int64(end)
    for fname, ftext in (files or {}).items():
        out['file_' + fname] = np.array(ftext)
    for k, v in fma.items():
        if k.startswith('rx'):
            out['fma_' + k] = v
    if refout:
        from gprmax_gb300.outputs import read_outputfile
        rxs, _ = read_outputfile(refout)
        for rx, comps in rxs.items():
            for comp, v in comps.items():
                out['refout_{}_{}'.format(rx, comp)] = v.astype(np.float32)
    np.savez_compressed(os.path.join(HERE, name + '.npz'), **out)
    print('wrote', name, sorted(k for k in out if not k.startswith(('rx', 'fma', 'refout')))[:6])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--src', default=build_ref.SOURCE)
    ap.add_argument('--only', nargs='*')
    a = ap.parse_args()
    from models import MODELS
    from gprmax_gb300.workloads import bscan_2d_input
    todo = {n: (t, None) for n, t in MODELS.items()}
    # the first and last model runs of a 6-trace 2D B-scan (antenna pair stepped per run)
    bscan = ''.join(bscan_2d_input())
    runs = {'bscan2d_run1': 1, 'bscan2d_run6': 6}
    for n in REFERENCE_MODELS:
        d = os.path.join(a.src, 'tests', 'models_basic', n)
        with open(os.path.join(d, n + '.in')) as f:
            text = f.read()
        ref = os.path.join(d, n + '_ref.out')
        todo['ref_' + n] = (text, ref if os.path.exists(ref) else None)
    for rel in PML_MODELS:
        with open(os.path.join(a.src, 'tests', 'models_pmls', rel)) as f:
            text = f.read()
        todo['ref_' + os.path.splitext(os.path.basename(rel))[0]] = (text, None)
    for name, (text, ref) in sorted(todo.items()):
        if a.only and name not in a.only:
            continue
        make(name, text, a.src, ref)
    for name, run in runs.items():
        if a.only and name not in a.only:
            continue
        make(name, bscan, a.src, None, run, 6)
    if not a.only or 'waveforms' in a.only:
        make('waveforms', WAVEFORMS, a.src, files={'exc.txt': excitation_text()})
    if not a.only or 'include' in a.only:
        make('include', INCLUDE, a.src, files={'parts.txt': INCLUDED})
    if not a.only or 'python_run2' in a.only:
        make('python_run2', PYTHON_BSCAN, a.src, None, 2, 3)
    # the reference's own B-scan example (user_models), first and last of its 60 model runs
    with open(os.path.join(a.src, 'user_models', 'cylinder_Bscan_2D.in')) as f:
        example = f.read()
    for run in (1, 60):
        name = 'ref_cylinder_Bscan_2D_run{}'.format(run)
        if not a.only or name in a.only:
            make(name, example, a.src, None, run, 60)
    shutil.copy(os.path.join(a.src, 'tests', 'models_basic', 'hertzian_dipole_dispersive',
                             HDF5_FIXTURE), os.path.join(HERE, HDF5_FIXTURE))
    with open(os.path.join(HERE, 'README.txt'), 'w') as f:
        f.write('Golden fixtures generated by make_golden.py from gprMax v3.1.7 itself; see its '
                'docstring for the content of each file.\n')


if __name__ == '__main__':
    main()
