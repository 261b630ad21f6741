"""Build recipe for the reference's own Cython/OpenMP solver kernels (test infrastructure).

This script is part of the ORACLE, i.e. test and baseline infrastructure. Nothing in the
product path (``gprmax_gb300``) imports or calls what it builds.

Two stages, both writing only under ``oracle/_ref/`` (git-ignored):

1. ``cythonize`` (needs Cython and the gprMax v3.1.7 sources): translates the reference's
   ``.pyx`` files (``gprMax/fields_updates_ext.pyx``, ``gprMax/pml_updates/*_ext.pyx`` and the
   build-time modules) into C under ``oracle/_ref/csrc/`` with the compiler directives of the
   reference's ``setup.py:208-215`` (boundscheck/wraparound/initializedcheck off).
2. ``compile`` (needs gcc, Python headers and numpy headers only): compiles every generated C
   file into an extension module under ``oracle/_ref/gprMax/`` with the reference's Linux
   flags (``setup.py:176-181``: ``-O3 -w -fopenmp -march=native``; ``-march=native`` is dropped
   when the compiler rejects it).

Stage 2 also runs where the sources are absent (the generated C travels with the repository
copy), so the reference kernels can be timed as the CPU baseline on any host.

``oracle/_ref/gprMax/__init__.py`` extends the package ``__path__`` with the reference source
directory when it exists, so ``import gprMax.grid`` etc. resolve to the reference's own
Python modules there while the compiled kernels come from ``oracle/_ref``.

A second variant, ``--variant nofma`` (output ``oracle/_ref/nofma/gprMax``), compiles the same
C with ``-ffp-contract=off`` added: every product and sum rounded as written. With it the
reference's results are reproducible bit for bit on any host, and they are what the golden
fixtures under ``tests/golden`` record.

Usage: python oracle/build_ref.py [--src PATH_TO_GPRMAX_CHECKOUT] [--jobs N] [--variant nofma]
"""
import argparse
import os
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
# where this recipe reads the reference checkout from: $GPRMAX_REFERENCE, else the read-only
# copy this build environment mounts; every other oracle script takes the location from here
SOURCE = os.environ.get('GPRMAX_REFERENCE', '/root/reference')
OUT = os.path.join(HERE, '_ref')
CSRC = os.path.join(OUT, 'csrc')
PKG = os.path.join(OUT, 'gprMax')

# module name -> path of the .pyx relative to the checkout root
KERNEL_MODULES = [
    'gprMax.fields_updates_ext',
    'gprMax.pml_updates.pml_updates_electric_HORIPML_ext',
    'gprMax.pml_updates.pml_updates_magnetic_HORIPML_ext',
    'gprMax.pml_updates.pml_updates_electric_MRIPML_ext',
    'gprMax.pml_updates.pml_updates_magnetic_MRIPML_ext',
]
BUILD_MODULES = [
    'gprMax.yee_cell_setget_rigid_ext',
    'gprMax.yee_cell_build_ext',
    'gprMax.geometry_primitives_ext',
    'gprMax.snapshots_ext',
    'gprMax.fractals_generate_ext',
    'gprMax.geometry_outputs_ext',
]
ALL_MODULES = KERNEL_MODULES + BUILD_MODULES

INIT_TEMPLATE = '''"""Package shim for the reference kernels compiled by oracle/build_ref.py (test infrastructure)."""
import os as _os
_src = {src!r}
if _src and _os.path.isdir(_src):
    __path__.append(_src)
'''


def _cythonize(mod, src):
    import Cython  # noqa: F401  (fail early with a clear message)
    rel = mod.replace('.', os.sep) + '.pyx'
    pyx = os.path.join(src, rel)
    out = os.path.join(CSRC, mod + '.c')
    directives = 'boundscheck=False,wraparound=False,initializedcheck=False,embedsignature=True,language_level=3'
    cmd = [sys.executable, '-m', 'cython', '-3', '--directive', directives, '-I', src,
           '--module-name', mod, '-o', out, pyx]
    subprocess.run(cmd, check=True, cwd=src)
    return out


def _march_ok(cc):
    try:
        r = subprocess.run([cc, '-march=native', '-x', 'c', '-c', '-o', os.devnull, '-'],
                           input=b'int x;', capture_output=True)
        return r.returncode == 0
    except OSError:
        return False


def _compile(mod, cc, march, variant=''):
    import numpy as np
    c_file = os.path.join(CSRC, mod + '.c')
    parts = mod.split('.')
    dest_dir = os.path.join(OUT, variant, *parts[:-1]) if variant else os.path.join(OUT, *parts[:-1])
    os.makedirs(dest_dir, exist_ok=True)
    so = os.path.join(dest_dir, parts[-1] + sysconfig.get_config_var('EXT_SUFFIX'))
    if os.path.exists(so) and os.path.getmtime(so) >= os.path.getmtime(c_file):
        return so
    flags = ['-O3', '-w', '-fopenmp', '-fPIC', '-shared']
    if march:
        flags.append('-march=native')
    if variant == 'nofma':
        flags.append('-ffp-contract=off')
    cmd = [cc] + flags + ['-I', sysconfig.get_paths()['include'], '-I', np.get_include(),
                          c_file, '-o', so + '.tmp', '-fopenmp']
    subprocess.run(cmd, check=True)
    os.replace(so + '.tmp', so)
    return so


def build(src=None, jobs=8, modules=None, quiet=False, variant=''):
    """Cythonize (when ``src`` exists and Cython is importable) then compile into oracle/_ref
    (``oracle/_ref/nofma`` for the no-contraction variant)."""
    modules = modules or ALL_MODULES
    os.makedirs(CSRC, exist_ok=True)
    os.makedirs(os.path.join(PKG, 'pml_updates'), exist_ok=True)
    have_src = bool(src) and os.path.isdir(os.path.join(src, 'gprMax'))
    if have_src:
        try:
            import Cython  # noqa: F401
        except ImportError:
            have_src = False
    if have_src:
        todo = []
        for mod in modules:
            out = os.path.join(CSRC, mod + '.c')
            pyx = os.path.join(src, mod.replace('.', os.sep) + '.pyx')
            if not os.path.exists(out) or os.path.getmtime(out) < os.path.getmtime(pyx):
                todo.append(mod)
        with ThreadPoolExecutor(jobs) as ex:
            list(ex.map(lambda m: _cythonize(m, src), todo))
    available = [m for m in modules if os.path.exists(os.path.join(CSRC, m + '.c'))]
    if not available:
        raise FileNotFoundError('no generated reference C sources under ' + CSRC)
    cc = os.environ.get('CC', 'gcc')
    march = _march_ok(cc)
    with ThreadPoolExecutor(jobs) as ex:
        sos = list(ex.map(lambda m: _compile(m, cc, march, variant), available))
    pkg = os.path.join(OUT, variant, 'gprMax') if variant else PKG
    os.makedirs(os.path.join(pkg, 'pml_updates'), exist_ok=True)
    with open(os.path.join(pkg, '__init__.py'), 'w') as f:
        f.write(INIT_TEMPLATE.format(src=os.path.join(src, 'gprMax') if have_src else ''))
    with open(os.path.join(pkg, 'pml_updates', '__init__.py'), 'w') as f:
        f.write(INIT_TEMPLATE.format(
            src=os.path.join(src, 'gprMax', 'pml_updates') if have_src else ''))
    if not quiet:
        print('reference kernels built: %d modules (march=native: %s)' % (len(sos), march))
    return sos


if __name__ == '__main__':
    ap = argparse.ArgumentParser()
    ap.add_argument('--src', default=SOURCE)
    ap.add_argument('--jobs', type=int, default=os.cpu_count() or 4)
    ap.add_argument('--kernels-only', action='store_true')
    ap.add_argument('--variant', choices=['', 'nofma'], default='')
    a = ap.parse_args()
    build(a.src, a.jobs, KERNEL_MODULES if a.kernels_only else ALL_MODULES, variant=a.variant)
