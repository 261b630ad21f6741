"""Drive the reference gprMax v3.1.7 solver in-process (test infrastructure only).

This module is part of the ORACLE. It is used by ``tests/golden/make_golden.py`` to produce
golden vectors from the reference itself, and by nothing in the product path.

It needs the reference Python sources (a gprMax v3.1.7 checkout) and the kernels compiled by
``oracle/build_ref.py``. Three packages the reference imports are absent here and are replaced
by inert stand-ins: ``colorama`` (terminal colours), ``terminaltables`` (materials table
printing) and ``h5py`` (only used by the output writer, which is intercepted).

``run_reference(inputfile)`` follows ``gprMax/gprMax.py:api -> run_std_sim -> run_model``
(``gprMax/model_build_run.py:84-405``) for one model and returns the built grid ``G`` captured
where ``run_model`` calls ``write_hdf5_outputfile`` (``model_build_run.py:376``), i.e. after
``solve_cpu`` (``model_build_run.py:408-474``) finished.
"""
import contextlib
import io
import os
import sys
import types

HERE = os.path.dirname(os.path.abspath(__file__))
REF_BUILD = os.path.join(HERE, '_ref')


def _install_shims():
    if 'colorama' not in sys.modules:
        m = types.ModuleType('colorama')
        m.init = lambda *a, **k: None

        class _Blank:
            def __getattr__(self, name):
                return ''
        m.Fore = _Blank()
        m.Style = _Blank()
        sys.modules['colorama'] = m
    if 'terminaltables' not in sys.modules:
        m = types.ModuleType('terminaltables')

        class AsciiTable:
            def __init__(self, data):
                self.data = data
                self.outer_border = True
                self.justify_columns = {}

            @property
            def table(self):
                return '\n'.join(' '.join(str(c) for c in row) for row in self.data)
        m.AsciiTable = AsciiTable
        sys.modules['terminaltables'] = m
    if 'h5py' not in sys.modules:
        sys.modules['h5py'] = types.ModuleType('h5py')


def load(src=None, variant=''):
    """Import the reference's model driver; returns the ``gprMax.model_build_run`` module.
    ``variant='nofma'`` selects the kernels compiled without floating-point contraction."""
    global REF_BUILD
    if src is None:
        import build_ref
        src = build_ref.SOURCE
    if variant:
        REF_BUILD = os.path.join(HERE, '_ref', variant)
    if not os.path.isdir(os.path.join(REF_BUILD, 'gprMax')):
        raise RuntimeError('reference kernels not built: run python oracle/build_ref.py')
    if not os.path.isdir(os.path.join(src, 'gprMax')):
        raise RuntimeError('reference sources not found at ' + src)
    _install_shims()
    if REF_BUILD not in sys.path:
        sys.path.insert(0, REF_BUILD)
    import gprMax  # noqa: F401  (the oracle/_ref package shim)
    import gprMax.model_build_run as mbr
    return mbr


class _Args:
    def __init__(self):
        self.n = 1
        self.task = None
        self.restart = None
        self.mpi = False
        self.mpi_no_spawn = False
        self.mpicomm = None
        self.gpu = None
        self.benchmark = False
        self.geometry_only = False
        self.geometry_fixed = False
        self.write_processed = False
        self.opt_taguchi = False


def run_reference(inputfile, src=None, currentmodelrun=1, modelend=1,
                  nthreads=None, quiet=True, variant=''):
    """Run one model through the reference and return its grid object after the solve."""
    if src is None:
        import build_ref
        src = build_ref.SOURCE
    mbr = load(src, variant)
    from gprMax.constants import c, e0, m0, z0
    from gprMax.materials import Material
    Material.maxpoles = 0   # class attribute; reset so models do not leak into each other
    if nthreads is not None:
        os.environ['OMP_NUM_THREADS'] = str(nthreads)
    captured = {}

    def capture(outputfile, G):
        captured['G'] = G
        captured['outputfile'] = outputfile
    mbr.write_hdf5_outputfile = capture
    # Snapshot .vti files are not needed; keep their stored arrays
    args = _Args()
    args.inputfile = inputfile
    usernamespace = {'c': c, 'e0': e0, 'm0': m0, 'z0': z0, 'number_model_runs': modelend,
                     'inputfile': os.path.abspath(inputfile)}
    sink = io.StringIO()
    with open(inputfile) as f:
        ctx = contextlib.redirect_stdout(sink) if quiet else contextlib.nullcontext()
        with ctx:
            G = None
            orig_del = None
            # run_model deletes its global G at the end; the capture keeps a reference
            tsolve = mbr.run_model(args, currentmodelrun, modelend, modelend, f, usernamespace)
    G = captured['G']
    G.tsolve = tsolve
    G.maxpoles = Material.maxpoles
    return G
