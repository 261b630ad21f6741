"""The reference's own compiled CPU kernels driven by the ``solve_cpu`` loop (test and baseline
infrastructure only; used by ``bench.py --impl reference`` and the CPU-baseline leg).

The kernels are gprMax v3.1.7's Cython/OpenMP modules compiled by ``oracle/build_ref.py`` into
``oracle/_ref`` (``fields_updates_ext``, ``pml_updates_{electric,magnetic}_{HORIPML,MRIPML}_ext``),
called with the reference's own signatures exactly as ``solve_cpu`` calls them
(``gprMax/model_build_run.py:424-470``; PML dispatch by name as ``gprMax/pml.py:276-296``).
The model arrays come from the front-end, which builds them identically to the reference.
"""
import os

from oracle import OracleSolver

HERE = os.path.dirname(os.path.abspath(__file__))
REF_BUILD = os.path.join(HERE, '_ref')


def available(variant=''):
    """True when the compiled reference kernels (``variant`` '' = the reference's own flags,
    'nofma' = the same C without floating-point contraction) can be imported."""
    try:
        _modules(variant)
        return True
    except Exception:
        return False


_loaded = {}


def _load_ext(variant, mod):
    """Import one compiled kernel module of a build variant from its file, under a package
    name of its own, so the two variants can be loaded side by side in one process."""
    import glob
    import importlib.util
    key = (variant, mod)
    if key not in _loaded:
        parts = mod.split('.')
        base = os.path.join(REF_BUILD, variant) if variant else REF_BUILD
        found = glob.glob(os.path.join(base, *parts[:-1], parts[-1] + '.*.so'))
        if not found:
            raise ImportError('reference kernel {} ({}) not built'.format(mod, variant or 'stock'))
        name = 'gbref_{}.{}'.format(variant or 'stock', parts[-1])
        spec = importlib.util.spec_from_file_location(name, found[0])
        m = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(m)
        _loaded[key] = m
    return _loaded[key]


def _modules(variant=''):
    fu = _load_ext(variant, 'gprMax.fields_updates_ext')
    pml = {}
    for kind in ('electric', 'magnetic'):
        for form in ('HORIPML', 'MRIPML'):
            pml[(kind, form)] = _load_ext(
                variant, 'gprMax.pml_updates.pml_updates_{}_{}_ext'.format(kind, form))
    return fu, pml


class RefCPUSolver(OracleSolver):
    """``solve_cpu`` over the reference's compiled kernels with ``nthreads`` OpenMP threads
    (``variant`` 'nofma': the build without floating-point contraction)."""

    def __init__(self, G, nthreads=None, variant=''):
        super().__init__(G)
        self.nthreads = nthreads or os.cpu_count() or 1
        self.fu, pml = _modules(variant)
        form = G.pmlformulation
        self.pml_e = [getattr(pml[('electric', form)], 'order{}_{}'.format(self.order, s.pml.direction))
                      for s in self.slabs]
        self.pml_h = [getattr(pml[('magnetic', form)], 'order{}_{}'.format(self.order, s.pml.direction))
                      for s in self.slabs]

    def step(self):
        G, fu, it, nt = self.G, self.fu, self.it, self.nthreads
        nx, ny, nz = G.nx, G.ny, G.nz
        Ex, Ey, Ez = self.E
        Hx, Hy, Hz = self.H
        self._store_outputs(it)
        for s, snap in enumerate(G.snapshots):
            if snap.time == it + 1:
                self._store_snapshot(s, snap)
        fu.update_magnetic(nx, ny, nz, nt, self.cH, self.ID, Ex, Ey, Ez, Hx, Hy, Hz)
        for st, f in zip(self.slabs, self.pml_h):
            p, r = st.pml, st.rows
            f(p.xs, p.xf, p.ys, p.yf, p.zs, p.zf, nt, self.cH, self.ID, Ex, Ey, Ez, Hx, Hy, Hz,
              st.HPhi1, st.HPhi2, r['HRA'], r['HRB'], r['HRE'], r['HRF'], p.d)
        self._sources_magnetic(it)
        if self.P == 0:
            fu.update_electric(nx, ny, nz, nt, self.cE, self.ID, Ex, Ey, Ez, Hx, Hy, Hz)
        elif self.P == 1:
            fu.update_electric_dispersive_1pole_A(nx, ny, nz, nt, self.cE, self.cD, self.ID,
                                                  *self.T, Ex, Ey, Ez, Hx, Hy, Hz)
        else:
            fu.update_electric_dispersive_multipole_A(nx, ny, nz, nt, self.P, self.cE, self.cD,
                                                      self.ID, *self.T, Ex, Ey, Ez, Hx, Hy, Hz)
        for st, f in zip(self.slabs, self.pml_e):
            p, r = st.pml, st.rows
            f(p.xs, p.xf, p.ys, p.yf, p.zs, p.zf, nt, self.cE, self.ID, Ex, Ey, Ez, Hx, Hy, Hz,
              st.EPhi1, st.EPhi2, r['ERA'], r['ERB'], r['ERE'], r['ERF'], p.d)
        self._sources_electric(it)
        if self.P == 1:
            fu.update_electric_dispersive_1pole_B(nx, ny, nz, nt, self.cD, self.ID, *self.T, Ex, Ey, Ez)
        elif self.P > 1:
            fu.update_electric_dispersive_multipole_B(nx, ny, nz, nt, self.P, self.cD, self.ID,
                                                      *self.T, Ex, Ey, Ez)
        self.it += 1


def make_solver(G, nthreads=None):
    """The reference-kernel solver when available, else the oracle port; returns (solver, kind)."""
    if available():
        return RefCPUSolver(G, nthreads), 'reference'
    os.environ.setdefault('OMP_NUM_THREADS', str(nthreads or os.cpu_count() or 1))
    return OracleSolver(G), 'port'
