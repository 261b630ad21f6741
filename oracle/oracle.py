"""ORACLE (test infrastructure only): CPU restatement of gprMax v3.1.7's time loop.

Used by ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg as the
checker of the GPU solver; the product path (``gprmax_gb300``) never imports it.

``OracleSolver(G)`` runs the iteration loop of ``solve_cpu`` (``gprMax/model_build_run.py:
408-474``) on a model built by the front-end: receiver store (``fields_outputs.py:40-67``),
snapshots (``snapshots.py:87-130``), H update, PML H in slab order, magnetic dipoles, E update
(or dispersive part A), PML E, voltage sources and Hertzian dipoles, dispersive part B. The
field kernels are the C restatements in ``fdtd_oracle.c`` (built with ``-ffp-contract=off``);
the per-source updates are numpy fp32 scalar arithmetic, as in ``gprMax/sources.py``.

Parity of this oracle with the reference itself is pinned by ``tests/golden`` (fixtures
produced by running the reference's own Cython solver on the same inputs).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, 'fdtd_oracle.c')
LIB = os.path.join(HERE, '_build', 'liboracle.so')
LIB64 = os.path.join(HERE, '_build', 'liboracle64.so')   # the same loops in fp64

_libs = {}


def build(force=False):
    """Compile ``fdtd_oracle.c`` into ``oracle/_build/liboracle.so`` (fp32) and
    ``liboracle64.so`` (fp64, ``-DORACLE_F64``)."""
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    cc = os.environ.get('CC', 'gcc')
    for out, extra in ((LIB, []), (LIB64, ['-DORACLE_F64'])):
        if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(SRC):
            continue
        cmd = [cc, '-O2', '-fopenmp', '-ffp-contract=off', '-fPIC', '-shared'] + extra + [
            SRC, '-o', out + '.tmp']
        subprocess.run(cmd, check=True)
        os.replace(out + '.tmp', out)
    return LIB


def lib(fp64=False):
    if fp64 not in _libs:
        build()
        L = ctypes.CDLL(LIB64 if fp64 else LIB)
        args = [ctypes.c_int] * 12 + [ctypes.c_void_p] * 16 + [
            ctypes.c_double if fp64 else ctypes.c_float]
        L.oracle_pml_electric.argtypes = args
        L.oracle_pml_magnetic.argtypes = args
        _libs[fp64] = L
    return _libs[fp64]


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


_DIRS = {'xminus': 0, 'yminus': 1, 'zminus': 2, 'xplus': 3, 'yplus': 4, 'zplus': 5}


class _SlabState:
    """Phi arrays of one slab in the reference's shapes (``gprMax/pml.py:202-219``)."""

    def __init__(self, pml, order, ft=np.float32):
        nx, ny, nz = pml.nx, pml.ny, pml.nz
        a = pml.direction[0]
        if a == 'x':
            shapes = [(nx + 1, ny, nz + 1), (nx + 1, ny + 1, nz), (nx, ny + 1, nz), (nx, ny, nz + 1)]
        elif a == 'y':
            shapes = [(nx, ny + 1, nz + 1), (nx + 1, ny + 1, nz), (nx + 1, ny, nz), (nx, ny, nz + 1)]
        else:
            shapes = [(nx, ny + 1, nz + 1), (nx + 1, ny, nz + 1), (nx + 1, ny, nz), (nx, ny + 1, nz)]
        self.EPhi1, self.EPhi2, self.HPhi1, self.HPhi2 = (
            np.zeros((order,) + s, dtype=ft) for s in shapes)
        self.dims = [np.array(s, dtype=np.int32) for s in shapes]
        self.pml = pml
        self.rows = {n: np.ascontiguousarray(getattr(pml, n), dtype=np.float32)
                     for n in ('ERA', 'ERB', 'ERE', 'ERF', 'HRA', 'HRB', 'HRE', 'HRF')}


def fp64_tables(G):
    """Material coefficient tables of ``G`` computed and kept in fp64: ``updatecoeffsE/H``
    float64 [nmat][5] and ``updatecoeffsdispersive`` complex128 [nmat][3P], the formulas of
    ``gprMax/materials.py:69-143, 204-208`` with no rounding to fp32 (what the reference computes
    when built with double ``floattype``). The model's own fp32 tables are left untouched."""
    import copy
    from gprmax_gb300 import materials as M
    nmat = len(G.materials)
    cE = np.zeros((nmat, 5), dtype=np.float64)
    cH = np.zeros((nmat, 5), dtype=np.float64)
    cD = np.zeros((nmat, 3 * G.maxpoles), dtype=np.complex128) if G.maxpoles else None
    keep = M.complextype
    M.complextype = np.complex128
    try:
        for m0 in G.materials:
            m = copy.copy(m0)
            m.calculate_update_coeffsE(G)
            m.calculate_update_coeffsH(G)
            cE[m.numID] = (m.CA, m.CBx, m.CBy, m.CBz, m.srce)
            cH[m.numID] = (m.DA, m.DBx, m.DBy, m.DBz, m.srcm)
            if G.maxpoles:
                for pole in range(G.maxpoles):
                    cD[m.numID, 3 * pole:3 * pole + 3] = (M.e0 * m.eqt2[pole], m.eqt[pole], m.zt[pole])
    finally:
        M.complextype = keep
    return cE, cH, cD


def fp64_pml_rows(G, pml):
    """A slab's RA..RF rows for E and H computed in fp64 (``gprMax/pml.py:221-274`` with a
    double ``floattype``), from the same sigma max the model's fp32 rows used."""
    import copy
    from gprmax_gb300 import pml as Pm
    q = copy.copy(pml)
    keep = Pm.floattype
    Pm.floattype = np.float64
    try:
        # sigma max is already set on the model's CFS terms, so it is reused as it is
        q.calculate_update_coeffs(0.0, 0.0, G)
    finally:
        Pm.floattype = keep
    return {n: np.ascontiguousarray(getattr(q, n), dtype=np.float64)
            for n in ('ERA', 'ERB', 'ERE', 'ERF', 'HRA', 'HRB', 'HRE', 'HRF')}


def fp64_waves(G, src):
    """A source's waveform at whole and half steps in fp64 (``gprMax/sources.py:47-68`` without
    the fp32 tables)."""
    waveform = next(x for x in G.waveforms if x.ID == src.waveformID)
    time = G.dt * np.arange(G.iterations, dtype=np.float64)
    active = (time >= src.start) & (time <= src.stop)
    t = time[active] - src.start
    whole = np.zeros(G.iterations)
    half = np.zeros(G.iterations)
    if t.size:
        whole[active] = waveform.values(t, G.dt)
        half[active] = waveform.values(t + 0.5 * G.dt, G.dt)
    return whole, half


class OracleSolver:
    """The reference's CPU time loop over a model built by the front-end.

    ``fp64=True`` runs the same loop in double precision with every table (material and PML
    coefficients, waveforms) computed and kept in fp64: the fp64 run of the same grid against
    which the fp32 solvers' error is stated. Transmission lines are not supported there."""

    def __init__(self, G, fp64=False):
        self.G = G
        self.fp64 = fp64
        self.L = lib(fp64)
        ft = np.float64 if fp64 else np.float32
        ct = np.complex128 if fp64 else np.complex64
        self.ft = ft
        shape = (G.nx + 1, G.ny + 1, G.nz + 1)
        self.E = [np.zeros(shape, dtype=ft) for _ in range(3)]
        self.H = [np.zeros(shape, dtype=ft) for _ in range(3)]
        self.ID = np.ascontiguousarray(G.ID, dtype=np.uint32)
        self.P = G.maxpoles
        if fp64:
            self.cE, self.cH, cD = fp64_tables(G)
        else:
            self.cE = np.ascontiguousarray(G.updatecoeffsE, dtype=np.float32)
            self.cH = np.ascontiguousarray(G.updatecoeffsH, dtype=np.float32)
            cD = G.updatecoeffsdispersive
        if self.P:
            self.cD = np.ascontiguousarray(cD, dtype=ct)
            self.T = [np.zeros((self.P,) + shape, dtype=ct) for _ in range(3)]
        self.order = max(len(G.cfs), 1)
        self.form = 0 if G.pmlformulation == 'HORIPML' else 1
        self.slabs = [_SlabState(p, self.order, ft) for p in G.pmls]
        if fp64:
            if G.transmissionlines:
                raise ValueError('the fp64 oracle does not model transmission lines')
            for st in self.slabs:
                st.rows = fp64_pml_rows(G, st.pml)
            self.waves = {id(s): fp64_waves(G, s) for s in
                          list(G.hertziandipoles) + list(G.voltagesources) + list(G.magneticdipoles)}
        self.rx = np.zeros((9, G.iterations, max(len(G.rxs), 1)), dtype=ft)
        self.snaps = {}
        self.it = 0
        # transmission lines advance on copies, so the model's own state stays untouched
        import copy
        self.tls = [copy.deepcopy(t) for t in G.transmissionlines]

    # -- receivers and snapshots -------------------------------------------------------
    def _store_outputs(self, it):
        G = self.G
        Hx, Hy, Hz = self.H
        for tl in self.tls:
            tl.Vtotal[it] = tl.voltage[tl.antpos]
            tl.Itotal[it] = tl.current[tl.antpos]
        for n, r in enumerate(G.rxs):
            x, y, z = r.xcoord, r.ycoord, r.zcoord
            for c in range(3):
                self.rx[c, it, n] = self.E[c][x, y, z]
                self.rx[3 + c, it, n] = self.H[c][x, y, z]
            # grid.py:413-461 (fp32 arithmetic with fp32-cast cell sizes)
            f = self.ft
            self.rx[6, it, n] = 0 if (y == 0 or z == 0) else (
                f(G.dy) * (Hy[x, y, z - 1] - Hy[x, y, z]) + f(G.dz) * (Hz[x, y, z] - Hz[x, y - 1, z]))
            self.rx[7, it, n] = 0 if (x == 0 or z == 0) else (
                f(G.dx) * (Hx[x, y, z] - Hx[x, y, z - 1]) + f(G.dz) * (Hz[x - 1, y, z] - Hz[x, y, z]))
            self.rx[8, it, n] = 0 if (x == 0 or y == 0) else (
                f(G.dx) * (Hx[x, y - 1, z] - Hx[x, y, z]) + f(G.dy) * (Hy[x, y, z] - Hy[x - 1, y, z]))

    def _store_snapshot(self, s, snap):
        sx = slice(snap.xs, snap.xf + snap.dx, snap.dx)
        sy = slice(snap.ys, snap.yf + snap.dy, snap.dy)
        sz = slice(snap.zs, snap.zf + snap.dz, snap.dz)
        Ex, Ey, Ez = (a[sx, sy, sz] for a in self.E)
        Hx, Hy, Hz = (a[sx, sy, sz] for a in self.H)
        nx, ny, nz = snap.nx, snap.ny, snap.nz
        out = np.zeros((6, nx, ny, nz), dtype=np.float32)
        out[0] = (Ex[:nx, :ny, :nz] + Ex[:nx, 1:ny + 1, :nz] + Ex[:nx, :ny, 1:nz + 1] + Ex[:nx, 1:ny + 1, 1:nz + 1]) / np.float32(4)
        out[1] = (Ey[:nx, :ny, :nz] + Ey[1:nx + 1, :ny, :nz] + Ey[:nx, :ny, 1:nz + 1] + Ey[1:nx + 1, :ny, 1:nz + 1]) / np.float32(4)
        out[2] = (Ez[:nx, :ny, :nz] + Ez[1:nx + 1, :ny, :nz] + Ez[:nx, 1:ny + 1, :nz] + Ez[1:nx + 1, 1:ny + 1, :nz]) / np.float32(4)
        out[3] = (Hx[:nx, :ny, :nz] + Hx[1:nx + 1, :ny, :nz]) / np.float32(2)
        out[4] = (Hy[:nx, :ny, :nz] + Hy[:nx, 1:ny + 1, :nz]) / np.float32(2)
        out[5] = (Hz[:nx, :ny, :nz] + Hz[:nx, :ny, 1:nz + 1]) / np.float32(2)
        self.snaps[s] = out

    # -- sources (gprMax/sources.py, numpy fp32 scalar arithmetic) ----------------------
    def _tl_current(self, tl):
        """The current around a transmission line's edge (grid.py Ix/Iy/Iz, fp32)."""
        G = self.G
        Hx, Hy, Hz = self.H
        x, y, z = tl.xcoord, tl.ycoord, tl.zcoord
        f = np.float32
        if tl.polarisation == 'x':
            return 0 if (y == 0 or z == 0) else (
                f(G.dy) * (Hy[x, y, z - 1] - Hy[x, y, z]) + f(G.dz) * (Hz[x, y, z] - Hz[x, y - 1, z]))
        if tl.polarisation == 'y':
            return 0 if (x == 0 or z == 0) else (
                f(G.dx) * (Hx[x, y, z] - Hx[x, y, z - 1]) + f(G.dz) * (Hz[x - 1, y, z] - Hz[x, y, z]))
        return 0 if (x == 0 or y == 0) else (
            f(G.dx) * (Hx[x, y - 1, z] - Hx[x, y, z]) + f(G.dy) * (Hy[x, y, z] - Hy[x - 1, y, z]))

    def _whole(self, src):
        return self.waves[id(src)][0] if self.fp64 else src.waveformvalues_wholestep

    def _half(self, src):
        return self.waves[id(src)][1] if self.fp64 else src.waveformvalues_halfstep

    def _sources_magnetic(self, it):
        """Transmission lines, then magnetic dipoles (model_build_run.py:440-442)."""
        G = self.G
        for tl in self.tls:
            if it * G.dt >= tl.start and it * G.dt <= tl.stop:
                tl.update_current(it, G)
                tl.current[tl.antpos] = self._tl_current(tl)
        for m in G.magneticdipoles:
            if it * G.dt >= m.start and it * G.dt <= m.stop:
                c = 'xyz'.index(m.polarisation)
                i, j, k = m.xcoord, m.ycoord, m.zcoord
                self.H[c][i, j, k] -= (self.cH[self.ID[3 + c, i, j, k], 4]
                                       * self._half(m)[it] * (1 / (G.dx * G.dy * G.dz)))

    def _sources_electric(self, it):
        G = self.G
        for v in G.voltagesources:
            if it * G.dt >= v.start and it * G.dt <= v.stop:
                c = 'xyz'.index(v.polarisation)
                i, j, k = v.xcoord, v.ycoord, v.zcoord
                if v.resistance != 0:
                    other = {'x': G.dy * G.dz, 'y': G.dx * G.dz, 'z': G.dx * G.dy}[v.polarisation]
                    self.E[c][i, j, k] -= (self.cE[self.ID[c, i, j, k], 4]
                                           * self._whole(v)[it] * (1 / (v.resistance * other)))
                else:
                    d = {'x': G.dx, 'y': G.dy, 'z': G.dz}[v.polarisation]
                    self.E[c][i, j, k] = -self._half(v)[it] / d
        for tl in self.tls:
            if it * G.dt >= tl.start and it * G.dt <= tl.stop:
                c = 'xyz'.index(tl.polarisation)
                d = {'x': G.dx, 'y': G.dy, 'z': G.dz}[tl.polarisation]
                tl.update_voltage(it, G)
                self.E[c][tl.xcoord, tl.ycoord, tl.zcoord] = - tl.voltage[tl.antpos] / d
        for h in G.hertziandipoles:
            if it * G.dt >= h.start and it * G.dt <= h.stop:
                c = 'xyz'.index(h.polarisation)
                i, j, k = h.xcoord, h.ycoord, h.zcoord
                self.E[c][i, j, k] -= (self.cE[self.ID[c, i, j, k], 4] * self._whole(h)[it]
                                       * h.dl * (1 / (G.dx * G.dy * G.dz)))

    # -- the loop -------------------------------------------------------------------------
    def _d(self, d):
        return ctypes.c_double(d) if self.fp64 else ctypes.c_float(d)

    def step(self):
        G, L, it = self.G, self.L, self.it
        nx, ny, nz = G.nx, G.ny, G.nz
        E, H = self.E, self.H
        self._store_outputs(it)
        for s, snap in enumerate(G.snapshots):
            if snap.time == it + 1:
                self._store_snapshot(s, snap)
        L.oracle_update_magnetic(nx, ny, nz, _p(self.cH), _p(self.ID), *(_p(a) for a in E),
                                 *(_p(a) for a in H))
        for st in self.slabs:
            p = st.pml
            r = st.rows
            L.oracle_pml_magnetic(self.form, self.order, _DIRS[p.direction], p.xs, p.xf, p.ys, p.yf,
                                  p.zs, p.zf, nx, ny, nz, _p(self.cH), _p(self.ID),
                                  *(_p(a) for a in E), *(_p(a) for a in H), _p(st.HPhi1), _p(st.HPhi2),
                                  _p(st.dims[2]), _p(st.dims[3]), _p(r['HRA']), _p(r['HRB']),
                                  _p(r['HRE']), _p(r['HRF']), self._d(p.d))
        self._sources_magnetic(it)
        if self.P == 0:
            L.oracle_update_electric(nx, ny, nz, _p(self.cE), _p(self.ID), *(_p(a) for a in E),
                                     *(_p(a) for a in H))
        else:
            L.oracle_update_dispersive_A(nx, ny, nz, self.P, _p(self.cE), _p(self.cD), _p(self.ID),
                                         *(_p(t) for t in self.T), *(_p(a) for a in E),
                                         *(_p(a) for a in H))
        for st in self.slabs:
            p = st.pml
            r = st.rows
            L.oracle_pml_electric(self.form, self.order, _DIRS[p.direction], p.xs, p.xf, p.ys, p.yf,
                                  p.zs, p.zf, nx, ny, nz, _p(self.cE), _p(self.ID),
                                  *(_p(a) for a in E), *(_p(a) for a in H), _p(st.EPhi1), _p(st.EPhi2),
                                  _p(st.dims[0]), _p(st.dims[1]), _p(r['ERA']), _p(r['ERB']),
                                  _p(r['ERE']), _p(r['ERF']), self._d(p.d))
        self._sources_electric(it)
        if self.P:
            L.oracle_update_dispersive_B(nx, ny, nz, self.P, _p(self.cD), _p(self.ID),
                                         *(_p(t) for t in self.T), *(_p(a) for a in E))
        self.it += 1

    def run(self, nsteps=None):
        n = self.G.iterations - self.it if nsteps is None else nsteps
        for _ in range(n):
            self.step()
        return self

    def fields(self):
        return np.stack(self.E + self.H)

    def receivers(self):
        return self.rx[:, :, :len(self.G.rxs)]


