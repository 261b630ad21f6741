"""GB300 solver driver: the drop-in for the reference's ``solve_cpu``/``solve_gpu``.

``solve_gb300(currentmodelrun, modelend, G)`` reads the same grid object the reference's
solvers read (``model_build_run.py:369-373``), runs every iteration on the GPU through the C
ABI of ``libgbfdtd.so`` and fills ``G.rxs[*].outputs`` and the snapshots, so the output writer
is unchanged. :class:`DeviceModel` is the reusable form: build once, run, read back, reset.
"""
import ctypes
import time

import numpy as np

from . import _native
from .exceptions import SolverError
from .receivers import OUTPUT_INDEX
from .sources import active_range, kernel_record

PML_SLABS = ['x0', 'y0', 'z0', 'xmax', 'ymax', 'zmax']


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else ctypes.c_void_p(0)


def pole_count(G):
    """Dispersive poles per material: ``G.maxpoles`` on grids built by this package; the
    reference keeps the count on its ``Material`` class (``materials.py:30``), equal to the
    largest ``poles`` of the grid's materials."""
    mp = getattr(G, 'maxpoles', None)
    if mp is None:
        mp = max((int(getattr(m, 'poles', 0)) for m in G.materials), default=0)
    return int(mp)


def source_list(G):
    """Sources in the reference's application order: E sources (voltage sources, transmission
    lines, Hertzian dipoles; ``model_build_run.py:459-461``), then magnetic dipoles."""
    return (list(G.voltagesources) + list(getattr(G, 'transmissionlines', []))
            + list(G.hertziandipoles) + list(G.magneticdipoles))


_TL_STENCIL = {'x': ((4, 0, 0, -1), (4, 0, 0, 0), (5, 0, 0, 0), (5, 0, -1, 0)),
               'y': ((3, 0, 0, 0), (3, 0, 0, -1), (5, -1, 0, 0), (5, 0, 0, 0)),
               'z': ((3, 0, -1, 0), (3, 0, 0, 0), (4, 0, 0, 0), (4, -1, 0, 0))}


def tl_tables(G):
    """The transmission lines' device tables: info int32 [n][9], coefficients float64 [n][4],
    line state float32 [n][34], cell sizes float32 [n], waveforms float32 [n][2][iterations]."""
    from .sources import active_range
    tls = list(getattr(G, 'transmissionlines', []))
    n = len(tls)
    cells = 16
    info = np.zeros((max(n, 1), 9), dtype=np.int32)
    coef = np.zeros((max(n, 1), 4), dtype=np.float64)
    state = np.zeros((max(n, 1), 2 * cells + 2), dtype=np.float32)
    cell = np.zeros(max(n, 1), dtype=np.float32)
    waves = np.zeros((max(n, 1), 2, G.iterations), dtype=np.float32)
    for q, t in enumerate(tls):
        comp = 'xyz'.index(t.polarisation)
        first, last = active_range(t, G)
        info[q] = (comp, t.xcoord, t.ycoord, t.zcoord, first, last, t.nl, t.srcpos, t.antpos)
        coef[q] = t.ratios(G)
        state[q, :t.nl] = t.voltage[:t.nl]
        state[q, cells:cells + t.nl] = t.current[:t.nl]
        state[q, 2 * cells] = np.float32(t.abcv0)
        state[q, 2 * cells + 1] = np.float32(t.abcv1)
        cell[q] = np.float32({'x': G.dx, 'y': G.dy, 'z': G.dz}[t.polarisation])
        waves[q, 0] = t.waveformvalues_wholestep
        waves[q, 1] = t.waveformvalues_halfstep
        # the reference updates the lines before the magnetic dipoles: a dipole on an H value
        # of the line's current loop would be seen in a different order here
        for m in G.magneticdipoles:
            mc = 3 + 'xyz'.index(m.polarisation)
            for c, di, dj, dk in _TL_STENCIL[t.polarisation]:
                if (mc, m.xcoord, m.ycoord, m.zcoord) == (c, t.xcoord + di, t.ycoord + dj, t.zcoord + dk):
                    raise SolverError('a magnetic dipole on the current loop of a transmission line '
                                      'is not supported')
    return info, coef, state, cell, waves


def source_tables(G):
    """int32 [n][8] info, fp32 [n][2] scales and fp32 [n][iterations] waveform tables."""
    srcs = source_list(G)
    n = len(srcs)
    info = np.zeros((max(n, 1), 8), dtype=np.int32)
    scale = np.zeros((max(n, 1), 2), dtype=np.float32)
    waves = np.zeros((max(n, 1), G.iterations), dtype=np.float32)
    for s, src in enumerate(srcs):
        kind, comp, sc, table = kernel_record(src, G)
        first, last = active_range(src, G)
        info[s] = (kind, comp, src.xcoord, src.ycoord, src.zcoord, first, last, 0)
        scale[s] = sc
        waves[s] = table
    return info, scale, waves


def real_dispersive_state(G):
    """Whether the C ABI stores this model's dispersive state as real parts: poles present,
    packed material IDs (at most 1024 materials) and every pole Debye-like (eqt with imaginary
    part +0, zt with imaginary part +-0), the rule ``gbf_upload_materials`` applies."""
    if not pole_count(G) or len(G.materials) > 1024:
        return False
    d = np.ascontiguousarray(G.updatecoeffsdispersive, dtype=np.complex64)
    bits = d.view(np.float32).reshape(d.shape[0], -1, 3, 2).view(np.uint32)
    return bool((bits[:, :, 1, 1] == 0).all() and ((bits[:, :, 2, 1] & 0x7fffffff) == 0).all())


def model_inputs(G, options=0, ids=True):
    """Everything the C ABI receives for grid ``G``: the descriptor and the host arrays, in
    the reference's layouts (without the ID array when ``ids`` is false). Reads only attributes
    that the reference's own grid object also carries, so a grid built by the reference's
    ``run_model`` can be handed over unchanged."""
    d = _native.GridDesc()
    d.nx, d.ny, d.nz = G.nx, G.ny, G.nz
    d.iterations = G.iterations
    d.nmat = len(G.materials)
    d.maxpoles = pole_count(G)
    d.pml_formulation = 0 if G.pmlformulation == 'HORIPML' else 1
    d.pml_order = max(len(G.cfs), 1)
    thick = {pml.ID: pml.thickness for pml in G.pmls}
    for s, key in enumerate(PML_SLABS):
        d.pml_thickness[s] = thick.get(key, 0)
    d.dx, d.dy, d.dz = np.float32(G.dx), np.float32(G.dy), np.float32(G.dz)
    d.nsrc = len(source_list(G))
    d.nrx = len(G.rxs)
    d.nsnap = len(G.snapshots)
    d.ntl = len(getattr(G, 'transmissionlines', []))
    d.options = options
    inp = {'desc': d,
           'ID': (np.ascontiguousarray(G.ID, dtype=np.uint32)
                  if ids and getattr(G, 'geom', None) is None else None),
           'coeffE': np.ascontiguousarray(G.updatecoeffsE, dtype=np.float32),
           'coeffH': np.ascontiguousarray(G.updatecoeffsH, dtype=np.float32),
           'coeffD': None, 'pml': [], 'sources': None, 'rx': None, 'snapshots': None}
    if d.maxpoles > 0:
        inp['coeffD'] = np.ascontiguousarray(G.updatecoeffsdispersive, dtype=np.complex64)
    for pml in G.pmls:
        rows = [np.ascontiguousarray(getattr(pml, n), dtype=np.float32)
                for n in ('ERA', 'ERB', 'ERE', 'ERF', 'HRA', 'HRB', 'HRE', 'HRF')]
        inp['pml'].append((PML_SLABS.index(pml.ID), rows))
    if d.nsrc:
        inp['sources'] = source_tables(G)
    inp['tls'] = tl_tables(G) if d.ntl else None
    if G.rxs:
        inp['rx'] = np.array([[r.xcoord, r.ycoord, r.zcoord] for r in G.rxs], dtype=np.int32)
    if G.snapshots:
        inp['snapshots'] = np.array([[s.xs, s.ys, s.zs, s.dx, s.dy, s.dz, s.nx, s.ny, s.nz, s.time]
                                     for s in G.snapshots], dtype=np.int32)
    return inp


class PinnedWords:
    """A uint32 array in page-locked host memory from the library (``gbf_host_alloc``), released
    with the object."""

    def __init__(self, lib, n):
        self.lib = lib
        self.ptr = ctypes.c_void_p(0)
        rc = lib.gbf_host_alloc(4 * n, ctypes.byref(self.ptr))
        if rc != 0:
            buf = ctypes.create_string_buffer(256)
            lib.gbf_last_error(None, buf, 256)
            raise SolverError('libgbfdtd error {}: {}'.format(rc, buf.value.decode()))
        self.array = np.ctypeslib.as_array((ctypes.c_uint32 * n).from_address(self.ptr.value))

    def __del__(self):
        try:
            if self.ptr and self.ptr.value:
                self.lib.gbf_host_free(self.ptr)
        except Exception:
            pass
        self.ptr = ctypes.c_void_p(0)


def uniform_h(G):
    """Whether every material of ``G`` has the same H row (DA, DBx, DBy, DBz, srcm): true for
    any model without magnetic materials, whose H half-step then reads no material IDs."""
    h = np.asarray(G.updatecoeffsH, dtype=np.float32)
    return bool((h.view(np.uint32) == h[:1].view(np.uint32)).all())


def pack_materials(G):
    """The material IDs of ``G`` as packed words per node in page-locked host memory (E:
    ``IDx | IDy << 10 | IDz << 20``, H likewise; the H words only when the materials' H rows
    differ, else None in their place), the form ``DeviceModel(G, packed=...)`` uploads with a
    third (a sixth) of the bytes at the full copy rate. Packed on the host's cores
    (``gbf_pack_ids``). Returns None for models with more than 1024 materials or IDs built in
    device memory. The words are a copy: pack again after changing ``G.ID``."""
    if len(G.materials) > 1024 or getattr(G, 'geom', None) is not None:
        return None
    lib = _native.lib()
    ID = np.ascontiguousarray(G.ID, dtype=np.uint32)
    n = ID[0].size
    pe = PinnedWords(lib, n)
    ph = None if uniform_h(G) else PinnedWords(lib, n)
    mx = ctypes.c_uint32(0)
    rc = lib.gbf_pack_ids(_ptr(ID), n, pe.ptr, ph.ptr if ph is not None else None,
                          ctypes.byref(mx))
    if rc != 0:
        buf = ctypes.create_string_buffer(256)
        lib.gbf_last_error(None, buf, 256)
        raise SolverError('libgbfdtd error {}: {}'.format(rc, buf.value.decode()))
    return pe, ph


class DeviceModel:
    """One model resident on the GPU (fields, IDs, coefficients, PML and dispersive state).
    ``packed``: the material IDs as ``pack_materials(G)`` returns them, uploaded instead of
    ``G.ID``. ``share``: another DeviceModel of the same geometry whose material IDs and
    coefficient tables this one uses instead of uploading its own (``gbf_share_materials``)."""

    def __init__(self, G, options=0, packed=None, share=None):
        self.G = G
        self.lib = _native.lib()
        self.ctx = ctypes.c_void_p(0)
        self.packed = packed
        self.shared_from = share
        t0 = time.perf_counter()
        self.inputs = model_inputs(G, options, ids=share is None)
        d = self.desc = self.inputs['desc']
        self.maxpoles = d.maxpoles
        t1 = time.perf_counter()
        self._check(self.lib.gbf_create(ctypes.byref(d), ctypes.byref(self.ctx)), create=True)
        t2 = time.perf_counter()
        try:
            self._upload()
        except Exception:
            self.close()
            raise
        t3 = time.perf_counter()
        # seconds spent building the host arrays, creating the context and uploading
        self.timings = {'inputs_s': t1 - t0, 'create_s': t2 - t1, 'upload_s': t3 - t2}

    def _check(self, rc, create=False):
        if rc != 0:
            buf = ctypes.create_string_buffer(1024)
            self.lib.gbf_last_error(None if create else self.ctx, buf, 1024)
            raise SolverError('libgbfdtd error {}: {}'.format(rc, buf.value.decode()))

    def _upload(self):
        inp = self.inputs
        t0 = time.perf_counter()
        if self.shared_from is not None:
            self._check(self.lib.gbf_share_materials(self.ctx, self.shared_from.ctx))
        elif self.packed is not None:
            pe, ph = self.packed
            self._check(self.lib.gbf_upload_materials_packed(
                self.ctx, pe.ptr, ph.ptr if ph is not None else None, _ptr(inp['coeffE']),
                _ptr(inp['coeffH']), _ptr(inp['coeffD'])))
        elif inp['ID'] is None:
            # IDs built in device memory: copied device to device
            self._check(self.lib.gbf_upload_materials_geom(
                self.ctx, self.G.geom.h, _ptr(inp['coeffE']), _ptr(inp['coeffH']),
                _ptr(inp['coeffD'])))
        else:
            self._check(self.lib.gbf_upload_materials(
                self.ctx, _ptr(inp['ID']), _ptr(inp['coeffE']), _ptr(inp['coeffH']),
                _ptr(inp['coeffD'])))
        self.materials_s = time.perf_counter() - t0
        for slab, rows in inp['pml']:
            arr = (ctypes.c_void_p * 8)(*[r.ctypes.data for r in rows])
            self._check(self.lib.gbf_upload_pml(self.ctx, slab, arr))
        if inp['sources'] is not None:
            info, scale, waves = inp['sources']
            self._check(self.lib.gbf_upload_sources(self.ctx, _ptr(info), _ptr(scale), _ptr(waves)))
        if inp['tls'] is not None:
            self._check(self.lib.gbf_upload_tls(self.ctx, *(_ptr(a) for a in inp['tls'])))
        if inp['rx'] is not None:
            self._check(self.lib.gbf_set_receivers(self.ctx, _ptr(inp['rx'])))
        if inp['snapshots'] is not None:
            self._check(self.lib.gbf_set_snapshots(self.ctx, _ptr(inp['snapshots'])))
        self.reset()
        self.synchronize()
        self.inputs = None   # every host array has been copied to the device

    def reset(self):
        self._check(self.lib.gbf_reset(self.ctx))

    def run(self, nsteps=None, graph=True):
        """Advance ``nsteps`` iterations (default: all remaining) on the device stream."""
        if nsteps is None:
            nsteps = self.G.iterations - self.iteration()
        flags = _native.GBF_RUN_GRAPH if graph else 0
        self._check(self.lib.gbf_run(self.ctx, int(nsteps), flags))

    def run_timed(self, nsteps, graph=True):
        """Run ``nsteps`` iterations; device milliseconds from CUDA events on the solver stream."""
        ms = ctypes.c_float(0)
        flags = _native.GBF_RUN_GRAPH if graph else 0
        self._check(self.lib.gbf_run_timed(self.ctx, int(nsteps), flags, ctypes.byref(ms)))
        return ms.value

    def synchronize(self):
        self._check(self.lib.gbf_synchronize(self.ctx))

    def iteration(self):
        it = ctypes.c_int32(0)
        self._check(self.lib.gbf_current_iteration(self.ctx, ctypes.byref(it)))
        return it.value

    def receivers(self):
        """fp32 [9][iterations][nrx] receiver samples."""
        out = np.zeros((9, self.G.iterations, max(len(self.G.rxs), 1)), dtype=np.float32)
        if self.G.rxs:
            self._check(self.lib.gbf_download_rx(self.ctx, _ptr(out)))
        return out[:, :, :len(self.G.rxs)]

    def transmission_lines(self):
        """fp32 [ntl][2][iterations]: each line's Vtotal and Itotal."""
        n = self.desc.ntl
        out = np.zeros((max(n, 1), 2, self.G.iterations), dtype=np.float32)
        if n:
            self._check(self.lib.gbf_download_tls(self.ctx, _ptr(out)))
        return out[:n]

    def fields(self):
        """fp32 [6][nx+1][ny+1][nz+1] (Ex, Ey, Ez, Hx, Hy, Hz)."""
        G = self.G
        out = np.zeros((6, G.nx + 1, G.ny + 1, G.nz + 1), dtype=np.float32)
        self._check(self.lib.gbf_download_fields(self.ctx, _ptr(out)))
        return out

    def set_fields(self, fields):
        f = np.ascontiguousarray(fields, dtype=np.float32)
        self._check(self.lib.gbf_upload_fields(self.ctx, _ptr(f)))

    def dispersive(self):
        """complex64 [3][maxpoles][nx+1][ny+1][nz+1] (Tx, Ty, Tz)."""
        G = self.G
        out = np.zeros((3, self.maxpoles, G.nx + 1, G.ny + 1, G.nz + 1), dtype=np.complex64)
        self._check(self.lib.gbf_download_dispersive(self.ctx, _ptr(out)))
        return out

    def snapshot(self, s):
        snap = self.G.snapshots[s]
        out = np.zeros((6, snap.nx, snap.ny, snap.nz), dtype=np.float32)
        self._check(self.lib.gbf_download_snapshot(self.ctx, s, _ptr(out)))
        return out

    def profile(self, nsteps):
        """Device milliseconds of the H kernels, E kernels and whole steps over ``nsteps``."""
        h, e, t = ctypes.c_float(0), ctypes.c_float(0), ctypes.c_float(0)
        self._check(self.lib.gbf_profile(self.ctx, int(nsteps), ctypes.byref(h), ctypes.byref(e),
                                         ctypes.byref(t)))
        return h.value, e.value, t.value

    def step_info(self):
        """How the model steps: {'fused': bool, 'tj', 'nch', 'planes', 'blocks', 'tuned',
        'buffer', 'two_buffers', 'fused_available', 'staged', 'staged_h', 'forms_tuned',
        'staged_available', 'staged_h_available'} (``gbf_step_info``; 'staged', 'staged_h': the
        E, H half-step is the staged sweep)."""
        info = np.zeros(8, dtype=np.int32)
        self._check(self.lib.gbf_step_info(self.ctx, _ptr(info)))
        keys = ('fused', 'tj', 'nch', 'planes', 'blocks', 'tuned', 'buffer', 'two_buffers')
        out = {k: int(v) for k, v in zip(keys, info)}
        out['fused'] = bool(out['fused'])
        out['fused_available'] = bool(out['two_buffers'] & 2)
        out['staged'] = bool(out['two_buffers'] & 4)
        out['staged_h'] = bool(out['two_buffers'] & 8)
        out['forms_tuned'] = bool(out['two_buffers'] & 16)
        out['staged_available'] = bool(out['two_buffers'] & 32)
        out['staged_h_available'] = bool(out['two_buffers'] & 64)
        out['two_buffers'] = bool(out['two_buffers'] & 1)
        return out

    def set_step_forms(self, e_staged, h_staged):
        """Fix each half-step's form: the staged sweep or the plain kernel
        (``gbf_set_step_forms``; the results are the same bit for bit)."""
        self._check(self.lib.gbf_set_step_forms(self.ctx, int(bool(e_staged)) | 2 * int(bool(h_staged))))

    def set_fused_tiles(self, tj, nch):
        """Fix the fused step's tiling (tile height ``tj`` rows, ``nch`` chunks along x)."""
        self._check(self.lib.gbf_set_fused_tiles(self.ctx, int(tj), int(nch)))

    def device_bytes(self):
        b = ctypes.c_size_t(0)
        self._check(self.lib.gbf_device_bytes(self.ctx, ctypes.byref(b)))
        return b.value

    def close(self):
        if self.ctx and self.ctx.value:
            self.lib.gbf_destroy(self.ctx)
        self.ctx = ctypes.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def store_results(self, fields=True):
        """Copy receiver outputs, snapshots and (optionally) final fields into ``G``."""
        G = self.G
        rx = self.receivers()
        for n, r in enumerate(G.rxs):
            for name in r.outputs:
                r.outputs[name] = rx[OUTPUT_INDEX[name], :, n].copy()
        tls = list(getattr(G, 'transmissionlines', []))
        if tls:
            out = self.transmission_lines()
            for q, t in enumerate(tls):
                t.Vtotal = out[q, 0].copy()
                t.Itotal = out[q, 1].copy()
        for s, snap in enumerate(G.snapshots):
            f = self.snapshot(s)
            # the VTK point layout the reference's Snapshot.store leaves (snapshots.py:129-130)
            snap.electric = np.stack(f[:3]).reshape(-1, order='F')
            snap.magnetic = np.stack(f[3:]).reshape(-1, order='F')
        if fields:
            f = self.fields()
            G.Ex, G.Ey, G.Ez, G.Hx, G.Hy, G.Hz = (f[c] for c in range(6))
            if self.maxpoles > 0:
                T = self.dispersive()
                G.Tx, G.Ty, G.Tz = T[0], T[1], T[2]


def same_geometry(G, H):
    """Whether grids ``G`` and ``H`` have the same material IDs and coefficient tables (so one
    device copy serves both): the same object, or equal sizes and tables and then equal IDs
    (the tables, compared first, tell most different geometries apart cheaply)."""
    if G is H or G.ID is H.ID:
        return True
    if getattr(G, 'geom', None) is not None or getattr(H, 'geom', None) is not None:
        return False
    if (G.nx, G.ny, G.nz) != (H.nx, H.ny, H.nz) or len(G.materials) != len(H.materials):
        return False
    for a in ('updatecoeffsE', 'updatecoeffsH'):
        if not np.array_equal(getattr(G, a), getattr(H, a)):
            return False
    if pole_count(G) != pole_count(H):
        return False
    if pole_count(G) and not np.array_equal(G.updatecoeffsdispersive, H.updatecoeffsdispersive):
        return False
    return np.array_equal(G.ID, H.ID)


class BatchModel:
    """Many models advanced together: one persistent launch per half-step walks every model
    (``gbf_batch_*`` in the C ABI), and the requested time loop is replayed from one CUDA graph.
    The models may differ in size, geometry, sources and receivers; they must share the PML
    formulation and order, the pole count and the material-ID layout, and have no snapshots.
    Models of one geometry (a B-scan over a fixed model, the traces differing only in source
    and receiver positions) share one device copy of their material IDs and coefficient tables
    (``share_geometry``; found with :func:`same_geometry`)."""

    def __init__(self, grids, options=0, share_geometry=True):
        self.lib = _native.lib()
        self.models = []
        self.b = ctypes.c_void_p(0)
        # one layout of the dispersive state for the whole batch: real parts only if every
        # model allows it, else complex everywhere (option bit 2)
        if any(pole_count(G) for G in grids) and not all(real_dispersive_state(G) for G in grids):
            options |= 4
        try:
            owners = []
            for G in grids:
                owner = None
                if share_geometry:
                    owner = next((m for m in owners if same_geometry(G, m.G)), None)
                m = DeviceModel(G, options, share=owner)
                if owner is None:
                    owners.append(m)
                self.models.append(m)
            arr = (ctypes.c_void_p * len(self.models))(*[m.ctx.value for m in self.models])
            rc = self.lib.gbf_batch_create(arr, len(self.models), ctypes.byref(self.b))
            self._check(rc, created=False)
        except Exception:
            self.close()
            raise

    def _check(self, rc, created=True):
        if rc != 0:
            buf = ctypes.create_string_buffer(1024)
            self.lib.gbf_batch_last_error(self.b if created else None, buf, 1024)
            raise SolverError('libgbfdtd batch error {}: {}'.format(rc, buf.value.decode()))

    def iteration(self):
        return self.models[0].iteration()

    def run(self, nsteps=None, graph=True):
        """Advance every model ``nsteps`` iterations (default: to the end of the shortest)."""
        if nsteps is None:
            nsteps = min(m.G.iterations for m in self.models) - self.iteration()
        flags = _native.GBF_RUN_GRAPH if graph else 0
        self._check(self.lib.gbf_batch_run(self.b, int(nsteps), flags))

    def run_timed(self, nsteps, graph=True):
        """Run ``nsteps`` iterations; device milliseconds from CUDA events on the batch stream
        (the graph is captured before the timed region)."""
        ms = ctypes.c_float(0)
        flags = _native.GBF_RUN_GRAPH if graph else 0
        self._check(self.lib.gbf_batch_run_timed(self.b, int(nsteps), flags, ctypes.byref(ms)))
        return ms.value

    def synchronize(self):
        self._check(self.lib.gbf_batch_synchronize(self.b))

    def info(self):
        """{'tuned': bool, 'blocks_h', 'blocks_e', 'own_kernels'}: the grid sizes of the batched
        launches and how many (large) models step with their own kernels."""
        info = np.zeros(4, dtype=np.int32)
        self._check(self.lib.gbf_batch_info(self.b, _ptr(info)))
        return {'tuned': bool(info[0]), 'blocks_h': int(info[1]), 'blocks_e': int(info[2]),
                'own_kernels': int(info[3])}

    def receivers(self):
        """Per model, fp32 [9][iterations][nrx] receiver samples."""
        self.synchronize()
        return [m.receivers() for m in self.models]

    def store_results(self, fields=False):
        self.synchronize()
        for m in self.models:
            m.store_results(fields=fields)

    def close(self):
        if self.b and self.b.value:
            self.lib.gbf_batch_destroy(self.b)
        self.b = ctypes.c_void_p(0)
        for m in self.models:
            m.close()
        self.models = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def solve_gb300_batch(grids, fields=False, outputfile=None):
    """Run every grid of a B-scan or parameter sweep to its end in one batch; returns the solve
    seconds. Each grid's receiver outputs are stored as ``solve_gb300`` stores them; with
    ``outputfile`` the traces are also written as one merged ``.out`` file
    ([iterations][nmodels] per receiver output)."""
    bm = BatchModel(grids)
    try:
        t0 = time.perf_counter()
        bm.run()
        bm.synchronize()
        tsolve = time.perf_counter() - t0
        bm.store_results(fields=fields)
    finally:
        bm.close()
    if outputfile:
        from .outputs import write_merged_outputfile
        write_merged_outputfile(outputfile, grids)
    return tsolve


def solve_gb300(currentmodelrun, modelend, G, fields=True):
    """Run all iterations of ``G`` on the GPU; returns (tsolve seconds, device bytes)."""
    dm = DeviceModel(G)
    try:
        t0 = time.perf_counter()
        dm.run()
        dm.synchronize()
        tsolve = time.perf_counter() - t0
        dm.store_results(fields=fields)
        mem = dm.device_bytes()
    finally:
        dm.close()
    return tsolve, mem
