"""Model geometry built in device memory (``gbf_geom_*`` in the C ABI).

With ``build_grid(..., device_build=True)`` the grid's solid, rigid and ID arrays
(``gprMax/grid.py:157-169``) are never allocated on the host: the geometry primitives write
them on the GPU (``gbf_geom_cells`` / ``_voxels`` / ``_edges``), the E and H component build
(``gprMax/yee_cell_build_ext.pyx:110-257``) runs there, and the solver takes the finished ID
array device to device. The host keeps what is host work in the reference too: selecting the
cells of spheres and cylinders (the same arithmetic as :mod:`gprmax_gb300.geometry`), naming
and numbering averaged materials, PML face averages and voltage-source materials, for which it
reads the few values it needs.
"""
import ctypes

import numpy as np

from . import _native
from .exceptions import SolverError

SOLID, RIGID = 0, 1


def _box(xs, ys, zs, sx, sy, sz):
    return (ctypes.c_int32 * 6)(int(xs), int(ys), int(zs), int(sx), int(sy), int(sz))


class DeviceGeometry:
    """The geometry arrays of an ``nx x ny x nz`` grid on the current CUDA device."""

    def __init__(self, nx, ny, nz):
        self.lib = _native.lib()
        self.h = ctypes.c_void_p(0)
        self.nx, self.ny, self.nz = nx, ny, nz
        self._check(self.lib.gbf_geom_create(nx, ny, nz, ctypes.byref(self.h)), created=False)

    def _check(self, rc, created=True):
        if rc != 0:
            buf = ctypes.create_string_buffer(1024)
            self.lib.gbf_geom_last_error(self.h if created else None, buf, 1024)
            raise SolverError('libgbfdtd geometry error {}: {}'.format(rc, buf.value.decode()))

    # -- primitives --------------------------------------------------------------------------
    def cells(self, origin, shape, mask, num, averaging):
        """``build_voxel`` on the cells of a box (where ``mask`` is true, if given)."""
        if min(shape) <= 0:
            return
        m = None
        if mask is not None:
            m = np.ascontiguousarray(mask, dtype=np.uint8)
            if not m.any():
                return
        nums = (ctypes.c_uint32 * 4)(*[int(v) for v in num])
        self._check(self.lib.gbf_geom_cells(self.h, _box(*origin, *shape),
                                            None if m is None else m.ctypes.data, nums,
                                            1 if averaging else 0))

    def box(self, origin, shape, num, averaging):
        """``build_box``: the cells of a box and its per-component ID ranges."""
        if min(shape) <= 0:
            return
        nums = (ctypes.c_uint32 * 4)(*[int(v) for v in num])
        self._check(self.lib.gbf_geom_box(self.h, _box(*origin, *shape), nums,
                                          1 if averaging else 0))

    def voxels(self, origin, data, averaging):
        """``build_voxels_from_array`` for a block already clipped to the grid (material
        numbers, negative = leave the cell)."""
        if data.size == 0:
            return
        if data.max() > np.iinfo(np.int16).max:
            raise SolverError('voxel material numbers must fit in int16')
        d16 = np.ascontiguousarray(data, dtype=np.int16)
        self._check(self.lib.gbf_geom_voxels(self.h, _box(*origin, *d16.shape), d16.ctypes.data,
                                             0, 1 if averaging else 0))

    def edges(self, records):
        """Rigid E edges: rows (component, i, j, k, numID), a list or an (n, 5) array."""
        r = np.ascontiguousarray(np.asarray(records, dtype=np.int32).reshape(-1, 5))
        if r.shape[0] == 0:
            return
        bad = ((r[:, 1] < 0) | (r[:, 2] < 0) | (r[:, 3] < 0) | (r[:, 1] >= self.nx)
               | (r[:, 2] >= self.ny) | (r[:, 3] >= self.nz))
        if bad.any():
            raise IndexError('edge {} is outside the grid'.format(tuple(r[np.argmax(bad), :4])))
        self._check(self.lib.gbf_geom_edges(self.h, r.shape[0], r.ctypes.data))

    # -- component build -----------------------------------------------------------------------
    def components(self, electric, resolve, G):
        """Per-edge IDs of the E (or H) components; ``resolve(G, ids)`` names and numbers the
        averaged materials, called once per distinct neighbour combination in the order the
        reference's loops first meet it."""
        counts = (ctypes.c_int64 * 3)()
        self._check(self.lib.gbf_geom_components(self.h, 1 if electric else 0, counts))
        n = int(sum(counts))
        if n == 0:
            self._check(self.lib.gbf_geom_resolve(self.h, 0, None, None))
            return
        keys = np.empty(n, dtype=np.uint64)
        self._check(self.lib.gbf_geom_averaged_keys(self.h, keys.ctypes.data))
        table, first = np.unique(keys, return_index=True)
        numbers = np.empty(table.size, dtype=np.uint32)
        shifts = (48, 32, 16, 0) if electric else (16, 0)
        for idx in np.argsort(first, kind='stable'):
            key = int(table[idx])
            numbers[idx] = resolve(G, tuple((key >> s) & 0xFFFF for s in shifts))
        table = np.ascontiguousarray(table)
        self._check(self.lib.gbf_geom_resolve(self.h, table.size, table.ctypes.data,
                                              numbers.ctypes.data))

    # -- access --------------------------------------------------------------------------------
    def read(self, array, origin, shape):
        out = np.empty(shape, dtype=np.uint32)
        self._check(self.lib.gbf_geom_read(self.h, array, _box(*origin, *shape), out.ctypes.data))
        return out

    def fill(self, array, origin, shape, value):
        if min(shape) <= 0:
            return
        self._check(self.lib.gbf_geom_fill(self.h, array, _box(*origin, *shape), int(value)))

    def solid(self):
        return self.read(SOLID, (0, 0, 0), (self.nx, self.ny, self.nz))

    def rigid(self):
        """rigidE int8 [12][nx][ny][nz] and rigidH int8 [6][nx][ny][nz] from the packed flags."""
        w = self.read(RIGID, (0, 0, 0), (self.nx, self.ny, self.nz))
        bits = ((w[None] >> np.arange(18, dtype=np.uint32)[:, None, None, None]) & 1).astype(np.int8)
        return bits[:12], bits[12:]

    def ids(self, comp=None):
        """The ID array uint32 [6][nx+1][ny+1][nz+1] (or one component)."""
        shape = (self.nx + 1, self.ny + 1, self.nz + 1)
        if comp is not None:
            return self.read(2 + comp, (0, 0, 0), shape)
        return np.stack([self.read(2 + c, (0, 0, 0), shape) for c in range(6)])

    def id_at(self, comp, i, j, k):
        return int(self.read(2 + comp, (i, j, k), (1, 1, 1))[0, 0, 0])

    def set_id(self, comp, i, j, k, value):
        self.fill(2 + comp, (i, j, k), (1, 1, 1), value)

    def max_id(self):
        v = ctypes.c_uint32(0)
        self._check(self.lib.gbf_geom_max_id(self.h, ctypes.byref(v)))
        return v.value

    def close(self):
        if self.h and self.h.value:
            self.lib.gbf_geom_destroy(self.h)
        self.h = ctypes.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

