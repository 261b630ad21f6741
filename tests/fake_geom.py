"""A numpy stand-in for the ``gbf_geom_*`` entry points of the native library (test
infrastructure): the same arguments and results as the device builders, restated with plain
array operations, so that the host side of the device geometry build (dispatch of the
primitives, the key order and resolution of averaged materials, PML faces, 2D planes,
voltage-source materials) can be checked on a machine without a GPU."""
import ctypes

import numpy as np

_E_COMPS = (
    # comp, region start, neighbour cells (offsets subtracted), rigid (bit, offset)
    (0, (0, 1, 1), ((0, 0, 0), (0, 1, 0), (0, 1, 1), (0, 0, 1)),
     ((0, (0, 0, 0)), (1, (0, 1, 0)), (3, (0, 0, 1)), (2, (0, 1, 1)))),
    (1, (1, 0, 1), ((0, 0, 0), (1, 0, 0), (1, 0, 1), (0, 0, 1)),
     ((4, (0, 0, 0)), (7, (1, 0, 0)), (5, (0, 0, 1)), (6, (1, 0, 1)))),
    (2, (1, 1, 0), ((0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0)),
     ((8, (0, 0, 0)), (9, (1, 0, 0)), (11, (0, 1, 0)), (10, (1, 1, 0)))),
)
_H_COMPS = (
    (3, (1, 0, 0), ((0, 0, 0), (1, 0, 0)), ((12, (0, 0, 0)), (13, (1, 0, 0)))),
    (4, (0, 1, 0), ((0, 0, 0), (0, 1, 0)), ((14, (0, 0, 0)), (15, (0, 1, 0)))),
    (5, (0, 0, 1), ((0, 0, 0), (0, 0, 1)), ((16, (0, 0, 0)), (17, (0, 0, 1)))),
)


def _arr(ptr, dtype, shape):
    if isinstance(ptr, ctypes.Array):
        return np.frombuffer(ptr, dtype=dtype).reshape(shape)
    n = int(np.prod(shape))
    buf = (ctypes.c_char * (n * np.dtype(dtype).itemsize)).from_address(int(ptr))
    return np.frombuffer(buf, dtype=dtype).reshape(shape)


class _Geom:
    def __init__(self, nx, ny, nz):
        self.n = (nx, ny, nz)
        self.solid = np.ones((nx, ny, nz), np.uint32)
        self.rigid = np.zeros((nx, ny, nz), np.uint32)
        self.ID = np.ones((6, nx + 1, ny + 1, nz + 1), np.uint32)
        self.keys = None
        self.pos = None


class FakeGeomLib:
    """The ``gbf_geom_*`` functions; handles are indices into ``self.objs``."""

    def __init__(self):
        self.objs = {}
        self.next = 1

    @staticmethod
    def _h(h):
        return h.value if isinstance(h, ctypes.c_void_p) else int(h)

    def gbf_geom_create(self, nx, ny, nz, out):
        h = self.next
        self.next += 1
        self.objs[h] = _Geom(nx, ny, nz)
        out._obj.value = h
        return 0

    def gbf_geom_destroy(self, h):
        self.objs.pop(self._h(h), None)

    def gbf_geom_last_error(self, h, buf, n):
        return 0

    def _voxel(self, g, i, j, k, num, averaging):
        g.solid[i, j, k] = num[0]
        g.rigid[i, j, k] = 0 if averaging else 0x3FFFF
        if averaging:
            return
        for comp, v, nodes in ((0, num[1], ((0, 0, 0), (0, 1, 1), (0, 1, 0), (0, 0, 1))),
                               (1, num[2], ((0, 0, 0), (1, 0, 1), (1, 0, 0), (0, 0, 1))),
                               (2, num[3], ((0, 0, 0), (1, 1, 0), (1, 0, 0), (0, 1, 0)))):
            for a, b, c in nodes:
                g.ID[comp, i + a, j + b, k + c] = v
                g.ID[comp + 3, i + a, j + b, k + c] = v

    def gbf_geom_cells(self, h, box, mask, num, averaging):
        g = self.objs[self._h(h)]
        xs, ys, zs, sx, sy, sz = list(box)
        m = np.ones((sx, sy, sz), bool) if mask is None else _arr(mask, np.uint8, (sx, sy, sz)) != 0
        for i, j, k in zip(*np.nonzero(m)):
            self._voxel(g, xs + i, ys + j, zs + k, list(num), averaging)
        return 0

    def gbf_geom_box(self, h, box, num, averaging):
        g = self.objs[self._h(h)]
        xs, ys, zs, sx, sy, sz = list(box)
        xf, yf, zf = xs + sx, ys + sy, zs + sz
        n = list(num)
        g.solid[xs:xf, ys:yf, zs:zf] = n[0]
        g.rigid[xs:xf, ys:yf, zs:zf] = 0 if averaging else 0x3FFFF
        if averaging:
            return 0
        g.ID[0, xs:xf, ys:yf + 1, zs:zf + 1] = n[1]
        g.ID[1, xs:xf + 1, ys:yf, zs:zf + 1] = n[2]
        g.ID[2, xs:xf + 1, ys:yf + 1, zs:zf] = n[3]
        g.ID[3, xs:xf + 1, ys:yf, zs:zf] = n[1]
        g.ID[4, xs:xf, ys:yf + 1, zs:zf] = n[2]
        g.ID[5, xs:xf, ys:yf, zs:zf + 1] = n[3]
        return 0

    def gbf_geom_voxels(self, h, box, data, numexist, averaging):
        g = self.objs[self._h(h)]
        xs, ys, zs, sx, sy, sz = list(box)
        d = _arr(data, np.int16, (sx, sy, sz))
        for i, j, k in zip(*np.nonzero(d >= 0)):
            v = numexist + int(d[i, j, k])
            self._voxel(g, xs + i, ys + j, zs + k, (v, v, v, v), averaging)
        return 0

    def gbf_geom_edges(self, h, n, recs):
        g = self.objs[self._h(h)]
        r = _arr(recs, np.int32, (n, 5))
        for comp, i, j, k, v in r:
            sets = {0: ((0, 0, 0, 0), (1, 0, 1, 0), (3, 0, 0, 1), (2, 0, 1, 1)),
                    1: ((4, 0, 0, 0), (7, 1, 0, 0), (5, 0, 0, 1), (6, 1, 0, 1)),
                    2: ((8, 0, 0, 0), (9, 1, 0, 0), (11, 0, 1, 0), (10, 1, 1, 0))}[int(comp)]
            for bit, a, b, c in sets:
                if i - a >= 0 and j - b >= 0 and k - c >= 0:
                    g.rigid[i - a, j - b, k - c] |= np.uint32(1 << bit)
            g.ID[comp, i, j, k] = v
        return 0

    def gbf_geom_components(self, h, electric, counts):
        g = self.objs[self._h(h)]
        nx, ny, nz = g.n
        keys, pos = [], []
        for q, (comp, start, nbs, rig) in enumerate(_E_COMPS if electric else _H_COMPS):
            i0, j0, k0 = start
            R = (slice(i0, nx), slice(j0, ny), slice(k0, nz))

            def shifted(a, off):
                return a[i0 - off[0]:nx - off[0], j0 - off[1]:ny - off[1], k0 - off[2]:nz - off[2]]
            rigid = np.zeros(shifted(g.solid, (0, 0, 0)).shape, bool)
            for bit, off in rig:
                rigid |= (shifted(g.rigid, off) >> np.uint32(bit)) & np.uint32(1) != 0
            s = [shifted(g.solid, off).astype(np.uint64) for off in nbs]
            same = np.ones(rigid.shape, bool)
            for a in s[1:]:
                same &= a == s[0]
            target = g.ID[comp][R]
            plain = ~rigid & same
            target[plain] = s[0][plain]
            avg = ~rigid & ~same
            if len(s) == 4:
                k = (s[0] << np.uint64(48)) | (s[1] << np.uint64(32)) | (s[2] << np.uint64(16)) | s[3]
            else:
                k = (s[0] << np.uint64(16)) | s[1]
            idx = np.nonzero(avg)
            keys.append(k[idx])
            nodes = np.ravel_multi_index((idx[0] + i0, idx[1] + j0, idx[2] + k0), (nx + 1, ny + 1, nz + 1))
            pos.append(comp * (nx + 1) * (ny + 1) * (nz + 1) + nodes)
            counts[q] = int(idx[0].size)
        g.keys = np.concatenate(keys)
        g.pos = np.concatenate(pos)
        return 0

    def gbf_geom_averaged_keys(self, h, keys):
        g = self.objs[self._h(h)]
        _arr(keys, np.uint64, (g.keys.size,))[:] = g.keys
        return 0

    def gbf_geom_resolve(self, h, m, table, numbers):
        g = self.objs[self._h(h)]
        if g.keys is not None and g.keys.size:
            t = _arr(table, np.uint64, (m,))
            nb = _arr(numbers, np.uint32, (m,))
            at = np.searchsorted(t, g.keys)
            assert (t[at] == g.keys).all()
            g.ID.reshape(-1)[g.pos] = nb[at]
        g.keys = g.pos = None
        return 0

    def _array(self, g, array):
        return {0: g.solid, 1: g.rigid}.get(array) if array < 2 else g.ID[array - 2]

    def gbf_geom_fill(self, h, array, box, value):
        g = self.objs[self._h(h)]
        xs, ys, zs, sx, sy, sz = list(box)
        self._array(g, array)[xs:xs + sx, ys:ys + sy, zs:zs + sz] = value
        return 0

    def gbf_geom_read(self, h, array, box, out):
        g = self.objs[self._h(h)]
        xs, ys, zs, sx, sy, sz = list(box)
        _arr(out, np.uint32, (sx, sy, sz))[:] = self._array(g, array)[xs:xs + sx, ys:ys + sy, zs:zs + sz]
        return 0

    def gbf_geom_max_id(self, h, out):
        out._obj.value = int(self.objs[self._h(h)].ID.max())
        return 0
