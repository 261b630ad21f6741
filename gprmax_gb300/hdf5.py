"""Minimal HDF5 writer and reader for gprMax ``.out`` files (no h5py or libhdf5 needed).

Implements the subset of the HDF5 File Format Specification (version 2.0 of the spec, the
"version 0" superblock family) that gprMax's output files use, as written by h5py with its
default settings (``gprMax/fields_outputs.py:111-161``):

* superblock version 0 with 8-byte offsets and lengths;
* groups as symbol tables: object header with a Symbol Table message, a version-1 B-tree of
  group nodes and a local heap of link names, symbol-table nodes (SNOD) holding the entries;
* datasets with contiguous storage (Dataspace v1, Datatype v1, Data Layout v3 messages);
* attributes (Attribute message v1) with scalar or 1-D data of fixed-point, IEEE float or
  fixed-length string type, and text attributes as h5py stores a Python ``str``: a scalar
  variable-length UTF-8 string (Datatype class 9 over unsigned bytes) whose characters lie in a
  global heap collection (GCOL), one collection per file.

The reader also follows object header continuation messages and skips messages it does not
use (fill value, modification time, ...), so it reads files produced by h5py, variable-length
strings included.
"""
import struct

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF
SIGNATURE = b'\x89HDF\r\n\x1a\n'
LEAF_K = 32        # symbols per SNOD: up to 2*LEAF_K
INTERNAL_K = 16    # children per B-tree node: up to 2*INTERNAL_K


def _pad8(n):
    return (n + 7) & ~7


# ----------------------------------------------------------------------------- datatypes
def _dtype_message(dt):
    """Datatype message body (version 1) for a numpy dtype."""
    dt = np.dtype(dt)
    if dt.kind == 'f':
        if dt.itemsize == 4:
            bits = (0x20, 31, 0)
            props = struct.pack('<HHBBBBI', 0, 32, 23, 8, 0, 23, 127)
        elif dt.itemsize == 8:
            bits = (0x20, 63, 0)
            props = struct.pack('<HHBBBBI', 0, 64, 52, 11, 0, 52, 1023)
        else:
            raise TypeError('unsupported float size')
        return bytes([0x10 | 1]) + bytes(bits) + struct.pack('<I', dt.itemsize) + props
    if dt.kind in 'iu':
        flags = 0x08 if dt.kind == 'i' else 0
        return (bytes([0x10 | 0, flags, 0, 0]) + struct.pack('<I', dt.itemsize)
                + struct.pack('<HH', 0, 8 * dt.itemsize))
    if dt.kind == 'S':
        # fixed-length string, null-terminated, ASCII
        return bytes([0x10 | 3, 0x00, 0, 0]) + struct.pack('<I', dt.itemsize)
    raise TypeError('unsupported dtype {}'.format(dt))


# a scalar variable-length UTF-8 string: class 9 (string, null padding, UTF-8), 16-byte element
# (length, global heap collection address, object index), base type one unsigned byte
_VLSTR_MESSAGE = (bytes([0x10 | 9, 0x01, 0x01, 0x00]) + struct.pack('<I', 16)
                  + bytes([0x10 | 0, 0, 0, 0]) + struct.pack('<IHH', 1, 0, 8))
GCOL_MIN = 4096   # smallest global heap collection


def _dataspace_message(shape):
    """Dataspace message body (version 1); shape () is scalar."""
    body = struct.pack('<BBBB4x', 1, len(shape), 0, 0)
    for d in shape:
        body += struct.pack('<Q', d)
    return body


def _as_array(value):
    if isinstance(value, str):
        b = value.encode('utf-8')
        return np.array(b, dtype='S{}'.format(max(len(b) + 1, 1)))
    if isinstance(value, bytes):
        return np.array(value, dtype='S{}'.format(max(len(value) + 1, 1)))
    a = np.asarray(value)
    if a.dtype == np.bool_:
        a = a.astype(np.int8)
    if a.dtype.kind == 'U':
        return _as_array(str(a))
    return a


# ----------------------------------------------------------------------------- writer
class _Node:
    def __init__(self, name):
        self.name = name
        self.attrs = {}


class _Group(_Node):
    def __init__(self, name):
        super().__init__(name)
        self.children = {}


class _Dataset(_Node):
    def __init__(self, name, data):
        super().__init__(name)
        self.data = np.ascontiguousarray(data)


class File:
    """Write-only HDF5 file built in memory and written on :meth:`close`.

    ``f.attrs[name] = value``, ``f.create_group('/a/b')``, ``f['/a/b/ds'] = array`` and
    ``group.attrs[...]`` mirror the h5py calls the reference's writer makes.
    """

    def __init__(self, path, mode='w'):
        if mode != 'w':
            raise ValueError('only mode "w" is supported; use read() to read')
        self.path = path
        self.root = _Group('')
        self.attrs = self.root.attrs

    def _walk(self, path, create=True):
        node = self.root
        for part in [p for p in path.split('/') if p]:
            if part not in node.children:
                if not create:
                    raise KeyError(path)
                node.children[part] = _Group(part)
            node = node.children[part]
            if not isinstance(node, _Group):
                raise KeyError('{} is not a group'.format(path))
        return node

    def create_group(self, path):
        return _GroupHandle(self._walk(path))

    def __setitem__(self, path, data):
        parts = [p for p in path.split('/') if p]
        parent = self._walk('/'.join(parts[:-1]))
        parent.children[parts[-1]] = _Dataset(parts[-1], data)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        if exc[0] is None:
            self.close()

    def close(self):
        _Writer(self.root).write(self.path)


class _GroupHandle:
    def __init__(self, g):
        self._g = g
        self.attrs = g.attrs

    def __setitem__(self, name, data):
        self._g.children[name] = _Dataset(name, data)


class _Writer:
    """Lays the objects out: superblock, then for each group its header, B-tree, SNODs and
    local heap, then dataset headers and raw data."""

    def __init__(self, root):
        self.root = root
        self.buf = bytearray()
        self.gcol = UNDEF      # the file's global heap collection (text attributes)
        self.gindex = {}       # text -> object index in it

    def alloc(self, n):
        off = len(self.buf)
        self.buf += b'\x00' * _pad8(n)
        return off

    def put(self, off, data):
        self.buf[off:off + len(data)] = data

    @staticmethod
    def _message(mtype, body):
        body = body + b'\x00' * (_pad8(len(body)) - len(body))
        return struct.pack('<HHB3x', mtype, len(body), 0) + body

    def _texts(self, node, out):
        for v in node.attrs.values():
            if isinstance(v, str) and v not in out:
                out.append(v)
        for c in getattr(node, 'children', {}).values():
            self._texts(c, out)
        return out

    def write_gheap(self):
        """One global heap collection with every text attribute of the file (objects numbered
        from 1, each padded to 8 bytes, then the free-space object filling the rest)."""
        texts = self._texts(self.root, [])
        if not texts:
            return
        objs = b''
        for n, t in enumerate(texts, 1):
            b = t.encode('utf-8')
            self.gindex[t] = n
            objs += struct.pack('<HHIQ', n, 0, 0, len(b)) + b + b'\x00' * (_pad8(len(b)) - len(b))
        size = max(GCOL_MIN, 16 + len(objs) + 16)
        body = b'GCOL' + struct.pack('<B3xQ', 1, size) + objs
        body += struct.pack('<HHIQ', 0, 0, 0, size - len(body))
        self.gcol = self.alloc(size)
        self.put(self.gcol, body)

    def _attr_messages(self, attrs):
        out = []
        for name, value in attrs.items():
            nm = name.encode('utf-8') + b'\x00'
            if isinstance(value, str):
                dtm, dsm = _VLSTR_MESSAGE, _dataspace_message(())
                data = struct.pack('<IQI', len(value.encode('utf-8')), self.gcol, self.gindex[value])
                body = struct.pack('<BxHHH', 1, len(nm), len(dtm), len(dsm))
                body += nm + b'\x00' * (_pad8(len(nm)) - len(nm))
                body += dtm + b'\x00' * (_pad8(len(dtm)) - len(dtm))
                body += dsm + b'\x00' * (_pad8(len(dsm)) - len(dsm))
                out.append(self._message(0x000C, body + data))
                continue
            a = _as_array(value)
            dtm = _dtype_message(a.dtype)
            dsm = _dataspace_message(a.shape)
            body = struct.pack('<BxHHH', 1, len(nm), len(dtm), len(dsm))
            body += nm + b'\x00' * (_pad8(len(nm)) - len(nm))
            body += dtm + b'\x00' * (_pad8(len(dtm)) - len(dtm))
            body += dsm + b'\x00' * (_pad8(len(dsm)) - len(dsm))
            body += a.astype(a.dtype.newbyteorder('<')).tobytes()
            out.append(self._message(0x000C, body))
        return out

    def _object_header(self, messages):
        payload = b''.join(messages)
        hdr = struct.pack('<BxHII4x', 1, len(messages), 1, len(payload))
        off = self.alloc(len(hdr) + len(payload))
        self.put(off, hdr + payload)
        return off

    def write_group(self, g):
        names = sorted(g.children)
        # local heap: empty name at offset 0, then the member names
        heap_data = bytearray(b'\x00' * 8)
        name_off = {}
        for n in names:
            name_off[n] = len(heap_data)
            b = n.encode('utf-8') + b'\x00'
            heap_data += b + b'\x00' * (_pad8(len(b)) - len(b))
        heap_data_addr = self.alloc(len(heap_data))
        self.put(heap_data_addr, bytes(heap_data))
        heap_addr = self.alloc(32)
        self.put(heap_addr, b'HEAP' + struct.pack('<B3xQQQ', 0, len(heap_data), UNDEF, heap_data_addr))
        # children first, so their header addresses are known
        entries = []
        for n in names:
            child = g.children[n]
            if isinstance(child, _Group):
                addr, btree, heap = self.write_group(child)
                entries.append((n, addr, 1, btree, heap))
            else:
                addr = self.write_dataset(child)
                entries.append((n, addr, 0, 0, 0))
        # symbol table nodes, 2*LEAF_K entries each
        cap = 2 * LEAF_K
        snods = []
        for s in range(0, max(len(entries), 1), cap):
            chunk = entries[s:s + cap]
            body = b'SNOD' + struct.pack('<BxH', 1, len(chunk))
            for (n, addr, cache, bt, hp) in chunk:
                scratch = struct.pack('<QQ', bt, hp) if cache == 1 else b'\x00' * 16
                body += struct.pack('<QQI4x', name_off[n], addr, cache) + scratch
            body += b'\x00' * (40 * (cap - len(chunk)))
            off = self.alloc(len(body))
            self.put(off, body)
            snods.append((off, name_off[chunk[-1][0]] if chunk else 0))
        if len(snods) > 2 * INTERNAL_K:
            raise ValueError('group with more than {} members'.format(cap * 2 * INTERNAL_K))
        # one level-0 B-tree node over the SNODs
        body = b'TREE' + struct.pack('<BBHQQ', 0, 0, len(snods) if entries else 0, UNDEF, UNDEF)
        body += struct.pack('<Q', 0)   # key 0: empty name
        for off, last in snods if entries else []:
            body += struct.pack('<QQ', off, last)
        # a node always occupies room for 2K children and 2K+1 keys
        body += b'\x00' * (24 + 8 + 16 * 2 * INTERNAL_K - len(body))
        btree = self.alloc(len(body))
        self.put(btree, body)
        msgs = [self._message(0x0011, struct.pack('<QQ', btree, heap_addr))]
        msgs += self._attr_messages(g.attrs)
        return self._object_header(msgs), btree, heap_addr

    def write_dataset(self, ds):
        a = ds.data
        if a.dtype.byteorder == '>':
            a = a.astype(a.dtype.newbyteorder('<'))
        raw = a.tobytes()
        data_addr = self.alloc(len(raw))
        self.put(data_addr, raw)
        msgs = [self._message(0x0001, _dataspace_message(a.shape)),
                self._message(0x0003, _dtype_message(a.dtype)),
                self._message(0x0008, struct.pack('<BBQQ', 3, 1, data_addr, len(raw)))]
        msgs += self._attr_messages(ds.attrs)
        return self._object_header(msgs)

    def write(self, path):
        sb = self.alloc(96)
        self.write_gheap()
        root_addr, btree, heap = self.write_group(self.root)
        eof = len(self.buf)
        hdr = SIGNATURE + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack('<HHI', LEAF_K, INTERNAL_K, 0)
        hdr += struct.pack('<QQQQ', 0, UNDEF, eof, UNDEF)
        hdr += struct.pack('<QQI4xQQ', 0, root_addr, 1, btree, heap)
        self.put(sb, hdr)
        with open(path, 'wb') as f:
            f.write(bytes(self.buf))


# ----------------------------------------------------------------------------- reader
class Node:
    """A group (``children``) or dataset (``data``) read from a file, with ``attrs``."""

    def __init__(self, name):
        self.name = name
        self.attrs = {}
        self.children = None
        self.data = None

    def __getitem__(self, path):
        node = self
        for part in [p for p in path.split('/') if p]:
            node = node.children[part]
        return node

    def keys(self):
        return list(self.children or {})

    def __contains__(self, path):
        try:
            self[path]
            return True
        except (KeyError, TypeError):
            return False


class _Reader:
    def __init__(self, buf):
        self.b = buf

    def u(self, fmt, off):
        return struct.unpack_from('<' + fmt, self.b, off)

    def messages(self, addr):
        """(type, body) of every message of a version-1 object header, with continuations."""
        ver, nmsg, _, size = self.u('BxHII', addr)
        if ver != 1:
            raise ValueError('object header version {} not supported'.format(ver))
        blocks = [(addr + 16, size)]
        out = []
        while blocks:
            off, size = blocks.pop(0)
            end = off + size
            while off + 8 <= end:
                mtype, msize, _ = self.u('HHB', off)
                body = self.b[off + 8:off + 8 + msize]
                if mtype == 0x0010:   # continuation
                    caddr, clen = struct.unpack_from('<QQ', body, 0)
                    blocks.append((caddr, clen))
                else:
                    out.append((mtype, body))
                off += 8 + msize
        return out

    @staticmethod
    def dtype(body):
        cls = body[0] & 0x0F
        bits0 = body[1]
        size = struct.unpack_from('<I', body, 4)[0]
        order = '>' if bits0 & 1 else '<'
        if cls == 1:
            return np.dtype('{}f{}'.format(order, size)), 8 + 12
        if cls == 0:
            signed = bool(bits0 & 0x08)
            return np.dtype('{}{}{}'.format(order, 'i' if signed else 'u', size)), 8 + 4
        if cls == 3:
            return np.dtype('S{}'.format(size)), 8
        if cls == 9:
            return None, None   # variable length
        raise ValueError('datatype class {} not supported'.format(cls))

    @staticmethod
    def dataspace(body):
        ver, ndim, flags = body[0], body[1], body[2]
        off = 8 if ver == 1 else 4
        dims = struct.unpack_from('<' + 'Q' * ndim, body, off)
        return tuple(dims)

    def attribute(self, body):
        ver = body[0]
        if ver != 1:
            return None, None
        nlen, tlen, slen = struct.unpack_from('<HHH', body, 2)
        off = 8
        name = bytes(body[off:off + nlen]).split(b'\x00')[0].decode('utf-8')
        off += _pad8(nlen)
        dt, _ = self.dtype(body[off:off + tlen])
        off += _pad8(tlen)
        shape = self.dataspace(body[off:off + slen])
        off += _pad8(slen)
        if dt is None:   # variable-length string: (length, collection address, index)
            if shape != ():
                return name, None
            length, addr, index = struct.unpack_from('<IQI', body, off)
            text = self.gheap_object(addr, index)
            return name, None if text is None else text[:length].decode('utf-8')
        n = int(np.prod(shape)) if shape else 1
        a = np.frombuffer(bytes(body[off:off + n * dt.itemsize]), dtype=dt).reshape(shape)
        if dt.kind == 'S':
            v = a[()] if shape == () else a
            return name, (v.split(b'\x00')[0].decode('utf-8') if shape == () else v)
        return name, (a[()] if shape == () else a.copy())

    def gheap_object(self, addr, index):
        """Object ``index`` of the global heap collection at ``addr`` (None if absent)."""
        if self.b[addr:addr + 4] != b'GCOL':
            return None
        size = self.u('Q', addr + 8)[0]
        off = addr + 16
        while off + 16 <= addr + size:
            idx, _, _, osize = self.u('HHIQ', off)
            if idx == 0:
                return None
            if idx == index:
                return bytes(self.b[off + 16:off + 16 + osize])
            off += 16 + _pad8(osize)
        return None

    def obj(self, name, addr):
        node = Node(name)
        msgs = self.messages(addr)
        layout = dtype = shape = None
        for mtype, body in msgs:
            if mtype == 0x0011:
                btree, heap = struct.unpack_from('<QQ', body, 0)
                node.children = self.group(btree, heap)
            elif mtype == 0x0001:
                shape = self.dataspace(body)
            elif mtype == 0x0003:
                dtype, _ = self.dtype(body)
            elif mtype == 0x0008:
                layout = body
            elif mtype == 0x000C:
                k, v = self.attribute(body)
                if k is not None:
                    node.attrs[k] = v
        if layout is not None:
            ver, cls = layout[0], layout[1]
            if ver != 3 or cls not in (0, 1):
                raise ValueError('only contiguous or compact datasets are supported')
            n = int(np.prod(shape)) if shape else 1
            if cls == 1:
                daddr, size = struct.unpack_from('<QQ', layout, 2)
                raw = bytes(self.b[daddr:daddr + n * dtype.itemsize]) if daddr != UNDEF else b''
            else:
                size = struct.unpack_from('<H', layout, 2)[0]
                raw = bytes(layout[4:4 + size])
            if len(raw) < n * dtype.itemsize:
                raw = raw + b'\x00' * (n * dtype.itemsize - len(raw))
            node.data = np.frombuffer(raw, dtype=dtype).reshape(shape).copy()
        return node

    def heap_names(self, heap):
        sig, ver, size, free, daddr = struct.unpack_from('<4sB3xQQQ', self.b, heap)
        if sig != b'HEAP':
            raise ValueError('bad local heap')
        return daddr

    def group(self, btree, heap):
        daddr = self.heap_names(heap)
        children = {}
        self._btree(btree, daddr, children)
        return children

    def _btree(self, addr, daddr, children):
        sig, ntype, level, used = struct.unpack_from('<4sBBH', self.b, addr)
        if sig != b'TREE':
            raise ValueError('bad B-tree node')
        off = addr + 24 + 8
        for _ in range(used):
            child = struct.unpack_from('<Q', self.b, off)[0]
            off += 16
            if level > 0:
                self._btree(child, daddr, children)
            else:
                self._snod(child, daddr, children)

    def _snod(self, addr, daddr, children):
        sig, ver, n = struct.unpack_from('<4sBxH', self.b, addr)
        if sig != b'SNOD':
            raise ValueError('bad symbol table node')
        off = addr + 8
        for _ in range(n):
            noff, oaddr = struct.unpack_from('<QQ', self.b, off)
            raw = bytes(self.b[daddr + noff:daddr + noff + 1024])
            name = raw.split(b'\x00')[0].decode('utf-8')
            children[name] = self.obj(name, oaddr)
            off += 40


def read(path):
    """Read a whole file into a tree of :class:`Node` (root group)."""
    with open(path, 'rb') as f:
        buf = f.read()
    base = buf.find(SIGNATURE)
    if base < 0:
        raise ValueError('not an HDF5 file')
    if base:
        buf = buf[base:]
    ver = buf[8]
    if ver not in (0, 1):
        raise ValueError('superblock version {} not supported'.format(ver))
    if buf[13] != 8 or buf[14] != 8:
        raise ValueError('only 8-byte offsets and lengths are supported')
    off = 24 + (4 if ver == 1 else 0)
    # base, free-space, eof, driver, then the root symbol table entry
    off += 32
    _, root_addr = struct.unpack_from('<QQ', buf, off)
    r = _Reader(memoryview(buf))
    return r.obj('', root_addr)
