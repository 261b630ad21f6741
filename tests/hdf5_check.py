"""A strict reader of the HDF5 file-format subset that gprMax ``.out`` files use (test
infrastructure: a second implementation, written from the HDF5 File Format Specification,
against which the package's own writer is checked; it shares no code with
``gprmax_gb300/hdf5.py``).

``walk(path)`` parses the file and returns a tree of groups, datasets and attributes with every
datatype, dataspace and layout decoded, while checking the structure as it goes:

* superblock version 0: signature, versions, 8-byte offsets and lengths, base address 0, no
  free-space or driver block, end-of-file address equal to the file size;
* version-1 object headers, their messages (8-byte aligned, inside the header or its
  continuation blocks), symbol-table groups (v1 B-tree of group nodes, local heap, SNOD
  symbol nodes with names in heap order), contiguous and compact dataset layouts, version-1
  attributes, variable-length strings in global heap collections;
* every block lies inside the file and no two blocks overlap.

Any violation raises ``FormatError``.
"""
import struct

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF


class FormatError(Exception):
    pass


def _need(cond, what):
    if not cond:
        raise FormatError(what)


class _File:
    def __init__(self, path):
        with open(path, 'rb') as f:
            self.b = f.read()
        self.blocks = []     # (start, end, what)
        self.gheaps = {}

    def take(self, start, size, what):
        _need(start != UNDEF and 0 <= start and start + size <= len(self.b),
              '{} at {} (+{}) lies outside the file ({} bytes)'.format(what, start, size, len(self.b)))
        for s, e, w in self.blocks:
            _need(start + size <= s or start >= e,
                  '{} [{}, {}) overlaps {} [{}, {})'.format(what, start, start + size, w, s, e))
        self.blocks.append((start, start + size, what))

    def u(self, fmt, off):
        return struct.unpack_from('<' + fmt, self.b, off)


def _datatype(body):
    cv, b0, b1, b2, size = struct.unpack_from('<BBBBI', body, 0)
    cls, ver = cv & 0x0F, cv >> 4
    _need(ver == 1, 'datatype version {}'.format(ver))
    bits = b0 | (b1 << 8) | (b2 << 16)
    if cls == 0:      # fixed point
        _need(bits & 1 == 0, 'big-endian integer')
        off, prec = struct.unpack_from('<HH', body, 8)
        _need(off == 0 and prec == 8 * size, 'integer bit offset/precision')
        return {'class': 'int', 'size': size, 'signed': bool(bits & 8)}
    if cls == 1:      # floating point
        _need(bits & 1 == 0, 'big-endian float')
        off, prec, eloc, esize, mloc, msize, ebias = struct.unpack_from('<HHBBBBI', body, 8)
        want = {4: (32, 23, 8, 0, 23, 127), 8: (64, 52, 11, 0, 52, 1023)}[size]
        _need((prec, eloc, esize, mloc, msize, ebias) == want and off == 0, 'IEEE float fields')
        return {'class': 'float', 'size': size}
    if cls == 3:      # fixed-length string
        return {'class': 'string', 'size': size, 'pad': bits & 0x0F, 'cset': (bits >> 4) & 0x0F}
    if cls == 9:      # variable length
        vtype, pad, cset = bits & 0x0F, (bits >> 4) & 0x0F, (bits >> 8) & 0x0F
        _need(vtype == 1, 'variable-length sequence (only strings are used)')
        base = _datatype(body[8:])
        return {'class': 'vlstring', 'size': size, 'pad': pad, 'cset': cset, 'base': base}
    raise FormatError('datatype class {}'.format(cls))


def _dataspace(body):
    ver, rank, flags = struct.unpack_from('<BBB', body, 0)
    _need(ver == 1, 'dataspace version {}'.format(ver))
    _need(body[3:8] == b'\0' * 5, 'dataspace reserved bytes')
    dims = struct.unpack_from('<{}Q'.format(rank), body, 8)
    if flags & 1:
        mx = struct.unpack_from('<{}Q'.format(rank), body, 8 + 8 * rank)
        _need(all(m == d or m == UNDEF for m, d in zip(mx, dims)), 'max dims')
    return tuple(dims)


def _gheap_string(f, addr, index):
    if addr not in f.gheaps:
        _need(f.b[addr:addr + 4] == b'GCOL', 'global heap signature at {}'.format(addr))
        ver, size = f.b[addr + 4], f.u('Q', addr + 8)[0]
        _need(ver == 1 and size >= 4096, 'global heap version/size')
        f.take(addr, size, 'global heap')
        objs = {}
        off = addr + 16
        while off + 16 <= addr + size:
            idx, ref, _, osize = f.u('HHIQ', off)
            if idx == 0:
                break
            objs[idx] = f.b[off + 16:off + 16 + osize]
            off += 16 + ((osize + 7) & ~7)
        f.gheaps[addr] = objs
    objs = f.gheaps[addr]
    _need(index in objs, 'global heap object {}'.format(index))
    return objs[index]


def _value(f, dt, shape, raw):
    n = int(np.prod(shape)) if shape else 1
    if dt['class'] == 'int':
        a = np.frombuffer(raw, dtype='<{}{}'.format('i' if dt['signed'] else 'u', dt['size']), count=n)
    elif dt['class'] == 'float':
        a = np.frombuffer(raw, dtype='<f{}'.format(dt['size']), count=n)
    elif dt['class'] == 'string':
        return raw[:dt['size']].split(b'\0')[0].decode()
    else:
        _need(n == 1 and dt['size'] == 16, 'one variable-length string')
        length, addr, index = struct.unpack_from('<IQI', raw, 0)
        s = _gheap_string(f, addr, index)
        _need(len(s) >= length, 'string length')
        return s[:length].decode()
    return a.reshape(shape) if shape else a[0]


def _messages(f, addr):
    ver, _, nmsg, refc, hsize = f.u('BBHII', addr)
    _need(ver == 1 and refc >= 1, 'object header version {} refcount {}'.format(ver, refc))
    f.take(addr, 16 + hsize, 'object header')
    blocks = [(addr + 16, hsize)]
    out = []
    total = 0
    while blocks:
        start, size = blocks.pop(0)
        off = start
        while off < start + size:
            mtype, msize, flags = f.u('HHB', off)
            _need(msize % 8 == 0 and off + 8 + msize <= start + size,
                  'message {} of {} bytes at {}'.format(mtype, msize, off))
            body = f.b[off + 8:off + 8 + msize]
            total += 1
            if mtype == 0x10:   # continuation
                caddr, clen = struct.unpack_from('<QQ', body, 0)
                f.take(caddr, clen, 'header continuation')
                blocks.append((caddr, clen))
            elif mtype:
                out.append((mtype, body))
            off += 8 + msize
    _need(total == nmsg, 'object header at {} lists {} messages, holds {}'.format(addr, nmsg, total))
    return out


def _attribute(f, body):
    ver, _, nsize, dsize, ssize = struct.unpack_from('<BBHHH', body, 0)
    _need(ver == 1, 'attribute version {}'.format(ver))
    p = 8
    name = body[p:p + nsize].split(b'\0')[0].decode()
    _need(body[p + nsize - 1] == 0, 'attribute name terminator')
    p += (nsize + 7) & ~7
    dt = _datatype(body[p:p + dsize])
    p += (dsize + 7) & ~7
    shape = _dataspace(body[p:p + ssize])
    p += (ssize + 7) & ~7
    return name, {'dtype': dt, 'shape': shape, 'value': _value(f, dt, shape, body[p:])}


def _object(f, addr):
    msgs = _messages(f, addr)
    attrs = {}
    node = {}
    kinds = [t for t, _ in msgs]
    for t, body in msgs:
        if t == 0x0C:
            name, a = _attribute(f, body)
            _need(name not in attrs, 'duplicate attribute ' + name)
            attrs[name] = a
    if 0x11 in kinds:           # group
        _, body = next(m for m in msgs if m[0] == 0x11)
        btree, heap = struct.unpack_from('<QQ', body, 0)
        node['kind'] = 'group'
        node['stab'] = (btree, heap)
        node['children'] = _group(f, btree, heap)
    else:
        _need(0x01 in kinds and 0x03 in kinds and 0x08 in kinds, 'dataset messages')
        shape = _dataspace(next(b for t, b in msgs if t == 0x01))
        dt = _datatype(next(b for t, b in msgs if t == 0x03))
        lay = next(b for t, b in msgs if t == 0x08)
        _need(lay[0] == 3, 'layout version {}'.format(lay[0]))
        n = int(np.prod(shape)) if shape else 1
        if lay[1] == 1:         # contiguous
            daddr, dsize = struct.unpack_from('<QQ', lay, 2)
            _need(dsize == n * dt['size'], 'contiguous size')
            f.take(daddr, dsize, 'dataset data')
            raw = f.b[daddr:daddr + dsize]
        elif lay[1] == 0:       # compact
            dsize = struct.unpack_from('<H', lay, 2)[0]
            raw = lay[4:4 + dsize]
        else:
            raise FormatError('layout class {}'.format(lay[1]))
        node['kind'] = 'dataset'
        node['dtype'] = dt
        node['shape'] = shape
        node['data'] = _value(f, dt, shape, raw)
    node['attrs'] = attrs
    return node


def _group(f, btree, heap):
    _need(f.b[heap:heap + 4] == b'HEAP' and f.b[heap + 4] == 0, 'local heap at {}'.format(heap))
    dsize, free, daddr = f.u('QQQ', heap + 8)
    f.take(heap, 32, 'local heap header')
    f.take(daddr, dsize, 'local heap data')
    _need(f.b[daddr:daddr + 1] == b'\0', 'local heap offset 0 is the empty name')

    def name_at(off):
        _need(off < dsize, 'name offset')
        return f.b[daddr + off:f.b.index(b'\0', daddr + off)].decode()
    children = {}
    order = []

    def tree(addr):
        _need(f.b[addr:addr + 4] == b'TREE', 'B-tree signature at {}'.format(addr))
        ntype, level, used = f.u('BBH', addr + 4)
        left, right = f.u('QQ', addr + 8)
        _need(ntype == 0, 'group B-tree node type')
        _need(used <= 2 * f.internal_k, 'B-tree node entries')
        f.take(addr, 24 + 8 * (4 * f.internal_k + 1), 'B-tree node')
        for q in range(used):
            child = f.u('Q', addr + 24 + 8 + 16 * q)[0]
            if level:
                tree(child)
            else:
                snod(child)

    def snod(addr):
        _need(f.b[addr:addr + 4] == b'SNOD' and f.b[addr + 4] == 1, 'symbol node at {}'.format(addr))
        n = f.u('H', addr + 6)[0]
        _need(n <= 2 * f.leaf_k, 'symbol node entries')
        f.take(addr, 8 + 40 * 2 * f.leaf_k, 'symbol node')
        for q in range(n):
            lo, oh, cache = f.u('QQI', addr + 8 + 40 * q)
            name = name_at(lo)
            order.append(name)
            _need(name not in children, 'duplicate link ' + name)
            children[name] = _object(f, oh)
    tree(btree)
    _need(order == sorted(order), 'symbol nodes out of name order')
    return children


def walk(path):
    """The file's tree: {'kind': 'group', 'attrs': {...}, 'children': {...}}."""
    f = _File(path)
    b = f.b
    _need(b[:8] == b'\x89HDF\r\n\x1a\n', 'signature')
    _need(tuple(b[8:12]) == (0, 0, 0, 0) and b[12] == 0, 'superblock/free-space/root/shared versions')
    _need(b[13] == 8 and b[14] == 8 and b[15] == 0, 'sizes of offsets and lengths')
    leaf_k, internal_k, flags = f.u('HHI', 16)
    _need(leaf_k > 0 and internal_k > 0 and flags == 0, 'group K / consistency flags')
    f.leaf_k, f.internal_k = leaf_k, internal_k
    base, free, eof, driver = f.u('QQQQ', 24)
    _need(base == 0 and free == UNDEF and driver == UNDEF, 'base / free-space / driver address')
    _need(eof == len(b), 'end-of-file address {} against {} bytes'.format(eof, len(b)))
    f.take(0, 56 + 40, 'superblock')
    lo, root, cache = f.u('QQI', 56)
    _need(cache == 1, 'root entry cache type')
    btree, heap = f.u('QQ', 56 + 24)
    node = _object(f, root)
    _need(node['kind'] == 'group', 'root is a group')
    # the root entry's scratch pad names the B-tree and heap of its Symbol Table message
    _need(node['stab'] == (btree, heap), 'root scratch pad')
    return node
