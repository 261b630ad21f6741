"""CPU check of the GPU kernels' PML index arithmetic (no GPU needed).

Mirrors, in numpy, how ``h_half_step``/``e_half_step`` (gprmax_gb300/csrc/fdtd_kernels.cuh)
decide which nodes take which slab correction and which Phi element they use: the kernel
domains, ``axis_member`` (one slab per axis: minus, plus or none) and ``phi_index``. For every
slab and component it checks that the set of
(node, profile index) pairs equals the reference's slab loops
(``gprMax/pml_updates/pml_updates_{electric,magnetic}_*_ext.pyx``, ``ii = xf - i`` etc.), that
every Phi index lies inside that slab's array, and that no two nodes share a Phi element.
"""
import itertools

import numpy as np
import pytest

# slab positions in kernel order: x0, y0, z0, xmax, ymax, zmax
# tangential components (component index, Phi array 1 or 2) per slab axis, E and H
E_COMPS = {0: ((1, 1), (2, 2)), 1: ((0, 1), (2, 2)), 2: ((0, 1), (1, 2))}
H_COMPS = {0: ((4, 1), (5, 2)), 1: ((3, 1), (5, 2)), 2: ((3, 1), (4, 2))}


def axis_member(c, n, Tm, Tp, electric):
    """Vectorised ``axis_member``: (where, pr) with where 0 outside, 1 minus, 2 plus."""
    c = np.asarray(c)
    pm = (Tm - c) if electric else (Tm - 1 - c)
    pp = c - (n - Tp)
    inm = (pm >= 0) & (pm < Tm)
    inp = (pp >= 0) & (pp < Tp)
    where = np.where(inp, 2, np.where(inm, 1, 0))
    pr = np.where(inp, pp, pm)
    return where, pr


def phi_index(axis, i, j, k, p, T, ny, nz):
    if axis == 0:
        return (p * ny + j) * nz + k
    if axis == 1:
        return (i * T + p) * nz + k
    return (i * ny + j) * T + p


def kernel_pairs(n3, thick, electric):
    """{(slab, comp): set of (i, j, k, p, phi_index)} as the kernels compute them."""
    nx, ny, nz = n3
    if electric:
        dom = [np.arange(nx), np.arange(ny), np.arange(nz)]
    else:
        dom = [np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1)]
    I, J, K = np.meshgrid(*dom, indexing='ij')
    inside = np.ones(I.shape, bool) if electric else (I < nx) & (J < ny) & (K < nz)
    out = {}
    for axis in range(3):
        Tm, Tp = thick[axis], thick[axis + 3]
        where, pr = axis_member((I, J, K)[axis], n3[axis], Tm, Tp, electric)
        for side, s in ((1, axis), (2, axis + 3)):
            T = thick[s]
            if not T:
                continue
            mem = (where == side) & inside
            comps = (E_COMPS if electric else H_COMPS)[axis]
            for comp, arr in comps:
                ii, jj, kk, pp = I[mem], J[mem], K[mem], pr[mem]
                idx = phi_index(axis, ii, jj, kk, pp, T, ny, nz)
                out[(s, comp)] = set(zip(ii.tolist(), jj.tolist(), kk.tolist(), pp.tolist(),
                                         idx.tolist()))
    return out


def reference_pairs(n3, thick, electric):
    """{(slab, comp): set of (ii, jj, kk, p)} from the reference's slab loops."""
    nx, ny, nz = n3
    out = {}
    for s in range(6):
        T = thick[s]
        if not T:
            continue
        axis, minus = s % 3, s < 3
        # slab extents as build_pmls makes them (pml.py:367-429)
        ext = [[0, nx], [0, ny], [0, nz]]
        ext[axis] = [0, T] if minus else [n3[axis] - T, n3[axis]]
        (xs, xf), (ys, yf), (zs, zf) = ext
        pairs = set()
        for i, j, k in itertools.product(range(xf - xs), range(yf - ys), range(zf - zs)):
            loc = [i, j, k]
            node = [i + xs, j + ys, k + zs]
            f = (xf, yf, zf)[axis]
            if minus:
                node[axis] = f - loc[axis] if electric else f - (loc[axis] + 1)
            pairs.add((node[0], node[1], node[2], loc[axis]))
        for comp, arr in (E_COMPS if electric else H_COMPS)[axis]:
            out[(s, comp)] = pairs
    return out


CASES = [((12, 10, 9), (3, 2, 2, 3, 2, 2)), ((13, 11, 14), (4, 0, 3, 2, 3, 0)),
         ((9, 12, 10), (0, 5, 0, 0, 4, 3)), ((30, 28, 26), (6, 6, 6, 6, 6, 6))]


@pytest.mark.parametrize('n3,thick', CASES)
@pytest.mark.parametrize('electric', [True, False])
def test_slab_nodes_and_phi_indices(n3, thick, electric):
    nx, ny, nz = n3
    k = kernel_pairs(n3, thick, electric)
    r = reference_pairs(n3, thick, electric)
    assert set(k) == set(r)
    for key in r:
        s = key[0]
        T = thick[s]
        axis = s % 3
        nu = ny if axis == 0 else nx
        nv = ny if axis == 2 else nz
        ocount = T * nu * nv
        got = k[key]
        assert {q[:4] for q in got} == r[key], 'slab {} comp {}: node sets differ'.format(*key)
        idx = [q[4] for q in got]
        assert min(idx) >= 0 and max(idx) < ocount, 'slab {} comp {}: Phi index out of range'.format(*key)
        assert len(set(idx)) == len(idx), 'slab {} comp {}: Phi element shared'.format(*key)


def _boxes(lib, n3, thick, electric):
    import ctypes
    out = np.zeros((6, 10), dtype=np.int32)
    t = np.asarray(thick, dtype=np.int32)
    rc = lib.gbf_sweep_boxes(n3[0], n3[1], n3[2], t.ctypes.data_as(ctypes.c_void_p),
                             1 if electric else 0, out.ctypes.data_as(ctypes.c_void_p))
    assert rc == 0
    return out


@pytest.fixture(scope='module')
def native_lib():
    from gprmax_gb300 import _native
    _native.build()
    return _native.load()


@pytest.mark.parametrize('n3,thick', CASES + [((7, 9, 5), (0, 0, 0, 0, 0, 0)),
                                              ((400, 400, 200), (10,) * 6)])
@pytest.mark.parametrize('electric', [True, False])
def test_sweep_boxes_cover_the_domain_once(native_lib, n3, thick, electric):
    """The boxes the half-step kernels walk (host ``make_boxes``): every node of the kernel's
    domain exactly once, the walk's virtual index contiguous, and the core box (box 0) only on
    rows whose i and j have both neighbours inside the arrays and lie outside the x and y
    slabs (the kernels handle z per node)."""
    nx, ny, nz = n3
    ext = (nx, ny, nz) if electric else (nx + 1, ny + 1, nz + 1)
    boxes = _boxes(native_lib, n3, thick, electric)
    seen = np.zeros(ext, dtype=np.int32)
    start = 0
    for b, (i0, j0, k0, bi, bj, bk, ksplit, kgap, st, count) in enumerate(boxes):
        assert st == start
        start += count
        if count == 0:
            continue
        assert count == bi * bj * bk
        c = np.arange(bk)
        kk = k0 + c + np.where(c >= ksplit, kgap, 0)
        ii = i0 + np.arange(bi)
        jj = j0 + np.arange(bj)
        assert ii.min() >= 0 and jj.min() >= 0 and kk.min() >= 0
        assert ii.max() < ext[0] and jj.max() < ext[1] and kk.max() < ext[2]
        seen[np.ix_(ii, jj, kk)] += 1
        if b == 0:
            for axis, idx in enumerate((ii, jj)):
                where, _ = axis_member(idx, n3[axis], thick[axis], thick[axis + 3], electric)
                assert not where.any(), 'core box reaches an x or y slab'
                assert idx.min() >= 1 and idx.max() <= n3[axis] - 1
    assert start == np.prod(ext)
    assert (seen == 1).all()
