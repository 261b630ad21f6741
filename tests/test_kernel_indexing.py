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


def _fused_tiles(lib, n3, tj, nch):
    import ctypes
    out = np.zeros(6, dtype=np.int32)
    rc = lib.gbf_fused_tiles(n3[0], n3[1], n3[2], tj, nch, out.ctypes.data_as(ctypes.c_void_p))
    assert rc == 0
    return [int(v) for v in out]


@pytest.mark.parametrize('n3', [(7, 9, 5), (23, 19, 40), (12, 30, 62), (31, 8, 31)])
@pytest.mark.parametrize('tj', [7, 15])
@pytest.mark.parametrize('nch', [1, 3, 7, 1000])
def test_fused_tiles_cover_the_grid_once(native_lib, n3, tj, nch):
    """The fused step's tiling (fused_step.cuh, decomposition from the library's own
    ``gbf_fused_tiles``), restated: block b has tj + 1 warps; warp w, lane l works on row
    j = tile * tj - 1 + w and column k = seg * K - 1 + l over planes [i0 - 1 or 0, i1); warp 0
    and lane 0 are halo. Checks that every H node of [0,nx]x[0,ny]x[0,nz] and every E node of
    [0,nx)x[0,ny)x[0,nz) is stored by exactly one thread, that every guarded load lies inside
    the arrays, and that each E update finds the H values it needs (j-1 from the warp below,
    k-1 from the lane below, i-1 from the same thread's previous plane)."""
    nx, ny, nz = n3
    nseg, njt, nchunks, L, nblocks, K = _fused_tiles(native_lib, n3, tj, nch)
    assert K == 31 and nblocks == nseg * njt * nchunks
    assert nseg * K >= nz + 1 and njt * tj >= ny + 1 and nchunks * L >= nx + 1
    assert (nchunks - 1) * L < nx + 1
    hcount = np.zeros((nx + 1, ny + 1, nz + 1), dtype=np.int32)
    ecount = np.zeros((nx, ny, nz), dtype=np.int32)
    lane = np.arange(32)
    for b in range(nblocks):
        seg, rest = b % nseg, b // nseg
        jt, ch = rest % njt, rest // njt
        k = seg * K - 1 + lane
        kv = (k >= 0) & (k <= nz)
        assert ((k >= 0) | (lane == 0)).all()        # only the halo lane can fall below 0
        i0 = ch * L
        i1 = min(i0 + L, nx + 1)
        assert i0 <= nx
        ib = i0 - 1 if i0 > 0 else 0
        for w in range(tj + 1):
            j = jt * tj - 1 + w
            jv = 0 <= j <= ny
            own = (lane > 0) & (w > 0) & kv & jv
            eown = (lane > 0) & (w > 0) & (k < nz) & (j < ny)
            assert j >= 0 or w == 0                  # only the halo warp can fall below 0
            for i in range(ib, i1):
                # loads at planes i .. i + 2 are guarded by pl <= nx and the node's validity;
                # the last lane's k + 1 and the top warp's j + 1 by k + 1 <= nz, j + 1 <= ny
                if jv:
                    assert k[kv].min() >= 0 and k[kv].max() <= nz
                halo = i < i0
                if not halo and jv:
                    hcount[i, j, k[own]] += 1
                if not halo and i < nx and eown.any():
                    ecount[i, j, k[eown]] += 1
                    # H(j - 1) from warp w - 1 >= 0 of the same block; H(k - 1) from lane - 1 >= 0;
                    # H(i - 1) formed by this thread at the previous plane i - 1 >= ib
                    assert w - 1 >= 0 and (lane[eown] >= 1).all()
                    assert i == 0 or i - 1 >= ib
    assert (hcount == 1).all(), 'H nodes stored {}..{} times'.format(hcount.min(), hcount.max())
    assert (ecount == 1).all(), 'E nodes stored {}..{} times'.format(ecount.min(), ecount.max())


def test_fused_tiles_at_the_benchmark_size(native_lib):
    """The decomposition of the 400 x 400 x 200 soil covers it with whole tiles and stays far
    inside int32 node indices."""
    nseg, njt, nchunks, L, nblocks, K = _fused_tiles(native_lib, (400, 400, 200), 7, 2)
    assert (nseg, njt) == (7, 58)
    assert nchunks * L >= 401 and (nchunks - 1) * L < 401
    assert nblocks == 7 * 58 * nchunks
    assert 401 * 401 * 201 < 2 ** 31


def test_pack_ids_on_the_host(native_lib):
    """``gbf_pack_ids`` (host arithmetic): the E and H words are the three 10-bit IDs of each
    node, the largest ID is reported, and IDs above 1023 are refused."""
    import ctypes
    rng = np.random.default_rng(3)
    n = 100003
    ID = rng.integers(0, 1024, size=(6, n), dtype=np.uint32)
    pe = np.zeros(n, np.uint32)
    ph = np.zeros(n, np.uint32)
    mx = ctypes.c_uint32(0)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    assert native_lib.gbf_pack_ids(p(ID), n, p(pe), p(ph), ctypes.byref(mx)) == 0
    np.testing.assert_array_equal(pe, ID[0] | (ID[1] << 10) | (ID[2] << 20))
    np.testing.assert_array_equal(ph, ID[3] | (ID[4] << 10) | (ID[5] << 20))
    assert mx.value == ID.max()
    ID[4, 777] = 1024
    assert native_lib.gbf_pack_ids(p(ID), n, p(pe), p(ph), ctypes.byref(mx)) == -1
    assert mx.value == 1024
    # the E words only: H IDs are not read
    pe2 = np.zeros(n, np.uint32)
    assert native_lib.gbf_pack_ids(p(ID), n, p(pe2), None, ctypes.byref(mx)) == 0
    np.testing.assert_array_equal(pe2, ID[0] | (ID[1] << 10) | (ID[2] << 20))
    assert mx.value == ID[:3].max()


def _staged_consumers():
    """kStagedC of staged.cuh: consumer warps per block, one node per consumer thread per
    chunk (chunks of L = 32 kStagedC nodes, copies of L + 8 floats)."""
    import os
    import re
    src = open(os.path.join(os.path.dirname(os.path.abspath(__file__)), '..', 'gprmax_gb300',
                            'csrc', 'staged.cuh')).read()
    assert re.search(r'kStageL = 32 \* kStagedC;', src)
    assert re.search(r'kStageSpan = kStageL \+ 8;', src)
    return int(re.search(r'kStagedC = (\d+);', src).group(1))


def _fast_div(d):
    """FastDiv's constants for divisor d (gbfdtd.cu fast_div) and its quotient function."""
    l = 0
    while (1 << l) < d:
        l += 1
    m = ((1 << (31 + l)) + d - 1) // d
    assert m < 2 ** 32
    return lambda n: ((np.asarray(n, dtype=np.uint64) * np.uint64(m)) >> np.uint64(32)) >> np.uint64(l - 1)


def test_fast_division():
    """The multiply-high division the staged sweep uses for n / sy and n / cpp is exact for
    every n in [0, 2^31) (theorem 4.2 of Granlund and Montgomery, PLDI 1994): checked on every
    divisor up to 1200 and on the divisors of large grids, at the multiples of d and their
    neighbours and at random n."""
    rng = np.random.default_rng(5)
    top = 2 ** 31 - 1
    for d in list(range(2, 1201)) + [4095, 4097, 8191, 8192, 32769, 65535, 65536, 80601, 80602]:
        q = _fast_div(d)
        mult = np.arange(0, top, d * max(1, top // d // 2000), dtype=np.int64)
        n = np.concatenate([mult, mult + 1, mult + d - 1, rng.integers(0, top, 2000), [top]])
        n = n[(n >= 0) & (n <= top)]
        np.testing.assert_array_equal(q(n).astype(np.int64), n // d)


def _staged_sweep(lib, n3, thick, electric=True, planes=None):
    """The staged sweep's chunks (E, or H), restated: host geometry (gbfdtd.cu staged_geom) and
    device arithmetic (staged.cuh stage_chunk's header, the consumer loop). Checks every copy
    and every shared-memory read a node makes, and returns the flat indices of the updated
    nodes and each chunk's core flag."""
    nx, ny, nz = n3
    T = 32 * _staged_consumers()
    L = T
    W = L + 8
    sy, sx = nz + 1, (ny + 1) * (nz + 1)
    npts = (nx + 1) * sx
    ncomp = (npts + 63) & ~63
    assert ncomp >= 2 * W, 'grid too small for the staged sweep'
    i0, j0, _, bi, bj, _, _, _, _, count = _boxes(lib, n3, thick, electric)[0]
    ilo, ihi = i0, i0 + (bi if count else 0)
    jlo, jhi = j0, j0 + (bj if count else 0)
    plen = ny * sy if electric else sx
    nplanes = nx if electric else nx + 1
    cpp = (plen + 3 + L - 1) // L
    amax = ncomp - W
    c = np.arange(nplanes * cpp, dtype=np.int64)
    if planes is not None:
        c = np.concatenate([np.arange(p * cpp, (p + 1) * cpp) for p in planes])
    i = c if cpp == 1 else _fast_div(cpp)(c).astype(np.int64)
    np.testing.assert_array_equal(i, c // cpp)
    s = ((i * sx) & ~3) + (c - i * cpp) * L
    dj, di = (-sy, -sx) if electric else (sy, sx)
    clamp = lambda a: np.clip(a, 0, amax)
    aE, aH = clamp(s), clamp(s - 4 if electric else s)
    aJ, aI = clamp((s + dj) & ~3), clamp((s + di) & ~3)
    for a in (aE, aH, aJ, aI):      # 16-byte aligned starts, copies inside their arrays
        assert (a % 4 == 0).all() and (a >= 0).all() and (a + W <= ncomp).all()
    shE, shH = s - aE, s - aH
    shJ, shI = s + dj - aJ, s + di - aI
    # the header's row and column of node s, and each consumer thread's offsets from it
    by_sy = _fast_div(sy)
    f = s - i * sx
    jf = np.where(f >= 0, by_sy(np.maximum(f, 0)).astype(np.int64), -1)
    kf = f - jf * sy
    assert ((kf >= 0) & (kf < sy)).all()
    t = np.arange(T)
    tq = by_sy(t).astype(np.int64)
    tr = t - tq * sy
    J = jf[:, None] + tq[None, :]
    K = kf[:, None] + tr[None, :]
    wrap = K >= sy
    K = np.where(wrap, K - sy, K)
    J = np.where(wrap, J + 1, J)
    r = t[None, :]
    assert (J * sy + K == f[:, None] + r).all() and (K >= 0).all() and (K < sy).all()
    I = np.broadcast_to(i[:, None], J.shape)
    # every shared-memory read a node makes lies inside its stream's span
    inspan = lambda x, m: ((x >= 0) & (x < W))[m].all()
    if electric:
        valid = (J >= 0) & (J < ny) & (K < nz)
        assert inspan(shE[:, None] + r, valid)                    # E, packed word, pole state
        assert inspan(shH[:, None] + r, valid)                    # own H
        assert inspan(shH[:, None] + r - 1, valid & (K >= 1))     # H at k - 1
        assert inspan(shJ[:, None] + r, valid & (J >= 1))         # H at j - 1
        assert inspan(shI[:, None] + r, valid & (I >= 1))         # H at i - 1
    else:
        valid = (J >= 0) & (J <= ny)
        assert (shH == shE).all()
        assert inspan(shE[:, None] + r, valid)                    # own E, H, packed word
        assert inspan(shE[:, None] + r + 1, valid & (K < nz))     # E at k + 1
        assert inspan(shJ[:, None] + r, valid & (J < ny))         # E at j + 1
        assert inspan(shI[:, None] + r, valid & (I < nx))         # E at i + 1
    # the core test: a core chunk's nodes lie in the core box, so its node code may skip the x
    # and y tests
    jl = by_sy(np.minimum(f + L - 1, plen - 1)).astype(np.int64)
    core = (i >= ilo) & (i < ihi) & (jf >= jlo) & (jl < jhi)
    m = valid & core[:, None]
    assert ((I[m] >= ilo) & (I[m] < ihi) & (J[m] >= jlo) & (J[m] < jhi)).all()
    assert (I[m] >= 1).all() and (J[m] >= 1).all() and (I[m] < nx).all() and (J[m] < ny).all()
    # the z slabs' Phi state: the copies of the chunk's rows hold every element its slab nodes
    # read, for each CFS order (the second order's elements ocount further on)
    Tz = (thick[2], thick[5])
    if max(Tz):
        zspan = ((((L + 2) // sy + 2) * max(Tz) + 3 + 3) // 4) * 4
        j0 = np.maximum(jf, 0)
        j1 = np.minimum(jl, ny - 1)
        zrows = (j0 <= j1) & (True if electric else (i < nx))
        for side in (0, 1):
            T = Tz[side]
            if not T:
                continue
            where, pr = axis_member(K, nz, Tz[0], Tz[1], electric)
            node = valid & (where == side + 1)
            if not electric:
                node &= (I < nx) & (J < ny) & (K < nz)
            assert not (node & ~zrows[:, None]).any()
            ocount = T * nx * ny
            pidx = (I * ny + J) * T + pr
            lo = (i * ny + j0) * T
            for o in range(2):
                a = (lo + o * ocount) & ~3
                off = pidx + o * ocount - a[:, None]
                assert ((off >= 0) & (off < zspan))[node].all()
    idx = (s[:, None] + r)[valid]
    assert (idx == (I * sx + J * sy + K)[valid]).all()
    return idx, core


@pytest.mark.parametrize('n3,thick', [((13, 11, 14), (4, 0, 3, 2, 3, 0)),
                                      ((30, 28, 26), (6, 6, 6, 6, 6, 6)),
                                      ((41, 7, 9), (0, 0, 0, 0, 0, 0)),
                                      ((20, 18, 16), (0, 0, 0, 0, 0, 0)),
                                      ((20, 37, 64), (3, 5, 10, 2, 4, 10)),
                                      ((60, 50, 40), (10, 0, 5, 10, 7, 0))])
@pytest.mark.parametrize('electric', [True, False])
def test_staged_sweep_covers_the_domain_once(native_lib, n3, thick, electric):
    """The staged half-steps (staged.cuh) update every node of their domain exactly once, read
    only inside the spans their bulk copies filled (copies aligned, inside their arrays), and
    run the core node code only on chunks inside the core box."""
    nx, ny, nz = n3
    W = 32 * _staged_consumers() + 8
    if ((nx + 1) * (ny + 1) * (nz + 1) + 63) & ~63 < 2 * W:
        pytest.skip('grid below the staged sweep\'s minimum')
    idx, core = _staged_sweep(native_lib, n3, thick, electric)
    sy, sx = nz + 1, (ny + 1) * (nz + 1)
    ext = (nx, ny, nz) if electric else (nx + 1, ny + 1, nz + 1)
    ii, jj, kk = np.meshgrid(*(np.arange(e) for e in ext), indexing='ij')
    want = np.sort((ii * sx + jj * sy + kk).ravel())
    np.testing.assert_array_equal(np.sort(idx), want)


@pytest.mark.parametrize('electric', [True, False])
def test_staged_sweep_at_the_benchmark_size(native_lib, electric):
    """The 400 x 400 x 200 soil: the first, second, a middle, the second-last and the last
    planes, checked as above; most chunks of a middle plane take the core code."""
    n3, thick = (400, 400, 200), (10,) * 6
    planes = (0, 1, 11, 200, 389, 390, 398, 399) + (() if electric else (400,))
    idx, core = _staged_sweep(native_lib, n3, thick, electric, planes)
    sy, sx = 201, 401 * 201
    for p in planes:
        got = np.sort(idx[(idx >= p * sx) & (idx < (p + 1) * sx)])
        ext = (400, 200) if electric else (401, 201)
        jj, kk = np.meshgrid(np.arange(ext[0]), np.arange(ext[1]), indexing='ij')
        np.testing.assert_array_equal(got, np.sort((p * sx + jj * sy + kk).ravel()))
    L = 32 * _staged_consumers()
    cpp = ((400 * 201 if electric else sx) + 3 + L - 1) // L
    mid = core[planes.index(200) * cpp:(planes.index(200) + 1) * cpp]
    assert mid.mean() > 0.85 and not core[:cpp].any()


def _batch_tile():
    """kBatchTile of fdtd_kernels.cuh: nodes a block sweeps per model visit."""
    import os
    import re
    src = open(os.path.join(os.path.dirname(os.path.abspath(__file__)), '..', 'gprmax_gb300',
                            'csrc', 'fdtd_kernels.cuh')).read()
    threads = int(re.search(r'constexpr int kThreads = (\d+);', src).group(1))
    per = int(re.search(r'constexpr int kBatchTile = (\d+) \* kThreads;', src).group(1))
    return per * threads, threads


def _box_walk(boxes, q, base, stride, lim):
    """h_sweep / e_sweep with TILE, restated with BoxWalk's incremental steps: the nodes one
    thread updates from virtual position q (its model's sweep starting at base) until lim."""
    out = []
    q -= base
    lim -= base
    for b, (i0, j0, k0, bi, bj, bk, ksplit, kgap, st, count) in enumerate(boxes):
        end = st + count
        if b > 0 and q >= lim:
            break
        if q >= end or q >= lim:
            continue
        plane = bj * bk
        r = q - st
        a, r = divmod(r, plane)
        bb, c = divmod(r, bk)
        sa, r = divmod(stride, plane)
        sb, sc = divmod(r, bk)
        while q < end and q < lim:
            out.append((i0 + a, j0 + bb, k0 + c + (kgap if c >= ksplit else 0)))
            q += stride
            c += sc
            if c >= bk:
                c -= bk
                bb += 1
            bb += sb
            if bb >= bj:
                bb -= bj
                a += 1
            a += sa
    return out


@pytest.mark.parametrize('electric', [True, False])
@pytest.mark.parametrize('grid', [1, 3, 7])
def test_batch_tiles_cover_every_model_once(native_lib, electric, grid):
    """The batched half-steps (h_half_step_batch, e_half_step_batch): ranges padded to whole
    tiles (gbf_batch_create), blocks taking tiles in turn and finding each tile's model, every
    thread sweeping its tile's nodes with the block's stride. Every node of every batched model
    is updated exactly once; a model with its own kernels (an empty range) is never entered."""
    tile, threads = _batch_tile()
    shapes = [((7, 9, 5), (2, 2, 1, 2, 2, 1)), ((12, 10, 14), (3, 3, 3, 3, 3, 3)),
              None, ((5, 6, 8), (0, 0, 0, 0, 0, 0)), ((20, 11, 9), (4, 0, 2, 4, 0, 2))]
    boxes, ranges = [], [0]
    for s in shapes:
        if s is None:   # a model with its own kernels
            boxes.append(None)
            ranges.append(ranges[-1])
            continue
        bx = _boxes(native_lib, s[0], s[1], electric)
        boxes.append(bx)
        n = int(bx[-1][8] + bx[-1][9])
        ranges.append(ranges[-1] + -(-n // tile) * tile)
    total = ranges[-1]
    seen = {}
    for blk in range(grid):
        m, mend = 0, -1
        for t0 in range(blk * tile, total, grid * tile):
            if t0 >= mend:
                while ranges[m + 1] <= t0:
                    m += 1
                mbeg, mend = ranges[m], ranges[m + 1]
            assert boxes[m] is not None and mbeg <= t0 and t0 + tile <= mend
            for t in range(threads):
                for node in _box_walk(boxes[m], t0 + t, mbeg, threads, t0 + tile):
                    key = (m,) + node
                    seen[key] = seen.get(key, 0) + 1
    for m, s in enumerate(shapes):
        if s is None:
            assert not any(k[0] == m for k in seen)
            continue
        nx, ny, nz = s[0]
        ext = (nx, ny, nz) if electric else (nx + 1, ny + 1, nz + 1)
        got = sorted(k[1:] for k in seen if k[0] == m)
        want = sorted(itertools.product(*(range(e) for e in ext)))
        assert got == want
    assert all(v == 1 for v in seen.values())
