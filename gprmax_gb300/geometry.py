"""Voxelisation of geometry primitives into the solid, rigid and ID arrays.

Semantics follow ``gprMax/geometry_primitives_ext.pyx``: a primitive built without dielectric
smoothing writes the solid array, marks its cells rigid and writes the 12 edge IDs of each
cell (``build_voxel`` :314-377; ``build_box`` :618-691 writes whole index ranges instead);
with smoothing it only writes the solid array and clears the rigid flags, and the edge IDs are
derived later by :mod:`gprmax_gb300.yee_build`. Cell selection for spheres and cylinders uses
the reference's fp32 geometry inputs (``build_sphere`` :873, ``build_cylinder`` :692).
All writes here are whole-array numpy operations; one primitive writes one material, so the
order of its cells does not matter. On a grid built in device memory (``G.geom``, see
:mod:`gprmax_gb300.devgeom`) the same cell selections are handed to the device builders.
"""
import numpy as np

from .exceptions import CmdInputError
from .utilities import round_value

# rigidE holds 12 edge flags per cell, rigidH 6 (``yee_cell_setget_rigid_ext.pyx:24-157``)


def _set_cells(G, I, J, K, numID, numIDx, numIDy, numIDz, averaging):
    """``build_voxel`` applied to every cell (I, J, K)."""
    G.solid[I, J, K] = numID
    if averaging:
        G.rigidE[:, I, J, K] = 0
        G.rigidH[:, I, J, K] = 0
        return
    G.rigidE[:, I, J, K] = 1
    G.rigidH[:, I, J, K] = 1
    ID = G.ID
    for comp, val in ((0, numIDx), (3, numIDx)):
        ID[comp, I, J, K] = val
        ID[comp, I, J + 1, K + 1] = val
        ID[comp, I, J + 1, K] = val
        ID[comp, I, J, K + 1] = val
    for comp, val in ((1, numIDy), (4, numIDy)):
        ID[comp, I, J, K] = val
        ID[comp, I + 1, J, K + 1] = val
        ID[comp, I + 1, J, K] = val
        ID[comp, I, J, K + 1] = val
    for comp, val in ((2, numIDz), (5, numIDz)):
        ID[comp, I, J, K] = val
        ID[comp, I + 1, J + 1, K] = val
        ID[comp, I + 1, J, K] = val
        ID[comp, I, J + 1, K] = val


def build_voxels_mask(G, mask, origin, numID, numIDx, numIDy, numIDz, averaging):
    """Build every cell where ``mask`` (a box starting at ``origin``) is true."""
    geom = getattr(G, 'geom', None)
    if geom is not None:
        geom.cells(origin, mask.shape, mask, (numID, numIDx, numIDy, numIDz), averaging)
        return
    I, J, K = np.nonzero(mask)
    I = I + origin[0]
    J = J + origin[1]
    K = K + origin[2]
    if I.size:
        _set_cells(G, I, J, K, numID, numIDx, numIDy, numIDz, averaging)


def build_box(G, xs, xf, ys, yf, zs, zf, numID, numIDx, numIDy, numIDz, averaging):
    """Axis-aligned box of cells [xs, xf) x [ys, yf) x [zs, zf) (``build_box`` :618-691)."""
    geom = getattr(G, 'geom', None)
    if geom is not None:
        geom.box((xs, ys, zs), (xf - xs, yf - ys, zf - zs), (numID, numIDx, numIDy, numIDz),
                 averaging)
        return
    G.solid[xs:xf, ys:yf, zs:zf] = numID
    if averaging:
        G.rigidE[:, xs:xf, ys:yf, zs:zf] = 0
        G.rigidH[:, xs:xf, ys:yf, zs:zf] = 0
        return
    G.rigidE[:, xs:xf, ys:yf, zs:zf] = 1
    G.rigidH[:, xs:xf, ys:yf, zs:zf] = 1
    ID = G.ID
    ID[0, xs:xf, ys:yf + 1, zs:zf + 1] = numIDx
    ID[1, xs:xf + 1, ys:yf, zs:zf + 1] = numIDy
    ID[2, xs:xf + 1, ys:yf + 1, zs:zf] = numIDz
    ID[3, xs:xf + 1, ys:yf, zs:zf] = numIDx
    ID[4, xs:xf, ys:yf + 1, zs:zf] = numIDy
    ID[5, xs:xf, ys:yf, zs:zf + 1] = numIDz


def _clip(lo, hi, n):
    return max(lo, 0), min(hi, n)


def build_sphere(G, xc, yc, zc, r, numID, numIDx, numIDy, numIDz, averaging):
    """Cells whose centre lies within ``r`` of node (xc, yc, zc) (``build_sphere`` :873-928)."""
    dx, dy, dz, rf = (np.float32(G.dx), np.float32(G.dy), np.float32(G.dz), np.float32(r))
    xs = round_value(((xc * dx) - rf) / dx) - 1
    xf = round_value(((xc * dx) + rf) / dx) + 1
    ys = round_value(((yc * dy) - rf) / dy) - 1
    yf = round_value(((yc * dy) + rf) / dy) + 1
    zs = round_value(((zc * dz) - rf) / dz) - 1
    zf = round_value(((zc * dz) + rf) / dz) + 1
    xs, xf = _clip(xs, xf, G.nx)
    ys, yf = _clip(ys, yf, G.ny)
    zs, zf = _clip(zs, zf, G.nz)
    if xs >= xf or ys >= yf or zs >= zf:
        return
    i = np.arange(xs, xf, dtype=np.float64)[:, None, None]
    j = np.arange(ys, yf, dtype=np.float64)[None, :, None]
    k = np.arange(zs, zf, dtype=np.float64)[None, None, :]
    # fp32 squares of the cell sizes, promoted to double as in the compiled reference
    dx2, dy2, dz2 = (np.float64(dx * dx), np.float64(dy * dy), np.float64(dz * dz))
    dist = np.sqrt((i + 0.5 - xc) ** 2 * dx2 + (j + 0.5 - yc) ** 2 * dy2
                   + (k + 0.5 - zc) ** 2 * dz2)
    build_voxels_mask(G, dist <= np.float64(rf), (xs, ys, zs), numID, numIDx, numIDy, numIDz,
                      averaging)


def build_cylinder(G, x1, y1, z1, x2, y2, z2, r, numID, numIDx, numIDy, numIDz, averaging):
    """Cylinder between face centres (x1,y1,z1) and (x2,y2,z2) (``build_cylinder`` :692-871)."""
    f32 = np.float32
    x1, y1, z1, x2, y2, z2, r = (f32(x1), f32(y1), f32(z1), f32(x2), f32(y2), f32(z2), f32(r))
    dx, dy, dz = f32(G.dx), f32(G.dy), f32(G.dz)
    x_align = y_align = z_align = False
    if round_value(y1 / dy) == round_value(y2 / dy) and round_value(z1 / dz) == round_value(z2 / dz):
        x_align = True
    elif round_value(x1 / dx) == round_value(x2 / dx) and round_value(z1 / dz) == round_value(z2 / dz):
        y_align = True
    elif round_value(x1 / dx) == round_value(x2 / dx) and round_value(y1 / dy) == round_value(y2 / dy):
        z_align = True

    def bounds(a1, a2, d, aligned):
        lo, hi = (a1, a2) if a1 < a2 else (a2, a1)
        if aligned:
            return round_value(lo / d), round_value(hi / d)
        return round_value((lo - r) / d) - 1, round_value((hi + r) / d) + 1
    xs, xf = _clip(*bounds(x1, x2, dx, x_align), G.nx)
    ys, yf = _clip(*bounds(y1, y2, dy, y_align), G.ny)
    zs, zf = _clip(*bounds(z1, z2, dz, z_align), G.nz)
    if xs >= xf or ys >= yf or zs >= zf:
        return

    def centre(n0, n1, d, a):
        # (n * d) in fp32, plus 0.5 * d and minus the face centre in double
        n = np.arange(n0, n1)
        return (n.astype(f32) * d).astype(np.float64) + 0.5 * np.float64(d) - np.float64(a)

    cx = centre(xs, xf, dx, x1)
    cy = centre(ys, yf, dy, y1)
    cz = centre(zs, zf, dz, z1)
    shape = (xf - xs, yf - ys, zf - zs)
    if x_align:
        m2 = np.sqrt(cy[:, None] ** 2 + cz[None, :] ** 2) <= np.float64(r)
        mask = np.broadcast_to(m2[None, :, :], shape)
    elif y_align:
        m2 = np.sqrt(cx[:, None] ** 2 + cz[None, :] ** 2) <= np.float64(r)
        mask = np.broadcast_to(m2[:, None, :], shape)
    elif z_align:
        m2 = np.sqrt(cx[:, None] ** 2 + cy[None, :] ** 2) <= np.float64(r)
        mask = np.broadcast_to(m2[:, :, None], shape)
    else:
        mask = _oblique_cylinder_mask(xs, xf, ys, yf, zs, zf, dx, dy, dz, x1, y1, z1, x2, y2, z2, r)
    build_voxels_mask(G, mask, (xs, ys, zs), numID, numIDx, numIDy, numIDz, averaging)


def _oblique_cylinder_mask(xs, xf, ys, yf, zs, zf, dx, dy, dz, x1, y1, z1, x2, y2, z2, r):
    """Point-to-axis distance test of a cylinder not aligned with an axis (fp32 vectors)."""
    f32 = np.float32
    f1f2 = np.array([x2 - x1, y2 - y1, z2 - z1], dtype=f32)
    f2f1 = np.array([x1 - x2, y1 - y2, z1 - z2], dtype=f32)
    f1f2mag = np.sqrt((f1f2 * f1f2).sum(axis=0))
    f2f1mag = np.sqrt((f2f1 * f2f1).sum(axis=0))
    out = np.zeros((xf - xs, yf - ys, zf - zs), dtype=bool)
    with np.errstate(invalid='ignore'):
        for i in range(xs, xf):
            for j in range(ys, yf):
                for k in range(zs, zf):
                    px = i * dx + 0.5 * dx
                    py = j * dy + 0.5 * dy
                    pz = k * dz + 0.5 * dz
                    f1pt = np.array([px - x1, py - y1, pz - z1], dtype=f32)
                    f2pt = np.array([px - x2, py - y2, pz - z2], dtype=f32)
                    f1ptmag = np.sqrt((f1pt * f1pt).sum(axis=0))
                    f2ptmag = np.sqrt((f2pt * f2pt).sum(axis=0))
                    if f1ptmag == 0 or f2ptmag == 0:
                        out[i - xs, j - ys, k - zs] = True
                        continue
                    factor1 = np.float32(np.dot(f1f2, f1pt) / (f1f2mag * f1ptmag))
                    factor2 = np.float32(np.dot(f2f1, f2pt) / (f2f1mag * f2ptmag))
                    theta1 = np.arccos(factor1)
                    theta2 = np.arccos(factor2)
                    theta1 = f32(0) if np.isnan(theta1) else f32(theta1)
                    theta2 = f32(0) if np.isnan(theta2) else f32(theta2)
                    distance1 = f32(f1ptmag * np.sin(theta1))
                    distance2 = f32(f2ptmag * np.sin(theta2))
                    if ((distance1 <= r or distance2 <= r) and theta1 <= np.pi / 2
                            and theta2 <= np.pi / 2):
                        out[i - xs, j - ys, k - zs] = True
    return out


def build_edge(G, xs, ys, zs, xf, yf, zf, numID):
    """Single-material line of edges (``input_cmds_geometry.py`` #edge; ``build_edge_*``)."""
    geom = getattr(G, 'geom', None)
    if geom is not None:
        if xs != xf:
            geom.edges([(0, i, ys, zs, numID) for i in range(xs, xf)])
        elif ys != yf:
            geom.edges([(1, xs, j, zs, numID) for j in range(ys, yf)])
        elif zs != zf:
            geom.edges([(2, xs, ys, k, numID) for k in range(zs, zf)])
        return
    if xs != xf:
        for i in range(xs, xf):
            _rigid_edge(G, 0, i, ys, zs)
            G.ID[0, i, ys, zs] = numID
    elif ys != yf:
        for j in range(ys, yf):
            _rigid_edge(G, 1, xs, j, zs)
            G.ID[1, xs, j, zs] = numID
    elif zs != zf:
        for k in range(zs, zf):
            _rigid_edge(G, 2, xs, ys, k)
            G.ID[2, xs, ys, k] = numID


def _rigid_edge(G, comp, i, j, k):
    """``set_rigid_Ex/Ey/Ez`` (``yee_cell_setget_rigid_ext.pyx:72-97``)."""
    r = G.rigidE
    if comp == 0:
        r[0, i, j, k] = 1
        if j != 0:
            r[1, i, j - 1, k] = 1
        if k != 0:
            r[3, i, j, k - 1] = 1
        if j != 0 and k != 0:
            r[2, i, j - 1, k - 1] = 1
    elif comp == 1:
        r[4, i, j, k] = 1
        if i != 0:
            r[7, i - 1, j, k] = 1
        if k != 0:
            r[5, i, j, k - 1] = 1
        if i != 0 and k != 0:
            r[6, i - 1, j, k - 1] = 1
    else:
        r[8, i, j, k] = 1
        if i != 0:
            r[9, i - 1, j, k] = 1
        if j != 0:
            r[11, i, j - 1, k] = 1
        if i != 0 and j != 0:
            r[10, i - 1, j - 1, k] = 1


def build_plate(G, xs, xf, ys, yf, zs, zf, numIDs):
    """Zero-thickness plate of E edges on one grid plane (#plate; ``build_face_*`` :230-312).
    ``numIDs`` holds one or two material numbers (isotropic or anisotropic): the first for the
    lower in-plane component (Ey on an x plane, Ex otherwise), the last for the other."""
    if xs == xf:
        axes, level, r1, r2 = (1, 2, 0), xs, range(ys, yf), range(zs, zf)
    elif ys == yf:
        axes, level, r1, r2 = (0, 2, 1), ys, range(xs, xf), range(zs, zf)
    elif zs == zf:
        axes, level, r1, r2 = (0, 1, 2), zs, range(xs, xf), range(ys, yf)
    else:
        return
    I, J = np.meshgrid(np.arange(r1.start, r1.stop), np.arange(r2.start, r2.stop), indexing='ij')
    _write_faces(G, I.ravel(), J.ravel(), level, axes, numIDs[0], numIDs[-1])


def _triangle_cells(v, normal, d):
    """Cells (i, j) of the triangle's plane whose centres lie strictly inside it, with the plane
    index ``level`` and the axes (a, b) that i and j count along (``build_triangle``,
    ``geometry_primitives_ext.pyx:378-486``). The arithmetic keeps the reference's C types:
    vertices, cell sizes, the area and the two barycentric sums are fp32, the cell centres
    (i + 1/2) * d are fp64 and promote the sums they enter, as the compiled reference does."""
    f32, f64 = np.float32, np.float64
    a, b = {'x': (1, 2), 'y': (0, 2), 'z': (0, 1)}[normal]
    n = 'xyz'.index(normal)
    P = [[f32(c) for c in p] for p in v]
    A1, B1 = P[0][a], P[0][b]
    A2, B2 = P[1][a], P[1][b]
    A3, B3 = P[2][a], P[2][b]
    da, db, dn = f32(d[a]), f32(d[b]), f32(d[n])
    area = f32(f64(0.5) * f64(-B2 * A3 + B1 * (-A2 + A3) + A1 * (B2 - B3) + A2 * B3))
    sign = int(np.sign(float(area)))
    i1 = round_value(float(min(A1, A2, A3)) / float(da)) - 1
    i2 = round_value(float(max(A1, A2, A3)) / float(da)) + 1
    j1 = round_value(float(min(B1, B2, B3)) / float(db)) - 1
    j2 = round_value(float(max(B1, B2, B3)) / float(db)) + 1
    level = round_value(float(P[0][n] / dn))
    I, J = np.meshgrid(np.arange(i1, i2), np.arange(j1, j2), indexing='ij')
    ir = (I + 0.5) * f64(da)
    jr = (J + 0.5) * f64(db)
    s = (f64(sign) * (f64(B1 * A3 - A1 * B3) + f64(B3 - B1) * ir + f64(A1 - A3) * jr)).astype(f32)
    t = (f64(sign) * (f64(A1 * B2 - B1 * A2) + f64(B1 - B2) * ir + f64(A2 - A1) * jr)).astype(f32)
    bound = f32(f32(2) * area) * f32(sign)
    inside = (s > 0) & (t > 0) & ((s + t) < bound)
    return I[inside], J[inside], level, (a, b, n), dn


def build_triangle(G, v, normal, thickness, numID, numIDx, numIDy, numIDz, averaging):
    """#triangle: a triangle in a grid plane (zero thickness: the faces of the cells inside it,
    ``build_face_*``) or a triangular prism of ``thickness`` metres (``build_voxel`` on those
    cells of every layer from the triangle's plane up), ``geometry_primitives_ext.pyx:378-486``.
    ``v``: the three vertices in metres (on grid nodes)."""
    d = (G.dx, G.dy, G.dz)
    I, J, level, axes, dn = _triangle_cells(v, normal, d)
    thicknesscells = round_value(float(np.float32(thickness) / dn))
    _build_in_plane(G, I, J, level, axes, thicknesscells, numID, numIDx, numIDy, numIDz,
                    averaging)


def _sector_cells(ctr1, ctr2, sectorstartangle, sectorangle, radius, normal, d, shape):
    """Cells (i, j) of the sector's plane whose centres are inside the sector
    (``build_cylindrical_sector`` :489-617 and ``is_inside_sector`` :73-110): anticlockwise of
    the start arm, clockwise of the end arm and within the radius. fp32 like the reference: the
    centre, radius, angles and cell sizes, each cell centre (i * d in fp32, plus d / 2 in fp64,
    rounded to fp32), the arm end points (radius times the fp64 cosine and sine, rounded to fp32)
    and both arm tests and the radius test."""
    f32, f64 = np.float32, np.float64
    a, b = {'x': (1, 2), 'y': (0, 2), 'z': (0, 1)}[normal]
    c1, c2, r = f32(ctr1), f32(ctr2), f32(radius)
    sa, ang = f32(sectorstartangle), f32(sectorangle)
    da, db = f32(d[a]), f32(d[b])
    i1 = max(round_value(float((c1 - r) / da)), 0)
    i2 = min(round_value(float((c1 + r) / da)), shape[a])
    j1 = max(round_value(float((c2 - r) / db)), 0)
    j2 = min(round_value(float((c2 + r) / db)), shape[b])
    if i1 >= i2 or j1 >= j2:
        return np.zeros(0, int), np.zeros(0, int), (a, b)
    I, J = np.meshgrid(np.arange(i1, i2), np.arange(j1, j2), indexing='ij')
    px = (f64(I.astype(f32) * da) + f64(0.5) * f64(da)).astype(f32)
    py = (f64(J.astype(f32) * db) + f64(0.5) * f64(db)).astype(f32)
    s1 = f32(f64(r) * np.cos(f64(sa)))
    s2 = f32(f64(r) * np.sin(f64(sa)))
    e1 = f32(f64(r) * np.cos(f64(f32(sa + ang))))
    e2 = f32(f64(r) * np.sin(f64(f32(sa + ang))))
    v1 = px - c1
    v2 = py - c2

    def clockwise(ux, uy):
        return (-ux) * v2 + uy * v1 > 0

    inside = ~clockwise(s1, s2) & clockwise(e1, e2) & (v1 * v1 + v2 * v2 <= r * r)
    return I[inside], J[inside], (a, b)


def build_cylindrical_sector(G, ctr1, ctr2, level, sectorstartangle, sectorangle, radius, normal,
                             thickness, numID, numIDx, numIDy, numIDz, averaging):
    """#cylindrical_sector: the cells of a circular sector in a grid plane (zero thickness: their
    faces) or of a sector prism of ``thickness`` metres from plane ``level`` up
    (``geometry_primitives_ext.pyx:489-617``). Centre in metres on grid nodes, angles in
    radians, anticlockwise from the first in-plane axis."""
    d = (G.dx, G.dy, G.dz)
    I, J, (a, b) = _sector_cells(ctr1, ctr2, sectorstartangle, sectorangle, radius, normal, d,
                                 (G.nx, G.ny, G.nz))
    n = 'xyz'.index(normal)
    thicknesscells = round_value(float(np.float32(thickness) / np.float32(d[n])))
    _build_in_plane(G, I, J, level, (a, b, n), thicknesscells, numID, numIDx, numIDy, numIDz,
                    averaging)


def _rigid_edges(G, comp, x, y, z):
    """``_rigid_edge`` for arrays of edges of one component (the flags are only ever set)."""
    r = G.rigidE
    if comp == 0:
        own, nb = 0, ((1, y != 0, (0, -1, 0)), (3, z != 0, (0, 0, -1)),
                      (2, (y != 0) & (z != 0), (0, -1, -1)))
    elif comp == 1:
        own, nb = 4, ((7, x != 0, (-1, 0, 0)), (5, z != 0, (0, 0, -1)),
                      (6, (x != 0) & (z != 0), (-1, 0, -1)))
    else:
        own, nb = 8, ((9, x != 0, (-1, 0, 0)), (11, y != 0, (0, -1, 0)),
                      (10, (x != 0) & (y != 0), (-1, -1, 0)))
    r[own, x, y, z] = 1
    for flag, m, (ox, oy, oz) in nb:
        r[flag, x[m] + ox, y[m] + oy, z[m] + oz] = 1


def _write_faces(G, I, J, level, axes, va, vb):
    """The faces of cells (I, J) of the grid plane ``level`` normal to axis ``axes[2]``
    (``build_face_yz/xz/xy`` :230-312): per face the near and far edges of the two in-plane
    components, component ``axes[0]`` taking ``va`` and ``axes[1]`` taking ``vb``, with their
    rigid flags; in face order on a device-built grid."""
    a, b, n = axes
    m = I.size
    if m == 0:
        return
    ii = np.stack([I, I, I, I + 1], axis=1).ravel()
    jj = np.stack([J, J, J + 1, J], axis=1).ravel()
    comp = np.tile(np.array([a, b, a, b]), m)
    val = np.tile(np.array([va, vb, va, vb], dtype=np.int64), m)
    idx = [None, None, None]
    idx[a], idx[b], idx[n] = ii, jj, np.full(ii.shape, level)
    geom = getattr(G, 'geom', None)
    if geom is not None:
        geom.edges(np.stack([comp, idx[0], idx[1], idx[2], val], axis=1))
        return
    for c in (a, b):
        sel = comp == c
        x, y, z = idx[0][sel], idx[1][sel], idx[2][sel]
        _rigid_edges(G, c, x, y, z)
        G.ID[c, x, y, z] = val[sel]


def _build_in_plane(G, I, J, level, axes, thicknesscells, numID, numIDx, numIDy, numIDz,
                    averaging):
    """Cells (I, J) of a grid plane at ``level``: with no thickness the faces of those cells
    (``build_face_yz/xz/xy`` :230-312: rigid edges and IDs of the two in-plane components),
    otherwise ``build_voxel`` on them in every layer from ``level`` up."""
    a, b, n = axes
    if I.size == 0 or thicknesscells < 0:
        return
    shape = (G.nx, G.ny, G.nz)
    if thicknesscells == 0:
        # the rigid flags of a face's far edges sit one cell on; on the domain's last cell row
        # or its upper boundary plane that is past the end of the (cell-sized) rigid arrays
        if level >= shape[n] or int(I.max()) + 1 >= shape[a] or int(J.max()) + 1 >= shape[b]:
            raise CmdInputError('a zero-thickness face on the last cell row or the upper '
                                'boundary of the domain is not built: its rigid edge flags would '
                                'lie outside the grid')
        # face numbers: the two in-plane components (yz face: Ey, Ez; xz: Ex, Ez; xy: Ex, Ey)
        nums = (numIDx, numIDy, numIDz)
        _write_faces(G, I, J, level, axes, nums[a], nums[b])
        return
    ks = np.arange(level, min(level + thicknesscells, shape[n]))
    if ks.size == 0:
        return
    lo = [0, 0, 0]
    hi = [0, 0, 0]
    lo[a], hi[a] = int(I.min()), int(I.max()) + 1
    lo[b], hi[b] = int(J.min()), int(J.max()) + 1
    lo[n], hi[n] = int(ks[0]), int(ks[-1]) + 1
    mask = np.zeros([hi[q] - lo[q] for q in range(3)], dtype=bool)
    sel = [None, None, None]
    sel[a] = I - lo[a]
    sel[b] = J - lo[b]
    for k in ks:
        sel[n] = np.full(I.shape, k - lo[n])
        mask[sel[0], sel[1], sel[2]] = True
    build_voxels_mask(G, mask, tuple(lo), numID, numIDx, numIDy, numIDz, averaging)


# Edge offsets written by ``build_voxel`` for one cell, per component (E and H alike):
# x-directed components take (0,0,0), (0,1,1), (0,1,0), (0,0,1) and so on.
_VOXEL_EDGE_OFFSETS = {
    0: ((0, 0, 0), (0, 1, 1), (0, 1, 0), (0, 0, 1)),
    1: ((0, 0, 0), (1, 0, 1), (1, 0, 0), (0, 0, 1)),
    2: ((0, 0, 0), (1, 1, 0), (1, 0, 0), (0, 1, 0)),
}


def build_voxels_array(G, origin, numids, averaging):
    """``build_voxels_from_array`` (``geometry_primitives_ext.pyx:930-980``) for a block of
    per-cell material numbers (negative = leave the cell alone), clipped to the domain.

    Cells sharing an edge write it in the reference's (i, j, k) loop order, so the edge ends
    with the material of the last such cell; the writes below are issued in that order.
    """
    xs, ys, zs = origin
    n = numids[:max(0, min(numids.shape[0], G.nx - xs)), :max(0, min(numids.shape[1], G.ny - ys)),
               :max(0, min(numids.shape[2], G.nz - zs))]
    geom = getattr(G, 'geom', None)
    if geom is not None:
        geom.voxels((xs, ys, zs), n, averaging)
        return
    built = n >= 0
    if not built.any():
        return
    X = slice(xs, xs + n.shape[0])
    Y = slice(ys, ys + n.shape[1])
    Z = slice(zs, zs + n.shape[2])
    solid = G.solid[X, Y, Z]
    solid[built] = n[built]
    for r in (G.rigidE, G.rigidH):
        view = r[:, X, Y, Z]
        view[:, built] = 0 if averaging else 1
    if averaging:
        return
    sx, sy, sz = n.shape
    for comp in range(3):
        offs = _VOXEL_EDGE_OFFSETS[comp]
        # a cell with a larger (i, j, k) writes later; offsets ordered by how late the writing
        # cell comes relative to the edge: the edge at cell + o is written by cell = edge - o
        order = sorted(offs, key=lambda o: (-o[0], -o[1], -o[2]))
        for o in order:
            for c in (comp, comp + 3):
                target = G.ID[c, xs + o[0]:xs + o[0] + sx, ys + o[1]:ys + o[1] + sy,
                              zs + o[2]:zs + o[2] + sz]
                target[built] = n[built]
