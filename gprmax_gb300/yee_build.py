"""Per-edge material IDs from the solid array, with dielectric smoothing.

Follows ``gprMax/yee_cell_build_ext.pyx:110-257``: every E edge not marked rigid takes the
material of its 4 surrounding cells when they agree, otherwise an averaged material; every H
edge uses its 2 neighbouring cells. Averaged materials are looked up, or created, by the
reference's name-matching rule (``create_electric_average`` :31-68,
``create_magnetic_average`` :71-108), in the order the reference's (i, j, k) loops first meet
each neighbour combination, so new materials receive identical numbers. The loops are done as
whole-array numpy operations; only distinct combinations are resolved one by one. On a grid
built in device memory the device classifies the edges and lists the combinations in the same
order (:meth:`gprmax_gb300.devgeom.DeviceGeometry.components`); their resolution is the same.
"""
import numpy as np

from .materials import Material


def _rigid_edges(G):
    """Per-component rigid masks over each component's build range (``get_rigid_*``)."""
    rE, rH = G.rigidE, G.rigidH
    nx, ny, nz = G.nx, G.ny, G.nz
    ex = (rE[0, :, 1:, 1:] | rE[1, :, :-1, 1:] | rE[3, :, 1:, :-1] | rE[2, :, :-1, :-1])
    ey = (rE[4, 1:, :, 1:] | rE[7, :-1, :, 1:] | rE[5, 1:, :, :-1] | rE[6, :-1, :, :-1])
    ez = (rE[8, 1:, 1:, :] | rE[9, :-1, 1:, :] | rE[11, 1:, :-1, :] | rE[10, :-1, :-1, :])
    hx = rH[0, 1:, :, :] | rH[1, :-1, :, :]
    hy = rH[2, :, 1:, :] | rH[3, :, :-1, :]
    hz = rH[4, :, :, 1:] | rH[5, :, :, :-1]
    del nx, ny, nz
    return ex, ey, ez, hx, hy, hz


def _first_occurrence_unique(keys):
    """Distinct rows of ``keys`` (n x m) ordered by first appearance, and the inverse map."""
    if keys.shape[0] == 0:
        return keys, np.zeros(0, dtype=np.int64)
    uniq, first, inverse = np.unique(keys, axis=0, return_index=True, return_inverse=True)
    order = np.argsort(first, kind='stable')
    rank = np.empty_like(order)
    rank[order] = np.arange(order.size)
    return uniq[order], rank[inverse.ravel()]


def _electric_average(G, ids):
    """Material number for 4 neighbour IDs (``create_electric_average``)."""
    mats = G.materials
    requiredID = '+'.join(mats[n].ID for n in ids)
    tmp = requiredID.split('+')
    for x in mats:
        if (x.ID.count(tmp[0]) == requiredID.count(tmp[0]) and
                x.ID.count(tmp[1]) == requiredID.count(tmp[1]) and
                x.ID.count(tmp[2]) == requiredID.count(tmp[2]) and
                x.ID.count(tmp[3]) == requiredID.count(tmp[3])):
            return x.numID
    m = Material(len(mats), requiredID)
    m.type = 'dielectric-smoothed'
    m.er = np.mean(tuple(mats[n].er for n in ids), axis=0)
    m.se = np.mean(tuple(mats[n].se for n in ids), axis=0)
    m.mr = np.mean(tuple(mats[n].mr for n in ids), axis=0)
    m.sm = np.mean(tuple(mats[n].sm for n in ids), axis=0)
    mats.append(m)
    return m.numID


def _magnetic_average(G, ids):
    """Material number for 2 neighbour IDs (``create_magnetic_average``)."""
    mats = G.materials
    requiredID = mats[ids[0]].ID + '+' + mats[ids[1]].ID
    tmp = requiredID.split('+')
    for x in mats:
        c0 = x.ID.count(tmp[0])
        c1 = x.ID.count(tmp[1])
        if ((c0 == requiredID.count(tmp[0]) and c1 == requiredID.count(tmp[1]))
                or (c0 % 2 == 0 and c1 % 2 == 0)):
            return x.numID
    m = Material(len(mats), requiredID)
    m.type = 'dielectric-smoothed'
    m.er = np.mean((mats[ids[0]].er, mats[ids[1]].er), axis=0)
    m.se = np.mean((mats[ids[0]].se, mats[ids[1]].se), axis=0)
    m.mr = np.mean((mats[ids[0]].mr, mats[ids[1]].mr), axis=0)
    m.sm = np.mean((mats[ids[0]].sm, mats[ids[1]].sm), axis=0)
    mats.append(m)
    return m.numID


def _assign(G, comp, region, rigid, neighbours, resolve):
    """Write ID[comp][region] for the non-rigid edges of one component."""
    n1 = neighbours[0]
    same = np.ones(n1.shape, dtype=bool)
    for nb in neighbours[1:]:
        same &= (nb == n1)
    free = ~rigid.astype(bool)
    target = G.ID[comp][region]
    plain = free & same
    target[plain] = n1[plain]
    avg = free & ~same
    if avg.any():
        keys = np.stack([nb[avg] for nb in neighbours], axis=1).astype(np.int64)
        uniq, inv = _first_occurrence_unique(keys)
        numbers = np.array([resolve(G, tuple(int(v) for v in row)) for row in uniq],
                           dtype=np.uint32)
        target[avg] = numbers[inv]
    G.ID[comp][region] = target


def build_electric_components(G):
    """E-edge IDs for Ex, Ey, Ez in that order."""
    if getattr(G, 'geom', None) is not None:
        G.geom.components(True, _electric_average, G)
        return
    s = G.solid
    ex, ey, ez, _, _, _ = _rigid_edges(G)
    # Ex: i in [0,nx), j in [1,ny), k in [1,nz)
    _assign(G, 0, (slice(0, G.nx), slice(1, G.ny), slice(1, G.nz)), ex,
            (s[:, 1:, 1:], s[:, :-1, 1:], s[:, :-1, :-1], s[:, 1:, :-1]), _electric_average)
    # Ey: i in [1,nx), j in [0,ny), k in [1,nz)
    _assign(G, 1, (slice(1, G.nx), slice(0, G.ny), slice(1, G.nz)), ey,
            (s[1:, :, 1:], s[:-1, :, 1:], s[:-1, :, :-1], s[1:, :, :-1]), _electric_average)
    # Ez: i in [1,nx), j in [1,ny), k in [0,nz)
    _assign(G, 2, (slice(1, G.nx), slice(1, G.ny), slice(0, G.nz)), ez,
            (s[1:, 1:, :], s[:-1, 1:, :], s[:-1, :-1, :], s[1:, :-1, :]), _electric_average)


def build_magnetic_components(G):
    """H-edge IDs for Hx, Hy, Hz in that order."""
    if getattr(G, 'geom', None) is not None:
        G.geom.components(False, _magnetic_average, G)
        return
    s = G.solid
    _, _, _, hx, hy, hz = _rigid_edges(G)
    _assign(G, 3, (slice(1, G.nx), slice(0, G.ny), slice(0, G.nz)), hx,
            (s[1:, :, :], s[:-1, :, :]), _magnetic_average)
    _assign(G, 4, (slice(0, G.nx), slice(1, G.ny), slice(0, G.nz)), hy,
            (s[:, 1:, :], s[:, :-1, :]), _magnetic_average)
    _assign(G, 5, (slice(0, G.nx), slice(0, G.ny), slice(1, G.nz)), hz,
            (s[:, :, 1:], s[:, :, :-1]), _magnetic_average)
