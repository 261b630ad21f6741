"""Pure-torch restatement of the differentiable FDTD model of ``gprmax_gb300.adjoint``
(test infrastructure): the same updates, ranges, PML slab corrections, sources and receivers,
written with tensor slices so torch's autograd gives reference gradients on small grids.
"""
import torch

# tangential components per slab axis: (first, second) with their H (or E) difference
# component and sign, as the reference's PML kernels apply them
E_SLAB = {0: ((1, 2, -1.0), (2, 1, +1.0)), 1: ((0, 2, +1.0), (2, 0, -1.0)),
          2: ((0, 1, -1.0), (1, 0, +1.0))}
H_SLAB = {0: ((4, 2, +1.0), (5, 1, -1.0)), 1: ((3, 2, -1.0), (5, 0, +1.0)),
          2: ((3, 1, +1.0), (4, 0, -1.0))}


def _box(axis, minus, T, n3, electric):
    """Slices of a slab box and the profile index of each plane along the axis."""
    n = n3[axis]
    if minus:
        lo, hi = (1, T + 1) if electric else (0, T)
        prof = [T - c for c in range(lo, hi)] if electric else [T - 1 - c for c in range(lo, hi)]
    else:
        lo, hi = n - T, n
        prof = [c - (n - T) for c in range(lo, hi)]
    sl = [slice(0, n3[0]), slice(0, n3[1]), slice(0, n3[2])]
    sl[axis] = slice(lo, hi)
    return sl, torch.tensor(prof)


def _shift(sl, axis, delta):
    out = list(sl)
    out[axis] = slice(sl[axis].start + delta, sl[axis].stop + delta)
    return tuple(out)


def _bcast(v, axis):
    shape = [1, 1, 1]
    shape[axis] = -1
    return v.reshape(shape)


def forward(model, CA, CB, dtype=torch.float64):
    """Receiver traces [nrx][iterations] of the model for per-edge CA, CB [3][nx+1][ny+1][nz+1]."""
    nx, ny, nz = model.nx, model.ny, model.nz
    n3 = (nx, ny, nz)
    d = model.d
    shape = (nx + 1, ny + 1, nz + 1)
    dev = CA.device
    CA = CA.to(dtype)
    CB = CB.to(dtype)
    CBd = CB / d
    dbd = model.dbd
    srcm = model.srcm
    F = [torch.zeros(shape, dtype=dtype, device=dev) for _ in range(6)]   # Ex Ey Ez Hx Hy Hz
    slabs = []
    for s in range(6):
        T = model.thickness[s]
        if not T:
            continue
        rows = [torch.tensor(r, dtype=dtype, device=dev) for r in model.pml_rows[s]]
        axis, minus = s % 3, s < 3
        eb, ep = _box(axis, minus, T, n3, True)
        hb, hp = _box(axis, minus, T, n3, False)
        box_shape = lambda b: tuple(x.stop - x.start for x in b)
        slabs.append({'axis': axis, 'rows': rows, 'eb': eb, 'ep': ep, 'hb': hb, 'hp': hp,
                      'phiE': [torch.zeros(box_shape(eb), dtype=dtype, device=dev) for _ in range(2)],
                      'phiH': [torch.zeros(box_shape(hb), dtype=dtype, device=dev) for _ in range(2)]})
    traces = [[] for _ in model.receivers]
    for n in range(model.iterations):
        for r, (c, i, j, k) in enumerate(model.receivers):
            traces[r].append(F[c][i, j, k])
        Ex, Ey, Ez, Hx, Hy, Hz = F
        # H main update (update_magnetic ranges)
        nHx = Hx.clone()
        nHx[1:, :ny, :nz] = Hx[1:, :ny, :nz] - dbd * (Ez[1:, 1:, :nz] - Ez[1:, :ny, :nz]) \
            + dbd * (Ey[1:, :ny, 1:] - Ey[1:, :ny, :nz])
        nHy = Hy.clone()
        nHy[:nx, 1:, :nz] = Hy[:nx, 1:, :nz] - dbd * (Ex[:nx, 1:, 1:] - Ex[:nx, 1:, :nz]) \
            + dbd * (Ez[1:, 1:, :nz] - Ez[:nx, 1:, :nz])
        nHz = Hz.clone()
        nHz[:nx, :ny, 1:] = Hz[:nx, :ny, 1:] - dbd * (Ey[1:, :ny, 1:] - Ey[:nx, :ny, 1:]) \
            + dbd * (Ex[:nx, 1:, 1:] - Ex[:nx, :ny, 1:])
        Hn = [nHx, nHy, nHz]
        for sd in slabs:
            axis, rows = sd['axis'], sd['rows']
            RA, RB, RE, RF = (_bcast(rows[4 + q][sd['hp'].to(dev)], axis) for q in range(4))
            for which, (comp, dcomp, sign) in enumerate(H_SLAB[axis]):
                b = tuple(sd['hb'])
                dF = (F[dcomp][_shift(b, axis, 1)] - F[dcomp][b]) / d
                phi = sd['phiH'][which]
                X = (RA - 1) * dF + RB * phi
                h = Hn[comp - 3].clone()
                h[b] = h[b] + sign * srcm * X
                Hn[comp - 3] = h
                sd['phiH'][which] = RE * phi - RF * dF
        Hx, Hy, Hz = Hn
        # E main update (update_electric ranges; CA = 1, CB = 0 off them)
        nEx = CA[0] * Ex
        nEx = nEx.clone()
        nEx[:nx, 1:ny, 1:nz] = nEx[:nx, 1:ny, 1:nz] + CBd[0, :nx, 1:ny, 1:nz] * (
            (Hz[:nx, 1:ny, 1:nz] - Hz[:nx, :ny - 1, 1:nz]) - (Hy[:nx, 1:ny, 1:nz] - Hy[:nx, 1:ny, :nz - 1]))
        nEy = (CA[1] * Ey).clone()
        nEy[1:nx, :ny, 1:nz] = nEy[1:nx, :ny, 1:nz] + CBd[1, 1:nx, :ny, 1:nz] * (
            (Hx[1:nx, :ny, 1:nz] - Hx[1:nx, :ny, :nz - 1]) - (Hz[1:nx, :ny, 1:nz] - Hz[:nx - 1, :ny, 1:nz]))
        nEz = (CA[2] * Ez).clone()
        nEz[1:nx, 1:ny, :nz] = nEz[1:nx, 1:ny, :nz] + CBd[2, 1:nx, 1:ny, :nz] * (
            (Hy[1:nx, 1:ny, :nz] - Hy[:nx - 1, 1:ny, :nz]) - (Hx[1:nx, 1:ny, :nz] - Hx[1:nx, :ny - 1, :nz]))
        En = [nEx, nEy, nEz]
        Hall = [None, None, None, Hx, Hy, Hz]
        for sd in slabs:
            axis, rows = sd['axis'], sd['rows']
            RA, RB, RE, RF = (_bcast(rows[q][sd['ep'].to(dev)], axis) for q in range(4))
            for which, (comp, dcomp, sign) in enumerate(E_SLAB[axis]):
                b = tuple(sd['eb'])
                dF = (Hall[3 + dcomp][b] - Hall[3 + dcomp][_shift(b, axis, -1)]) / d
                phi = sd['phiE'][which]
                X = (RA - 1) * dF + RB * phi
                e = En[comp].clone()
                e[b] = e[b] + sign * CB[comp][b] * X
                En[comp] = e
                sd['phiE'][which] = RE * phi - RF * dF
        for comp, i, j, k, scale, wave in model.sources:
            e = En[comp].clone()
            e[i, j, k] = e[i, j, k] - CB[comp, i, j, k] * float(wave[n]) * scale
            En[comp] = e
        F = En + [Hx, Hy, Hz]
    return torch.stack([torch.stack(t) for t in traces])
