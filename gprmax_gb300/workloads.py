"""Synthetic models with the shapes, sizes and value distributions of the benchmark
configurations (no external data is involved; every draw is seeded).

* :func:`freespace_dipole`    100^3 free-space Hertzian dipole, 10-cell CFS PML, Ricker 1.5 GHz
* :func:`dispersive_soil`     400x400x200 heterogeneous 50-material Debye soil with a PEC
                              cylinder, x-dipole and receiver above the surface
* :func:`throughput_cube`     N^3 grid with a seeded dielectric block in the central half
The soil is binned from a fractal field made with the reference's fractal-volume recipe
(``gprMax/fractals.py:141-194``): FFT of seeded Gaussian noise, scaled by 1/r^D about the
spectrum centre, inverse FFT, then ``np.digitize`` into equal-width bins.
"""
import numpy as np

from .geometry import build_voxels_array
from .grid import FDTDGrid
from .materials import Material
from .model import build_grid, finish_build


def fractal_volume(shape, dimension, seed, nbins, device=False):
    """Bin indices 0..nbins-1 of a seeded fractal field of the given shape (``device``: the
    transforms and filter on the GPU, equal to the host's field to rounding)."""
    nx, ny, nz = shape
    weighting = np.array([1.0, 1.0, 1.0]) * (np.amin(np.array(shape)) / np.array(shape, dtype=np.float64))
    v1 = np.array([weighting[0] * nx / 2, weighting[1] * ny / 2, weighting[2] * nz / 2])
    rng = np.random.default_rng(seed=seed)
    A = rng.standard_normal(size=shape)
    if device:
        from .fractals import device_field
        vol = device_field(A, weighting, float(np.float32(dimension)))
        bins = np.linspace(np.amin(vol), np.amax(vol), nbins)
        return np.digitize(vol, bins, right=True).astype(np.int64)
    A = np.fft.fftshift(np.fft.fftn(A))
    i = (weighting[0] * np.arange(nx) - v1[0])[:, None, None]
    j = (weighting[1] * np.arange(ny) - v1[1])[None, :, None]
    k = (weighting[2] * np.arange(nz) - v1[2])[None, None, :]
    rr = np.sqrt(i ** 2 + j ** 2 + k ** 2)
    B = rr ** dimension
    B[B == 0] = 0.9
    A /= B
    A = np.fft.ifftshift(A)
    A[0, 0, 0] = 0
    vol = np.real(np.fft.ifftn(A)).astype(np.float32)
    bins = np.linspace(np.amin(vol), np.amax(vol), nbins)
    return np.digitize(vol, bins, right=True).astype(np.int64)


def freespace_dipole(n=100, timewindow='3e-9', pml=10, messages=False):
    """Free-space z-dipole at the centre, receiver 10 cells along x (1 mm cells)."""
    d = 0.001
    c = n * d / 2
    lines = ['#domain: {0:g} {0:g} {0:g}'.format(n * d), '#dx_dy_dz: 0.001 0.001 0.001',
             '#time_window: {}'.format(timewindow), '#pml_cells: {}'.format(pml),
             '#waveform: ricker 1 1.5e9 w',
             '#hertzian_dipole: z {0:g} {0:g} {0:g} w'.format(c),
             '#rx: {:g} {:g} {:g} rx1 Ez Hx Hy'.format(c + 10 * d, c, c)]
    return build_grid([l + '\n' for l in lines], messages=messages)


def dispersive_soil(nx=400, ny=400, nz=200, dx=0.002, surface=150, nmat=50, seed=1,
                    timewindow='12e-9', cylinder=True, pml=10, messages=False, device_build=False,
                    snapshot_at=0, device_fractals=False, extra_lines=()):
    """Heterogeneous single-pole Debye soil below ``surface`` cells, air above.

    Per material: eps_s ~ U[5,20], eps_inf ~ U[3,6], tau ~ logU[1e-10,1e-8] s,
    sigma ~ logU[1e-4,1e-2] S/m. A PEC cylinder of radius 20 mm runs along y at depth 60 mm;
    an x-polarised dipole and a receiver 40 mm apart sit 10 mm above the surface.
    ``snapshot_at`` > 0 adds a snapshot of the whole domain (every cell) at that iteration;
    ``extra_lines`` are further input commands (a PML formulation, CFS parameters).
    """
    rng = np.random.default_rng(seed)
    es = rng.uniform(5, 20, nmat)
    einf = rng.uniform(3, 6, nmat)
    tau = 10 ** rng.uniform(-10, -8, nmat)
    sig = 10 ** rng.uniform(-4, -2, nmat)
    zsurf = surface * dx
    xc = nx * dx / 2
    yc = ny * dx / 2
    lines = ['#domain: {:g} {:g} {:g}'.format(nx * dx, ny * dx, nz * dx),
             '#dx_dy_dz: {0:g} {0:g} {0:g}'.format(dx), '#time_window: {}'.format(timewindow),
             '#pml_cells: {}'.format(pml), '#waveform: ricker 1 1.5e9 w',
             '#hertzian_dipole: x {:g} {:g} {:g} w'.format(xc - 0.02, yc, zsurf + 0.01),
             '#rx: {:g} {:g} {:g}'.format(xc + 0.02, yc, zsurf + 0.01)]
    for m in range(nmat):
        lines.append('#material: {!r} {!r} 1 0 soil{}'.format(float(einf[m]), float(sig[m]), m))
        lines.append('#add_dispersion_debye: 1 {!r} {!r} soil{}'.format(
            float(es[m] - einf[m]), float(tau[m]), m))
    if cylinder:
        lines.append('#cylinder: {0:g} 0 {1:g} {0:g} {2:g} {1:g} 0.02 pec'.format(
            xc, zsurf - 0.06, ny * dx))
    if snapshot_at:
        lines.append('#snapshot: 0 0 0 {:g} {:g} {:g} {d:g} {d:g} {d:g} {} soil_snapshot'.format(
            nx * dx, ny * dx, nz * dx, int(snapshot_at), d=dx))
    lines.extend(extra_lines)
    first_soil = 2

    def soil(G):
        bins = fractal_volume((nx, ny, surface), 1.5, seed, nmat, device=device_fractals)
        build_voxels_array(G, (0, 0, 0), bins + first_soil, averaging=False)
    return build_grid([l + '\n' for l in lines], messages=messages, geometry_hook=soil,
                      device_build=device_build)


def throughput_cube(n, iterations=2000, seed=0, pml=10, messages=False, device_build=False):
    """N^3 cube at 1 mm with a seeded dielectric block filling the central half."""
    rng = np.random.default_rng(seed)
    er = rng.uniform(2, 20)
    se = rng.uniform(0, 0.01)
    d = 0.001
    L = n * d
    c = L / 2
    lines = ['#domain: {0:g} {0:g} {0:g}'.format(L), '#dx_dy_dz: 0.001 0.001 0.001',
             '#time_window: {}'.format(iterations), '#pml_cells: {}'.format(pml),
             '#waveform: ricker 1 1.5e9 w', '#material: {!r} {!r} 1 0 block'.format(er, se),
             '#box: {0:g} {0:g} {0:g} {1:g} {1:g} {1:g} block'.format(L / 4, 3 * L / 4),
             '#hertzian_dipole: z {0:g} {0:g} {1:g} w'.format(c, L / 4 - 5 * d),
             '#rx: {0:g} {0:g} {1:g}'.format(c + 5 * d, L / 4 - 5 * d)]
    return build_grid([l + '\n' for l in lines], messages=messages, device_build=device_build)


def bscan_input(shape, seed, position, dx=0.002, timewindow='10e-9', pml=10):
    """Input-file lines of one model of an uneven B-scan: a seeded 3-layer soil (per layer
    eps_r ~ U[3,15], sigma ~ logU[1e-4,1e-2] S/m) filling the lower 70 % of the domain, one
    buried PEC sphere of radius U[15,30] mm at a random position in the soil, and a y-directed
    Hertzian dipole with a receiver 40 mm away in x, 10 mm above the surface, moved 4 mm per
    model along x (``position``, wrapped to the positions that keep the pair 30 mm clear of the
    far side); Ricker 1.5 GHz."""
    nx, ny, nz = shape
    rng = np.random.default_rng(seed)
    er = rng.uniform(3, 15, 3)
    sig = 10 ** rng.uniform(-4, -2, 3)
    surf = int(nz * 0.7)
    cuts = np.sort(rng.choice(np.arange(int(surf * 0.2), int(surf * 0.9)), 2, replace=False))
    lines = ['#domain: {:g} {:g} {:g}'.format(nx * dx, ny * dx, nz * dx),
             '#dx_dy_dz: {0:g} {0:g} {0:g}'.format(dx), '#time_window: {}'.format(timewindow),
             '#pml_cells: {}'.format(pml), '#waveform: ricker 1 1.5e9 w']
    for layer in range(3):
        lines.append('#material: {!r} {!r} 1 0 layer{}'.format(float(er[layer]), float(sig[layer]), layer))
    z = [0, int(cuts[0]), int(cuts[1]), surf]
    for layer in range(3):
        lines.append('#box: 0 0 {:g} {:g} {:g} {:g} layer{}'.format(
            z[layer] * dx, nx * dx, ny * dx, z[layer + 1] * dx, layer))
    r = rng.uniform(0.015, 0.030)
    c = (rng.uniform(0.2, 0.8) * nx * dx, rng.uniform(0.2, 0.8) * ny * dx,
         rng.uniform(r + 0.03, max(surf * dx - r, r + 0.03)))
    lines.append('#sphere: {:g} {:g} {:g} {:g} pec'.format(c[0], c[1], c[2], r))
    x = 0.06 + 0.004 * (position % max(1, int((nx * dx - 0.13) / 0.004 + 1e-9) + 1))
    zs = surf * dx + 0.01
    lines.append('#hertzian_dipole: y {:g} {:g} {:g} w'.format(x, ny * dx / 2, zs))
    lines.append('#rx: {:g} {:g} {:g}'.format(x + 0.04, ny * dx / 2, zs))
    return [line + '\n' for line in lines]


def bscan_models(nmodels=128, shapes=((200, 200, 100), (300, 300, 150)), seed=11,
                 messages=False, device_build=False):
    """The uneven B-scan: ``nmodels`` grids, the first half of the first shape and the second
    half of the second, each with its own seed; the dipole/receiver pair of model m of each half
    sits 4 mm * m along x."""
    half = nmodels // 2
    grids = []
    for m in range(nmodels):
        shape = shapes[0] if m < half else shapes[1]
        pos = m if m < half else m - half
        grids.append(build_grid(bscan_input(shape, seed + m, pos), messages=messages,
                                device_build=device_build))
    return grids


def bscan_2d_input(shape=(120, 105), dx=0.002, timewindow='3e-9', seed=31):
    """Input-file lines of a 2D (TMz, one cell in z) B-scan: a seeded dielectric half-space
    (eps_r ~ U[4, 9], sigma ~ logU[1e-4, 1e-2] S/m) filling the lower 80 % of the domain, a PEC
    cylinder along z of radius U[8, 14] mm buried in it, and a z-directed Hertzian dipole with a
    receiver 40 mm away in x, 10 mm above the surface, both stepped one cell in x per trace
    (``#src_steps`` / ``#rx_steps``); Ricker 1.5 GHz; the default 10-cell PML (none along z)."""
    nx, ny = shape
    rng = np.random.default_rng(seed)
    er = rng.uniform(4, 9)
    sig = 10 ** rng.uniform(-4, -2)
    surf = int(ny * 0.8)
    r = rng.uniform(0.008, 0.014)
    cx = rng.uniform(0.4, 0.6) * nx * dx
    cy = rng.uniform(0.3, 0.6) * surf * dx
    ys = surf * dx + 0.01
    return [line + '\n' for line in (
        '#domain: {:g} {:g} {:g}'.format(nx * dx, ny * dx, dx),
        '#dx_dy_dz: {0:g} {0:g} {0:g}'.format(dx), '#time_window: {}'.format(timewindow),
        '#material: {!r} {!r} 1 0 half_space'.format(float(er), float(sig)),
        '#waveform: ricker 1 1.5e9 w',
        '#hertzian_dipole: z {:g} {:g} 0 w'.format(0.04, ys),
        '#rx: {:g} {:g} 0'.format(0.08, ys),
        '#src_steps: {:g} 0 0'.format(dx), '#rx_steps: {:g} 0 0'.format(dx),
        '#box: 0 0 0 {:g} {:g} {:g} half_space'.format(nx * dx, surf * dx, dx),
        '#cylinder: {0:g} {1:g} 0 {0:g} {1:g} {2:g} {3:g} pec'.format(cx, cy, dx, r))]


def bscan_2d_models(ntraces=60, shape=(120, 105), seed=31, messages=False, device_build=False):
    """The grids of every trace of the 2D B-scan, each stepped to its model run as the
    reference's ``-n`` loop steps them (``model_build_run.py:308-324``)."""
    from .model import step_sources_receivers
    lines = bscan_2d_input(shape, seed=seed)
    grids = []
    for m in range(ntraces):
        G = build_grid(lines, messages=messages, device_build=device_build)
        step_sources_receivers(G, m + 1, ntraces)
        grids.append(G)
    return grids


def gaussian_random_field(shape, corr_cells, seed, lo=1.0, hi=20.0, mean=8.0, std=4.0):
    """Seeded smooth Gaussian random field: white noise filtered in Fourier space by a Gaussian
    of correlation length ``corr_cells``, scaled to ``mean`` +/- ``std`` and clipped to
    [lo, hi]."""
    rng = np.random.default_rng(seed)
    noise = rng.standard_normal(shape)
    k = [np.fft.fftfreq(n) for n in shape]
    kk = sum(np.meshgrid(*[(2 * np.pi * x) ** 2 for x in k], indexing='ij'))
    field = np.real(np.fft.ifftn(np.fft.fftn(noise) * np.exp(-0.5 * kk * corr_cells ** 2)))
    field = (field - field.mean()) / (field.std() + 1e-30)
    return np.clip(mean + std * field, lo, hi)


def adjoint_problem(shape=(200, 200, 100), dx=0.002, timewindow='8e-9', seed=21, pml=10):
    """The gradient workload: per-cell eps_r from a seeded Gaussian random field (correlation
    20 mm, clipped to [1, 20]), sigma ~ U[0, 0.01] S/m, four z-directed dipoles and eight
    receivers on a plane 5 cells below the top PML, Ricker 1 GHz. Returns the input lines,
    eps_r and sigma [nx][ny][nz], and the 'true' eps_r of the observed data (eps_r with a
    buried 40 mm box raised by 5 %)."""
    nx, ny, nz = shape
    rng = np.random.default_rng(seed)
    eps = gaussian_random_field(shape, 0.020 / dx, seed)
    sig = rng.uniform(0, 0.01, shape)
    top = (nz - pml - 5) * dx
    lines = ['#domain: {:g} {:g} {:g}'.format(nx * dx, ny * dx, nz * dx),
             '#dx_dy_dz: {0:g} {0:g} {0:g}'.format(dx), '#time_window: {}'.format(timewindow),
             '#pml_cells: {}'.format(pml), '#waveform: ricker 1 1e9 w']
    for s in range(4):
        x = (0.3 + 0.4 * (s % 2)) * nx * dx
        y = (0.3 + 0.4 * (s // 2)) * ny * dx
        lines.append('#hertzian_dipole: z {:g} {:g} {:g} w'.format(x, y, top))
    for r in range(8):
        x = (0.2 + 0.6 * (r % 4) / 3) * nx * dx
        y = (0.35 + 0.3 * (r // 4)) * ny * dx
        lines.append('#rx: {:g} {:g} {:g}'.format(x, y, top))
    true = eps.copy()
    b = int(round(0.040 / dx))
    c = (nx // 2, ny // 2, nz // 2 - b)
    true[c[0] - b // 2:c[0] + b // 2, c[1] - b // 2:c[1] + b // 2, c[2] - b // 2:c[2] + b // 2] *= 1.05
    return [line + '\n' for line in lines], eps, sig, true
