"""Fractal volumes for ``#fractal_box`` (``gprMax/fractals.py:141-194``) and the Peplinski soil
mixing model for ``#soil_peplinski`` (``gprMax/materials.py:244-330``).

The volume is generated with the same library calls and the same floating-point operations as
the reference, so the binned material numbers (and hence the material-ID array) agree bit for
bit: seeded standard normals (``numpy.random.default_rng``), ``scipy.fftpack`` FFTs and shifts,
the 1/r^D filter of ``fractals_generate_ext.pyx:56-86`` (rr = (dx^2 + dy^2 + dz^2)^(1/2) and
B = rr^D, every power through the C library's ``pow`` in float64, D rounded to float32 as the
extension's ``float D`` argument, B = 0.9 where it is zero, the complex value divided by the
real B component-wise), the DC term
zeroed, the real part of the inverse FFT in float32, and ``numpy.digitize`` into ``nbins``
bins row by row.

With ``device=True`` (an opt-in for building many realisations) the same seeded noise goes
through the transforms and the filter on the GPU (``gbf_fractal_field``, double precision); the
field then agrees with the reference's to rounding, so a cell whose value lies at a bin edge can
land in the neighbouring bin.
"""
import math

import numpy as np
from scipy import fftpack

from .constants import floattype
from .materials import Material


def _fractal_filter(A, w, v1, dimension):
    """A / r^D with r the weighted distance of each index from v1 (``fractals_generate_ext.pyx``
    ``generate_fractal2D`` :24-50 and ``generate_fractal3D`` :53-86). Every power goes through
    the C library's pow (math.pow), as the compiled filter does (numpy's vectorised power
    differs from it in the last bit); D is rounded to float32 as the extension's ``float D``
    argument; r^D = 0 becomes 0.9; the complex value is divided by the real B component-wise."""
    cpow = np.frompyfunc(math.pow, 2, 1)
    nd = A.ndim
    d = [cpow(w[a] * np.arange(A.shape[a], dtype=np.float64) - v1[a], 2.0).astype(np.float64)
         for a in range(nd)]
    if nd == 3:
        s = d[0][:, None, None] + d[1][None, :, None] + d[2][None, None, :]
    else:
        s = d[0][:, None] + d[1][None, :]
    rr = cpow(s, 0.5)
    B = cpow(rr, float(np.float32(dimension))).astype(np.float64)
    B[B == 0] = 0.9
    out = np.empty(A.shape, dtype=np.complex128)
    out.real = A.real / B
    out.imag = A.imag / B
    return out


def device_field(noise, weights, dimension):
    """The fp32 fractal field of ``noise`` (float64, 2D or 3D) computed on the GPU: the filtered
    inverse FFT's real part, ``dimension`` taken as float32 as the reference's filter takes it."""
    import ctypes
    from . import _native
    from .exceptions import SolverError
    lib = _native.lib()
    noise = np.ascontiguousarray(noise, dtype=np.float64)
    dims = np.array(noise.shape, dtype=np.int32)
    w = np.ascontiguousarray(weights, dtype=np.float64)
    out = np.empty(noise.shape, dtype=np.float32)
    p = lambda a: ctypes.c_void_p(a.ctypes.data)
    rc = lib.gbf_fractal_field(noise.ndim, p(dims), p(w), ctypes.c_float(float(np.float32(dimension))),
                               p(noise), p(out))
    if rc != 0:
        raise SolverError('gbf_fractal_field failed ({})'.format(rc))
    return out


class FractalSurface:
    """A fractal surface on one face of a fractal box (``#add_surface_roughness``,
    ``gprMax/fractals.py:29-111``): heights in cells, scaled into ``fractalrange``."""

    surfaceIDs = ['xminus', 'xplus', 'yminus', 'yplus', 'zminus', 'zplus']

    def __init__(self, xs, xf, ys, yf, zs, zf, dimension, seed):
        self.ID = None
        self.surfaceID = None
        self.xs, self.xf, self.ys, self.yf, self.zs, self.zf = xs, xf, ys, yf, zs, zf
        self.nx = xf - xs
        self.ny = yf - ys
        self.nz = zf - zs
        self.seed = seed
        self.dimension = dimension
        self.weighting = np.array([1, 1], dtype=np.float64)
        self.fractalrange = (0, 0)
        self.filldepth = 0
        self.operatingonID = None

    def generate_fractal_surface(self, device=False):
        """Heights (float32 [n1][n2]) of the surface (``device``: transforms on the GPU)."""
        if self.xs == self.xf:
            dims = (self.ny, self.nz)
        elif self.ys == self.yf:
            dims = (self.nx, self.nz)
        else:
            dims = (self.nx, self.ny)
        w = self.weighting
        v1 = np.array([w[0] * dims[0] / 2, w[1] * dims[1] / 2])
        rng = np.random.default_rng(seed=self.seed)
        A = rng.standard_normal(size=(dims[0], dims[1]))
        if device:
            surf = device_field(A, w, self.dimension)
        else:
            A = fftpack.fftshift(fftpack.fftn(A))
            surf = fftpack.ifftshift(_fractal_filter(A, w, v1, self.dimension))
            surf[0, 0] = 0
            surf = np.real(fftpack.ifftn(surf)).astype(floattype, copy=False)
        # scaled to the requested range (the reference's expression, types as numpy gives them)
        fmin = np.amin(surf)
        fmax = np.amax(surf)
        frange = fmax - fmin
        r0, r1 = self.fractalrange
        surf = surf * ((r1 - r0) / frange) + r0 - ((r1 - r0) / frange) * fmin
        self.fractalsurface = surf
        return surf


class FractalVolume:
    """A box whose cells take one of ``nbins`` materials from a seeded fractal field."""

    def __init__(self, xs, xf, ys, yf, zs, zf, dimension, seed):
        self.ID = None
        self.operatingonID = None
        self.xs, self.xf, self.ys, self.yf, self.zs, self.zf = xs, xf, ys, yf, zs, zf
        self.nx = xf - xs
        self.ny = yf - ys
        self.nz = zf - zs
        self.averaging = False
        self.seed = seed
        self.dimension = dimension
        self.weighting = np.array([1, 1, 1], dtype=np.float64)
        self.nbins = 0
        self.fractalsurfaces = []

    def extend_for_surfaces(self):
        """Grow the box to take in the ranges of its rough surfaces, keeping the original
        extent (``input_cmds_geometry.py:1266-1298``)."""
        self.originalxs, self.originalxf = self.xs, self.xf
        self.originalys, self.originalyf = self.ys, self.yf
        self.originalzs, self.originalzf = self.zs, self.zf
        for surface in self.fractalsurfaces:
            lo, hi = surface.fractalrange
            if surface.surfaceID == 'xminus' and lo < self.xs:
                self.nx += self.xs - lo
                self.xs = lo
            elif surface.surfaceID == 'xplus' and hi > self.xf:
                self.nx += hi - self.xf
                self.xf = hi
            elif surface.surfaceID == 'yminus' and lo < self.ys:
                self.ny += self.ys - lo
                self.ys = lo
            elif surface.surfaceID == 'yplus' and hi > self.yf:
                self.ny += hi - self.yf
                self.yf = hi
            elif surface.surfaceID == 'zminus' and lo < self.zs:
                self.nz += self.zs - lo
                self.zs = lo
            elif surface.surfaceID == 'zplus' and hi > self.zf:
                self.nz += hi - self.zf
                self.zf = hi

    def generate_volume_mask(self):
        """1 inside the original box, 0 in the extension (``fractals.py:196-210``), then each
        rough surface in order: 1 below (or above, on a plus face) the surface, 2 (water) where
        it lies between the surface and the fill depth, 0 elsewhere in the surface's range
        (``input_cmds_geometry.py:1312-1470`` without grass)."""
        mask = np.zeros((self.nx, self.ny, self.nz), dtype=np.int8)
        mx = self.originalxs - self.xs
        my = self.originalys - self.ys
        mz = self.originalzs - self.zs
        mask[mx:mx + self.originalxf - self.originalxs, my:my + self.originalyf - self.originalys,
             mz:mz + self.originalzf - self.originalzs] = 1
        for s in self.fractalsurfaces:
            lo, hi = s.fractalrange
            axis = 'xyz'.index(s.surfaceID[0])
            minus = s.surfaceID.endswith('minus')
            pos = np.arange(lo, hi)
            h = s.fractalsurface
            if axis == 0:
                P = pos[:, None, None]
                H = h[None, :, :]
                region = (slice(lo - self.xs, hi - self.xs), slice(s.ys - self.ys, s.yf - self.ys),
                          slice(s.zs - self.zs, s.zf - self.zs))
            elif axis == 1:
                P = pos[None, :, None]
                H = h[:, None, :]
                region = (slice(s.xs - self.xs, s.xf - self.xs), slice(lo - self.ys, hi - self.ys),
                          slice(s.zs - self.zs, s.zf - self.zs))
            else:
                P = pos[None, None, :]
                H = h[:, :, None]
                region = (slice(s.xs - self.xs, s.xf - self.xs), slice(s.ys - self.ys, s.yf - self.ys),
                          slice(lo - self.zs, hi - self.zs))
            below = (P > H) if minus else (P < H)
            wet = (P > s.filldepth) if minus else (P < s.filldepth)
            wet = wet & (s.filldepth > 0)
            m = np.where(below, 1, np.where(wet, 2, 0)).astype(np.int8)
            mask[region] = np.broadcast_to(m, mask[region].shape)
        self.mask = mask
        return mask

    def generate_fractal_volume(self, device=False):
        """Bin numbers (float32 array [nx][ny][nz], values 0..nbins-1) of the fractal field
        (``device``: transforms on the GPU, binned in one pass)."""
        n = np.array([self.nx, self.ny, self.nz])
        if self.nx == 1:
            scaling = np.insert(np.amin(n[1:]) / n[1:], 0, 1)
        elif self.ny == 1:
            scaling = np.insert(np.amin(n[[0, 2]]) / n[[0, 2]], 1, 1)
        elif self.nz == 1:
            scaling = np.insert(np.amin(n[:2]) / n[:2], 2, 1)
        else:
            scaling = np.amin(n) / n
        self.weighting = np.multiply(self.weighting, scaling)
        w = self.weighting
        v1 = np.array([w[0] * self.nx / 2, w[1] * self.ny / 2, w[2] * self.nz / 2])
        rng = np.random.default_rng(seed=self.seed)
        A = rng.standard_normal(size=(self.nx, self.ny, self.nz))
        if device:
            vol = device_field(A, w, self.dimension)
            bins = np.linspace(np.amin(vol), np.amax(vol), self.nbins)
            # the same rule as the row-by-row loop below, applied to every cell at once
            vol = np.digitize(vol, bins, right=True).astype(floattype)
            self.fractalvolume = vol
            return vol
        A = fftpack.fftshift(fftpack.fftn(A))
        vol = fftpack.ifftshift(_fractal_filter(A, w, v1, self.dimension))
        vol[0, 0, 0] = 0
        vol = np.real(fftpack.ifftn(vol)).astype(floattype, copy=False)
        bins = np.linspace(np.amin(vol), np.amax(vol), self.nbins)
        for j in range(self.ny):
            for k in range(self.nz):
                vol[:, j, k] = np.digitize(vol[:, j, k], bins, right=True)
        self.fractalvolume = vol
        return vol


class PeplinskiSoil:
    """Soil whose materials come from the Peplinski mixing model
    (http://dx.doi.org/10.1109/36.387598): one single-pole Debye material per bin of the
    volumetric water fraction."""

    def __init__(self, ID, sandfraction, clayfraction, bulkdensity, sandpartdensity,
                 watervolfraction):
        self.ID = ID
        self.S = sandfraction
        self.C = clayfraction
        self.rb = bulkdensity
        self.rs = sandpartdensity
        self.mu = watervolfraction
        self.startmaterialnum = 0

    def calculate_debye_properties(self, nbins, G, fractalboxname):
        """Append the ``nbins`` materials named ``|<box>_<n>|`` to ``G.materials``."""
        self.startmaterialnum = len(G.materials)
        f = 1.3e9
        w = 2 * np.pi * f
        erealw = Material.watereri + ((Material.waterdeltaer) / (1 + (w * Material.watertau) ** 2))
        a = 0.65
        es = (1.01 + 0.44 * self.rs) ** 2 - 0.062
        b1 = 1.2748 - 0.519 * self.S - 0.152 * self.C
        b2 = 1.33797 - 0.603 * self.S - 0.166 * self.C
        sigf = 0.0467 + 0.2204 * self.rb - 0.411 * self.S + 0.6614 * self.C
        mubins = np.linspace(self.mu[0], self.mu[1], nbins)
        mumaterials = mubins + (mubins[1] - mubins[0]) / 2
        digits = len(str(int(nbins)))
        it = np.nditer(mumaterials, flags=['c_index'])
        while not it.finished:
            mu = it[0]
            er = (1 + (self.rb / self.rs) * ((es ** a) - 1) + (mu ** b1 * erealw ** a) - mu) ** (1 / a)
            er = 1.15 * er - 0.68
            eri = er - (mu ** (b2 / a) * Material.waterdeltaer)
            sig = mu ** (b2 / a) * ((sigf * (self.rs - self.rb)) / (self.rs * mu))
            m = Material(len(G.materials), '|{}_{}|'.format(fractalboxname,
                                                         str(it.index + 1).zfill(digits)))
            m.type = 'debye'
            m.averagable = False
            m.poles = 1
            if m.poles > G.maxpoles:
                G.maxpoles = m.poles
            m.er = eri
            m.se = sig
            m.deltaer.append(er - eri)
            m.tau.append(Material.watertau)
            G.materials.append(m)
            it.iternext()
