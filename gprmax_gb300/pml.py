"""CFS perfectly matched layers: profiles and update coefficients (``gprMax/pml.py``).

A model has up to six slabs, built in the fixed order x0, y0, z0, xmax, ymax, zmax
(``grid.py:132-136``); the solver applies their corrections in that order. Each slab carries
per-depth coefficient rows ``ERA, ERB, ERE, ERF`` (electric) and ``HRA..HRF`` (magnetic),
fp32 [n_cfs][thickness], for the HORIPML (https://doi.org/10.1109/TAP.2011.2180344) or MRIPML
(https://doi.org/10.1109/TAP.2018.2823864) formulation. The coefficient arithmetic keeps the
reference's array dtypes (``pml.py:221-274``) so the fp32 rows agree bit for bit.
"""
from collections import OrderedDict

import numpy as np

from .constants import e0, z0, floattype


class CFSParameter:
    """One CFS parameter (alpha, kappa or sigma) with its grading profile."""

    scalingprofiles = {'constant': 0, 'linear': 1, 'quadratic': 2, 'cubic': 3, 'quartic': 4,
                       'quintic': 5, 'sextic': 6, 'septic': 7, 'octic': 8}
    scalingdirections = ['forward', 'reverse']

    def __init__(self, ID=None, scaling='polynomial', scalingprofile=None,
                 scalingdirection='forward', min=0, max=0):
        self.ID = ID
        self.scaling = scaling
        self.scalingprofile = scalingprofile
        self.scalingdirection = scalingdirection
        self.min = min
        self.max = max


class CFS:
    """One CFS term (one PML order): alpha, kappa, sigma (defaults ``pml.py:67-69``)."""

    def __init__(self):
        self.alpha = CFSParameter(ID='alpha', scalingprofile='constant')
        self.kappa = CFSParameter(ID='kappa', scalingprofile='constant', min=1, max=1)
        self.sigma = CFSParameter(ID='sigma', scalingprofile='quartic', min=0, max=None)

    def calculate_sigmamax(self, d, er, mr):
        """Optimum sigma max (http://dx.doi.org/10.1109/8.546249; ``pml.py:71-83``)."""
        m = CFSParameter.scalingprofiles[self.sigma.scalingprofile]
        self.sigma.max = (0.8 * (m + 1)) / (z0 * d * np.sqrt(er * mr))

    @staticmethod
    def scaling_polynomial(order, Evalues, Hvalues):
        """Polynomial sampled at whole (E) and half (H) cells from the inner face."""
        tmp = (np.linspace(0, (len(Evalues) - 1) + 0.5, num=2 * len(Evalues))
               / (len(Evalues) - 1)) ** order
        return tmp[0:-1:2], tmp[1::2]

    def calculate_values(self, thickness, parameter):
        """Profile of one parameter at E and H depths (``pml.py:104-146``)."""
        Evalues = np.zeros(thickness + 1, dtype=floattype)
        Hvalues = np.zeros(thickness + 1, dtype=floattype)
        if parameter.scalingprofile == 'constant':
            Evalues += parameter.max
            Hvalues += parameter.max
        elif parameter.scaling == 'polynomial':
            Evalues, Hvalues = self.scaling_polynomial(
                CFSParameter.scalingprofiles[parameter.scalingprofile], Evalues, Hvalues)
            p = {'alpha': self.alpha, 'kappa': self.kappa, 'sigma': self.sigma}[parameter.ID]
            Evalues = Evalues * (p.max - p.min) + p.min
            Hvalues = Hvalues * (p.max - p.min) + p.min
        if parameter.scalingdirection == 'reverse':
            Evalues = Evalues[::-1]
            Hvalues = Hvalues[::-1]
            # magnetic samples move one element left after the reversal
            Hvalues = np.roll(Hvalues, -1)
        return Evalues[:-1], Hvalues[:-1]


class PML:
    """One PML slab: extent, grading direction and fp32 coefficient rows."""

    formulations = ['HORIPML', 'MRIPML']
    boundaryIDs = ['x0', 'y0', 'z0', 'xmax', 'ymax', 'zmax']
    directions = ['xminus', 'yminus', 'zminus', 'xplus', 'yplus', 'zplus']

    def __init__(self, G, ID=None, direction=None, xs=0, xf=0, ys=0, yf=0, zs=0, zf=0):
        self.ID = ID
        self.direction = direction
        self.xs, self.xf, self.ys, self.yf, self.zs, self.zf = xs, xf, ys, yf, zs, zf
        self.nx = xf - xs
        self.ny = yf - ys
        self.nz = zf - zs
        if direction[0] == 'x':
            self.d = G.dx
            self.thickness = self.nx
        elif direction[0] == 'y':
            self.d = G.dy
            self.thickness = self.ny
        else:
            self.d = G.dz
            self.thickness = self.nz
        self.CFS = G.cfs

    @property
    def axis(self):
        return 'xyz'.index(self.direction[0])

    @property
    def minus(self):
        return self.direction.endswith('minus')

    def calculate_update_coeffs(self, er, mr, G):
        """Coefficient rows for this slab (``pml.py:221-274``). Sigma max is filled in only
        when it is unset; CFS terms are shared by all slabs, so the first slab built fixes it."""
        n = len(self.CFS)
        shape = (n, self.thickness)
        self.ERA = np.zeros(shape, dtype=floattype)
        self.ERB = np.zeros(shape, dtype=floattype)
        self.ERE = np.zeros(shape, dtype=floattype)
        self.ERF = np.zeros(shape, dtype=floattype)
        self.HRA = np.zeros(shape, dtype=floattype)
        self.HRB = np.zeros(shape, dtype=floattype)
        self.HRE = np.zeros(shape, dtype=floattype)
        self.HRF = np.zeros(shape, dtype=floattype)
        for x, cfs in enumerate(self.CFS):
            if not cfs.sigma.max:
                cfs.calculate_sigmamax(self.d, er, mr)
            Ealpha, Halpha = cfs.calculate_values(self.thickness, cfs.alpha)
            Ekappa, Hkappa = cfs.calculate_values(self.thickness, cfs.kappa)
            Esigma, Hsigma = cfs.calculate_values(self.thickness, cfs.sigma)
            dt = G.dt
            if G.pmlformulation == 'HORIPML':
                tmp = (2 * e0 * Ekappa) + dt * (Ealpha * Ekappa + Esigma)
                self.ERA[x, :] = (2 * e0 + dt * Ealpha) / tmp
                self.ERB[x, :] = (2 * e0 * Ekappa) / tmp
                self.ERE[x, :] = ((2 * e0 * Ekappa) - dt * (Ealpha * Ekappa + Esigma)) / tmp
                self.ERF[x, :] = (2 * Esigma * dt) / (Ekappa * tmp)
                tmp = (2 * e0 * Hkappa) + dt * (Halpha * Hkappa + Hsigma)
                self.HRA[x, :] = (2 * e0 + dt * Halpha) / tmp
                self.HRB[x, :] = (2 * e0 * Hkappa) / tmp
                self.HRE[x, :] = ((2 * e0 * Hkappa) - dt * (Halpha * Hkappa + Hsigma)) / tmp
                self.HRF[x, :] = (2 * Hsigma * dt) / (Hkappa * tmp)
            elif G.pmlformulation == 'MRIPML':
                tmp = 2 * e0 + dt * Ealpha
                self.ERA[x, :] = Ekappa + (dt * Esigma) / tmp
                self.ERB[x, :] = (2 * e0) / tmp
                self.ERE[x, :] = ((2 * e0) - dt * Ealpha) / tmp
                self.ERF[x, :] = (2 * Esigma * dt) / tmp
                tmp = 2 * e0 + dt * Halpha
                self.HRA[x, :] = Hkappa + (dt * Hsigma) / tmp
                self.HRB[x, :] = (2 * e0) / tmp
                self.HRE[x, :] = ((2 * e0) - dt * Halpha) / tmp
                self.HRF[x, :] = (2 * Hsigma * dt) / tmp


def default_pml_thickness():
    """Ordered slab thicknesses; the order fixes the order corrections are applied in."""
    return OrderedDict((key, 10) for key in PML.boundaryIDs)


def _face_average(G, face):
    """Sequential (left-to-right) float sums of er and mr over a solid face, divided by its
    size, as the reference's loops accumulate them (``pml.py:397-427``)."""
    er_of = np.array([m.er for m in sorted(G.materials, key=lambda m: m.numID)], dtype=np.float64)
    mr_of = np.array([m.mr for m in sorted(G.materials, key=lambda m: m.numID)], dtype=np.float64)
    ids = face.ravel()
    sumer = np.cumsum(er_of[ids])[-1] if ids.size else 0.0
    summr = np.cumsum(mr_of[ids])[-1] if ids.size else 0.0
    return float(sumer) / ids.size, float(summr) / ids.size


def _solid_face(G, axis, index):
    """One plane of the solid array (read from the device for a grid built there)."""
    geom = getattr(G, 'geom', None)
    if geom is None:
        return G.solid[(slice(None),) * axis + (index,)]
    origin = [0, 0, 0]
    shape = [G.nx, G.ny, G.nz]
    origin[axis] = index
    shape[axis] = 1
    return geom.read(0, origin, shape).squeeze(axis)


def build_pmls(G):
    """Create the slabs of ``G.pmlthickness`` and their coefficients (``pml.py:367-429``)."""
    G.pmls = []
    for key, value in G.pmlthickness.items():
        if value <= 0:
            continue
        if key[0] == 'x':
            if key == 'x0':
                pml = PML(G, ID=key, direction='xminus', xf=value, yf=G.ny, zf=G.nz)
            else:
                pml = PML(G, ID=key, direction='xplus', xs=G.nx - value, xf=G.nx, yf=G.ny, zf=G.nz)
            face = _solid_face(G, 0, pml.xs)
        elif key[0] == 'y':
            if key == 'y0':
                pml = PML(G, ID=key, direction='yminus', yf=value, xf=G.nx, zf=G.nz)
            else:
                pml = PML(G, ID=key, direction='yplus', ys=G.ny - value, xf=G.nx, yf=G.ny, zf=G.nz)
            face = _solid_face(G, 1, pml.ys)
        else:
            if key == 'z0':
                pml = PML(G, ID=key, direction='zminus', zf=value, xf=G.nx, yf=G.ny)
            else:
                pml = PML(G, ID=key, direction='zplus', zs=G.nz - value, xf=G.nx, yf=G.ny, zf=G.nz)
            face = _solid_face(G, 2, pml.zs)
        G.pmls.append(pml)
        averageer, averagemr = _face_average(G, face)
        pml.calculate_update_coeffs(averageer, averagemr, G)
