"""Simple sources: Hertzian dipole, voltage source and magnetic dipole (``gprMax/sources.py``).

The host side precomputes each source's fp32 waveform tables at whole and half steps
(``sources.py:47-68``) and the per-source scale factors; the GPU applies the injection inside
the fused half-step kernels with the reference's fp32 operation order:

* Hertzian dipole (``sources.py:163-193``): E -= ((srce * w[it]) * dl) * (1/(dx dy dz))
* resistive voltage source (``sources.py:81-120``): E -= (srce * w[it]) * (1/(R d d)), plus an
  extra material carrying the source conductivity (``sources.py:122-153``)
* hard voltage source (R == 0): E = (-w_half[it]) / d
* magnetic dipole (``sources.py:202-232``): H -= (srcm * w_half[it]) * (1/(dx dy dz))
"""
from copy import deepcopy

import numpy as np

from .constants import floattype

# source kinds understood by the native solver
KIND_HERTZIAN = 0
KIND_VOLTAGE_RESISTIVE = 1
KIND_VOLTAGE_HARD = 2
KIND_MAGNETIC = 3


class Source:
    """A point source bound to a waveform and an active time interval."""

    def __init__(self):
        self.ID = None
        self.polarisation = None
        self.xcoord = self.ycoord = self.zcoord = None
        self.xcoordorigin = self.ycoordorigin = self.zcoordorigin = None
        self.start = None
        self.stop = None
        self.waveformID = None

    def calculate_waveform_values(self, G):
        """fp32 waveform tables at t = it*dt and t = (it+1/2)*dt over the active interval."""
        waveform = next(x for x in G.waveforms if x.ID == self.waveformID)
        time = G.dt * np.arange(G.iterations, dtype=np.float64)
        active = (time >= self.start) & (time <= self.stop)
        t = time[active] - self.start
        self.waveformvalues_wholestep = np.zeros(G.iterations, dtype=floattype)
        self.waveformvalues_halfstep = np.zeros(G.iterations, dtype=floattype)
        if t.size:
            self.waveformvalues_wholestep[active] = waveform.values(t, G.dt)
            self.waveformvalues_halfstep[active] = waveform.values(t + 0.5 * G.dt, G.dt)


class VoltageSource(Source):
    """Hard (R = 0) or resistive voltage source on one E edge."""

    def __init__(self):
        super().__init__()
        self.resistance = None

    def create_material(self, G):
        """Add the source conductivity on the source edge as a new material."""
        if self.resistance == 0:
            return
        i, j, k = self.xcoord, self.ycoord, self.zcoord
        comp = 'xyz'.index(self.polarisation)
        requirednumID = G.ID[comp, i, j, k]
        material = next(x for x in G.materials if x.numID == requirednumID)
        newmaterial = deepcopy(material)
        newmaterial.ID = material.ID + '+' + self.ID
        newmaterial.numID = len(G.materials)
        newmaterial.averagable = False
        newmaterial.type += ',\nvoltage-source'
        if self.polarisation == 'x':
            newmaterial.se += G.dx / (self.resistance * G.dy * G.dz)
        elif self.polarisation == 'y':
            newmaterial.se += G.dy / (self.resistance * G.dx * G.dz)
        else:
            newmaterial.se += G.dz / (self.resistance * G.dx * G.dy)
        G.ID[comp, i, j, k] = newmaterial.numID
        G.materials.append(newmaterial)

class HertzianDipole(Source):
    """Additive electric current element of length ``dl`` on one E edge."""

    def __init__(self):
        super().__init__()
        self.dl = None

class MagneticDipole(Source):
    """Additive magnetic current element on one H edge."""


def active_range(src, G):
    """First and last iteration (inclusive) at which the source is active: those whose time
    ``G.dt * iteration`` lies in [start, stop] (``sources.py:61-64``); (0, -1) when none."""
    t = G.dt * np.arange(G.iterations, dtype=np.float64)
    idx = np.nonzero((t >= src.start) & (t <= src.stop))[0]
    if idx.size == 0:
        return 0, -1
    return int(idx[0]), int(idx[-1])


def kernel_record(src, G):
    """(kind, component, (s0, s1), waveform table) of one source for the native solver.

    Reads only attributes the reference's own source objects carry (``polarisation``,
    ``resistance``, ``dl``, ``waveformvalues_wholestep``/``_halfstep``), so it serves sources
    built by this package's parser and by the reference's alike."""
    name = type(src).__name__
    if name == 'VoltageSource':
        comp = 'xyz'.index(src.polarisation)
        if src.resistance != 0:
            other = {'x': G.dy * G.dz, 'y': G.dx * G.dz, 'z': G.dx * G.dy}[src.polarisation]
            scale = (np.float32(1 / (src.resistance * other)), np.float32(1))
            return KIND_VOLTAGE_RESISTIVE, comp, scale, src.waveformvalues_wholestep
        d = {'x': G.dx, 'y': G.dy, 'z': G.dz}[src.polarisation]
        return KIND_VOLTAGE_HARD, comp, (np.float32(d), np.float32(1)), src.waveformvalues_halfstep
    if name == 'HertzianDipole':
        comp = 'xyz'.index(src.polarisation)
        scale = (np.float32(src.dl), np.float32(1 / (G.dx * G.dy * G.dz)))
        return KIND_HERTZIAN, comp, scale, src.waveformvalues_wholestep
    if name == 'MagneticDipole':
        comp = 3 + 'xyz'.index(src.polarisation)
        scale = (np.float32(1 / (G.dx * G.dy * G.dz)), np.float32(1))
        return KIND_MAGNETIC, comp, scale, src.waveformvalues_halfstep
    raise TypeError('source type {} is not supported by the GB300 solver core'.format(name))
