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
KIND_TRANSMISSION_LINE = 4


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
        geom = getattr(G, 'geom', None)
        requirednumID = G.ID[comp, i, j, k] if geom is None else geom.id_at(comp, i, j, k)
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
        if geom is None:
            G.ID[comp, i, j, k] = newmaterial.numID
        else:
            geom.set_id(comp, i, j, k, newmaterial.numID)
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
    if name == 'TransmissionLine':
        comp = 'xyz'.index(src.polarisation)
        d = {'x': G.dx, 'y': G.dy, 'z': G.dz}[src.polarisation]
        # the E edge is set to -V/d from the line's state (the table is unused)
        return KIND_TRANSMISSION_LINE, comp, (np.float32(d), np.float32(1)), src.waveformvalues_wholestep
    if name == 'MagneticDipole':
        comp = 3 + 'xyz'.index(src.polarisation)
        scale = (np.float32(1 / (G.dx * G.dy * G.dz)), np.float32(1))
        return KIND_MAGNETIC, comp, scale, src.waveformvalues_halfstep
    raise TypeError('source type {} is not supported by the GB300 solver core'.format(name))


class TransmissionLine(Source):
    """One-dimensional transmission line attached to one E edge (``sources.py:286-451``).

    The line's own 1D update (voltage, current, a first-order absorbing end) runs on the host
    once, unconnected and long, for the incident voltage and current (``calculate_incident_V_I``);
    its end state seeds the short connected line (``antpos + 1`` cells) that the GPU then advances
    every iteration: after the H half-step the line current is updated and its value at the
    antenna cell replaced by the current around the edge (grid.py's Ix/Iy/Iz), then the line
    voltage is updated and the edge's E set to -V/d. The arithmetic follows the reference's numpy
    expressions: the line updates are evaluated in float64 (the step ratio is a float64 scalar)
    and rounded to float32 on assignment."""

    def __init__(self, G=None):
        super().__init__()
        self.resistance = None
        self.abcv0 = 0
        self.abcv1 = 0
        if G is not None:
            self.bind(G)

    def bind(self, G):
        """Line discretisation for grid ``G``."""
        from .constants import c
        from .utilities import round_value
        self.dl = np.sqrt(3) * c * G.dt
        self.nl = round_value(0.667 * G.iterations)
        self.srcpos = 5
        self.antpos = 10
        self.voltage = np.zeros(self.nl, dtype=floattype)
        self.current = np.zeros(self.nl, dtype=floattype)
        self.Vtotal = np.zeros(G.iterations, dtype=floattype)
        self.Itotal = np.zeros(G.iterations, dtype=floattype)

    def ratios(self, G):
        """float64 coefficients of the line updates: I/V (1/R c dt/dl), V/I (R c dt/dl), the
        injection ratio c dt/dl and the absorbing end's h."""
        from .constants import c
        r = c * G.dt / self.dl
        h = (c * G.dt - self.dl) / (c * G.dt + self.dl)
        return (np.float64((1 / self.resistance) * r), np.float64(self.resistance * r),
                np.float64(r), np.float64(h))

    def update_abc(self, G):
        from .constants import c
        h = (c * G.dt - self.dl) / (c * G.dt + self.dl)
        self.voltage[0] = h * (self.voltage[1] - self.abcv0) + self.abcv1
        self.abcv0 = self.voltage[0]
        self.abcv1 = self.voltage[1]

    def update_voltage(self, iteration, G):
        from .constants import c
        nl = self.nl
        self.voltage[1:nl] -= (self.resistance * (c * G.dt / self.dl)
                               * (self.current[1:nl] - self.current[0:nl - 1]))
        self.voltage[self.srcpos] += ((c * G.dt / self.dl) * self.waveformvalues_wholestep[iteration])
        self.update_abc(G)

    def update_current(self, iteration, G):
        from .constants import c
        nl = self.nl
        self.current[0:nl - 1] -= ((1 / self.resistance) * (c * G.dt / self.dl)
                                   * (self.voltage[1:nl] - self.voltage[0:nl - 1]))
        self.current[self.srcpos - 1] += ((1 / self.resistance) * (c * G.dt / self.dl)
                                          * self.waveformvalues_halfstep[iteration])

    def calculate_incident_V_I(self, G):
        """Incident voltage and current of the long, unconnected line; then shorten it."""
        self.Vinc = np.zeros(G.iterations, dtype=floattype)
        self.Iinc = np.zeros(G.iterations, dtype=floattype)
        for iteration in range(G.iterations):
            self.Iinc[iteration] = self.current[self.antpos]
            self.Vinc[iteration] = self.voltage[self.antpos]
            self.update_current(iteration, G)
            self.update_voltage(iteration, G)
        self.nl = self.antpos + 1
