"""Materials and their fp32 update coefficients (``gprMax/materials.py:26-241``).

The coefficient formulas are the reference's (Yee update with conductivity; the ADE
recursion of http://dx.doi.org/10.1109/TAP.2014.2308549 for Debye, Lorentz and Drude poles).
They are evaluated with the same numpy scalar types as the reference so that the fp32/complex64
tables agree bit for bit: the per-pole terms live in complex64 arrays, which makes the
dispersive E coefficients fp32 arithmetic under numpy's promotion rules.
"""
import numpy as np

from .constants import e0, m0, complextype, floattype


class Material:
    """One material: constitutive parameters, dispersion poles and update coefficients."""

    # Properties of water (http://dx.doi.org/10.1109/TGRS.2006.873208)
    waterer = 80.1
    watereri = 4.9
    waterdeltaer = waterer - watereri
    watertau = 9.231e-12

    def __init__(self, numID, ID):
        self.numID = numID
        self.ID = ID
        self.type = ''
        self.averagable = True
        self.er = 1.0
        self.se = 0.0
        self.mr = 1.0
        self.sm = 0.0
        self.poles = 0
        self.deltaer = []
        self.tau = []
        self.alpha = []

    def calculate_update_coeffsH(self, G):
        """Magnetic coefficients DA, DBx, DBy, DBz, srcm (``materials.py:63-82``)."""
        HA = (m0 * self.mr / G.dt) + 0.5 * self.sm
        HB = (m0 * self.mr / G.dt) - 0.5 * self.sm
        self.DA = HB / HA
        self.DBx = (1 / G.dx) * 1 / HA
        self.DBy = (1 / G.dy) * 1 / HA
        self.DBz = (1 / G.dz) * 1 / HA
        self.srcm = 1 / HA

    def calculate_update_coeffsE(self, G):
        """Electric coefficients CA, CBx, CBy, CBz, srce and pole terms (``materials.py:84-143``)."""
        maxpoles = G.maxpoles
        if maxpoles > 0:
            self.w = np.zeros(maxpoles, dtype=complextype)
            self.q = np.zeros(maxpoles, dtype=complextype)
            self.zt = np.zeros(maxpoles, dtype=complextype)
            self.zt2 = np.zeros(maxpoles, dtype=complextype)
            self.eqt = np.zeros(maxpoles, dtype=complextype)
            self.eqt2 = np.zeros(maxpoles, dtype=complextype)
            for x in range(self.poles):
                if 'debye' in self.type:
                    self.w[x] = self.deltaer[x] / self.tau[x]
                    self.q[x] = -1 / self.tau[x]
                elif 'lorentz' in self.type:
                    # tau holds pole frequencies and alpha damping coefficients
                    wp2 = (2 * np.pi * self.tau[x]) ** 2
                    self.w[x] = -1j * ((wp2 * self.deltaer[x]) / np.sqrt(wp2 - self.alpha[x] ** 2))
                    self.q[x] = -self.alpha[x] + (1j * np.sqrt(wp2 - self.alpha[x] ** 2))
                elif 'drude' in self.type:
                    # tau holds pole frequencies and alpha inverse relaxation times
                    wp2 = (2 * np.pi * self.tau[x]) ** 2
                    self.se += wp2 / self.alpha[x]
                    self.w[x] = -(wp2 / self.alpha[x])
                    self.q[x] = -self.alpha[x]
                self.eqt[x] = np.exp(self.q[x] * G.dt)
                self.eqt2[x] = np.exp(self.q[x] * (G.dt / 2))
                self.zt[x] = (self.w[x] / self.q[x]) * (1 - self.eqt[x]) / G.dt
                self.zt2[x] = (self.w[x] / self.q[x]) * (1 - self.eqt2[x])
            EA = (e0 * self.er / G.dt) + 0.5 * self.se - (e0 / G.dt) * np.sum(self.zt2.real)
            EB = (e0 * self.er / G.dt) - 0.5 * self.se - (e0 / G.dt) * np.sum(self.zt2.real)
        else:
            EA = (e0 * self.er / G.dt) + 0.5 * self.se
            EB = (e0 * self.er / G.dt) - 0.5 * self.se

        if self.ID == 'pec' or self.se == float('inf'):
            self.CA = 0
            self.CBx = 0
            self.CBy = 0
            self.CBz = 0
            self.srce = 0
        else:
            self.CA = EB / EA
            self.CBx = (1 / G.dx) * 1 / EA
            self.CBy = (1 / G.dy) * 1 / EA
            self.CBz = (1 / G.dz) * 1 / EA
            self.srce = 1 / EA

    def calculate_er(self, freq):
        """Complex relative permittivity at ``freq`` (``materials.py:145-174``)."""
        er = self.er
        if self.poles > 0:
            w = 2 * np.pi * freq
            er += self.se / (1j * w * e0)
            if 'debye' in self.type:
                for pole in range(self.poles):
                    er += self.deltaer[pole] / (1 + 1j * w * self.tau[pole])
            elif 'lorentz' in self.type:
                for pole in range(self.poles):
                    er += ((self.deltaer[pole] * self.tau[pole] ** 2)
                           / (self.tau[pole] ** 2 + 2j * w * self.alpha[pole] - w ** 2))
            elif 'drude' in self.type:
                ersum = 0
                for pole in range(self.poles):
                    ersum += self.tau[pole] ** 2 / (w ** 2 - 1j * w * self.alpha[pole])
                    er -= ersum
        return er


def builtin_materials():
    """The two materials every model starts with: pec (0) and free_space (1)."""
    pec = Material(0, 'pec')
    pec.se = float('inf')
    pec.type = 'builtin'
    pec.averagable = False
    fs = Material(1, 'free_space')
    fs.type = 'builtin'
    return [pec, fs]


def process_materials(G):
    """Fill ``G.updatecoeffsE/H`` (fp32 [nmat][5]) and ``G.updatecoeffsdispersive``
    (complex64 [nmat][3*maxpoles]) from ``G.materials`` (``materials.py:177-241``)."""
    nmat = len(G.materials)
    G.updatecoeffsE = np.zeros((nmat, 5), dtype=floattype)
    G.updatecoeffsH = np.zeros((nmat, 5), dtype=floattype)
    if G.maxpoles > 0:
        G.updatecoeffsdispersive = np.zeros((nmat, 3 * G.maxpoles), dtype=complextype)
    else:
        G.updatecoeffsdispersive = None
    for material in G.materials:
        material.calculate_update_coeffsE(G)
        material.calculate_update_coeffsH(G)
        G.updatecoeffsE[material.numID, :] = (material.CA, material.CBx, material.CBy,
                                              material.CBz, material.srce)
        G.updatecoeffsH[material.numID, :] = (material.DA, material.DBx, material.DBy,
                                              material.DBz, material.srcm)
        if G.maxpoles > 0:
            z = 0
            for pole in range(G.maxpoles):
                G.updatecoeffsdispersive[material.numID, z:z + 3] = (
                    e0 * material.eqt2[pole], material.eqt[pole], material.zt[pole])
                z += 3
