"""The model description handed to the solver (the reference's ``FDTDGrid``, ``grid.py:80-272``).

``FDTDGrid`` holds what the front-end builds: sizes, dt, iteration count, the solid/rigid/ID
arrays, the material list and coefficient tables, PML slabs, sources, receivers and snapshots.
Field arrays are not kept on the host during a run; after a solve the final fields are
downloaded into ``Ex..Hz`` (fp32 [nx+1][ny+1][nz+1]) and ``Tx..Tz`` for dispersive models.
"""
import numpy as np

from .constants import floattype, complextype
from .pml import default_pml_thickness


class FDTDGrid:
    """Attributes of one model."""

    def __init__(self):
        self.inputfilename = ''
        self.inputdirectory = ''
        self.outputdirectory = None
        self.title = ''
        self.messages = True
        self.nthreads = 0
        self.nx = self.ny = self.nz = 0
        self.dx = self.dy = self.dz = 0
        self.dt = 0
        self.mode = None
        self.iterations = 0
        self.timewindow = 0
        self.pmlthickness = default_pml_thickness()
        self.cfs = []
        self.pmls = []
        self.pmlformulation = 'HORIPML'
        self.materials = []
        self.maxpoles = 0
        self.mixingmodels = []
        self.fractalvolumes = []
        self.averagevolumeobjects = True
        self.waveforms = []
        self.voltagesources = []
        self.hertziandipoles = []
        self.magneticdipoles = []
        self.transmissionlines = []
        self.rxs = []
        self.srcsteps = [0, 0, 0]
        self.rxsteps = [0, 0, 0]
        self.snapshots = []
        self.geometryviews = []
        self.geometryobjectswrite = []
        self.IDlookup = {'Ex': 0, 'Ey': 1, 'Ez': 2, 'Hx': 3, 'Hy': 4, 'Hz': 5}
        self.updatecoeffsE = None
        self.updatecoeffsH = None
        self.updatecoeffsdispersive = None

    def within_bounds(self, **kwargs):
        for co, val in kwargs.items():
            if val < 0 or val > getattr(self, 'n' + co):
                raise ValueError(co)

    def calculate_coord(self, coord, val):
        from .utilities import round_value
        return round_value(float(val) / getattr(self, 'd' + coord))

    def initialise_geometry_arrays(self, device=False):
        """solid and ID start as free_space (1); nothing is rigid (``grid.py:157-169``).
        ``device``: the arrays live on the GPU instead (:mod:`gprmax_gb300.devgeom`)."""
        if device:
            from .devgeom import DeviceGeometry
            self.geom = DeviceGeometry(self.nx, self.ny, self.nz)
            self.solid = self.rigidE = self.rigidH = self.ID = None
            return
        self.solid = np.ones((self.nx, self.ny, self.nz), dtype=np.uint32)
        self.rigidE = np.zeros((12, self.nx, self.ny, self.nz), dtype=np.int8)
        self.rigidH = np.zeros((6, self.nx, self.ny, self.nz), dtype=np.int8)
        self.ID = np.ones((6, self.nx + 1, self.ny + 1, self.nz + 1), dtype=np.uint32)

    def field_shape(self):
        return (self.nx + 1, self.ny + 1, self.nz + 1)

    def initialise_field_arrays(self):
        shape = self.field_shape()
        for name in ('Ex', 'Ey', 'Ez', 'Hx', 'Hy', 'Hz'):
            setattr(self, name, np.zeros(shape, dtype=floattype))

    def initialise_dispersive_arrays(self):
        shape = (self.maxpoles,) + self.field_shape()
        for name in ('Tx', 'Ty', 'Tz'):
            setattr(self, name, np.zeros(shape, dtype=complextype))

    def memory_estimate(self):
        """Bytes the GPU solver allocates for this model (fields, IDs, PML, dispersion)."""
        npts = (self.nx + 1) * (self.ny + 1) * (self.nz + 1)
        total = npts * (6 * 4 + 6 * 4)
        if self.maxpoles:
            total += npts * 3 * self.maxpoles * 8
        for pml in self.pmls:
            total += 4 * 4 * len(self.cfs) * pml.thickness * max(
                (self.ny + 1) * (self.nz + 1), (self.nx + 1) * (self.nz + 1),
                (self.nx + 1) * (self.ny + 1))
        return total
