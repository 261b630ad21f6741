"""Field snapshots (``gprMax/snapshots.py:26-130``).

A snapshot samples a strided sub-volume at one iteration: E from the mean of the 4 edge values
and H from the mean of 2 face values of each output cell (``snapshots_ext.pyx:24-71``). The
averaging runs on the GPU; ``electric``/``magnetic`` hold the result in the reference's
Fortran-ordered (component, i, j, k) layout used by its VTK writer.
"""
import sys
from struct import pack

import numpy as np

from .constants import floattype
from .utilities import round_value


class Snapshot:
    """One requested snapshot."""

    def __init__(self, xs=None, ys=None, zs=None, xf=None, yf=None, zf=None, dx=None, dy=None,
                 dz=None, time=None, filename=None):
        self.xs, self.ys, self.zs = xs, ys, zs
        self.xf, self.yf, self.zf = xf, yf, zf
        self.dx, self.dy, self.dz = dx, dy, dz
        self.nx = round_value((self.xf - self.xs) / self.dx)
        self.ny = round_value((self.yf - self.ys) / self.dy)
        self.nz = round_value((self.zf - self.zs) / self.dz)
        self.ncells = self.nx * self.ny * self.nz
        self.datasizefield = 3 * np.dtype(floattype).itemsize * self.ncells
        self.time = time
        self.basefilename = filename
        self.electric = None
        self.magnetic = None

    def set_fields(self, ex, ey, ez, hx, hy, hz):
        """Store the averaged components ([nx][ny][nz] each) in the VTK point layout."""
        self.electric = np.stack((ex, ey, ez)).reshape(-1, order='F')
        self.magnetic = np.stack((hx, hy, hz)).reshape(-1, order='F')

    def write_vtk_imagedata(self, filename, G):
        """Write a VTK ImageData (.vti) file with appended raw E and H cell data."""
        byteorder = 'LittleEndian' if sys.byteorder == 'little' else 'BigEndian'
        self.filename = filename
        hdr = ('<?xml version="1.0"?>\n<VTKFile type="ImageData" version="1.0" byte_order="{}">\n'
               '<ImageData WholeExtent="{} {} {} {} {} {}" Origin="0 0 0" Spacing="{:.3} {:.3} {:.3}">\n'
               '<Piece Extent="{} {} {} {} {} {}">\n<CellData Vectors="E-field H-field">\n'
               '<DataArray type="Float32" Name="E-field" NumberOfComponents="3" format="appended" offset="0" />\n'
               '<DataArray type="Float32" Name="H-field" NumberOfComponents="3" format="appended" offset="{}" />\n'
               '</CellData>\n</Piece>\n</ImageData>\n<AppendedData encoding="raw">\n_').format(
            byteorder, self.xs, round_value(self.xf / self.dx), self.ys,
            round_value(self.yf / self.dy), self.zs, round_value(self.zf / self.dz),
            self.dx * G.dx, self.dy * G.dy, self.dz * G.dz, self.xs,
            round_value(self.xf / self.dx), self.ys, round_value(self.yf / self.dy), self.zs,
            round_value(self.zf / self.dz), self.datasizefield + np.dtype(np.uint32).itemsize)
        with open(filename, 'wb') as f:
            f.write(hdr.encode('utf-8'))
            f.write(pack('I', self.datasizefield))
            f.write(self.electric.astype(floattype).tobytes())
            f.write(pack('I', self.datasizefield))
            f.write(self.magnetic.astype(floattype).tobytes())
            f.write('\n</AppendedData>\n</VTKFile>'.encode('utf-8'))
