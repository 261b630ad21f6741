"""Receivers: point samples of the fields each step (``gprMax/receivers.py``,
``gprMax/fields_outputs.py:40-67``). Samples are taken at the start of every iteration, before
the H update, and include the currents Ix, Iy, Iz from the circulation of H (``grid.py:413-461``).
"""
from collections import OrderedDict

import numpy as np

from .constants import floattype

OUTPUT_INDEX = {'Ex': 0, 'Ey': 1, 'Ez': 2, 'Hx': 3, 'Hy': 4, 'Hz': 5, 'Ix': 6, 'Iy': 7, 'Iz': 8}


class Rx:
    """A receiver at one grid node with an ordered set of outputs."""

    allowableoutputs = ['Ex', 'Ey', 'Ez', 'Hx', 'Hy', 'Hz', 'Ix', 'Iy', 'Iz']
    defaultoutputs = allowableoutputs[:-3]

    def __init__(self):
        self.ID = None
        self.outputs = OrderedDict()
        self.xcoord = self.ycoord = self.zcoord = None
        self.xcoordorigin = self.ycoordorigin = self.zcoordorigin = None


def allocate_outputs(rx, names, iterations):
    for name in names:
        rx.outputs[name] = np.zeros(iterations, dtype=floattype)
