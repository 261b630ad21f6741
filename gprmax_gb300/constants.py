"""Physical constants and storage types of the solver.

The constants come from ``scipy.constants`` at run time, exactly as the reference takes them
(``gprMax/constants.py:20-25``), so update coefficients agree bit for bit with a reference run
on the same host. Field storage is fp32 and dispersive state complex64 (``constants.py:34-40``).
"""
import numpy as np
from scipy.constants import c
from scipy.constants import mu_0 as m0
from scipy.constants import epsilon_0 as e0

# Impedance of free space (Ohms)
z0 = np.sqrt(m0 / e0)

floattype = np.float32
complextype = np.complex64
