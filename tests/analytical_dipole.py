"""Fields of an infinitesimal (Hertzian) dipole in free space, in the time domain (test
infrastructure). For a z-directed element of length dl at the origin carrying current I(t),
with retarded time tau = t - r/c and charge q = integral of I:

    E_r     = dl cos(th) / (2 pi e0) * ( q/r^3 + I/(c r^2) )
    E_theta = dl sin(th) / (4 pi e0) * ( q/r^3 + I/(c r^2) + I'/(c^2 r) )
    H_phi   = dl sin(th) / (4 pi)    * ( I/r^2 + I'/(c r) )

(the textbook near-, intermediate- and far-field terms of the radiating dipole). Ez follows from
Ez = E_r cos(th) - E_theta sin(th).
"""
import numpy as np
from scipy.constants import c, epsilon_0 as e0


def dipole_ez(current, t, dl, x, y, z, oversample=64):
    """Ez at offset (x, y, z) from a z-directed dipole for the current waveform ``current``
    (a function of time, seconds) at times ``t``."""
    r = np.sqrt(x * x + y * y + z * z)
    cos = z / r
    sin = np.sqrt(x * x + y * y) / r
    tau = np.asarray(t, dtype=np.float64) - r / c
    # fine grid for the derivative and the charge integral
    step = (t[1] - t[0]) / oversample
    fine = np.arange(min(tau.min(), 0.0) - step, tau.max() + 2 * step, step)
    i_f = current(fine)
    di_f = np.gradient(i_f, step)
    q_f = np.concatenate(([0.0], np.cumsum(0.5 * (i_f[1:] + i_f[:-1]) * step)))
    I = np.interp(tau, fine, i_f)
    dI = np.interp(tau, fine, di_f)
    q = np.interp(tau, fine, q_f)
    er = dl * cos / (2 * np.pi * e0) * (q / r ** 3 + I / (c * r ** 2))
    eth = dl * sin / (4 * np.pi * e0) * (q / r ** 3 + I / (c * r ** 2) + dI / (c ** 2 * r))
    return er * cos - eth * sin
