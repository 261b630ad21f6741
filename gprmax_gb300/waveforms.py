"""Source waveform shapes (``gprMax/waveforms.py:24-122``).

Values are evaluated in float64 over whole time vectors with the same operation order as the
reference's scalar code, then stored as fp32 tables by the sources.
"""
import numpy as np


class Waveform:
    """A named waveform: shape, amplitude scaling and centre frequency."""

    types = ['gaussian', 'gaussiandot', 'gaussiandotnorm', 'gaussiandotdot', 'gaussiandotdotnorm',
             'gaussianprime', 'gaussiandoubleprime', 'ricker', 'sine', 'contsine', 'impulse', 'user']

    def __init__(self):
        self.ID = None
        self.type = None
        self.amp = 1
        self.freq = None
        self.userfunc = None
        self.chi = 0
        self.zeta = 0
        self.delay = 0

    def calculate_coefficients(self):
        """Time shift ``chi`` and exponent scale ``zeta`` of the Gaussian family."""
        if self.type in ('gaussian', 'gaussiandot', 'gaussiandotnorm', 'gaussianprime',
                         'gaussiandoubleprime'):
            self.chi = 1 / self.freq
            self.zeta = 2 * np.pi ** 2 * self.freq ** 2
        elif self.type in ('gaussiandotdot', 'gaussiandotdotnorm', 'ricker'):
            self.chi = np.sqrt(2) / self.freq
            self.zeta = np.pi ** 2 * self.freq ** 2

    def values(self, time, dt):
        """Waveform values (float64) at the times in ``time`` (array, seconds)."""
        self.calculate_coefficients()
        t = np.asarray(time, dtype=np.float64)
        z = self.zeta
        if self.type == 'gaussian':
            delay = t - self.chi
            out = np.exp(-z * delay ** 2)
        elif self.type in ('gaussiandot', 'gaussianprime'):
            delay = t - self.chi
            out = -2 * z * delay * np.exp(-z * delay ** 2)
        elif self.type == 'gaussiandotnorm':
            delay = t - self.chi
            normalise = np.sqrt(np.exp(1) / (2 * z))
            out = -2 * z * delay * np.exp(-z * delay ** 2) * normalise
        elif self.type in ('gaussiandotdot', 'gaussiandoubleprime'):
            delay = t - self.chi
            out = 2 * z * (2 * z * delay ** 2 - 1) * np.exp(-z * delay ** 2)
        elif self.type == 'gaussiandotdotnorm':
            delay = t - self.chi
            normalise = 1 / (2 * z)
            out = 2 * z * (2 * z * delay ** 2 - 1) * np.exp(-z * delay ** 2) * normalise
        elif self.type == 'ricker':
            delay = t - self.chi
            normalise = 1 / (2 * z)
            out = -(2 * z * (2 * z * delay ** 2 - 1) * np.exp(-z * delay ** 2)) * normalise
        elif self.type == 'sine':
            out = np.sin(2 * np.pi * self.freq * t)
            out = np.where(t * self.freq > 1, 0.0, out)
        elif self.type == 'contsine':
            rampamp = 0.25
            ramp = np.minimum(rampamp * t * self.freq, 1.0)
            out = ramp * np.sin(2 * np.pi * self.freq * t)
        elif self.type == 'impulse':
            out = np.where((t == 0) | (t < dt), 1.0, 0.0)
        elif self.type == 'user':
            out = np.asarray([float(self.userfunc(x)) for x in t], dtype=np.float64)
        else:
            raise ValueError('unknown waveform type {}'.format(self.type))
        return np.asarray(out, dtype=np.float64) * self.amp

    def calculate_value(self, time, dt):
        """Scalar form of :meth:`values`."""
        return float(self.values(np.array([time]), dt)[0])
