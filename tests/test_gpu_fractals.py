"""GPU: fractal fields transformed on the device (``gbf_fractal_field``) against the host
restatement, which reproduces the reference's field bit for bit (``gprMax/fractals.py:141-194``,
``fractals_generate_ext.pyx:24-86``). The device transforms round differently, so the field
agrees to rounding and a cell whose value sits at a bin edge can change bin; the tests bound
the field difference and the share of cells that change bin, and print both."""
import time

import numpy as np
import pytest

from models import MODELS

pytestmark = pytest.mark.gpu


def _host_field(A, w, D):
    from scipy import fftpack
    from gprmax_gb300.fractals import _fractal_filter
    v1 = np.array([w[a] * A.shape[a] / 2 for a in range(A.ndim)])
    F = fftpack.fftshift(fftpack.fftn(A))
    F = fftpack.ifftshift(_fractal_filter(F, w, v1, D))
    F[(0,) * A.ndim] = 0
    return np.real(fftpack.ifftn(F)).astype(np.float32)


@pytest.mark.parametrize('shape,w,D', [((40, 33, 27), (1.0, 0.5, 2.0), 1.5),
                                       ((64, 48), (1.0, 1.0), 2.2),
                                       ((101, 80, 75), (0.8, 1.0, 1.0), 2.7)])
def test_device_field_equals_host_field(native, shape, w, D):
    from gprmax_gb300.fractals import device_field
    A = np.random.default_rng(11).standard_normal(size=shape)
    host = _host_field(A, np.array(w), D)
    dev = device_field(A, np.array(w), D)
    err = np.abs(dev.astype(np.float64) - host).max() / (host.max() - host.min())
    print('\n{}: max |device - host| / field range = {:.2e}'.format(shape, err))
    assert err <= 1e-5


@pytest.mark.parametrize('name', ['fractal', 'rough'])
def test_device_fractals_in_model_builds(native, name):
    """The fixtures' fractal boxes (Peplinski soil, rough and wet surfaces) built with the
    transforms on the device: the material IDs differ from the host build only at bin edges."""
    from gprmax_gb300.model import build_grid
    host = build_grid(MODELS[name].splitlines(True), messages=False)
    dev = build_grid(MODELS[name].splitlines(True), messages=False, device_fractals=True)
    flips = float(np.mean(host.ID != dev.ID))
    print('\n{}: share of edge IDs that differ from the host build = {:.2e}'.format(name, flips))
    assert flips <= 1e-3


def test_device_fractal_volume_at_the_soil_size(native):
    """The benchmark soil's 400 x 400 x 150 fractal volume binned into 50 materials."""
    from gprmax_gb300.workloads import fractal_volume
    t0 = time.perf_counter()
    host = fractal_volume((400, 400, 150), 1.5, 1, 50)
    t1 = time.perf_counter()
    dev = fractal_volume((400, 400, 150), 1.5, 1, 50, device=True)
    t2 = time.perf_counter()
    flips = float(np.mean(host != dev))
    print('\nsoil volume: host {:.2f} s, device {:.2f} s (both with the host noise), share of cells '
          'in another bin {:.2e}'.format(t1 - t0, t2 - t1, flips))
    assert flips <= 1e-4
    assert np.abs(host - dev).max() <= 1
