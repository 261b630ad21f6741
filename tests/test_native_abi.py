"""The C ABI library without a GPU: it builds, loads, exports every function that
include/gbfdtd.h declares, and its host-only parts behave (CPU only)."""
import os
import re
from fractions import Fraction

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, 'include', 'gbfdtd.h')


def _declared():
    text = open(HEADER).read()
    text = re.sub(r'/\*.*?\*/', '', text, flags=re.S)
    return sorted(set(re.findall(r'\b(gbf_\w+)\s*\(', text)))


@pytest.fixture(scope='module')
def lib():
    from gprmax_gb300 import _native
    _native.build()
    return _native.load()


def test_header_and_bindings_agree():
    from gprmax_gb300 import _native
    assert _declared() == _native.exported_symbols()


def test_library_exports_every_declared_function(lib):
    for name in _declared():
        assert hasattr(lib, name), name
    assert lib.gbf_version().startswith(b'gbfdtd')


def test_last_error_rejects_empty_buffer(lib):
    import ctypes
    assert lib.gbf_last_error(None, None, 0) == -1
    buf = ctypes.create_string_buffer(64)
    assert lib.gbf_last_error(None, buf, 64) == 0


def test_create_rejects_bad_descriptions(lib):
    """Argument checks run before any CUDA call, so they answer without a GPU."""
    import ctypes
    from gprmax_gb300 import _native
    d = _native.GridDesc()
    d.nx, d.ny, d.nz, d.iterations, d.nmat = 20, 20, 20, 10, 2
    d.pml_order = 1
    d.dx = d.dy = d.dz = 1e-3
    ctx = ctypes.c_void_p(0)
    cases = [('pml_thickness', [10, 0, 0, 0, 0, 0]),   # 2 T >= n
             ('maxpoles', 5), ('pml_order', 3), ('options', 64), ('nz', 0)]
    for field, value in cases:
        bad = _native.GridDesc.from_buffer_copy(d)
        if field == 'pml_thickness':
            for s, t in enumerate(value):
                bad.pml_thickness[s] = t
        else:
            setattr(bad, field, value)
        rc = lib.gbf_create(ctypes.byref(bad), ctypes.byref(ctx))
        assert rc == -1, (field, rc)
        buf = ctypes.create_string_buffer(256)
        lib.gbf_last_error(None, buf, 256)
        assert buf.value.startswith(b'gbf_create'), buf.value


def _rn32(x):
    """Round an exact rational to the nearest float32 (ties to even), for normal results."""
    if x == 0:
        return 0.0
    sign = -1 if x < 0 else 1
    a = abs(x)
    e = a.numerator.bit_length() - a.denominator.bit_length()
    while Fraction(2) ** e > a:
        e -= 1
    while Fraction(2) ** (e + 1) <= a:
        e += 1
    scale = Fraction(2) ** (e - 23)
    m = a / scale
    q, r = divmod(m.numerator, m.denominator)
    if 2 * r > m.denominator or (2 * r == m.denominator and q % 2):
        q += 1
    return float(sign * q * scale)


def _corrected_quotient(x, d):
    """q = RN(x*r); e = RN(x - q*d); RN(q + e*r), r = RN(1/d) (each fused step rounded once)."""
    X, D = Fraction(float(x)), Fraction(float(d))
    r = Fraction(_rn32(1 / D))
    q = Fraction(_rn32(X * r))
    e = Fraction(_rn32(X - q * D))
    return _rn32(q + e * r)


@pytest.mark.parametrize('d', [1e-3, 2e-3, 5e-4, 2.5e-3, 1e-2, 0.1])
def test_reciprocal_division_matches_ieee_quotient(d):
    """The product form of dF/d used by the PML kernels, restated in exact arithmetic, against
    numpy's IEEE float32 division on a seeded sample of significands; the library's own
    exhaustive check must agree for these cell sizes."""
    d32 = np.float32(d)
    rng = np.random.default_rng(7)
    xs = (1 + rng.random(400)).astype(np.float32) * np.float32(rng.choice([1e-3, 1, 7e2]))
    for x in xs:
        want = np.float32(x) / d32
        assert np.float32(_corrected_quotient(x, d32)) == want, (x, d)


@pytest.mark.parametrize('d', [1e-3, 2e-3, 5e-4, 1e-2])
def test_library_accepts_common_cell_sizes(lib, d):
    assert lib.gbf_check_cell_division(float(np.float32(d))) == 1


def test_library_refuses_cell_sizes_outside_its_window(lib):
    for d in (1e-7, 2e7, 0.0, -1e-3, float('nan')):
        assert lib.gbf_check_cell_division(d) == 0
