"""GPU: the material upload rejects IDs that do not index the coefficient tables, on both ID
layouts: packed words built by one kernel straight from the caller's array (at most 1024
materials) and the plain six ID arrays (more materials). The reference indexes its tables
unchecked (fields_updates_ext.pyx, boundscheck off); here an out-of-range ID is an error."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GBF_EINVAL = -1


def _desc(nmat, n=8):
    from gprmax_gb300 import _native
    d = _native.GridDesc()
    d.nx = d.ny = d.nz = n
    d.iterations = 4
    d.nmat = nmat
    d.pml_order = 1
    d.dx = d.dy = d.dz = np.float32(1e-3)
    return d


def _upload(lib, d, ID):
    ctx = ctypes.c_void_p(0)
    assert lib.gbf_create(ctypes.byref(d), ctypes.byref(ctx)) == 0
    try:
        cE = np.zeros((d.nmat, 5), np.float32)
        cH = np.zeros((d.nmat, 5), np.float32)
        cE[:, 0] = cH[:, 0] = 1
        rc = lib.gbf_upload_materials(ctx, ID.ctypes.data_as(ctypes.c_void_p),
                                      cE.ctypes.data_as(ctypes.c_void_p),
                                      cH.ctypes.data_as(ctypes.c_void_p), None)
        buf = ctypes.create_string_buffer(256)
        lib.gbf_last_error(ctx, buf, 256)
        return rc, buf.value.decode()
    finally:
        lib.gbf_destroy(ctx)


@pytest.mark.parametrize('nmat', [7, 1100])
def test_out_of_range_ids_are_rejected(native, nmat):
    d = _desc(nmat)
    ID = np.ones((6, 9, 9, 9), dtype=np.uint32)
    rc, msg = _upload(native, d, ID)
    assert rc == 0, msg
    for comp in (0, 4):
        bad = ID.copy()
        bad[comp, 3, 5, 2] = nmat
        rc, msg = _upload(native, d, bad)
        assert rc == GBF_EINVAL and str(nmat) in msg, (rc, msg)


@pytest.mark.parametrize('name', ['debye1', 'mixed', 'smoothed'])
def test_packed_upload_gives_the_same_run(native, name):
    """IDs packed on the host into page-locked memory (pack_materials) and uploaded as words
    give the same run bit for bit as the ID array itself."""
    from models import MODELS
    from gprmax_gb300.model import build_grid
    from gprmax_gb300.solver import DeviceModel, pack_materials
    G = build_grid(MODELS[name].splitlines(True), messages=False)
    words = pack_materials(G)
    # the H words only for a model with magnetic materials ('smoothed')
    assert (words[1] is None) == (name != 'smoothed')
    out = []
    for packed in (None, words):
        dm = DeviceModel(G, packed=packed)
        try:
            dm.run()
            out.append((dm.receivers(), dm.fields()))
        finally:
            dm.close()
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])


def test_packed_upload_rejects_bad_words(native):
    from gprmax_gb300.solver import PinnedWords
    d = _desc(7)
    n = 9 ** 3
    ctx = ctypes.c_void_p(0)
    assert native.gbf_create(ctypes.byref(d), ctypes.byref(ctx)) == 0
    try:
        pe, ph = PinnedWords(native, n), PinnedWords(native, n)
        cE = np.zeros((7, 5), np.float32)
        cH = np.zeros((7, 5), np.float32)
        for bad in (7, 1 << 31):
            pe.array[:] = 1 | (1 << 10) | (1 << 20)
            ph.array[:] = 1
            pe.array[100] = bad
            rc = native.gbf_upload_materials_packed(ctx, pe.ptr, ph.ptr,
                                                    cE.ctypes.data_as(ctypes.c_void_p),
                                                    cH.ctypes.data_as(ctypes.c_void_p), None)
            assert rc == GBF_EINVAL
        pe.array[100] = 1
        rc = native.gbf_upload_materials_packed(ctx, pe.ptr, ph.ptr, cE.ctypes.data_as(ctypes.c_void_p),
                                                cH.ctypes.data_as(ctypes.c_void_p), None)
        assert rc == 0
        # no H words: accepted while every H row is the same, refused otherwise
        rc = native.gbf_upload_materials_packed(ctx, pe.ptr, None, cE.ctypes.data_as(ctypes.c_void_p),
                                                cH.ctypes.data_as(ctypes.c_void_p), None)
        assert rc == 0
        cH[3, 0] = 0.5
        rc = native.gbf_upload_materials_packed(ctx, pe.ptr, None, cE.ctypes.data_as(ctypes.c_void_p),
                                                cH.ctypes.data_as(ctypes.c_void_p), None)
        assert rc == GBF_EINVAL
    finally:
        native.gbf_destroy(ctx)


def test_device_division_check_agrees_with_the_host_loop():
    """gbf_create decides the PML kernels' division form per axis on the device; for cell sizes
    across the range (the soil's 2 mm, round sizes, significands at both ends of the binade,
    seeded random ones) the device's answer is the host loop's, and sizes outside the window
    are refused without a launch."""
    from gprmax_gb300 import _native
    lib = _native.lib()
    rng = np.random.default_rng(11)
    ds = [2e-3, 1e-3, 5e-4, 1e-2, 0.1, 1.0, 1.5]
    ds += [float(np.float32(1 + 2.0 ** -23)), float(np.float32(2 - 2.0 ** -23))]
    ds += [float(v) for v in (10 ** rng.uniform(-5, 2, 12)).astype(np.float32)]
    for d in ds:
        d = float(np.float32(d))
        ok = ctypes.c_int32(-1)
        assert lib.gbf_check_cell_division_device(d, ctypes.byref(ok)) == 0
        assert ok.value == lib.gbf_check_cell_division(d), d
    for d in (1e-7, 2e7, 0.0, -1e-3, float('nan')):
        ok = ctypes.c_int32(-1)
        assert lib.gbf_check_cell_division_device(d, ctypes.byref(ok)) == 0
        assert ok.value == 0
