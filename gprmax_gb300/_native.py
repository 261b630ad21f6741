"""Build and load the native solver library ``csrc/libgbfdtd.so`` (sm_103a CUDA + C ABI).

The library is compiled in-tree with nvcc. There is no fallback: if the library cannot be
built or loaded, :func:`lib` raises, so a model never runs anywhere but the GPU kernels.
"""
import ctypes
import os
import subprocess
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
LIBPATH = os.path.join(CSRC, 'libgbfdtd.so')
SOURCES = ['gbfdtd.cu', 'kernels_inst.cu', 'fused_inst.cu', 'staged_inst.cu', 'adjoint.cu',
           'geom.cu', 'fractal.cu', 'fdtd_kernels.cuh', 'fused_step.cuh', 'staged.cuh']
PML_KINDS = 5       # kernels_inst.cu and staged_inst.cu are compiled once per PML kind
FUSED_TJ = (7, 15)  # fused_inst.cu once per PML kind and tile height
HEADER = os.path.join(os.path.dirname(HERE), 'include', 'gbfdtd.h')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
# --fmad=false: every product and sum is rounded as written, which makes the GPU results
# bit-identical to the reference's CPU kernels compiled without floating-point contraction
NVCC_FLAGS = ['-O3', '-lineinfo', '-std=c++17', '--fmad=false', '-Xcompiler', '-fPIC',
              '-Xcompiler', '-ffp-contract=off', '-shared']

_lock = threading.Lock()
_lib = None


def _nvcc():
    for cand in (os.environ.get('NVCC'), '/usr/local/cuda/bin/nvcc', 'nvcc'):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return 'nvcc'


def _stale():
    if not os.path.exists(LIBPATH):
        return True
    t = os.path.getmtime(LIBPATH)
    deps = [os.path.join(CSRC, s) for s in SOURCES] + [HEADER]
    return any(os.path.getmtime(p) > t for p in deps if os.path.exists(p))


def build(force=False, verbose=False):
    """Compile ``libgbfdtd.so`` for sm_103a if it is missing or older than its sources.

    The main translation unit, one half-step and one staged half-step instantiation unit per
    PML kind and one fused-step unit per PML kind and tile height are compiled in parallel, then
    linked."""
    if not force and not _stale():
        return LIBPATH
    import shutil
    import tempfile
    from concurrent.futures import ThreadPoolExecutor
    # objects in a scratch folder, removed once the library is linked
    objdir = tempfile.mkdtemp(prefix='gbfdtd_build_')
    compile_flags = [f for f in NVCC_FLAGS if f != '-shared']
    jobs = [(os.path.join(CSRC, 'gbfdtd.cu'), os.path.join(objdir, 'gbfdtd.o'), []),
            (os.path.join(CSRC, 'adjoint.cu'), os.path.join(objdir, 'adjoint.o'), []),
            (os.path.join(CSRC, 'geom.cu'), os.path.join(objdir, 'geom.o'), []),
            (os.path.join(CSRC, 'fractal.cu'), os.path.join(objdir, 'fractal.o'), [])]
    for pk in range(PML_KINDS):
        jobs.append((os.path.join(CSRC, 'kernels_inst.cu'),
                     os.path.join(objdir, 'kernels_pk{}.o'.format(pk)), ['-DGBF_PK={}'.format(pk)]))
        jobs.append((os.path.join(CSRC, 'staged_inst.cu'),
                     os.path.join(objdir, 'staged_pk{}.o'.format(pk)), ['-DGBF_PK={}'.format(pk)]))
        for tj in FUSED_TJ:
            jobs.append((os.path.join(CSRC, 'fused_inst.cu'),
                         os.path.join(objdir, 'fused_pk{}_tj{}.o'.format(pk, tj)),
                         ['-DGBF_PK={}'.format(pk), '-DGBF_TJ={}'.format(tj)]))
    # the longest units first, so the pool ends together
    jobs.sort(key=lambda j: 'fused_inst' not in j[0])

    def compile_one(job):
        src, obj, extra = job
        cmd = [_nvcc()] + ARCH + compile_flags + extra + ['-c', src, '-o', obj]
        if verbose:
            print(' '.join(cmd))
        subprocess.run(cmd, check=True, cwd=CSRC)
        return obj
    with ThreadPoolExecutor(min(len(jobs), max(os.cpu_count() or 1, 1))) as ex:
        objs = list(ex.map(compile_one, jobs))
    # cuFFT for the fractal fields' transforms (fractal.cu)
    cmd = [_nvcc()] + ARCH + ['-shared'] + objs + ['-lcufft', '-o', LIBPATH + '.tmp']
    if verbose:
        print(' '.join(cmd))
    try:
        subprocess.run(cmd, check=True, cwd=CSRC)
    finally:
        shutil.rmtree(objdir, ignore_errors=True)
    os.replace(LIBPATH + '.tmp', LIBPATH)
    return LIBPATH


class AdjDesc(ctypes.Structure):
    _fields_ = [('nx', ctypes.c_int32), ('ny', ctypes.c_int32), ('nz', ctypes.c_int32),
                ('iterations', ctypes.c_int32), ('d', ctypes.c_float), ('dt', ctypes.c_float),
                ('dbd', ctypes.c_float), ('srcm', ctypes.c_float),
                ('pml_thickness', ctypes.c_int32 * 6), ('nsrc', ctypes.c_int32),
                ('nrx', ctypes.c_int32), ('checkpoint_interval', ctypes.c_int32),
                ('reserved', ctypes.c_int32 * 3)]


class GridDesc(ctypes.Structure):
    _fields_ = [('nx', ctypes.c_int32), ('ny', ctypes.c_int32), ('nz', ctypes.c_int32),
                ('iterations', ctypes.c_int32), ('nmat', ctypes.c_int32),
                ('maxpoles', ctypes.c_int32), ('pml_formulation', ctypes.c_int32),
                ('pml_order', ctypes.c_int32), ('pml_thickness', ctypes.c_int32 * 6),
                ('dx', ctypes.c_float), ('dy', ctypes.c_float), ('dz', ctypes.c_float),
                ('nsrc', ctypes.c_int32), ('nrx', ctypes.c_int32), ('nsnap', ctypes.c_int32),
                ('options', ctypes.c_int32), ('ntl', ctypes.c_int32),
                ('reserved', ctypes.c_int32 * 2)]


GBF_RUN_GRAPH = 1
GBF_RUN_CHECK = 2

_P = ctypes.c_void_p
_SIGS = {
    'gbf_create': (ctypes.c_int, [ctypes.POINTER(GridDesc), ctypes.POINTER(_P)]),
    'gbf_destroy': (None, [_P]),
    'gbf_upload_materials': (ctypes.c_int, [_P, _P, _P, _P, _P]),
    'gbf_upload_pml': (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(_P)]),
    'gbf_upload_materials_packed': (ctypes.c_int, [_P, _P, _P, _P, _P, _P]),
    'gbf_pack_ids': (ctypes.c_int, [_P, ctypes.c_int64, _P, _P, _P]),
    'gbf_host_alloc': (ctypes.c_int, [ctypes.c_size_t, ctypes.POINTER(_P)]),
    'gbf_host_free': (None, [_P]),
    'gbf_upload_sources': (ctypes.c_int, [_P, _P, _P, _P]),
    'gbf_set_receivers': (ctypes.c_int, [_P, _P]),
    'gbf_set_snapshots': (ctypes.c_int, [_P, _P]),
    'gbf_reset': (ctypes.c_int, [_P]),
    'gbf_run': (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_uint32]),
    'gbf_run_timed': (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_uint32, ctypes.POINTER(ctypes.c_float)]),
    'gbf_current_iteration': (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int32)]),
    'gbf_synchronize': (ctypes.c_int, [_P]),
    'gbf_download_rx': (ctypes.c_int, [_P, _P]),
    'gbf_download_fields': (ctypes.c_int, [_P, _P]),
    'gbf_upload_fields': (ctypes.c_int, [_P, _P]),
    'gbf_download_dispersive': (ctypes.c_int, [_P, _P]),
    'gbf_download_snapshot': (ctypes.c_int, [_P, ctypes.c_int, _P]),
    'gbf_step_info': (ctypes.c_int, [_P, _P]),
    'gbf_batch_info': (ctypes.c_int, [_P, _P]),
    'gbf_fractal_field': (ctypes.c_int, [ctypes.c_int32, _P, _P, ctypes.c_float, _P, _P]),
    'gbf_set_fused_tiles': (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int32]),
    'gbf_set_step_forms': (ctypes.c_int, [_P, ctypes.c_int32]),
    'gbf_share_materials': (ctypes.c_int, [_P, _P]),
    'gbf_fused_tiles': (ctypes.c_int, [ctypes.c_int32] * 5 + [_P]),
    'gbf_profile': (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(ctypes.c_float),
                                   ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]),
    'gbf_device_bytes': (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_size_t)]),
    'gbf_set_device': (ctypes.c_int, [ctypes.c_int32]),
    'gbf_last_error': (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_size_t]),
    'gbf_version': (ctypes.c_char_p, []),
    'gbf_check_cell_division': (ctypes.c_int, [ctypes.c_float]),
    'gbf_check_cell_division_device': (ctypes.c_int, [ctypes.c_float, ctypes.POINTER(ctypes.c_int32)]),
    'gbf_upload_tls': (ctypes.c_int, [_P, _P, _P, _P, _P, _P]),
    'gbf_download_tls': (ctypes.c_int, [_P, _P]),
    'gbf_adj_create': (ctypes.c_int, [_P, ctypes.POINTER(_P)]),
    'gbf_adj_destroy': (None, [_P]),
    'gbf_adj_last_error': (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_size_t]),
    'gbf_adj_upload_pml': (ctypes.c_int, [_P, ctypes.c_int32, ctypes.POINTER(_P)]),
    'gbf_adj_upload_sources': (ctypes.c_int, [_P, _P, _P, _P]),
    'gbf_adj_set_receivers': (ctypes.c_int, [_P, _P]),
    'gbf_adj_forward': (ctypes.c_int, [_P, _P, _P, _P]),
    'gbf_adj_backward': (ctypes.c_int, [_P, _P, _P, _P, _P, _P]),
    'gbf_adj_backward_static': (ctypes.c_int, [_P, _P, _P, _P, _P, _P]),
    'gbf_batch_create': (ctypes.c_int, [_P, ctypes.c_int32, ctypes.POINTER(_P)]),
    'gbf_batch_destroy': (None, [_P]),
    'gbf_batch_run': (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_uint32]),
    'gbf_batch_run_timed': (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_uint32,
                                           ctypes.POINTER(ctypes.c_float)]),
    'gbf_batch_synchronize': (ctypes.c_int, [_P]),
    'gbf_batch_last_error': (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_size_t]),
    'gbf_sweep_boxes': (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, _P,
                                       ctypes.c_int32, _P]),
    'gbf_geom_create': (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                       ctypes.POINTER(_P)]),
    'gbf_geom_destroy': (None, [_P]),
    'gbf_geom_last_error': (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_size_t]),
    'gbf_geom_cells': (ctypes.c_int, [_P, _P, _P, _P, ctypes.c_int32]),
    'gbf_geom_box': (ctypes.c_int, [_P, _P, _P, ctypes.c_int32]),
    'gbf_geom_voxels': (ctypes.c_int, [_P, _P, _P, ctypes.c_int32, ctypes.c_int32]),
    'gbf_geom_edges': (ctypes.c_int, [_P, ctypes.c_int32, _P]),
    'gbf_geom_components': (ctypes.c_int, [_P, ctypes.c_int32, _P]),
    'gbf_geom_averaged_keys': (ctypes.c_int, [_P, _P]),
    'gbf_geom_resolve': (ctypes.c_int, [_P, ctypes.c_int64, _P, _P]),
    'gbf_geom_fill': (ctypes.c_int, [_P, ctypes.c_int32, _P, ctypes.c_uint32]),
    'gbf_geom_read': (ctypes.c_int, [_P, ctypes.c_int32, _P, _P]),
    'gbf_geom_max_id': (ctypes.c_int, [_P, _P]),
    'gbf_upload_materials_geom': (ctypes.c_int, [_P, _P, _P, _P, _P]),
}


def exported_symbols():
    """Names the C ABI exports (the functions declared in include/gbfdtd.h)."""
    return sorted(_SIGS)


def load(path=LIBPATH):
    """Load the library without building (raises OSError if it is absent)."""
    lib_ = ctypes.CDLL(path)
    for name, (res, args) in _SIGS.items():
        f = getattr(lib_, name)
        f.restype = res
        f.argtypes = args
    return lib_


def lib():
    """The loaded native library, built on first use when nvcc is available."""
    global _lib
    with _lock:
        if _lib is None:
            if _stale():
                build()
            _lib = load()
    return _lib
