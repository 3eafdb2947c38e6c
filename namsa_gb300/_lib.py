"""ctypes binding of libmsx.so (the C ABI declared in include/msx.h).

The library is built in-tree by ``namsa_gb300.build``.  There is no CPU
fallback: if the shared object is missing or fails to load, importing the
engine raises ``MsxLibraryError``.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, 'libmsx.so')

MSX_OK = 0
MSX_ERR_INVALID = -1
MSX_ERR_UNSUPPORTED = -2
MSX_ERR_CUDA = -3
MSX_ERR_ALLOC = -4
MSX_ERR_TIMEOUT = -5

# (name, restype, argtypes) for every entry point of include/msx.h
_c = ctypes
_vp = _c.c_void_p
SIGNATURES = [
    ('msx_version', _c.c_int, []),
    ('msx_last_error', _c.c_int, [_c.c_char_p, _c.c_size_t]),
    ('msx_supported_size', _c.c_int, [_c.c_int]),
    ('msx_num_schedules', _c.c_int, [_c.c_int]),
    ('msx_schedule_name', _c.c_int, [_c.c_int, _c.c_int, _c.c_char_p, _c.c_size_t]),
    ('msx_schedule_col_tile', _c.c_int, [_c.c_int, _c.c_int, _c.POINTER(_c.c_int)]),
    ('msx_band_columns', _c.c_int, [_c.c_int, _c.c_float, _c.c_float, _c.c_int, _c.POINTER(_c.c_int),
                                    _c.POINTER(_c.c_int)]),
    ('msx_atom_windows', _c.c_int, [_vp, _c.c_int, _c.c_int, _c.c_int, _c.c_int, _c.c_double, _vp, _vp]),
    ('msx_build_transmission', _c.c_int, [_vp, _vp, _c.c_int, _vp, _c.c_int, _c.c_int, _c.c_int, _c.c_int,
                                          _c.c_float, _vp, _vp, _vp]),
    ('msx_build_probe', _c.c_int, [_c.c_int, _c.c_int, _c.c_float, _c.c_double, _c.c_float, _c.c_double,
                                   _c.c_double, _c.c_double, _c.c_int, _vp, _vp, _vp, _vp]),
    ('msx_plan_create', _c.c_int, [_c.c_int, _c.c_int, _c.c_int, _c.POINTER(_vp)]),
    ('msx_plan_destroy', _c.c_int, [_vp]),
    ('msx_plan_set_schedule', _c.c_int, [_vp, _c.c_int, _c.c_int, _c.c_int]),
    ('msx_plan_get_schedule', _c.c_int, [_vp, _c.POINTER(_c.c_int), _c.POINTER(_c.c_int), _c.POINTER(_c.c_int)]),
    ('msx_plan_set_graph', _c.c_int, [_vp, _c.c_int]),
    ('msx_plan_set_tma', _c.c_int, [_vp, _c.c_int]),
    ('msx_plan_check', _c.c_int, [_vp]),
    ('msx_multislice', _c.c_int, [_vp, _vp, _c.c_int, _vp, _vp, _vp, _c.c_int, _c.c_float, _c.c_double,
                                  _c.c_double, _c.c_float, _vp, _c.c_int, _c.c_int, _vp]),
    ('msx_multislice_host', _c.c_int, [_vp, _vp, _c.c_int, _vp, _c.c_double, _vp, _c.c_int, _c.c_float,
                                       _c.c_double, _c.c_double, _c.c_float, _vp, _c.c_int, _c.c_int, _vp]),
    ('msx_propagator_table', _c.c_int, [_c.c_int, _c.c_int, _c.c_float, _c.c_double, _c.c_double, _c.c_float, _vp,
                                        _vp]),
    ('msx_plan_probe_waves', _c.c_int, [_vp, _vp, _vp, _c.c_int, _c.c_float, _vp, _vp]),
    ('msx_plan_probe_stack', _c.c_int, [_vp, _vp, _vp, _vp, _c.c_int, _c.c_float, _vp, _vp]),
    ('msx_plan_step_waves', _c.c_int, [_vp, _vp, _c.c_int, _vp, _vp, _vp]),
    ('msx_plan_cbed_waves', _c.c_int, [_vp, _vp, _c.c_int, _vp, _vp, _c.c_int, _c.c_int, _vp]),
    ('msx_multislice_detect', _c.c_int, [_vp, _vp, _c.c_int, _vp, _vp, _vp, _c.c_int, _c.c_float, _c.c_double,
                                         _c.c_double, _c.c_float, _vp, _c.c_int, _vp, _vp]),
    ('msx_multislice_noalloc', _c.c_int, [_vp, _c.c_int, _vp, _vp, _vp, _c.c_int, _c.c_int, _c.c_int, _c.c_float,
                                          _c.c_double, _c.c_double, _c.c_float, _vp, _c.c_int, _c.c_int, _vp]),
    ('msx_process_cbed', _c.c_int, [_vp, _c.c_int, _c.c_int, _c.c_int, _vp, _vp]),
    ('msx_integrate_cbed', _c.c_int, [_vp, _c.c_int, _c.c_int, _c.c_int, _vp, _c.c_int, _vp, _vp]),
    ('msx_process_potential', _c.c_int, [_vp, _c.c_int, _c.c_int, _c.c_int, _vp, _vp, _vp]),
    ('msx_integrate_potential', _c.c_int, [_vp, _vp, _c.c_int, _c.c_int, _c.c_int, _c.c_int, _c.c_int, _c.c_int,
                                           _c.c_float, _vp, _vp]),
    ('msx_batch_create', _c.c_int, [_c.c_int, _c.POINTER(_vp)]),
    ('msx_batch_destroy', _c.c_int, [_vp]),
    ('msx_batch_set_schedule', _c.c_int, [_vp, _c.c_int, _c.c_int, _c.c_int, _c.c_int, _c.c_int]),
    ('msx_batch_run', _c.c_int, [_vp, _vp, _c.c_int, _vp]),
    ('msx_batch_autotune', _c.c_int, [_vp, _vp, _c.c_int, _c.c_int, _vp]),
    ('msx_batch_check', _c.c_int, [_vp]),
    ('msx_gemm_bf16', _c.c_int, [_vp, _c.c_int, _vp, _c.c_int, _c.c_int, _c.c_int, _c.c_int, _vp, _c.c_int, _vp,
                                 _c.c_int, _vp]),
    ('msx_gemm_check', _c.c_int, []),
    ('msx_tc_dft', _c.c_int, [_vp, _c.c_int, _c.c_int, _c.c_int, _vp, _vp]),
    ('msx_step_waves_tc', _c.c_int, [_vp, _c.c_int, _c.c_int, _vp, _vp, _vp]),
    ('msx_tc_set_compensation', _c.c_int, [_c.c_int]),
    ('msx_tc_check', _c.c_int, []),
    ('msx_selftest_wait', _c.c_int, [_c.c_int, _c.c_int, _c.c_void_p]),
    ('msx_corrector_create', _c.c_int, [_c.c_int, _c.c_int, _c.c_int, _c.c_int, _c.c_int, _c.c_int, _c.c_int,
                                        _c.c_int, _c.POINTER(_vp)]),
    ('msx_corrector_destroy', _c.c_int, [_vp]),
    ('msx_corrector_params', _c.c_int, [_vp, _c.POINTER(_vp), _c.POINTER(_vp), _c.POINTER(_c.c_size_t)]),
    ('msx_corrector_layout', _c.c_int, [_vp, _c.POINTER(_c.c_size_t), _c.c_int]),
    ('msx_corrector_forward', _c.c_int, [_vp, _vp, _c.c_int, _vp, _vp]),
    ('msx_corrector_backward', _c.c_int, [_vp, _vp, _vp]),
    ('msx_corrector_adam', _c.c_int, [_vp, _c.c_float, _c.c_float, _c.c_float, _c.c_float, _vp]),
    ('msx_corrector_check', _c.c_int, [_vp]),
    ('msx_corrector_features', _c.c_int, [_vp, _c.c_int, _c.c_int, _c.c_int, _c.c_int, _c.c_float, _c.c_float, _vp,
                                          _vp]),
    ('msx_corrector_apply_map', _c.c_int, [_vp, _c.c_int, _c.c_int, _c.c_int, _vp, _c.c_int, _c.c_int, _c.c_int,
                                           _vp]),
    ('msx_corrector_mul_plane', _c.c_int, [_vp, _c.c_int, _c.c_int, _c.c_int, _vp, _c.c_int, _vp]),
    ('msx_corrector_map_trans', _c.c_int, [_vp, _c.c_int, _c.c_int, _vp, _c.c_int, _c.c_int, _vp, _vp]),
    ('msx_corrector_map_grad', _c.c_int, [_vp, _vp, _c.c_int, _c.c_int, _c.c_int, _c.c_int, _c.c_int, _c.c_int, _vp,
                                          _vp, _vp]),
    ('msx_corrector_residual', _c.c_int, [_vp, _vp, _c.c_int, _c.c_int, _c.c_int, _c.c_float, _c.c_int, _vp, _vp,
                                          _vp]),
    ('msx_plan_autotune', _c.c_int, [_vp, _vp, _c.c_int, _vp, _vp, _vp, _c.c_int, _c.c_float, _c.c_double,
                                     _c.c_double, _c.c_float, _c.c_int, _c.c_size_t, _c.POINTER(_c.c_float), _vp]),
    ('msx_plan_profile', _c.c_int, [_vp, _vp, _c.c_int, _vp, _vp, _vp, _c.c_int, _c.c_float, _c.c_double,
                                    _c.c_double, _c.c_float, _c.c_int, _c.POINTER(_c.c_float), _vp]),
]


class MsxJob(ctypes.Structure):
    """ctypes mirror of msx_job (include/msx.h)."""
    _fields_ = [('ny', ctypes.c_int), ('nx', ctypes.c_int), ('num_slices', ctypes.c_int), ('num_probes', ctypes.c_int),
                ('crop_y', ctypes.c_int), ('crop_x', ctypes.c_int), ('kmax', ctypes.c_float), ('k_band', ctypes.c_float),
                ('lambda_', ctypes.c_double), ('slice_t', ctypes.c_double), ('trans_dev', ctypes.c_void_p),
                ('psi_k_dev', ctypes.c_void_p), ('normalization_dev', ctypes.c_void_p),
                ('positions_dev', ctypes.c_void_p), ('cbed_out_dev', ctypes.c_void_p)]


class MsxLibraryError(ImportError):
    """libmsx.so is missing or does not load."""


class MsxError(RuntimeError):
    """A libmsx call returned a non-zero status."""

    def __init__(self, code, message):
        super().__init__(f'libmsx error {code}: {message}')
        self.code = code


_lib = None


def load():
    """Load libmsx.so once and attach the ctypes signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise MsxLibraryError(f'{LIB_PATH} not found; build it with `python -m namsa_gb300.build`')
    try:
        lib = ctypes.CDLL(LIB_PATH)
    except OSError as exc:
        raise MsxLibraryError(f'cannot load {LIB_PATH}: {exc}') from exc
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error():
    lib = load()
    buf = ctypes.create_string_buffer(1024)
    lib.msx_last_error(buf, len(buf))
    return buf.value.decode(errors='replace')


def check(rc):
    """Raise MsxError when a libmsx call failed."""
    if rc != MSX_OK:
        raise MsxError(rc, last_error())
    return rc
