"""libmsx.so loads and exports every entry point declared in include/msx.h;
calls that need no GPU behave.  CPU only."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, 'include', 'msx.h')).read()
    return re.findall(r'^MSX_API\s+int\s+(msx_\w+)\(', src, flags=re.M)


def test_header_matches_binding(libmsx):
    from namsa_gb300 import _lib
    names = declared_symbols()
    assert len(names) >= 14
    assert sorted(names) == sorted(n for n, _, _ in _lib.SIGNATURES)


def test_exports(libmsx):
    for name in declared_symbols():
        assert hasattr(libmsx, name), name


def test_host_only_calls(libmsx):
    assert libmsx.msx_version() == 10000
    for n in (64, 128, 256, 384, 512, 768, 1024):
        assert libmsx.msx_supported_size(n) == 1
        assert libmsx.msx_num_schedules(n) >= 1
    for n in (0, 100, 2048, 500):
        assert libmsx.msx_supported_size(n) == 0
        assert libmsx.msx_num_schedules(n) == 0
    buf = ctypes.create_string_buffer(64)
    assert libmsx.msx_schedule_name(512, 0, buf, 64) == 0 and buf.value.startswith(b't')
    assert libmsx.msx_schedule_name(512, 99, buf, 64) == -1


def test_argument_errors_without_device(libmsx):
    from namsa_gb300 import _lib
    h = ctypes.c_void_p()
    assert libmsx.msx_plan_create(500, 512, 0, ctypes.byref(h)) == _lib.MSX_ERR_UNSUPPORTED
    assert 'supported line lengths' in _lib.last_error()
    assert libmsx.msx_plan_create(512, 512, -1, ctypes.byref(h)) == _lib.MSX_ERR_INVALID
    assert libmsx.msx_build_probe(1, 512, 1.0, 0.02, 1.0, 0., 0., 0., 1, None, None, None, None) == _lib.MSX_ERR_INVALID
    assert libmsx.msx_multislice(None, None, 1, None, None, None, 1, 1.0, 0.02, 1.0, 1.0, None, 1, 1, None) == \
        _lib.MSX_ERR_INVALID
    assert libmsx.msx_plan_destroy(None) == 0
