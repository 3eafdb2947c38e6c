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
    # newer entry points reject bad arguments before touching a device
    assert libmsx.msx_multislice_host(None, None, 1, None, ctypes.c_double(1.0), None, 1, ctypes.c_float(1.0),
                                      ctypes.c_double(0.02), ctypes.c_double(1.0), ctypes.c_float(1.0), None, 1, 1,
                                      None) == _lib.MSX_ERR_INVALID
    assert libmsx.msx_batch_autotune(None, None, 0, 1, None) == _lib.MSX_ERR_INVALID
    assert libmsx.msx_selftest_wait(0, 5, None) == _lib.MSX_ERR_INVALID
    assert libmsx.msx_selftest_wait(0, 40, None) == _lib.MSX_ERR_INVALID
    assert 'limit_log2' in _lib.last_error()


def test_reference_gpu_harness_exports_and_site_layout():
    """The checker's reference-GPU harness (oracle/refgpu_harness.cu) loads, exports
    its entry points, and lays out site lists as the reference does (triplets of
    window index, y pixel, x pixel per slice) with the zero-window index as padding."""
    import numpy as np
    import pytest
    from oracle import msa_oracle as O
    from oracle import refgpu as R
    try:
        ref = R.RefGPU('c1')
    except R.RefGPUUnavailable as e:
        pytest.skip(str(e))
    for name in ['refgpu_build_potential', 'refgpu_build_probe', 'refgpu_ctx_create', 'refgpu_ctx_destroy',
                 'refgpu_propagator', 'refgpu_propagate', 'refgpu_shape', 'refgpu_last_error']:
        assert hasattr(ref.L, name)
    meta = ref.meta
    assert (ref.ny, ref.nx, ref.S) == (meta['ny'], meta['nx'], meta['num_slices'])
    sc = O.si_supercell(*meta['cells'])
    geom = O.Geometry(np.column_stack([sc['x'], sc['y'], sc['z']]), sc['atomic_number'], meta['kv'], meta['semi'],
                      [meta['ny'], meta['nx']])
    sites = ref.sites(geom, meta['slice_t'], 1)
    assert sites.shape == (ref.S, ref.sites_size)
    want = O.slice_sites_gpu(geom, meta['slice_t'])
    for s in range(ref.S):
        trip = sites[s].reshape(-1, 3)
        n = len(want[s])
        np.testing.assert_array_equal(trip[:n], want[s].astype(np.float32))
        assert np.all(trip[n:, 0] == 1)


def test_noalloc_rejects_misaligned_pointers(libmsx):
    """The allocation-free entry point checks the alignment its kernels need
    (8 bytes for complex64 and float64, as msx_multislice does) before any device
    work, so a pointer into the middle of a caller's pool returns an error status
    instead of faulting on the GPU."""
    from namsa_gb300 import _lib
    vp = ctypes.c_void_p
    good, odd = 0x10000, 0x10004

    def call(trans, psik, norm, pos, out):
        return libmsx.msx_multislice_noalloc(vp(trans), 2, vp(psik), vp(norm), vp(pos), 3, 256, 256, 12.8, 0.025,
                                             1.5, 4.0, vp(out), 128, 128, None)
    for args in [(odd, good, good, good, good), (good, odd, good, good, good), (good, good, odd, good, good),
                 (good, good, good, odd, good), (good, good, good, good, odd + 2)]:
        assert call(*args) == _lib.MSX_ERR_INVALID
        assert 'aligned' in _lib.last_error()


def test_newer_entry_points_reject_bad_arguments_without_device(libmsx):
    """Argument checks of the stored-stack detector reduction, the tensor-core GEMM, the
    probe stack and the corrector run on the host before any device work."""
    from namsa_gb300 import _lib
    vp = ctypes.c_void_p
    assert libmsx.msx_integrate_cbed(vp(0x1000), 2, 0, 8, None, 1, vp(0x2000), None) == _lib.MSX_ERR_INVALID
    assert libmsx.msx_integrate_cbed(vp(0x1000), 2, 8, 8, None, 3, vp(0x2000), None) == _lib.MSX_ERR_INVALID
    assert 'weights' in _lib.last_error()
    assert libmsx.msx_gemm_bf16(vp(0x1000), 4, vp(0x2000), 4, 8, 8, 8, vp(0x3000), 8, None, 0, None) == \
        _lib.MSX_ERR_INVALID  # leading dimensions shorter than the rows
    assert libmsx.msx_gemm_bf16(vp(0x1000), 8, vp(0x2000), 8, 8, 5000, 8, vp(0x3000), 5000, None, 0, None) == \
        _lib.MSX_ERR_INVALID  # n above 4096
    assert libmsx.msx_plan_probe_stack(None, None, None, None, 1, 1.0, None, None) == _lib.MSX_ERR_INVALID
    h = ctypes.c_void_p()
    assert libmsx.msx_corrector_create(256, 256, 6, 48, 4, 32, 64, 4, ctypes.byref(h)) == _lib.MSX_ERR_INVALID
    assert libmsx.msx_corrector_create(256, 256, 6, 32, 4, 200, 64, 4, ctypes.byref(h)) == _lib.MSX_ERR_INVALID
    assert libmsx.msx_corrector_apply_map(None, 1, 8, 8, None, 0, 0, 0, None) == _lib.MSX_ERR_INVALID
    assert libmsx.msx_corrector_map_grad(vp(0x1000), vp(0x2000), 1, 8, 8, 0, 0, 1, None, vp(0x3000), None) == \
        _lib.MSX_ERR_INVALID  # the phase form needs the maps
