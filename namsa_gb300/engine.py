"""Torch-tensor wrappers over the libmsx C ABI.

Every function takes and returns CUDA tensors; the work is queued on the
current torch stream.  Shapes and dtypes are checked here, argument ranges
in the library.  There is no CPU path.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib

_vp = ctypes.c_void_p


def _stream():
    return _vp(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return _vp(0) if t is None else _vp(t.data_ptr())


def _need_host(t, dtype, name, ndim=None):
    if not isinstance(t, torch.Tensor) or t.is_cuda:
        raise TypeError(f'{name} must be a host (CPU) torch tensor')
    if t.dtype != dtype:
        raise TypeError(f'{name} must be {dtype}, got {t.dtype}')
    if not t.is_contiguous():
        raise ValueError(f'{name} must be contiguous')
    if ndim is not None and t.dim() != ndim:
        raise ValueError(f'{name} must have {ndim} dimensions, got {tuple(t.shape)}')
    return t


def _need(t, dtype, name, ndim=None):
    if not isinstance(t, torch.Tensor):
        raise TypeError(f'{name} must be a torch tensor')
    if not t.is_cuda:
        raise ValueError(f'{name} must be a CUDA tensor')
    if t.dtype != dtype:
        raise TypeError(f'{name} must be {dtype}, got {t.dtype}')
    if not t.is_contiguous():
        raise ValueError(f'{name} must be contiguous')
    if ndim is not None and t.dim() != ndim:
        raise ValueError(f'{name} must have {ndim} dimensions, got {tuple(t.shape)}')
    return t


def lib():
    return _lib.load()


def supported_size(n):
    return bool(lib().msx_supported_size(int(n)))


def col_tile(n, index):
    """Columns per tile of schedule `index`'s column pass for line length n."""
    v = ctypes.c_int()
    _lib.check(lib().msx_schedule_col_tile(int(n), int(index), ctypes.byref(v)))
    return v.value


def band_columns(nx, kmax, k_band, tile):
    """[x_lo, x_hi): the columns the persistent passes keep from the second slice on."""
    lo, hi = ctypes.c_int(), ctypes.c_int()
    _lib.check(lib().msx_band_columns(int(nx), float(kmax), float(k_band), int(tile), ctypes.byref(lo),
                                      ctypes.byref(hi)))
    return lo.value, hi.value


def schedules(n):
    """Names of the compiled FFT schedules for line length n."""
    out = []
    buf = ctypes.create_string_buffer(64)
    for i in range(lib().msx_num_schedules(int(n))):
        _lib.check(lib().msx_schedule_name(int(n), i, buf, len(buf)))
        out.append(buf.value.decode())
    return out


def atom_windows(coeff, n0, n1, oversample=2, potential_range=8.0):
    """Kirkland projected-potential windows, (nspecies, n0/os, n1/os) float32.

    ``coeff`` is (nspecies, 4, 3) float64 on the device (rows a, b, c, d)."""
    _need(coeff, torch.float64, 'coeff', 3)
    ns = coeff.shape[0]
    out = torch.empty((ns, n0 // oversample, n1 // oversample), dtype=torch.float32, device=coeff.device)
    _lib.check(lib().msx_atom_windows(_ptr(coeff), ns, int(n0), int(n1), int(oversample), float(potential_range),
                                      _ptr(out), _stream()))
    return out


def build_transmission(sites, offsets, windows, ny, nx, sigma, want_potential=False):
    """Transmission slices (S, ny, nx) complex64 and optionally V (S, ny, nx) float32.

    ``sites``: (nsites, 4) int32 (species index, y pixel, x pixel, 0) grouped by slice;
    ``offsets``: (S+1,) int32 slice boundaries into ``sites``."""
    _need(sites, torch.int32, 'sites', 2)
    _need(offsets, torch.int32, 'offsets', 1)
    _need(windows, torch.float32, 'windows', 3)
    if sites.shape[1] != 4:
        raise ValueError('sites must have 4 columns')
    S = offsets.shape[0] - 1
    dev = windows.device
    trans = torch.empty((S, ny, nx), dtype=torch.complex64, device=dev)
    pot = torch.empty((S, ny, nx), dtype=torch.float32, device=dev) if want_potential else None
    if S > 0:
        if sites.shape[0] == 0:  # no atoms: keep a valid pointer for the kernel
            sites = torch.zeros((1, 4), dtype=torch.int32, device=dev)
        _lib.check(lib().msx_build_transmission(_ptr(sites), _ptr(offsets), S, _ptr(windows), windows.shape[1],
                                                windows.shape[2], int(ny), int(nx), float(sigma), _ptr(trans),
                                                _ptr(pot), _stream()))
    return trans, pot


def build_probe(ny, nx, kmax, lam, k_semi, c1, c3, c5, smooth, device=None):
    """k-space probe (ny, nx) complex64, aperture (ny, nx) float32 and the
    normalisation (1,) float64, all on the device."""
    dev = torch.device('cuda', torch.cuda.current_device()) if device is None else device
    psik = torch.empty((ny, nx), dtype=torch.complex64, device=dev)
    ap = torch.empty((ny, nx), dtype=torch.float32, device=dev)
    norm = torch.empty((1,), dtype=torch.float64, device=dev)
    _lib.check(lib().msx_build_probe(int(ny), int(nx), float(kmax), float(lam), float(k_semi), float(c1), float(c3),
                                     float(c5), int(bool(smooth)), _ptr(psik), _ptr(ap), _ptr(norm), _stream()))
    return psik, ap, norm


def process_cbed(cbed):
    """Per-pattern z-scored float16 copy of a (P, H, W) float32 CBED stack."""
    _need(cbed, torch.float32, 'cbed', 3)
    out = torch.empty(cbed.shape, dtype=torch.float16, device=cbed.device)
    _lib.check(lib().msx_process_cbed(_ptr(cbed), cbed.shape[0], cbed.shape[1], cbed.shape[2], _ptr(out), _stream()))
    return out


def integrate_cbed(cbed, weights=None):
    """Detector signals (P, ndet) float64 of a CBED stack (P, ny, nx) float32 with
    weights (ndet, ny, nx) float32; without weights the sum of each pattern (P, 1)."""
    _need(cbed, torch.float32, 'cbed', 3)
    P, ny, nx = cbed.shape
    nd = 1
    if weights is not None:
        _need(weights, torch.float32, 'weights', 3)
        if tuple(weights.shape[1:]) != (ny, nx):
            raise ValueError('weights must be (ndet, ny, nx) like the patterns')
        nd = weights.shape[0]
    out = torch.empty((P, nd), dtype=torch.float64, device=cbed.device)
    _lib.check(lib().msx_integrate_cbed(_ptr(cbed), P, ny, nx, _ptr(weights), nd, _ptr(out), _stream()))
    return out


def process_potential(trans):
    """Projected-potential label (1, w, w) float16 of a transmission stack (S, ny, nx)."""
    _need(trans, torch.complex64, 'trans', 3)
    S, ny, nx = trans.shape
    r0, r1 = ny // 4, 3 * nx // 4
    work = torch.empty(2 * ny * nx + 22, dtype=torch.float32, device=trans.device)
    out = torch.empty((1, r1 - r0, r1 - r0), dtype=torch.float16, device=trans.device)
    _lib.check(lib().msx_process_potential(_ptr(trans), S, ny, nx, _ptr(work), _ptr(out), _stream()))
    return out


def integrate_potential(pot, z, num_slices, sigma):
    """Transmission slices (num_slices, n, n) complex64 from a potential (nz, ny, nx)
    float32 sampled at z (nz,) float64, over the leading square n = min(ny, nx)."""
    _need(pot, torch.float32, 'pot', 3)
    _need(z, torch.float64, 'z', 1)
    nz, ly, lx = pot.shape
    n = min(ly, lx)
    out = torch.empty((num_slices, n, n), dtype=torch.complex64, device=pot.device)
    _lib.check(lib().msx_integrate_potential(_ptr(pot), _ptr(z), nz, ly, lx, n, n, int(num_slices), float(sigma),
                                             _ptr(out), _stream()))
    return out


def propagator_table(ny, nx, kmax, lam, slice_t, k_band, device=None):
    """P(k) mask(k) / N as a (ny, nx) complex64 device tensor."""
    dev = torch.device('cuda', torch.cuda.current_device()) if device is None else device
    out = torch.empty((ny, nx), dtype=torch.complex64, device=dev)
    _lib.check(lib().msx_propagator_table(int(ny), int(nx), float(kmax), float(lam), float(slice_t), float(k_band),
                                          _ptr(out), _stream()))
    return out


def tc_dft(x, sign):
    """Tensor-core split-BF16 DFT along the last axis of (lines, n) complex64, n in {256, 512}."""
    _need(x, torch.complex64, 'x', 2)
    z = torch.empty_like(x)
    _lib.check(lib().msx_tc_dft(_ptr(x), x.shape[0], x.shape[1], int(sign), _ptr(z), _stream()))
    return z


def step_waves_tc(waves, trans, ptab):
    """One slice on real-space waves (G, n, n) with the four 1-D DFTs on the tensor cores."""
    _need(waves, torch.complex64, 'waves', 3)
    _lib.check(lib().msx_step_waves_tc(_ptr(waves), waves.shape[0], waves.shape[1], _ptr(trans), _ptr(ptab),
                                       _stream()))
    return waves


def gemm_bf16(a, b, bias=None, out=None, accumulate=False):
    """a (m, k) @ b (n, k)^T (+ bias) in bfloat16 with FP32 accumulation on the
    tensor cores; FP32 row-major tensors (rows may be strided)."""
    for t, name in ((a, 'a'), (b, 'b')):
        if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float32 and t.dim() == 2
                and t.stride(1) == 1):
            raise TypeError(f'{name} must be a 2-D float32 CUDA tensor with unit column stride')
    m, k = a.shape
    n, k2 = b.shape
    if k2 != k:
        raise ValueError('inner dimensions differ')
    if out is None:
        out = torch.zeros((m, n), dtype=torch.float32, device=a.device)
    _lib.check(lib().msx_gemm_bf16(_ptr(a), a.stride(0), _ptr(b), b.stride(0), m, n, k, _ptr(out), out.stride(0),
                                   _ptr(bias), int(bool(accumulate)), _stream()))
    return out


def gemm_check():
    _lib.check(lib().msx_gemm_check())


def tc_set_compensation(enable):
    """Per-line norm compensation of the tensor-core DFTs (default on) for this host thread."""
    _lib.check(lib().msx_tc_set_compensation(int(bool(enable))))


def tc_check():
    _lib.check(lib().msx_tc_check())


def selftest_wait(arrive, limit_log2=22):
    """Run the bounded-wait self-test; raises MsxError (code TIMEOUT) when the wait ran out."""
    _lib.check(lib().msx_selftest_wait(int(bool(arrive)), int(limit_log2), _stream()))


class Plan:
    """A multislice plan: resident wave workspace, schedules and graph cache."""

    def __init__(self, ny, nx, group=0):
        self.ny, self.nx = int(ny), int(nx)
        h = _vp()
        _lib.check(lib().msx_plan_create(self.ny, self.nx, int(group), ctypes.byref(h)))
        self._h = h

    @property
    def handle(self):
        if self._h is None:
            raise RuntimeError('plan is closed')
        return self._h

    def close(self):
        if getattr(self, '_h', None) is not None:
            lib().msx_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_schedule(self, row=None, col=None, group=0):
        r, c, _ = self.schedule
        _lib.check(lib().msx_plan_set_schedule(self.handle, int(r if row is None else row),
                                               int(c if col is None else col), int(group)))

    @property
    def schedule(self):
        r, c, g = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _lib.check(lib().msx_plan_get_schedule(self.handle, ctypes.byref(r), ctypes.byref(c), ctypes.byref(g)))
        return r.value, c.value, g.value

    def set_graph(self, enable):
        _lib.check(lib().msx_plan_set_graph(self.handle, int(bool(enable))))

    def set_tma(self, enable):
        """Persistent TMA-pipelined passes (default) or the plain one-CTA-per-tile passes."""
        _lib.check(lib().msx_plan_set_tma(self.handle, int(bool(enable))))

    def check(self):
        """Synchronise and raise MsxError(MSX_ERR_TIMEOUT) if a pipelined pass gave up waiting."""
        _lib.check(lib().msx_plan_check(self.handle))

    def multislice(self, trans, psik, norm, positions, kmax, lam, slice_t, k_band, crop=None, out=None):
        """CBED stack (P, crop_y, crop_x) float32 for positions (P, 2) [y, x] float32.

        ``kmax`` and ``k_band`` are float32 values (the reference passes
        ``float32(kmax)`` and ``float32(bandwidth * kmax)`` to its kernels)."""
        _need(trans, torch.complex64, 'trans', 3)
        _need(psik, torch.complex64, 'psi_k', 2)
        _need(norm, torch.float64, 'normalization', 1)
        _need(positions, torch.float32, 'positions', 2)
        S, ny, nx = trans.shape
        if (ny, nx) != (self.ny, self.nx) or tuple(psik.shape) != (ny, nx):
            raise ValueError(f'grid mismatch: plan {self.ny}x{self.nx}, trans {tuple(trans.shape)}, psi_k {tuple(psik.shape)}')
        if positions.shape[1] != 2:
            raise ValueError('positions must be (P, 2) [y, x]')
        cy, cx = (ny, nx) if crop is None else ((crop, crop) if isinstance(crop, int) else crop)
        P = positions.shape[0]
        if out is None:
            out = torch.empty((P, cy, cx), dtype=torch.float32, device=trans.device)
        else:
            _need(out, torch.float32, 'out', 3)
            if tuple(out.shape) != (P, cy, cx):
                raise ValueError('out has the wrong shape')
        _lib.check(lib().msx_multislice(self.handle, _ptr(trans), S, _ptr(psik), _ptr(norm), _ptr(positions), P,
                                        float(kmax), float(lam), float(slice_t), float(k_band), _ptr(out),
                                        int(cy), int(cx), _stream()))
        return out

    def multislice_host(self, trans, psik, norm, positions, kmax, lam, slice_t, k_band, crop=None, out=None):
        """multislice() with host tensors in and out (page-locked for overlapped copies):
        trans (S, ny, nx) and psik (ny, nx) complex64, norm a float, positions (P, 2)
        float32; returns the (P, crop_y, crop_x) float32 host stack.  Enqueued on the
        current stream; synchronise before reading the result."""
        _need_host(trans, torch.complex64, 'trans', 3)
        _need_host(psik, torch.complex64, 'psi_k', 2)
        _need_host(positions, torch.float32, 'positions', 2)
        S, ny, nx = trans.shape
        if (ny, nx) != (self.ny, self.nx) or tuple(psik.shape) != (ny, nx):
            raise ValueError(f'grid mismatch: plan {self.ny}x{self.nx}, trans {tuple(trans.shape)}, psi_k {tuple(psik.shape)}')
        cy, cx = (ny, nx) if crop is None else ((crop, crop) if isinstance(crop, int) else crop)
        P = positions.shape[0]
        if out is None:
            out = torch.empty((P, cy, cx), dtype=torch.float32, pin_memory=True)
        else:
            _need_host(out, torch.float32, 'out', 3)
            if tuple(out.shape) != (P, cy, cx):
                raise ValueError('out has the wrong shape')
        _lib.check(lib().msx_multislice_host(self.handle, _ptr(trans), S, _ptr(psik), float(norm), _ptr(positions), P,
                                             float(kmax), float(lam), float(slice_t), float(k_band), _ptr(out),
                                             int(cy), int(cx), _stream()))
        return out

    def probe_waves(self, psik, positions, kmax):
        """Real-space probe wavefunctions (P, ny, nx) complex64 (unnormalised ifft, fftshifted)."""
        out = torch.empty((positions.shape[0], self.ny, self.nx), dtype=torch.complex64, device=psik.device)
        _lib.check(lib().msx_plan_probe_waves(self.handle, _ptr(psik), _ptr(positions), positions.shape[0],
                                              float(kmax), _ptr(out), _stream()))
        return out

    def probe_stack(self, psik, norm, positions, kmax, out=None):
        """Unit-norm real-space probes (P, ny, nx) complex64 at each position, no
        propagation: fftshift(ifft2_u(psi_k * ramp)) / sqrt(norm)."""
        _need(psik, torch.complex64, 'psi_k', 2)
        _need(norm, torch.float64, 'normalization', 1)
        _need(positions, torch.float32, 'positions', 2)
        P = positions.shape[0]
        if out is None:
            out = torch.empty((P, self.ny, self.nx), dtype=torch.complex64, device=psik.device)
        else:
            _need(out, torch.complex64, 'out', 3)
            if tuple(out.shape) != (P, self.ny, self.nx):
                raise ValueError('out has the wrong shape')
        _lib.check(lib().msx_plan_probe_stack(self.handle, _ptr(psik), _ptr(norm), _ptr(positions), P, float(kmax),
                                              _ptr(out), _stream()))
        return out

    def step_waves(self, waves, trans, ptab):
        """One slice in place on real-space waves (G, ny, nx): psi <- ifft2(ptab * fft2(t * psi))."""
        _need(waves, torch.complex64, 'waves', 3)
        _lib.check(lib().msx_plan_step_waves(self.handle, _ptr(waves), waves.shape[0], _ptr(trans), _ptr(ptab),
                                             _stream()))
        return waves

    def cbed_waves(self, waves, norm, crop=None):
        """CBED patterns of real-space waves (overwrites the waves)."""
        _need(waves, torch.complex64, 'waves', 3)
        cy, cx = (self.ny, self.nx) if crop is None else ((crop, crop) if isinstance(crop, int) else crop)
        out = torch.empty((waves.shape[0], cy, cx), dtype=torch.float32, device=waves.device)
        _lib.check(lib().msx_plan_cbed_waves(self.handle, _ptr(waves), waves.shape[0], _ptr(norm), _ptr(out),
                                             int(cy), int(cx), _stream()))
        return out

    def detect(self, trans, psik, norm, positions, kmax, lam, slice_t, k_band, detectors, out=None):
        """Detector signals (P, ndet) float32: sum over each CBED pattern weighted by
        detectors (ndet, ny, nx) float32, fused into the last pass."""
        _need(trans, torch.complex64, 'trans', 3)
        _need(detectors, torch.float32, 'detectors', 3)
        P = positions.shape[0]
        nd = detectors.shape[0]
        if out is None:
            out = torch.empty((P, nd), dtype=torch.float32, device=trans.device)
        _lib.check(lib().msx_multislice_detect(self.handle, _ptr(trans), trans.shape[0], _ptr(psik), _ptr(norm),
                                               _ptr(positions), P, float(kmax), float(lam), float(slice_t),
                                               float(k_band), _ptr(detectors), nd, _ptr(out), _stream()))
        return out

    def profile(self, trans, psik, norm, positions, kmax, lam, slice_t, k_band, iters=20):
        """Mean duration (ms) of one row pass and one column pass over the plan's
        first group, timed with CUDA events on the current stream; also returns
        the waves per launch."""
        out = (ctypes.c_float * 3)()
        S = trans.shape[0]
        _lib.check(lib().msx_plan_profile(self.handle, _ptr(trans), S, _ptr(psik), _ptr(norm), _ptr(positions),
                                          positions.shape[0], float(kmax), float(lam), float(slice_t), float(k_band),
                                          int(iters), out, _stream()))
        return float(out[0]), float(out[1]), int(out[2])

    def autotune(self, trans, psik, norm, positions, kmax, lam, slice_t, k_band, iters=8, max_workspace_bytes=0):
        """Pick the fastest (row schedule, column schedule, group) on these inputs;
        returns (schedule tuple, ns per wave and slice)."""
        best = ctypes.c_float()
        S = trans.shape[0]
        _lib.check(lib().msx_plan_autotune(self.handle, _ptr(trans), S, _ptr(psik), _ptr(norm), _ptr(positions),
                                           positions.shape[0], float(kmax), float(lam), float(slice_t),
                                           float(k_band), int(iters), int(max_workspace_bytes), ctypes.byref(best),
                                           _stream()))
        return self.schedule, float(best.value)


class Batch:
    """Uneven batch of multislice jobs run as one CUDA graph over parallel branches."""

    def __init__(self, branches=0):
        h = _vp()
        _lib.check(lib().msx_batch_create(int(branches), ctypes.byref(h)))
        self._h = h
        self._keep = []

    def close(self):
        if getattr(self, '_h', None) is not None:
            lib().msx_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_schedule(self, ny, nx, row, col, group=0):
        _lib.check(lib().msx_batch_set_schedule(self._h, int(ny), int(nx), int(row), int(col), int(group)))

    @staticmethod
    def _jobs(jobs):
        arr = (_lib.MsxJob * len(jobs))()
        for j, d in zip(arr, jobs):
            _need(d['trans'], torch.complex64, 'trans', 3)
            _need(d['psik'], torch.complex64, 'psi_k', 2)
            _need(d['norm'], torch.float64, 'normalization', 1)
            _need(d['positions'], torch.float32, 'positions', 2)
            _need(d['out'], torch.float32, 'out', 3)
            S, ny, nx = d['trans'].shape
            j.ny, j.nx, j.num_slices, j.num_probes = ny, nx, S, d['positions'].shape[0]
            j.crop_y, j.crop_x = d['out'].shape[1], d['out'].shape[2]
            j.kmax, j.k_band, j.lambda_, j.slice_t = float(d['kmax']), float(d['k_band']), float(d['lam']), float(d['slice_t'])
            j.trans_dev, j.psi_k_dev = d['trans'].data_ptr(), d['psik'].data_ptr()
            j.normalization_dev, j.positions_dev = d['norm'].data_ptr(), d['positions'].data_ptr()
            j.cbed_out_dev = d['out'].data_ptr()
        return arr

    def run(self, jobs):
        """jobs: list of dicts with keys trans, psik, norm, positions, kmax, lam, slice_t,
        k_band, out (CUDA tensors / numbers as for Plan.multislice).  Returns the outs."""
        arr = self._jobs(jobs)
        _lib.check(lib().msx_batch_run(self._h, ctypes.cast(arr, _vp), len(jobs), _stream()))
        self._keep = jobs  # the graph refers to these buffers until the next run
        return [d['out'] for d in jobs]

    def autotune(self, jobs, iters=8):
        """Autotune every grid size of `jobs` on its largest job; the winners become
        the batch's schedules (and replace those of existing plans)."""
        arr = self._jobs(jobs)
        _lib.check(lib().msx_batch_autotune(self._h, ctypes.cast(arr, _vp), len(jobs), int(iters), _stream()))

    def check(self):
        _lib.check(lib().msx_batch_check(self._h))


class _DevView:
    """A device buffer of the library exposed to torch (no copy)."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {'shape': (int(n),), 'typestr': '<f4', 'data': (int(ptr), False),
                                         'version': 3, 'strides': None}


class Corrector:
    """Learned coarse-slice corrector network of libmsx (msx_corrector_*): maps
    the features of S coarse slices (S, ny, nx, in_channels) to the correction
    maps (S, ny, nx, 4) = (Re A, Im A, Re B, Im B) of the corrected coarse step
    psi <- (1 + A) ifft2(P_c fft2((1 + B) t_c psi))."""

    def __init__(self, ny, nx, in_channels=6, channels=32, layers=4, modes_x=32, modes_y=64, max_samples=16):
        h = _vp()
        _lib.check(lib().msx_corrector_create(int(ny), int(nx), int(in_channels), int(channels), int(layers),
                                              int(modes_x), int(modes_y), int(max_samples), ctypes.byref(h)))
        self._h = h
        self.ny, self.nx, self.in_channels, self.channels, self.layers = ny, nx, in_channels, channels, layers
        self.modes_x, self.modes_y, self.max_samples = modes_x, modes_y, max_samples
        p, g = _vp(), _vp()
        n = ctypes.c_size_t()
        _lib.check(lib().msx_corrector_params(self._h, ctypes.byref(p), ctypes.byref(g), ctypes.byref(n)))
        dev = torch.device('cuda', torch.cuda.current_device())
        self.count = n.value
        self.params = torch.as_tensor(_DevView(p.value, n.value), device=dev)
        self.grads = torch.as_tensor(_DevView(g.value, n.value), device=dev)
        offs = (ctypes.c_size_t * (6 + 3 * layers))()
        _lib.check(lib().msx_corrector_layout(self._h, offs, 6 + 3 * layers))
        self.offsets = [int(o) for o in offs]

    def views(self, flat=None):
        """Named views (W0, b0, R1, W1, b1, ..., P1, c1, P2, c2) into `flat` (default: the parameters)."""
        flat = self.params if flat is None else flat
        C, Ci, L = self.channels, self.in_channels, self.layers
        shapes = [('W0', (C, Ci)), ('b0', (C,))]
        for l in range(L):
            shapes += [(f'R{l + 1}', (self.modes_x, self.modes_y, C, C, 2)), (f'W{l + 1}', (C, C)), (f'b{l + 1}', (C,))]
        shapes += [('P1', (C, C)), ('c1', (C,)), ('P2', (4, C)), ('c2', (4,))]
        out = {}
        for (name, shape), off in zip(shapes, self.offsets):
            n = 1
            for d in shape:
                n *= d
            out[name] = flat[off:off + n].view(shape)
        return out

    def close(self):
        if getattr(self, '_h', None) is not None:
            lib().msx_corrector_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def forward(self, features, out=None):
        _need(features, torch.float32, 'features', 4)
        S = features.shape[0]
        if tuple(features.shape[1:]) != (self.ny, self.nx, self.in_channels):
            raise ValueError(f'features must be (S, {self.ny}, {self.nx}, {self.in_channels})')
        if out is None:
            out = torch.empty((S, self.ny, self.nx, 4), dtype=torch.float32, device=features.device)
        _lib.check(lib().msx_corrector_forward(self._h, _ptr(features), S, _ptr(out), _stream()))
        return out

    def backward(self, dmaps):
        """Parameter gradients (into self.grads) for d loss / d maps of the last forward."""
        _need(dmaps, torch.float32, 'dmaps', 4)
        _lib.check(lib().msx_corrector_backward(self._h, _ptr(dmaps), _stream()))

    def adam(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        _lib.check(lib().msx_corrector_adam(self._h, float(lr), float(beta1), float(beta2), float(eps), _stream()))

    def check(self):
        _lib.check(lib().msx_corrector_check(self._h))


def corrector_features(pot, ratio, sigma, tval, out=None):
    """Network inputs (S, ny, nx, ratio + 2) of S = pot.shape[0] // ratio coarse slices
    from fine potential slices pot (S * ratio, ny, nx) float32."""
    _need(pot, torch.float32, 'pot', 3)
    S = pot.shape[0] // ratio
    ny, nx = pot.shape[1], pot.shape[2]
    if out is None:
        out = torch.empty((S, ny, nx, ratio + 2), dtype=torch.float32, device=pot.device)
    _lib.check(lib().msx_corrector_features(_ptr(pot), S, int(ratio), ny, nx, float(sigma), float(tval), _ptr(out),
                                            _stream()))
    return out


def apply_map(waves, maps, which, conj=False, form=0):
    """waves (num, ny, nx) complex64 *= factor (or its conjugate); maps (ny, nx, 4), M = A (0) or B (1);
    factor 1 + M (form 0) or exp(i Im M) (form 1)."""
    _need(waves, torch.complex64, 'waves', 3)
    _need(maps, torch.float32, 'maps', 3)
    _lib.check(lib().msx_corrector_apply_map(_ptr(waves), waves.shape[0], waves.shape[1], waves.shape[2], _ptr(maps),
                                             int(which), int(bool(conj)), int(form), _stream()))
    return waves


def mul_plane(waves, plane, conj=False):
    """waves (num, ny, nx) complex64 *= plane (ny, nx) complex64 (or its conjugate)."""
    _need(waves, torch.complex64, 'waves', 3)
    _need(plane, torch.complex64, 'plane', 2)
    _lib.check(lib().msx_corrector_mul_plane(_ptr(waves), waves.shape[0], waves.shape[1], waves.shape[2], _ptr(plane),
                                             int(bool(conj)), _stream()))
    return waves


def map_trans(trans, maps, which, out=None, form=0):
    """trans (ny, nx) complex64 times the factor of map M (1 + M, or exp(i Im M) for form 1)."""
    _need(trans, torch.complex64, 'trans', 2)
    _need(maps, torch.float32, 'maps', 3)
    if out is None:
        out = torch.empty_like(trans)
    _lib.check(lib().msx_corrector_map_trans(_ptr(trans), trans.shape[0], trans.shape[1], _ptr(maps), int(which),
                                             int(form), _ptr(out), _stream()))
    return out


def map_grad(u, g, which, dmaps, accumulate=False, form=0, maps=None):
    """Gradient of the loss with respect to map M (into dmaps (ny, nx, 4)) for a factor that
    multiplied u, g the adjoint of the product; form 1 needs the maps."""
    _need(u, torch.complex64, 'u', 3)
    _need(g, torch.complex64, 'g', 3)
    _need(dmaps, torch.float32, 'dmaps', 3)
    _lib.check(lib().msx_corrector_map_grad(_ptr(u), _ptr(g), u.shape[0], u.shape[1], u.shape[2], int(which),
                                            int(bool(accumulate)), int(form), _ptr(maps), _ptr(dmaps), _stream()))
    return dmaps


def residual(psi, target, weight, adjoint, loss_out, accumulate=False):
    """adjoint (+)= weight (psi - target); loss_out[0] = weight sum |psi - target|^2."""
    _need(psi, torch.complex64, 'psi', 3)
    _need(target, torch.complex64, 'target', 3)
    _need(adjoint, torch.complex64, 'adjoint', 3)
    _lib.check(lib().msx_corrector_residual(_ptr(psi), _ptr(target), psi.shape[0], psi.shape[1], psi.shape[2],
                                            float(weight), int(bool(accumulate)), _ptr(adjoint), _ptr(loss_out),
                                            _stream()))
