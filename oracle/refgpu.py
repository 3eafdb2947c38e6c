"""ctypes front end of the reference-GPU harness -- TEST INFRASTRUCTURE ONLY.

Runs the reference's own rendered CUDA kernels and cuFFT (oracle/refgpu_harness.cu,
built by oracle/build_ref.py) on torch device buffers, mirroring what
``MSAGPU.build_potential_slices``, ``build_probe`` and ``multislice`` do
(namsa/msa.py:580-992).  Used by tests/test_gpu_refgpu.py as the parity target
"the reference's own GPU multislice on identical inputs" and by bench.py's
reference arm for the reference-GPU timing.
"""
from __future__ import annotations

import ctypes
import json
import os

import numpy as np

from . import build_ref
from . import msa_oracle as O

_LIBS = {}


class RefGPUUnavailable(RuntimeError):
    pass


def workloads():
    path = os.path.join(build_ref.OUT, 'workloads.json')
    if not os.path.exists(path):
        return {}
    return json.load(open(path))


def _lib(tag):
    if tag in _LIBS:
        return _LIBS[tag]
    path = build_ref.lib_path(tag)
    if not os.path.exists(path):
        raise RefGPUUnavailable(f'{path} is not built (render the reference kernels with oracle/render_ref_kernels.py '
                                'where the reference checkout exists, then run oracle/build_ref.py)')
    L = ctypes.CDLL(path)
    vp, f, i = ctypes.c_void_p, ctypes.c_float, ctypes.c_int
    L.refgpu_last_error.restype = ctypes.c_char_p
    L.refgpu_shape.argtypes = [ctypes.POINTER(i)] * 6
    L.refgpu_build_potential.argtypes = [vp, vp, vp, f, vp]
    L.refgpu_build_probe.argtypes = [f, f, f, f, f, f, i, vp, vp, vp, vp]
    L.refgpu_ctx_create.argtypes = [i, ctypes.POINTER(vp)]
    L.refgpu_ctx_destroy.argtypes = [vp]
    L.refgpu_propagator.argtypes = [vp, f, f, f, f, vp]
    L.refgpu_propagate.argtypes = [vp, vp, i, vp, vp, f, vp, vp]
    for name in ['refgpu_build_potential', 'refgpu_build_probe', 'refgpu_ctx_create', 'refgpu_propagator',
                 'refgpu_propagate']:
        getattr(L, name).restype = i
    _LIBS[tag] = L
    return L


def _stream():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


class RefGPU:
    """The reference GPU path for one rendered workload (grid, slices, window shape)."""

    def __init__(self, tag):
        self.tag = tag
        self.L = _lib(tag)
        v = [ctypes.c_int() for _ in range(6)]
        self.L.refgpu_shape(*[ctypes.byref(x) for x in v])
        self.ny, self.nx, self.S, self.pot_y, self.pot_x, self.sites_size = [x.value for x in v]
        self.meta = workloads()[tag]

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(self.L.refgpu_last_error().decode())

    def sites(self, geom, slice_t, species):
        """(S, sites_size) float32 site lists in the reference's layout (msa.py:589-605):
        (window index, y pixel, x pixel) triplets, padded with the index of an
        all-zero window (`species`) instead of -1."""
        sites = O.slice_sites_gpu(geom, slice_t)
        assert len(sites) == self.S, (len(sites), self.S)
        out = np.empty((self.S, self.sites_size), np.float32)
        out[:] = -1
        out.reshape(self.S, -1, 3)[:, :, 0] = species
        for s, st in enumerate(sites):
            out[s, :3 * len(st)] = st.astype(np.float32).ravel()
        return out

    def build_potential(self, geom, slice_t, windows):
        """Transmission slices exp(i sigma V) from BuildScatteringPotential."""
        import torch
        w = np.concatenate([windows, np.zeros((1,) + windows.shape[1:], np.float32)]).astype(np.float32)
        assert w.shape[1:] == (self.pot_y, self.pot_x), (w.shape, self.pot_y, self.pot_x)
        dev = torch.device('cuda', torch.cuda.current_device())
        wd = torch.from_numpy(np.ascontiguousarray(w)).to(dev)
        sd = torch.from_numpy(self.sites(geom, slice_t, len(windows))).to(dev)
        out = torch.empty((self.S, self.ny, self.nx), dtype=torch.complex64, device=dev)
        self._check(self.L.refgpu_build_potential(_ptr(out), _ptr(wd), _ptr(sd), np.float32(geom.sigma), _stream()))
        return out

    def build_probe(self, kmax, k_semi, lam, c1, c3, c5, smooth):
        """(psi_k, psi_x, aperture, normalisation) as build_probe leaves them
        (normalisation = FP64 sum of |psi_x|^2 on the host, msa.py:729)."""
        import torch
        dev = torch.device('cuda', torch.cuda.current_device())
        psi_k = torch.empty((self.ny, self.nx), dtype=torch.complex64, device=dev)
        psi_x = torch.empty_like(psi_k)
        ap = torch.empty((self.ny, self.nx), dtype=torch.float32, device=dev)
        self._check(self.L.refgpu_build_probe(np.float32(kmax), np.float32(k_semi), np.float32(lam), np.float32(c1),
                                              np.float32(c3), np.float32(c5), int(bool(smooth)), _ptr(psi_k),
                                              _ptr(psi_x), _ptr(ap), _stream()))
        px = psi_x.cpu().numpy()
        norm = float(np.sum(np.abs(px.astype(np.complex128)) ** 2))
        return psi_k, psi_x, ap, norm

    def context(self, P):
        ctx = ctypes.c_void_p()
        self._check(self.L.refgpu_ctx_create(int(P), ctypes.byref(ctx)))
        return ctx

    def destroy(self, ctx):
        self.L.refgpu_ctx_destroy(ctx)

    def propagator(self, ctx, kmax, k_band, slice_t, lam):
        self._check(self.L.refgpu_propagator(ctx, np.float32(kmax), np.float32(k_band), np.float32(slice_t),
                                             np.float32(lam), _stream()))

    def propagate(self, ctx, trans, psi_k, pos, kmax, psi):
        """One __propagate_beams batch into `psi` (|psi|^2 in the real parts)."""
        self._check(self.L.refgpu_propagate(ctx, _ptr(trans), int(trans.shape[0]), _ptr(psi_k), _ptr(pos),
                                            np.float32(kmax), _ptr(psi), _stream()))

    def multislice(self, trans, psi_k, pos, kmax, k_band, slice_t, lam, normalization):
        """CBED stack (P, ny, nx) float32: the whole multislice call of one batch,
        including the host-side division by the normalisation (msa.py:910-924)."""
        import torch
        P = int(pos.shape[0])
        ctx = self.context(P)
        try:
            self.propagator(ctx, kmax, k_band, slice_t, lam)
            psi = torch.empty((P, self.ny, self.nx), dtype=torch.complex64, device=trans.device)
            self.propagate(ctx, trans, psi_k, pos, kmax, psi)
            torch.cuda.synchronize()
        finally:
            self.destroy(ctx)
        return (psi.cpu().numpy() / normalization).real.astype(np.float32)
