"""CPU oracle for namsa's STEM/CBED multislice path -- TEST INFRASTRUCTURE ONLY.

This module restates, in NumPy, the arithmetic of the reference's multislice
path so that the CUDA engine in ``namsa_gb300`` can be checked against it.  It
is imported only by ``tests/``, by ``__graft_entry__.smoke()`` (as the checker)
and by ``bench.py``'s CPU-baseline / reference arm.  The product path never
imports it and has no CPU fallback.

Two convention sets exist in the reference and both are restated here:

* ``"gpu"`` -- the ``MSAGPU`` path (namsa/msa.py:529-992 with the kernels in
  namsa/probe_kernels.cu and namsa/potential_kernels.cu).  This is the path
  the engine replaces and the one parity is defined against.
* ``"cpu"`` -- the ``MSA`` CPU path (namsa/msa.py:61-361).  It differs in slice
  order (reversed, msa.py:337,346), aperture smoothing (``apert_smooth``
  instead of the kernel's fixed 80, probe_kernels.cu:203-204), window
  placement (``int()`` truncation, msa.py:169-171, instead of ``rintf`` around
  an integer centre, potential_kernels.cu:30-33), the bandwidth mask
  (pixel-radius ``N*bw`` around ``N/2``, msa.py:245-251, instead of
  ``k < bw*kmax``, msa.py:833), and the Scherzer rule (only when C3 > 1,
  optics.py:84-88).  The CPU conventions are pinned against the reference
  CPU class itself (``tests/golden``); the shared pieces (Kirkland windows,
  k-grid, propagator phase, FFT sequence) carry that pin over to the GPU
  conventions, whose remaining differences are restated from the kernel
  source lines cited below.

Precision: ``dtype=np.float64`` evaluates everything in FP64 (the accuracy
oracle).  ``potential_slices_gpu(..., mode="f32")`` reproduces the kernel's
sequential float32 accumulation bit for bit (one thread per pixel adds the
sites of its slice in site order, potential_kernels.cu:25-41).
"""
from __future__ import annotations

import math
import numpy as np
from scipy.constants import electron_mass, elementary_charge, speed_of_light
from scipy.special import k0 as _bessel_k0

XYZ_DTYPE = [('atomic_number', 'i'), ('x', 'f'), ('y', 'f'), ('z', 'f'), ('occ', 'f'), ('DW', 'f')]


# --------------------------------------------------------------------------- optics
def voltage2lambda(voltage):
    """Relativistic electron wavelength in Angstrom (namsa/optics.py:4-12)."""
    return 12.2643 / np.sqrt(voltage + 0.97845e-6 * voltage ** 2)


def sigma_int(voltage):
    """Interaction parameter sigma in rad/(V*Angstrom) (namsa/optics.py:100-108)."""
    mc2 = electron_mass * speed_of_light ** 2
    ev = elementary_charge * voltage
    return 2 * np.pi * (mc2 + ev) / (2 * mc2 + ev) / (voltage2lambda(voltage) * voltage)


def scherzer_defocus(lam, cs):
    """Scherzer defocus sqrt(1.5*Cs*lambda) (namsa/optics.py:69-72, first return value)."""
    return np.sqrt(1.5) * np.sqrt(cs * lam)


# --------------------------------------------------------------------------- geometry
class Geometry:
    """Simulation geometry as set up by ``MSA.__init__`` (namsa/msa.py:66-127).

    ``xyz`` is cast to float32 like msa.py:96; ``dims`` is the atom extent
    (msa.py:110); ``kmax = min(N/dims)`` (msa.py:114); ``pix_size`` is in
    (y, x) order (msa.py:121).  Debye-Waller jitter is not applied (the
    reference draws it unseeded, msa.py:102-107; callers pass displaced
    coordinates if they want it).
    """

    def __init__(self, xyz, Z, energy_kev, semi_angle, sampling):
        self.xyz = np.asarray(xyz, dtype=np.float32)
        self.Z = np.asarray(Z).astype(np.int64)
        self.E = energy_kev
        self.lam = voltage2lambda(energy_kev * 1e3)
        self.semi_ang = semi_angle
        self.sampling = np.asarray(sampling)
        self.dims = self.xyz.max(0) - self.xyz.min(0)
        self.kmax = np.min(self.sampling / self.dims[:2])
        self.pix_size = self.dims[:2][::-1] / self.sampling
        self.sigma = sigma_int(energy_kev * 1e3)

    def num_slices(self, slice_t):
        """``floor(dims_z / t)`` in the reference's float32 (msa.py:584)."""
        return int(np.int32(np.floor(self.dims[-1] / slice_t)))


# --------------------------------------------------------------------------- atom windows
def atom_potential(params, pix_size, potential_range=8, oversample=2):
    """Projected Kirkland potential window of one species.

    Follows ``calc_atomic_potentials``/``_get_potential`` (namsa/msa.py:137-146,
    180-196) and ``bin_2d_array`` (namsa/utils.py:101-108): an oversampled
    grid over [-range/2, range/2] with ``floor(range/pix)*oversample``
    inclusive points per axis, the Kirkland sum with a 0.1 Angstrom Bessel
    offset, 2x2 mean binning, minus its minimum, cast to float32.
    """
    start = potential_range / 2
    n = (np.floor(potential_range / np.asarray(pix_size)).astype(np.int64) * oversample)
    gx, gy = np.mgrid[-start:start:1j * n[0], -start:start:1j * n[1]]
    r = np.sqrt(gx ** 2 + gy ** 2)
    a0, e = 0.529, 14.4
    pre = 4 * np.pi ** 2 * a0 * e
    a, b, c, d = params
    v = (pre * a * _bessel_k0(2 * np.pi * r[:, :, None] * np.sqrt(b) + 0.1)
         + pre / 2. * c / d * np.exp(-np.pi ** 2 * r[:, :, None] ** 2 / d)).sum(-1)
    h0, h1 = v.shape
    v = v.reshape(h0 // oversample, oversample, h1 // oversample, oversample).mean(-1).mean(-2)
    v -= v.min()
    return v.astype(np.float32)


def atom_windows(geom, kirkland, potential_range=8, oversample=2):
    """Windows for the unique species in ascending Z order (msa.py:145, 589, 607)."""
    uz = np.unique(geom.Z)
    return uz, np.stack([atom_potential(kirkland[z - 1], geom.pix_size, potential_range, oversample) for z in uz])


# --------------------------------------------------------------------------- slices
def slice_masks(geom, slice_t):
    """Atom membership per slice, ``z`` in [s*t, (s+1)*t) compared in float32 (msa.py:585-587)."""
    S = geom.num_slices(slice_t)
    z = geom.xyz[:, -1]
    return [np.logical_and(z >= s * slice_t, z < (s + 1) * slice_t) for s in range(S)]


def slice_sites_gpu(geom, slice_t):
    """Per-slice integer sites (Z index, y pixel, x pixel) (msa.py:589-604).

    Pixel centres are ``int32`` truncations of ``xyz/pix`` (msa.py:592, 596);
    the Z index is the rank of Z among the unique species (msa.py:589-590).
    Returns a list of (n_s, 3) int64 arrays in supercell order.
    """
    uz = np.unique(geom.Z)
    zidx = np.searchsorted(uz, geom.Z)
    pix = geom.xyz[:, :2] / geom.pix_size[::-1]          # columns (x/px, y/py), float64
    out = []
    for m in slice_masks(geom, slice_t):
        yx = pix[m]
        out.append(np.column_stack([zidx[m], yx[:, 1], yx[:, 0]]).astype(np.int32).astype(np.int64))
    return out


def potential_slices_gpu(sites, windows, sampling, mode="f64"):
    """Summed projected potential V per slice with the kernel's windowing.

    ``BuildScatteringPotential`` (namsa/potential_kernels.cu:5-60): window start
    ``rintf(c - h/2)``, end ``rintf(c + h/2)``, clipped to the grid without
    periodic wrap, window row ``pix - start`` kept while ``< h``.  ``mode="f32"``
    accumulates in float32 in site order exactly as one thread per pixel does;
    ``"f64"`` accumulates in float64.  Padded sites of the reference (Z = -1,
    which read before the window stack, msa.py:603) are not materialised.
    """
    Ny, Nx = int(sampling[0]), int(sampling[1])
    H, W = windows.shape[1:]
    acc = np.float32 if mode == "f32" else np.float64
    V = np.zeros((len(sites), Ny, Nx), dtype=acc)
    win = windows.astype(acc)
    for s, st in enumerate(sites):
        for zi, yc, xc in st:
            ys = int(np.rint(np.float32(yc) - np.float32(H * 0.5)))
            ye = int(np.rint(np.float32(yc) + np.float32(H * 0.5)))
            xs = int(np.rint(np.float32(xc) - np.float32(W * 0.5)))
            xe = int(np.rint(np.float32(xc) + np.float32(W * 0.5)))
            r0, r1 = max(ys, 0), min(ye, Ny, ys + H)
            c0, c1 = max(xs, 0), min(xe, Nx, xs + W)
            if r1 <= r0 or c1 <= c0:
                continue
            V[s, r0:r1, c0:c1] += win[zi, r0 - ys:r1 - ys, c0 - xs:c1 - xs]
    return V


def transmission(V, sigma, mode="f64"):
    """t = exp(i sigma V) (potential_kernels.cu:48-57; msa.py:334 for the CPU path)."""
    if mode == "f32":
        arg = V.astype(np.float32) * np.float32(sigma)
        t = np.empty(V.shape, np.complex64)
        t.real = np.cos(arg)
        t.imag = np.sin(arg)
        return t
    return np.exp(1j * float(sigma) * V.astype(np.float64))


def potential_slices_cpu(geom, windows, slice_t):
    """CPU ``make_slice`` (namsa/msa.py:162-178): ``int()`` windows, float32 sums."""
    uz = np.unique(geom.Z)
    out = []
    for m in slice_masks(geom, slice_t):
        arr = np.zeros(tuple(int(v) for v in geom.sampling), dtype=np.float32)
        for Z, xyz in zip(geom.Z[m], geom.xyz[m]):
            pot = windows[int(np.searchsorted(uz, Z))]
            y_pix, x_pix = xyz[:2][::-1] / geom.pix_size
            y0, y1 = int(y_pix - pot.shape[0] / 2), int(y_pix + pot.shape[0] / 2)
            x0, x1 = int(x_pix - pot.shape[1] / 2), int(x_pix + pot.shape[1] / 2)
            ry, rx = slice(max(y0, 0), y1), slice(max(x0, 0), x1)
            oy, ox = abs(min(y0, 0)), abs(min(x0, 0))
            shp = arr[ry, rx].shape
            arr[ry, rx] += pot[oy:shp[0] + oy, ox:shp[1] + ox]
        out.append(arr)
    return np.array(out)


# --------------------------------------------------------------------------- k grid, probe
def kgrid_gpu(kmax32, n):
    """Centred linspace k axis of ``calc_krad`` (probe_kernels.cu:11-16), float64."""
    k = np.float64(np.float32(kmax32))
    j = np.arange(n, dtype=np.float64)
    return j * k / (n - 1) - k / 2.


def probe_gpu(geom, probe_dict, dtype=np.float64):
    """k-space probe psi_k = A(k) exp(-i chi(k)) and the normalisation of the GPU path.

    ``MSAGPU.build_probe`` (namsa/msa.py:669-735) with ``soft_aperture``
    (smoothing fixed at 80, probe_kernels.cu:196-206), ``hard_aperture``
    (probe_kernels.cu:180-194) and ``spherical_phase_error``
    (probe_kernels.cu:208-222).  Scherzer defocus replaces C1 whenever
    ``probe_dict['scherzer']`` is set (msa.py:677-679).  The normalisation is
    ``sum |fftshift(ifft_unnormalised(psi_k))|^2`` (msa.py:721-727).

    Returns (psi_k, aperture, normalization) in ``dtype`` precision.
    """
    Ny, Nx = int(geom.sampling[0]), int(geom.sampling[1])
    kmax32 = np.float32(geom.kmax)
    lam = np.float32(geom.lam) if dtype == np.float32 else geom.lam
    ab = probe_dict['aberration_dict']
    C1, C3, C5 = ab['C1'], ab['C3'], ab['C5']
    if probe_dict['scherzer']:
        C1 = scherzer_defocus(geom.lam, C3)
    if dtype == np.float32:
        C1, C3, C5 = np.float32(C1), np.float32(C3), np.float32(C5)
    k_semi = np.float32(geom.semi_ang / geom.lam)
    ky = kgrid_gpu(kmax32, Ny)[:, None]
    kx = kgrid_gpu(kmax32, Nx)[None, :]
    krad = np.sqrt(kx * kx + ky * ky)
    krad32 = krad.astype(np.float32)
    if probe_dict['smooth_apert']:
        with np.errstate(over='ignore'):
            if dtype == np.float32:
                ap = (np.float32(1) / (np.float32(1) + np.exp(np.float32(-160.) * (k_semi - krad32)))).astype(np.float32)
            else:
                ap = 1. / (1. + np.exp(-160. * (np.float64(k_semi) - krad)))
    else:
        ap = (krad32 < k_semi).astype(dtype)
    kl = krad * float(lam)
    chi = 2. * np.pi / float(lam) * (-0.5 * float(C1) * kl ** 2 + 0.25 * float(C3) * kl ** 4
                                     + float(C5) / 6. * kl ** 6)
    ctype = np.complex128 if dtype == np.float64 else np.complex64
    psi_k = (ap * np.exp(-1j * chi)).astype(ctype)
    psi_x = np.fft.fftshift(np.fft.ifft2(psi_k.astype(np.complex128)) * (Ny * Nx))
    normalization = float(np.sum(np.abs(psi_x) ** 2))
    return psi_k, ap.astype(dtype), normalization


def propagator_gpu(geom, slice_t, bandwidth, dtype=np.float64):
    """Fresnel propagator times the bandwidth mask of the GPU path.

    ``propagator`` (probe_kernels.cu:167-178): P = exp(-i pi lambda t k^2) on the
    centred grid; ``hard_aperture`` with ``k_semi = bandwidth*kmax``
    (msa.py:833-839): the mask keeps ``float(k) < float(bw*kmax)`` (the
    comparison is done in float32 exactly like the kernel, so the mask is
    identical in both precisions).
    """
    Ny, Nx = int(geom.sampling[0]), int(geom.sampling[1])
    kmax32 = np.float32(geom.kmax)
    ky = kgrid_gpu(kmax32, Ny)[:, None]
    kx = kgrid_gpu(kmax32, Nx)[None, :]
    krad = np.sqrt(kx * kx + ky * ky)
    krad32 = krad.astype(np.float32)
    mask = (krad32 < np.float32(bandwidth * geom.kmax))
    if dtype == np.float32:
        k = krad32.astype(np.float64)
        arg = (np.pi * k * k * float(np.float32(geom.lam)) * float(np.float32(slice_t))).astype(np.float32)
        P = (np.cos(arg) - 1j * np.sin(arg)).astype(np.complex64)
    else:
        P = np.exp(-1j * np.pi * geom.lam * slice_t * krad ** 2)
    return P * mask, mask


def probe_cpu(geom, probe_dict, position=(0., 0.)):
    """CPU ``MSA.build_probe`` (namsa/msa.py:198-236): returns (psi_x, psi_k, aperture)."""
    Ny, Nx = int(geom.sampling[0]), int(geom.sampling[1])
    ky, kx = np.mgrid[-geom.kmax / 2:geom.kmax / 2:1j * Ny, -geom.kmax / 2:geom.kmax / 2:1j * Nx]
    krad = np.sqrt(kx ** 2 + ky ** 2)
    k_semi = geom.semi_ang / geom.lam
    if probe_dict['smooth_apert']:
        with np.errstate(over='ignore'):
            ap = 1 / (1 + np.exp(-2 * probe_dict['apert_smooth'] * (k_semi - krad)))
    else:
        ap = np.heaviside(k_semi - krad, 0.5)
    ab = probe_dict['aberration_dict']
    C1, C3, C5 = ab['C1'], ab['C3'], ab['C5']
    if probe_dict['scherzer'] and C3 > 1.0:
        C1 = scherzer_defocus(geom.lam, C3)
    lam = geom.lam
    chi = 2 * np.pi / lam * (-0.5 * C1 * (krad * lam) ** 2 + 0.25 * C3 * (krad * lam) ** 4
                             + C5 / 6. * (krad * lam) ** 6)
    psi_k = ap * np.exp(-1j * chi)
    x, y = position
    ramp = np.exp(2 * np.pi * 1j * (-kx * x - ky * y))
    psi_x = np.fft.fftshift(np.fft.ifft2(psi_k * ramp, norm='ortho'))
    psi_x /= np.sqrt(np.sum(np.abs(psi_x) ** 2))
    return psi_x, psi_k, ap


def propagator_cpu(geom, slice_t, bandwidth):
    """CPU ``build_propagator`` x ``bandwidth_limit_mask`` (namsa/msa.py:238-251, 323-324)."""
    Ny, Nx = int(geom.sampling[0]), int(geom.sampling[1])
    ky, kx = np.mgrid[-geom.kmax / 2:geom.kmax / 2:1j * Ny, -geom.kmax / 2:geom.kmax / 2:1j * Nx]
    P = np.exp(-np.pi * 1j * geom.lam * slice_t * (kx ** 2 + ky ** 2))
    gx, gy = np.mgrid[-Ny // 2:Ny // 2, -Nx // 2:Nx // 2]
    mask = np.heaviside(max(Ny, Nx) * bandwidth - np.sqrt(gx ** 2 + gy ** 2), 0)
    return P * mask


# --------------------------------------------------------------------------- multislice
def probe_ramp_gpu(geom, position_yx, n_yx):
    """Per-position phase ramp exp(2 pi i (-kx x - ky y)) (probe_kernels.cu:37-57, 239-253).

    Evaluated in float64 on the same centred grid; ``position_yx`` is the
    reference's ``[y, x]`` pair (msa.py:265, 887)."""
    kmax32 = np.float32(geom.kmax)
    ky = kgrid_gpu(kmax32, n_yx[0])[:, None]
    kx = kgrid_gpu(kmax32, n_yx[1])[None, :]
    y, x = float(position_yx[0]), float(position_yx[1])
    return np.exp(2j * np.pi * (-kx * x - ky * y))


def multislice_gpu(t, psi_k, P, positions_yx, normalization, geom, crop=None, dtype=np.float64):
    """CBED stack of the GPU path (``MSAGPU.__propagate_beams``, namsa/msa.py:926-992).

    For each position: psi = fftshift(ifft2_u(psi_k * ramp)) (msa.py:959-964);
    for i = 0..S-1 (forward order, msa.py:971): psi = ifft2_u(P * fft2_u(psi * t_i / N))
    (msa.py:973-981); then I = |fft2_u(psi / N) * sqrt(N)|^2 / normalization
    (msa.py:985-990, 905).  ``crop`` keeps rows/cols N/2-crop/2 .. N/2+crop/2-1.
    ``t`` is (S, Ny, Nx); all FFTs are unnormalised like cuFFT's C2C.
    """
    import scipy.fft as sfft  # pocketfft, as numpy.fft, with threads over the rows
    ct = np.complex128 if dtype == np.float64 else np.complex64
    fft2 = lambda a: sfft.fft2(a, workers=-1)
    ifft2 = lambda a: sfft.ifft2(a, workers=-1)
    S, Ny, Nx = t.shape
    N = Ny * Nx
    out = []
    Pc = P.astype(ct)
    for pos in np.asarray(positions_yx):
        psi = np.fft.fftshift(ifft2(psi_k.astype(ct) * probe_ramp_gpu(geom, pos, (Ny, Nx)).astype(ct)) * N)
        for i in range(S):
            psi = psi * t[i].astype(ct) / N
            psi = ifft2(fft2(psi) * Pc) * N
        I = np.abs(fft2(psi / N) * np.sqrt(N)) ** 2 / normalization
        if crop is not None and crop < min(Ny, Nx):
            I = I[Ny // 2 - crop // 2:Ny // 2 + crop // 2, Nx // 2 - crop // 2:Nx // 2 + crop // 2]
        out.append(I.astype(np.float64 if dtype == np.float64 else np.float32))
    return np.array(out)


def probe_stack_gpu(psi_k, positions_yx, normalization, geom):
    """Probe stack of ``multislice(transmit=False)`` (namsa/msa.py:959-964, 970, 914-915).

    For each position fftshift(ifft2_u(psi_k * ramp)) / sqrt(normalization),
    complex128: the probes are formed and shifted, no slice is applied, and
    the stack is divided by the square root of the normalisation."""
    Ny, Nx = psi_k.shape
    out = []
    for pos in np.asarray(positions_yx):
        psi = np.fft.fftshift(np.fft.ifft2(psi_k.astype(np.complex128) * probe_ramp_gpu(geom, pos, (Ny, Nx))) * Ny * Nx)
        out.append(psi / np.sqrt(normalization))
    return np.array(out)


def bandwidth_limit_mask(shape, radius):
    """Disc of pixel radius max(shape)*radius about the centre (namsa/msa.py:246-251)."""
    gx, gy = np.mgrid[-shape[0] // 2:shape[0] // 2, -shape[1] // 2:shape[1] // 2]
    r = np.sqrt(gx ** 2 + gy ** 2)
    return np.heaviside(max(shape[0], shape[1]) * radius - r, 0).astype(np.float32)


def annular_detector(sampling, kpix_size, lam, inner_angle, outer_angle):
    """Annular detector of ``integrate_cbed`` (namsa/msa.py:428-435): the radii are
    angle / (kpix * lambda * N) / 2 per axis, the first axis's is used, and the
    annulus is where the outer and inner discs differ."""
    sampling = np.asarray(sampling)
    inner = inner_angle / (np.asarray(kpix_size) * lam * sampling) / 2
    outer = outer_angle / (np.asarray(kpix_size) * lam * sampling) / 2
    inner_seg = bandwidth_limit_mask(sampling, inner[0]).astype(bool)
    outer_seg = bandwidth_limit_mask(sampling, outer[0]).astype(bool)
    return np.logical_not(outer_seg == inner_seg)


def integrate_cbed(cbed, grid_steps, detector):
    """STEM image of ``integrate_cbed`` (namsa/msa.py:436-439): the CBED stack
    reshaped to (grid_steps..., Ny, Nx) and summed over each pattern times the
    detector, in float64."""
    stack = np.asarray(cbed, np.float64).reshape(list(grid_steps) + list(np.shape(cbed)[-2:]))
    return np.sum(stack * np.asarray(detector, np.float64), axis=(-2, -1))


def exit_wave_cpu(V, sigma, psi0, Pmask):
    """CPU ``propagate_beam`` (namsa/msa.py:320-361): reversed slice order, returns the exit wave."""
    t = np.exp(1j * sigma * V.astype(np.float64))
    psi = psi0.astype(np.complex128)
    for ti in t[::-1]:
        psi = np.fft.ifft2(np.fft.fft2(ti * psi) * Pmask)
    return psi


def _cpu_probe_worker(args):
    V, sigma, geom_state, probe_dict, slice_t, bandwidth, pos = args
    geom = Geometry.__new__(Geometry)
    geom.__dict__.update(geom_state)
    psi0, _, _ = probe_cpu(geom, probe_dict, (pos[1], pos[0]))
    P = propagator_cpu(geom, slice_t, bandwidth).astype(np.complex64)
    t = np.exp(1j * sigma * V).astype(np.complex64)
    psi = psi0.astype(np.complex64)
    for ti in t[::-1]:
        psi = np.fft.ifft2(np.fft.fft2(ti * psi) * P)
    return np.abs(np.fft.fft2(psi)) ** 2


def cbed_cpu_pool(V, geom, probe_dict, slice_t, bandwidth, positions_yx, processes):
    """The reference CPU path's per-position process pool (namsa/msa.py:280-318),
    complex64 NumPy FFTs like the reference under NumPy 2, one task per position.
    Used only as the timed CPU baseline.  The pool uses the ``spawn`` start method."""
    import multiprocessing as mp
    ctx = mp.get_context('spawn')
    state = dict(geom.__dict__)
    tasks = [(V, geom.sigma, state, probe_dict, slice_t, bandwidth, p) for p in np.asarray(positions_yx)]
    with ctx.Pool(processes=processes) as pool:
        return np.array(pool.map(_cpu_probe_worker, tasks, chunksize=max(1, len(tasks) // processes)))


# --------------------------------------------------------------------------- probe positions
def generate_probe_positions(dims, probe_step=np.array([0.1, 0.1]), probe_range=np.array([[0., 1.0], [0., 1.0]]),
                             grid_steps=None, fraction=0.5, origin=np.array([0, 0])):
    """``generate_probe_positions`` (namsa/msa.py:253-278); returns (positions[y,x], grid_steps, grid_range)."""
    dims = np.asarray(dims)
    if grid_steps is not None:
        start = (0.5 + origin[::-1] * dims[:2] - dims[:2] * fraction) / 2
        stop = (0.5 + origin[::-1] * dims[:2] + dims[:2] * fraction) / 2
        x_pos, y_pos = np.mgrid[start[0]:stop[0]:-1j * grid_steps[0], start[1]:stop[1]:-1j * grid_steps[1]]
        gsx, gsy = np.asarray(grid_steps).astype(int)
        grx = np.array([start[0], stop[0]])
        gry = np.array([start[1], stop[1]])
    else:
        gsx, gsy = np.floor(np.diff(probe_range).flatten() * dims[:2] / probe_step).astype(int)
        grx, gry = [(probe_range[i] - np.ones((2,)) * 0.5) * dims[i] for i in range(2)]
        x_pos, y_pos = np.mgrid[grx[0]:grx[1]:-1j * gsx, gry[0]:gry[1]:-1j * gsy]
    pos = np.array([[y, x] for y, x in zip(y_pos.flatten(), x_pos.flatten())])
    return pos, np.array([gsx, gsy]), np.array([grx, gry]).flatten()


# --------------------------------------------------------------------------- errors
def rel_l2(a, b, axes=(-2, -1)):
    """Per-pattern relative L2 error ||a-b|| / ||b||."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.sqrt(((a - b) ** 2).sum(axes)) / np.sqrt((b ** 2).sum(axes))


# --------------------------------------------------------------------------- crystals
def si_supercell(nx, ny, nz, a=5.431):
    """Face-inclusive diamond-cubic Si supercell as a reference XYZ structured array.

    Atoms with 0 <= r <= n*a on every axis are kept, matching the inclusive
    bounds of ``make_orthogonal_supercell`` (namsa/supercell.py:444)."""
    basis = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0],
                      [.25, .25, .25], [.25, .75, .75], [.75, .25, .75], [.75, .75, .25]])
    return _tile(basis, np.full(len(basis), 14), (nx, ny, nz), a)


def srtio3_supercell(nx, ny, nz, a=3.905):
    """Cubic perovskite SrTiO3: Sr (0,0,0), Ti (1/2,1/2,1/2), O at the face centres."""
    basis = np.array([[0, 0, 0], [.5, .5, .5], [.5, .5, 0], [.5, 0, .5], [0, .5, .5]])
    return _tile(basis, np.array([38, 22, 8, 8, 8]), (nx, ny, nz), a)


def random_supercell(seed, nx, ny, nz):
    """A seeded random cubic crystal of the uneven-batch kind: a ~ U[3, 8] Angstrom, 1-4
    species with Z ~ U{3..83}, 2-16 atoms at uniform fractional positions, each of one of
    the drawn species; tiled face-inclusive like si_supercell."""
    rng = np.random.default_rng(seed)
    a = rng.uniform(3.0, 8.0)
    ns = int(rng.integers(1, 5))
    zs = rng.integers(3, 84, size=ns)
    na = int(rng.integers(2, 17))
    basis = rng.uniform(0.0, 1.0, size=(na, 3))
    species = zs[rng.integers(0, ns, size=na)]
    return _tile(basis, species, (nx, ny, nz), a)


def _tile(basis, zs, n, a):
    n = np.asarray(n)
    cells = np.stack(np.meshgrid(*[np.arange(k + 1) for k in n], indexing='ij'), -1).reshape(-1, 3)
    pos = (cells[:, None, :] + basis[None, :, :]).reshape(-1, 3) * a
    zz = np.tile(zs, len(cells))
    keep = np.all((pos >= 0) & (pos <= n * a + 1e-6), axis=1)
    pos, zz = pos[keep], zz[keep]
    arr = np.zeros(len(pos), dtype=XYZ_DTYPE)
    arr['atomic_number'] = zz
    arr['x'], arr['y'], arr['z'] = pos[:, 0], pos[:, 1], pos[:, 2]
    arr['occ'] = 1
    return arr


# --------------------------------------------------------------------------- dataset post-processing
def process_cbed(cbed):
    """Per-pattern z-score to float16 (scripts/summit_scripts/utils.py:102-118)."""
    cbed = np.asarray(cbed)
    return ((cbed - np.mean(cbed, axis=(1, -1), keepdims=True)) / np.std(cbed, axis=(1, -1), keepdims=True)).astype(np.float16)


def process_potential(trans):
    """Projected-potential label (scripts/summit_scripts/utils.py:74-100): mean of Im t over
    slices, Gaussian filter sigma 1.2 (scipy, reflecting borders), the central crop
    [ny//4, 3*nx//4) on both axes, z-score with std floored at 1/sqrt(size), float16."""
    from scipy.ndimage import gaussian_filter
    proj = np.imag(trans).mean(0)
    proj = gaussian_filter(proj, 1.2)
    snap = slice(int(proj.shape[0] // 4), int(3 * proj.shape[1] // 4))
    proj = proj[snap, snap]
    proj = (proj - proj.mean()) / max(proj.std(), 1. / np.sqrt(proj.size))
    return np.expand_dims(proj, 0).astype(np.float16)


def integrate_potential_slices(pot, z, slice_t):
    """Slices of a sampled 3-D potential (namsa/msa.py:373-406): ``int(z_dim // t)``
    slices of ``nz // S`` samples each (trailing samples dropped), square crop to
    min(ny, nx), trapezoidal rule along z within each slice, negated."""
    z = np.asarray(z, np.float64)
    S = int((z[-1] - z[0]) // slice_t)
    n = min(pot.shape[1], pot.shape[2])
    pot = pot[:, :n, :n]
    d = pot.shape[0] // S
    out = []
    for s in range(S):
        p = pot[s * d:(s + 1) * d].astype(np.float64)
        zz = z[s * d:(s + 1) * d]
        out.append(-(np.diff(zz)[:, None, None] * (p[1:] + p[:-1]) * 0.5).sum(0))
    return np.array(out)
