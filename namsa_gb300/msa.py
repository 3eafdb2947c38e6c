"""``MSAGPU`` simulator surface over the libmsx engine.

The class keeps the method names, arguments and result attributes of namsa's
``MSAGPU`` (namsa/msa.py:529-992, inheriting ``MSA.__init__`` msa.py:66-127,
``generate_probe_positions`` msa.py:253-278, ``plan_simulation``
msa.py:445-461 and ``integrate_cbed`` msa.py:426-439), so driver scripts
written for the reference run unchanged:

    msa = MSAGPU(energy_kev, semi_angle, supercell_sites, sampling=np.array([512, 512]))
    msa.setup_device(gpu_id)
    msa.calc_atomic_potentials()
    msa.build_potential_slices(slice_thickness)
    msa.build_probe(probe_dict=...)
    msa.generate_probe_positions(...)      # or set msa.probe_positions directly
    msa.plan_simulation()
    msa.multislice(bandwidth=1/3)
    msa.probes                             # (P, Ny, Nx) float32 CBED stack

The host prepares small integer tables (slice membership, pixel sites) like
the reference does; every array operation on the potential, the probe and
the waves runs in libmsx.so.  Large results stay on the device as torch
tensors (``trans``, ``cbed``); the reference's host attributes
(``potential_slices``, ``probes``) are copies made on demand.
"""
from __future__ import annotations

import os
from warnings import warn

import numpy as np
import torch

from . import engine
from .optics import scherzer_defocus, sigma_int, voltage2Lambda

XYZ_dtype = [('atomic_number', 'i'), ('x', 'f'), ('y', 'f'), ('z', 'f'), ('occ', 'f'), ('DW', 'f')]
_DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'data')

DEFAULT_PROBE = {'smooth_apert': True, 'apert_smooth': 50, 'spherical_phase': True,
                 'aberration_dict': {'C1': 0., 'C3': 0., 'C5': 0.}, 'scherzer': True}


def kirkland_table():
    """(103, 4, 3) float64 Kirkland parameters indexed by Z-1 (namsa/database.py:7-8)."""
    return np.load(os.path.join(_DATA, 'kirkland_params.npy'))


# ----------------------------------------------------------------------------- host tables
def load_supercell(supercell):
    """Structured array with fields atomic_number, x, y, z, occ, DW (msa.py:76-95)."""
    if isinstance(supercell, np.ndarray):
        for field in ['x', 'y', 'z', 'occ', 'DW', 'atomic_number']:
            if field not in supercell.dtype.names:
                raise ValueError(f'supercell array lacks field {field!r}')
        return np.copy(supercell)
    if isinstance(supercell, str):
        if not os.path.exists(supercell):
            raise FileNotFoundError(supercell)
        return np.genfromtxt(supercell, skip_footer=1, skip_header=2, dtype=XYZ_dtype)
    raise TypeError('supercell must be a structured numpy array or an XYZ file path')


def window_grid(pix_size, potential_range=8, oversample=2):
    """Oversampled window grid points per axis, floor(range/pix)*oversample (msa.py:141-143)."""
    n = np.floor(potential_range / np.asarray(pix_size)).astype(np.int64) * oversample
    return int(n[0]), int(n[1])


def num_slices_of(dims_z, slice_t):
    """floor(dims_z / t) in float32 like the reference (msa.py:584)."""
    return int(np.int32(np.floor(np.float32(dims_z) / slice_t)))


def slice_sites(xyz, Z, pix_size, slice_t, num_slices):
    """Per-slice integer sites of the GPU path (msa.py:585-604).

    Returns ``sites`` (n, 4) int32 rows (species index, y pixel, x pixel, 0) in
    slice order, supercell order within a slice, and ``offsets`` (S+1,) int32.
    Atoms belong to slice s when s*t <= z < (s+1)*t in float32; pixel centres are
    int32 truncations of xyz/pix; species are ranked among the unique Z.
    """
    xyz = np.asarray(xyz, np.float32)
    Z = np.asarray(Z)
    uz = np.unique(Z)
    zidx = np.searchsorted(uz, Z)
    pix = xyz[:, :2] / np.asarray(pix_size)[::-1]
    z = xyz[:, 2]
    rows, offs = [], [0]
    for s in range(num_slices):
        m = np.logical_and(z >= s * slice_t, z < (s + 1) * slice_t)
        yx = pix[m]
        st = np.column_stack([zidx[m], yx[:, 1], yx[:, 0]]).astype(np.int32)
        rows.append(st)
        offs.append(offs[-1] + len(st))
    sites = np.zeros((offs[-1], 4), np.int32)
    if offs[-1]:
        sites[:, :3] = np.concatenate(rows)
    return sites, np.asarray(offs, np.int32)


def probe_positions_grid(dims, probe_step=np.array([0.1, 0.1]), probe_range=np.array([[0., 1.0], [0., 1.0]]),
                         grid_steps=None, fraction=0.5, origin=np.array([0, 0])):
    """Probe positions [y, x] (Angstrom) of ``generate_probe_positions`` (msa.py:253-278).

    Returns (positions, grid_steps, grid_range)."""
    dims = np.asarray(dims)
    if grid_steps is not None:
        start = (0.5 + origin[::-1] * dims[:2] - dims[:2] * fraction) / 2
        stop = (0.5 + origin[::-1] * dims[:2] + dims[:2] * fraction) / 2
        x_pos, y_pos = np.mgrid[start[0]:stop[0]:-1j * grid_steps[0], start[1]:stop[1]:-1j * grid_steps[1]]
        gsx, gsy = np.asarray(grid_steps).astype(int)
        grx, gry = np.array([start[0], stop[0]]), np.array([start[1], stop[1]])
    else:
        gsx, gsy = np.floor(np.diff(probe_range).flatten() * dims[:2] / probe_step).astype(int)
        grx, gry = [(probe_range[i] - np.ones((2,)) * 0.5) * dims[i] for i in range(2)]
        x_pos, y_pos = np.mgrid[grx[0]:grx[1]:-1j * gsx, gry[0]:gry[1]:-1j * gsy]
    pos = np.column_stack([y_pos.flatten(), x_pos.flatten()])
    return pos, np.array([gsx, gsy]), np.array([grx, gry]).flatten()


def max_probes_for(num_probes, sampling, slices_nbytes, free_bytes):
    """plan_simulation's batch heuristic (msa.py:445-461): shrink by 0.75 until
    probes + slices fit in half of the free device memory."""
    free = free_bytes / 1024e6
    n = int(num_probes)

    def need(k):
        return k * np.prod(sampling) * 8 / 1024e6 + slices_nbytes / 1024e6
    while need(n) > 0.5 * free and n > 0:
        n = int(n * 0.75)
    return n


def annular_detector(sampling, kpix_size, Lambda, inner_angle, outer_angle):
    """Annular detector mask of ``integrate_cbed`` (msa.py:426-435)."""
    sampling = np.asarray(sampling)
    inner = inner_angle / (np.asarray(kpix_size) * Lambda * sampling) / 2
    outer = outer_angle / (np.asarray(kpix_size) * Lambda * sampling) / 2

    def disk(radius):
        gx, gy = np.mgrid[-sampling[0] // 2:sampling[0] // 2, -sampling[1] // 2:sampling[1] // 2]
        r = np.sqrt(gx ** 2 + gy ** 2)
        return np.heaviside(max(sampling[0], sampling[1]) * radius - r, 0).astype(bool)
    return np.logical_not(disk(outer[0]) == disk(inner[0]))


# ----------------------------------------------------------------------------- simulator
class MSAGPU:
    """STEM/CBED multislice simulator on one GPU (drop-in for namsa's MSAGPU)."""

    def __init__(self, energy, semi_angle, supercell, sampling=np.array([512, 512]), max_angle=None, verbose=False,
                 debug=False, output_dir='', debye_waller=True, seed=None):
        self.E = energy
        self.Lambda = voltage2Lambda(self.E * 1e3)
        self.semi_ang = semi_angle
        self.verbose = verbose
        self.debug = debug
        self.output_dir = output_dir
        self.debye_waller = debye_waller
        arr = load_supercell(supercell)
        self.supercell_xyz = np.column_stack([arr['x'], arr['y'], arr['z']]).astype(np.float32)
        self.supercell_Z = arr['atomic_number']
        self.supercell_dw = arr['DW']
        self.supercell_occ = arr['occ']
        # thermal displacements (msa.py:101-107); the reference draws them unseeded
        rng = np.random.default_rng(seed) if seed is not None else np.random
        for Z in np.unique(self.supercell_Z):
            idx = np.where(self.supercell_Z == Z)[0]
            dw = self.supercell_dw[idx][0]
            self.supercell_xyz[idx] += float(self.debye_waller) * dw * rng.standard_normal(size=self.supercell_xyz[idx].shape)
        self.dims = self.supercell_xyz.max(0) - self.supercell_xyz.min(0)
        self.max_angle = max_angle
        if max_angle is None:
            self.sampling = np.asarray(sampling)
            self.kmax = np.min(self.sampling / self.dims[:2])
            self.max_ang = self.kmax * self.Lambda
        else:
            self.max_ang = max_angle
            self.kmax = self.max_ang / self.Lambda
            self.sampling = np.floor(self.kmax * self.dims[:2]).astype(int)[::-1]
        self.pix_size = self.dims[:2][::-1] / self.sampling
        self.kpix_size = self.kmax / self.sampling
        self.sigma = sigma_int(self.E * 1e3)
        self.device = None
        self.trans = None
        self.potential = None
        self.cbed = None
        self.probe_positions = None
        self.num_probes = 0
        self._plan = None
        self._probes_host = None
        self._last = None
        self.probe_stack = None
        self.print_verbose(f'grid {self.sampling[0]} x {self.sampling[1]} px over a {self.dims[0]:.3f} x '
                           f'{self.dims[1]:.3f} x {self.dims[2]:.3f} A cell; pixel {self.pix_size[0]:.4f} A, '
                           f'k pixel {self.kpix_size[0]:.4f} 1/A; largest angle {self.max_ang * 1e3:.1f} mrad')

    # ------------------------------------------------------------------ utilities
    def print_debug(self, *args, **kwargs):
        if self.debug:
            print(*args, **kwargs)

    def print_verbose(self, *args, **kwargs):
        if self.verbose:
            print(*args, **kwargs)

    def _dev(self):
        if self.device is None:
            self.setup_device(torch.cuda.current_device())
        return self.device

    def setup_device(self, gpu_id=0):
        """Select the GPU (msa.py:535-553; the context is torch's)."""
        if not torch.cuda.is_available():
            raise RuntimeError('MSAGPU needs a CUDA device')
        torch.cuda.set_device(gpu_id)
        self.device = torch.device('cuda', gpu_id)
        engine.lib()
        return self.device

    # ------------------------------------------------------------------ potential
    def calc_atomic_potentials(self, potential_range=8, oversample=2, kirkland=True):
        """Kirkland windows of every species, computed on the device (msa.py:137-146)."""
        if not kirkland:
            raise NotImplementedError('only Kirkland parameterised potentials exist in the reference')
        dev = self._dev()
        self.unique_Z = np.unique(self.supercell_Z)
        n0, n1 = window_grid(self.pix_size, potential_range, oversample)
        coeff = torch.from_numpy(np.ascontiguousarray(kirkland_table()[self.unique_Z - 1])).to(dev)
        self.windows = engine.atom_windows(coeff, n0, n1, oversample, potential_range)
        self._cached_pots = None

    @property
    def cached_pots(self):
        """Host copies of the windows keyed by Z, like the reference's dict (msa.py:144-146)."""
        if self._cached_pots is None:
            w = self.windows.cpu().numpy()
            self._cached_pots = {Z: w[i] for i, Z in enumerate(self.unique_Z)}
        return self._cached_pots

    def build_potential_slices(self, slice_thickness, keep_potential=False):
        """Transmission slices exp(i sigma V) on the device (msa.py:580-647)."""
        dev = self._dev()
        self.slice_t = slice_thickness
        self.num_slices = num_slices_of(self.dims[-1], slice_thickness)
        sites, offs = slice_sites(self.supercell_xyz, self.supercell_Z, self.pix_size, slice_thickness, self.num_slices)
        self.sites = torch.from_numpy(sites).to(dev)
        self.site_offsets = torch.from_numpy(offs).to(dev)
        self.trans, self.potential = engine.build_transmission(
            self.sites, self.site_offsets, self.windows, int(self.sampling[0]), int(self.sampling[1]),
            np.float32(self.sigma), want_potential=keep_potential)
        self.print_verbose('Built %d potential slices with shape:%s pixels' % (self.num_slices, self.sampling))

    def integrate_potential_slices(self, pot, grid, slice_thickness, output=False):
        """Transmission slices from a sampled 3-D potential (namsa/msa.py:373-424, 568-578).

        ``pot`` is (nz, ny, nx) in the reference's units, ``grid`` the (z, y, x)
        coordinate arrays.  The geometry is updated like the reference: square
        crop to min(ny, nx), dims from the coordinate maxima, sampling from the
        slice shape (or from ``max_angle``)."""
        dev = self._dev()
        z, y, x = [np.asarray(g, np.float64) for g in grid]
        self.slice_t = slice_thickness
        S = int((z[-1] - z[0]) // slice_thickness)
        n = min(x.size, y.size)
        self.num_slices = S
        self.dims = np.array([x.max(), y.max(), z.max()])
        if self.max_angle is None:
            self.sampling = np.array([n, n])
            self.kmax = np.min(self.sampling / self.dims[:2])
            self.max_ang = self.kmax * self.Lambda
        else:
            self.max_ang = self.max_angle
            self.kmax = self.max_ang / self.Lambda
            self.sampling = np.floor(self.kmax * self.dims[:2]).astype(int)[::-1]
        self.pix_size = self.dims[:2][::-1] / self.sampling
        self.kpix_size = self.kmax / self.sampling
        p = torch.as_tensor(np.ascontiguousarray(pot, np.float32), device=dev)
        zt = torch.as_tensor(z, device=dev)
        self.trans = engine.integrate_potential(p, zt, S, np.float32(self.sigma))
        self.potential = None
        if output:
            return self.trans

    def process_cbed(self):
        """Per-pattern z-scored float16 CBED stack (scripts/summit_scripts/utils.py:102-118)."""
        return engine.process_cbed(self.cbed)

    def process_potential(self):
        """Projected-potential label, float16 (scripts/summit_scripts/utils.py:74-100)."""
        return engine.process_potential(self.trans)

    @property
    def potential_slices(self):
        """Host copy of the transmission slices (the reference keeps them pinned on the host, msa.py:616-638)."""
        return None if self.trans is None else self.trans.cpu().numpy()

    # ------------------------------------------------------------------ probe
    def build_probe(self, probe_dict=DEFAULT_PROBE):
        """k-space probe psi_k = A exp(-i chi) and its normalisation (msa.py:669-735)."""
        self._dev()
        self.probe_dict = probe_dict
        ab = probe_dict['aberration_dict']
        C1, C3, C5 = ab['C1'], ab['C3'], ab['C5']
        if probe_dict['scherzer']:
            C1 = scherzer_defocus(self.Lambda, C3)
        if not probe_dict.get('spherical_phase', True):
            raise NotImplementedError('the reference implements only the rotationally invariant phase error')
        self.k_semi = np.float32(self.semi_ang / self.Lambda)
        self.psi_k_dev, self.apert_dev, self.norm_dev = engine.build_probe(
            int(self.sampling[0]), int(self.sampling[1]), np.float32(self.kmax), self.Lambda, self.k_semi,
            C1, C3, C5, probe_dict['smooth_apert'])
        self.normalization = float(self.norm_dev.item())

    @property
    def psi_k(self):
        return self.psi_k_dev.cpu().numpy()

    @property
    def apert(self):
        return self.apert_dev.cpu().numpy()

    @property
    def psi(self):
        """Unit-norm real-space probe at the origin, fftshift(ifft2(psi_k)) (msa.py:720-728).
        A host convenience view of the k-space probe, not part of the propagation."""
        psi = np.fft.fftshift(np.fft.ifft2(self.psi_k.astype(np.complex128))) * np.prod(self.sampling)
        return (psi / np.sqrt(self.normalization)).astype(np.complex64)

    # ------------------------------------------------------------------ positions and planning
    def generate_probe_positions(self, probe_step=np.array([0.1, 0.1]), probe_range=np.array([[0., 1.0], [0., 1.0]]),
                                 grid_steps=None, fraction=0.5, origin=np.array([0, 0])):
        pos, self.grid_steps, self.grid_range = probe_positions_grid(self.dims, probe_step, probe_range, grid_steps,
                                                                     fraction, origin)
        self.probe_positions = pos
        self.num_probes = np.int32(pos.shape[0])

    def plan_simulation(self, num_probes=None):
        """Batch size bound from free device memory (msa.py:445-461).  The engine
        itself streams probes through a resident group, so this only reports."""
        if num_probes is None:
            num_probes = self.num_probes
        free, _ = torch.cuda.mem_get_info(self._dev())
        nbytes = 0 if self.trans is None else self.trans.numel() * 8
        self.max_probes = max_probes_for(num_probes, self.sampling, nbytes, free)
        return self.max_probes

    def plan(self, group=0):
        """The engine plan of this grid (created on first use)."""
        if self._plan is None:
            self._plan = engine.Plan(int(self.sampling[0]), int(self.sampling[1]), group)
        return self._plan

    # ------------------------------------------------------------------ multislice
    def multislice(self, bandwidth=1 / 3, unified_mem=False, batch_size=None, transmit=True, crop=None):
        """CBED stack of every probe position (msa.py:767-992).

        ``crop`` (int or (cy, cx)) keeps the central window of each pattern;
        None keeps the full grid like the reference.  ``unified_mem`` and
        ``batch_size`` are accepted for compatibility; batching is the plan's.
        The result stays on the device in ``self.cbed``; ``self.probes`` is
        its host copy.  With ``transmit=False`` no slice is applied: the result
        is the unit-norm complex64 probe stack at every position
        (``self.probe_stack``; msa.py:970, 914-915)."""
        if self.trans is None:
            raise RuntimeError('Potential slices must be calculated first: call build_potential_slices().')
        if getattr(self, 'psi_k_dev', None) is None:
            raise RuntimeError('Probe must be initiated first: call build_probe().')
        if self.probe_positions is None:
            raise RuntimeError('Probe positions must be set first: call generate_probe_positions().')
        dev = self._dev()
        self.bandwidth = bandwidth
        pos = torch.from_numpy(np.ascontiguousarray(np.asarray(self.probe_positions, np.float32))).to(dev)
        self._probes_host = None
        if not transmit:
            # probe wavefunctions only (msa.py:970, 914-915): the unit-norm real-space
            # probe stack, complex64, with no slice applied
            self.probe_stack = self.plan().probe_stack(self.psi_k_dev, self.norm_dev, pos, np.float32(self.kmax))
            self._last = self.probe_stack
            return None
        self.cbed = self.plan().multislice(self.trans, self.psi_k_dev, self.norm_dev, pos, np.float32(self.kmax),
                                           self.Lambda, self.slice_t, np.float32(bandwidth * self.kmax), crop=crop)
        self._last = self.cbed
        return None

    @property
    def probes(self):
        """Host copy of the last multislice result: the float32 CBED stack, or with
        transmit=False the complex64 probe stack."""
        last = getattr(self, '_last', None)
        if last is None:
            return None
        if self._probes_host is None:
            self._probes_host = last.cpu().numpy()
        return self._probes_host

    @probes.setter
    def probes(self, value):
        self._probes_host = value

    def check_simulation(self):
        """Integrated intensity per pattern (msa.py:363-371).  Patterns that are not
        finite (NaN or Inf inputs) raise a RuntimeWarning naming how many."""
        prob = engine.integrate_cbed(self.cbed)[:, 0].cpu().numpy()
        bad = ~np.isfinite(prob)
        if bad.any():
            warn(f'{int(bad.sum())} of {prob.size} CBED patterns are not finite (NaN or Inf in the inputs)',
                 RuntimeWarning)
        elif prob.max() > 1.0 or prob.min() < 0.95:
            print('Significant deviation of the probability from unity is found.\n'
                  'Change the sampling and/or slice thickness!')
        return prob

    def integrate_cbed(self, detector_array=None, detector_params={'inner_angle': 50e-3, 'outer_angle': 100e-3}):
        """Annular-detector STEM image (msa.py:426-439)."""
        if detector_array is None:
            if not (detector_params['inner_angle'] < detector_params['outer_angle'] < self.max_ang):
                raise ValueError('Detector angles exceed maximum scattering angle simulated and/or are inconsistent')
            detector_array = annular_detector(self.sampling, self.kpix_size, self.Lambda,
                                              detector_params['inner_angle'], detector_params['outer_angle'])
        det = torch.as_tensor(np.asarray(detector_array, np.float32)[None], device=self.cbed.device).contiguous()
        img = engine.integrate_cbed(self.cbed, det)[:, 0]
        return img.reshape(tuple(int(g) for g in self.grid_steps)).cpu().numpy(), detector_array

    def close(self):
        if self._plan is not None:
            self._plan.close()
            self._plan = None
