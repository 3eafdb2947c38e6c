/*
 * msx.h -- C ABI of the GB300 multislice engine (libmsx.so).
 *
 * The engine replaces the GPU path of namsa's MSAGPU simulator
 * (namsa/msa.py:529-992 with the kernels of namsa/probe_kernels.cu and
 * namsa/potential_kernels.cu, launched through pycuda and cuFFT).  In the
 * reference that path is reached through the kernel loader
 * (namsa/cuda_kernels.py:8-57: ProbeKernels / PotentialKernels return
 * dicts of pycuda Functions taking raw device pointers).  This header is the
 * equivalent plugin boundary: plain pointers, sizes and a stream handle.
 *
 * Conventions
 *  - Every call returns an int status: MSX_OK (0) or a negative MSX_ERR_*.
 *    msx_last_error() copies the message of the last failure of the calling
 *    thread.
 *  - All array arguments named *_dev are device pointers owned by the caller,
 *    contiguous, row-major.  complex64 arrays are interleaved (re, im) float
 *    pairs.  Nothing is synchronised: work is ordered on `stream`
 *    (a cudaStream_t, NULL = the legacy default stream).
 *  - A plan owns its workspace and is not re-entrant; distinct plans may be
 *    used from distinct threads.
 *  - Supported grid line lengths (msx_supported_size): 64, 128, 256, 384,
 *    512, 768, 1024 on each axis.
 */
#ifndef MSX_H_
#define MSX_H_

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MSX_OK 0
#define MSX_ERR_INVALID -1      /* bad argument (size, pointer, range)          */
#define MSX_ERR_UNSUPPORTED -2  /* grid line length without a compiled schedule */
#define MSX_ERR_CUDA -3         /* CUDA runtime error (launch, configuration)   */
#define MSX_ERR_ALLOC -4        /* device allocation failed                     */
#define MSX_ERR_TIMEOUT -5      /* a bounded wait inside a kernel gave up       */

#if defined(__GNUC__)
#define MSX_API __attribute__((visibility("default")))
#else
#define MSX_API
#endif

typedef struct msx_plan msx_plan;
typedef struct msx_batch msx_batch;
typedef struct msx_corrector msx_corrector;

/* One crystal of an uneven batch (msx_batch_run): the arguments of
 * msx_multislice for one grid. */
typedef struct msx_job {
  int ny, nx;                       /* grid (supported line lengths)            */
  int num_slices, num_probes;
  int crop_y, crop_x;
  float kmax, k_band;               /* float32 k extent and mask radius          */
  double lambda, slice_t;
  const float* trans_dev;           /* (num_slices, ny, nx) complex64            */
  const float* psi_k_dev;           /* (ny, nx) complex64                        */
  const double* normalization_dev;  /* 1 float64                                 */
  const float* positions_dev;       /* (num_probes, 2) [y, x] Angstrom           */
  float* cbed_out_dev;              /* (num_probes, crop_y, crop_x) float32      */
} msx_job;

/* Library version (major*10000 + minor*100 + patch). */
MSX_API int msx_version(void);

/* Copies the last error message of the calling thread into buf (NUL-terminated).
 * Returns the message length. */
MSX_API int msx_last_error(char* buf, size_t len);

/* 1 if n is a supported grid line length, else 0. */
MSX_API int msx_supported_size(int n);

/* Number of compiled FFT schedules for line length n, and the name of one. */
MSX_API int msx_num_schedules(int n);
MSX_API int msx_schedule_name(int n, int index, char* buf, size_t len);
/* Columns per tile of a schedule's column pass. */
MSX_API int msx_schedule_col_tile(int n, int index, int* tile);

/*
 * Band-limited column range of the persistent passes (no counterpart in the
 * reference, whose every slice transforms the whole grid).  Every column with
 * |kx| >= k_band is zeroed whole by the bandwidth mask (msa.py:829-839), so from
 * the second slice on the passes leave the columns outside [x_lo, x_hi) alone
 * (they stay zero); the range is aligned to `tile` columns and keeps a 1e-6
 * relative margin on k_band.  Host only.
 */
MSX_API int msx_band_columns(int nx, float kmax, float k_band, int tile, int* x_lo, int* x_hi);

/*
 * Projected Kirkland potential windows of `nspecies` species.
 * Replaces MSA.calc_atomic_potentials / MSA._get_potential
 * (namsa/msa.py:137-146, 180-196) and bin_2d_array (namsa/utils.py:101-108),
 * which the reference evaluates on the host with scipy.
 *   coeff_dev     (nspecies, 4, 3) float64 Kirkland a, b, c, d rows
 *   n0, n1        oversampled grid points per axis (floor(range/pix) * oversample)
 *   windows_out   (nspecies, n0/oversample, n1/oversample) float32
 */
MSX_API int msx_atom_windows(const double* coeff_dev, int nspecies, int n0, int n1, int oversample, double potential_range,
                     float* windows_out_dev, void* stream);

/*
 * Transmission slices t = exp(i sigma V) of the supercell.
 * Replaces MSAGPU.build_potential_slices (namsa/msa.py:580-647) and the
 * BuildScatteringPotential kernel (namsa/potential_kernels.cu:5-60).
 *   sites_dev          (nsites, 4) int32 rows (species index, y pixel, x pixel, unused),
 *                      grouped by slice in supercell order
 *   slice_offsets_dev  (num_slices + 1) int32: sites of slice s are [off[s], off[s+1])
 *   windows_dev        (nspecies, window_h, window_w) float32
 *   trans_out_dev      (num_slices, ny, nx) complex64
 *   potential_out_dev  (num_slices, ny, nx) float32 summed potential V, or NULL
 */
MSX_API int msx_build_transmission(const int* sites_dev, const int* slice_offsets_dev, int num_slices, const float* windows_dev,
                           int window_h, int window_w, int ny, int nx, float sigma, float* trans_out_dev,
                           float* potential_out_dev, void* stream);

/*
 * k-space probe psi_k = A(k) exp(-i chi(k)) and its normalisation.
 * Replaces MSAGPU.build_probe (namsa/msa.py:669-735) with the soft_aperture,
 * hard_aperture, spherical_phase_error and mult_wise_c2d_re2d kernels
 * (namsa/probe_kernels.cu:126-134, 180-222).
 *   kmax               float32 k-grid extent (1/Angstrom)
 *   k_semi             float32 aperture radius semi_angle/lambda
 *   c1, c3, c5         defocus and spherical aberrations (Angstrom)
 *   smooth_aperture    1: 1/(1+exp(-160 (k_semi-k))), 0: k < k_semi
 *   psi_k_out_dev      (ny, nx) complex64
 *   aperture_out_dev   (ny, nx) float32 or NULL
 *   normalization_dev  1 float64: sum |fftshift(ifft2(psi_k))|^2 (unnormalised ifft), or NULL
 */
MSX_API int msx_build_probe(int ny, int nx, float kmax, double lambda, float k_semi, double c1, double c3, double c5,
                    int smooth_aperture, float* psi_k_out_dev, float* aperture_out_dev, double* normalization_dev,
                    void* stream);

/*
 * Multislice plan for an (ny, nx) grid.  `group` is the number of probe
 * wavefunctions kept resident per group (0 = about 1 GiB of waves, 4 to 512);
 * the workspace for it is allocated here.  The plan starts with the schedules
 * the autotuner picks on GB300 for the grid (msx_plan_autotune refines both
 * for given inputs).  Replaces the per-batch cuFFT plans and allocations of
 * MSAGPU.multislice (namsa/msa.py:843-881) and plan_simulation's batching
 * (namsa/msa.py:445-461).
 */
MSX_API int msx_plan_create(int ny, int nx, int group, msx_plan** plan);
MSX_API int msx_plan_destroy(msx_plan* plan);

/* Selects the FFT schedule of the row (x) and column (y) passes (index into
 * msx_num_schedules of nx / ny) and the group size; group 0 keeps the
 * current one.  The workspace grows when needed. */
MSX_API int msx_plan_set_schedule(msx_plan* plan, int row_schedule, int col_schedule, int group);

/* Reports the current row/column schedule indices and group size. */
MSX_API int msx_plan_get_schedule(const msx_plan* plan, int* row_schedule, int* col_schedule, int* group);

/* 1 = run the per-slice passes as persistent, TMA-pipelined kernels (default);
 * 0 = one CTA per tile, plain loads.  Both give the same results. */
MSX_API int msx_plan_set_tma(msx_plan* plan, int enable);

/* Synchronises the device and reports whether a pipelined pass of this plan
 * gave up on a bounded wait since the last check (MSX_ERR_TIMEOUT), or found
 * its shared memory misaligned for the paired row transform and did nothing
 * (MSX_ERR_CUDA); the error word is then cleared.  Kernels never trap: a
 * stuck copy makes the pass return early and flag the plan instead. */
MSX_API int msx_plan_check(msx_plan* plan);

/* 1 = record the launch sequence of msx_multislice in a CUDA graph and
 * replay it while the arguments repeat (default 1); 0 = launch directly. */
MSX_API int msx_plan_set_graph(msx_plan* plan, int enable);

/*
 * STEM/CBED multislice over num_probes positions.
 * Replaces MSAGPU.multislice / MSAGPU.__propagate_beams
 * (namsa/msa.py:767-992): probe stack with phase ramps, inverse FFT and
 * fftshift (build_probes_stack, fftshift_2d_stack), then for each slice
 * psi <- ifft2(P mask fft2(psi t_s / N)), then |fft2(psi / N) sqrt(N)|^2 / norm.
 *   trans_dev          (num_slices, ny, nx) complex64 transmission slices
 *   psi_k_dev          (ny, nx) complex64 k-space probe (msx_build_probe)
 *   normalization_dev  1 float64 (msx_build_probe)
 *   positions_dev      (num_probes, 2) float32 [y, x] in Angstrom, the reference's
 *                      probe_positions layout
 *   kmax               float32 k-grid extent; lambda, slice_t in Angstrom
 *   k_band             float32 radius of the bandwidth mask in 1/Angstrom, the reference's
 *                      float32(bandwidth * kmax) (msa.py:833; default bandwidth 1/3)
 *   cbed_out_dev       (num_probes, crop_y, crop_x) float32: rows ny/2-crop_y/2 ..
 *                      and columns nx/2-crop_x/2 .. of the CBED; crop = ny, nx keeps all
 */
MSX_API int msx_multislice(msx_plan* plan, const float* trans_dev, int num_slices, const float* psi_k_dev,
                   const double* normalization_dev, const float* positions_dev, int num_probes, float kmax,
                   double lambda, double slice_t, float k_band, float* cbed_out_dev, int crop_y, int crop_x,
                   void* stream);

/*
 * msx_multislice with host buffers, as the reference's multislice takes the
 * slices and probe from the host and returns the CBED stack there
 * (namsa/msa.py:767-924): trans_host (num_slices, ny, nx) complex64,
 * psi_k_host (ny, nx) complex64, the normalisation as a value, positions_host
 * (num_probes, 2) float32 [y, x], cbed_host (num_probes, crop_y, crop_x) float32.
 * The uploads run on the plan's copy stream in chunks of 8 slices while the
 * first group already computes, and each group's patterns are downloaded while
 * the next group computes.  Stream-ordered like msx_multislice: `stream` waits
 * for the last download, so the host buffers must stay valid until then; they
 * should be page-locked for the copies to overlap.  The plan holds the device
 * copies of the inputs and of the CBED stack.  With page-locked buffers (and
 * graphs enabled) the call is recorded as one CUDA graph and replayed while
 * the arguments, buffer addresses included, repeat; the copies read and write
 * the host buffers' contents at each replay.
 */
MSX_API int msx_multislice_host(msx_plan* plan, const float* trans_host, int num_slices, const float* psi_k_host,
                                double normalization, const float* positions_host, int num_probes, float kmax,
                                double lambda, double slice_t, float k_band, float* cbed_host, int crop_y, int crop_x,
                                void* stream);

/*
 * Real-space wave stepping, for workflows that act on the wave between slices
 * (the learned coarse-slice corrector).  No single reference counterpart: the
 * steps are those of namsa/msa.py:959-990 exposed one at a time.  waves are
 * (num, ny, nx) complex64 real-space arrays owned by the caller.
 *  msx_propagator_table: P(k) mask(k) / N (probe_kernels.cu:167-178, msa.py:833-839)
 *                        into ptab_out (ny, nx) complex64.
 *  msx_plan_probe_waves: fftshift(ifft2_u(psi_k * ramp)) per position (msa.py:959-964).
 *  msx_plan_step_waves:  in place, psi <- ifft2_u(ptab * fft2_u(t * psi)), one slice.
 *  msx_plan_cbed_waves:  |fft2_u(psi)|^2 / N / norm, cropped; the waves are overwritten.
 *  msx_plan_probe_stack: the probe stack of multislice(transmit=False)
 *                        (msa.py:959-964 then the division at msa.py:914-915):
 *                        fftshift(ifft2_u(psi_k * ramp)) / sqrt(norm) per position into
 *                        probes_out (num_probes, ny, nx) complex64, no propagation.
 */
MSX_API int msx_propagator_table(int ny, int nx, float kmax, double lambda, double slice_t, float k_band,
                                 float* ptab_out_dev, void* stream);
MSX_API int msx_plan_probe_waves(msx_plan* plan, const float* psi_k_dev, const float* positions_dev, int num_probes,
                                 float kmax, float* waves_out_dev, void* stream);
MSX_API int msx_plan_probe_stack(msx_plan* plan, const float* psi_k_dev, const double* normalization_dev,
                                 const float* positions_dev, int num_probes, float kmax, float* probes_out_dev,
                                 void* stream);
MSX_API int msx_plan_step_waves(msx_plan* plan, float* waves_dev, int num_waves, const float* trans_dev,
                                const float* ptab_dev, void* stream);
MSX_API int msx_plan_cbed_waves(msx_plan* plan, float* waves_dev, int num_waves, const double* normalization_dev,
                                float* cbed_out_dev, int crop_y, int crop_x, void* stream);

/*
 * Annular (or any) detector signals fused into the last pass instead of CBED
 * stacks: signals_out[p][d] = sum_k I_p(k) w_d(k), with I_p the CBED pattern of
 * msx_multislice (full grid, natural FFT order) and w_d the weights
 * detectors_dev[d] (num_detectors, ny, nx) float32, 1 <= num_detectors <= 8.
 * Replaces MSA.integrate_cbed (namsa/msa.py:426-439), which integrates an
 * already stored CBED stack on the host.  num_slices must be >= 1.
 * Launched directly (no graph).
 */
MSX_API int msx_multislice_detect(msx_plan* plan, const float* trans_dev, int num_slices, const float* psi_k_dev,
                                  const double* normalization_dev, const float* positions_dev, int num_probes,
                                  float kmax, double lambda, double slice_t, float k_band, const float* detectors_dev,
                                  int num_detectors, float* signals_out_dev, void* stream);

/*
 * msx_multislice without any device allocation, for callers that cannot call
 * cudaMalloc: applications whose device memory is entirely owned by their own
 * pool or allocator, plugin hosts that forbid allocation inside their callbacks,
 * and latency-critical loops that must not take cudaMalloc's implicit device
 * synchronisation.  No counterpart in the reference.
 *
 * Arguments are those of msx_multislice with the grid size given directly
 * (no plan).  Scratch -- twiddle tables, the propagator table and the resident
 * wave group -- lives in one static 32 MiB device array compiled into the
 * library; every GPU that loads the library holds it until the process exits.
 * A grid needs (2048 + 2*ny*nx) complex64 words of it at least, so every
 * supported size fits (1024 x 1024 runs 2 waves at a time); larger requests
 * return MSX_ERR_INVALID, and so do complex inputs, positions or the
 * normalisation that are not 8-byte aligned.  The first call on a device looks
 * up the array's device address (cudaGetSymbolAddress) with that device
 * current and keeps it for the life of the process; make that first call
 * before any stream capture.  A cudaDeviceReset on that device invalidates the
 * kept address, so this entry point must not be called on a device after it
 * was reset.  All calls share the array and it keeps
 * the last call's contents (nothing in it needs to start at zero): calls whose
 * work overlaps on the GPU -- on different streams, or from different host
 * threads -- race on it and must be serialised by the caller.  Uses the first
 * FFT schedule of each line length.
 */
MSX_API int msx_multislice_noalloc(const float* trans_dev, int num_slices, const float* psi_k_dev,
                                   const double* normalization_dev, const float* positions_dev, int num_probes,
                                   int ny, int nx, float kmax, double lambda, double slice_t, float k_band,
                                   float* cbed_out_dev, int crop_y, int crop_x, void* stream);

/*
 * Dataset post-processing of the reference's production runs
 * (scripts/summit_scripts/utils.py:74-118), on the device.
 *
 * msx_process_cbed: out[p] = (cbed[p] - mean_p) / std_p (population std) as
 * IEEE float16, for num_patterns patterns of height x width float32
 * (process_cbed, utils.py:102-118).
 *
 * msx_process_potential: the projected-potential label of a transmission stack
 * (num_slices, ny, nx) complex64: mean over slices of Im t, Gaussian filter
 * (sigma 1.2, 11 taps, half-sample reflecting borders, like
 * scipy.ndimage.gaussian_filter), the central crop rows and columns
 * [ny/4, 3*nx/4) (the reference applies one slice to both axes), then
 * (x - mean) / max(std, 1/sqrt(size)) as float16 (process_potential,
 * utils.py:74-100).  work_dev: 2*ny*nx + 22 floats of caller scratch (8-byte
 * aligned).  out: (3*nx/4 - ny/4)^2 halves.
 */
MSX_API int msx_process_cbed(const float* cbed_dev, int num_patterns, int height, int width, void* out_fp16_dev,
                             void* stream);

/*
 * Detector signals of a stored CBED stack: out[p][d] = sum_k cbed[p][k] w_d[k]
 * (float64, a fixed summation order), weights (num_detectors, height, width)
 * float32; with weights NULL and num_detectors 1, the plain sum of each
 * pattern.  Replaces MSA.integrate_cbed (namsa/msa.py:426-439) for stacks
 * already computed and the per-pattern sums of MSA.check_simulation
 * (namsa/msa.py:363-371).
 */
MSX_API int msx_integrate_cbed(const float* cbed_dev, int num_patterns, int height, int width, const float* weights_dev,
                               int num_detectors, double* out_dev, void* stream);
MSX_API int msx_process_potential(const float* trans_dev, int num_slices, int ny, int nx, float* work_dev,
                                  void* out_fp16_dev, void* stream);

/*
 * Transmission slices from a sampled 3-D potential (ab-initio input) instead
 * of Kirkland sites.  Replaces MSA/MSAGPU.integrate_potential_slices
 * (namsa/msa.py:373-424, 568-578): pot_dev (nz, ld_y, ld_x) float32 with the
 * z sample coordinates z_dev (nz) float64; slice s integrates its d = nz /
 * num_slices samples by the trapezoidal rule (samples past num_slices * d are
 * dropped, intervals between slices are not integrated, as in the reference),
 * V = -integral, t = exp(i sigma V) over the leading ny x nx window.
 */
MSX_API int msx_integrate_potential(const float* pot_dev, const double* z_dev, int nz, int ld_y, int ld_x, int ny,
                                    int nx, int num_slices, float sigma, float* trans_out_dev, void* stream);

/*
 * Uneven batches.  Replaces the reference's fan-out over materials and probe
 * blocks (MPI ranks with one crystal each, scripts/sim_batch.py:201,
 * namsa/msa.py:1014-1081) by one CUDA graph on one GPU: jobs of different grid
 * size, thickness, voltage and probe count are spread over `branches`
 * concurrent streams (0 = 4), longest first, each branch keeping one plan per
 * grid size.  The graph is captured on the first call for a job list and
 * replayed while the list repeats; it runs ordered on `stream`.
 */
MSX_API int msx_batch_create(int branches, msx_batch** batch);
MSX_API int msx_batch_destroy(msx_batch* batch);
/* Schedule and group size used for the (ny, nx) plans of the batch. */
MSX_API int msx_batch_set_schedule(msx_batch* batch, int ny, int nx, int row_schedule, int col_schedule, int group);
MSX_API int msx_batch_run(msx_batch* batch, const msx_job* jobs, int njobs, void* stream);
/* msx_plan_autotune for every grid size of the job list, on the job of that
 * size with the most positions (`iters` slices per candidate, workspace up to
 * the batch's 1 GiB per plan); the winners become the batch's schedules.
 * Synchronises `stream`. */
MSX_API int msx_batch_autotune(msx_batch* batch, const msx_job* jobs, int njobs, int iters, void* stream);
/* msx_plan_check over every plan of the batch. */
MSX_API int msx_batch_check(msx_batch* batch);

/*
 * Split-BF16 tensor-core DFT stages (precision study; no reference
 * counterpart).  A length-n DFT of complex lines as a 2n x 2n real GEMM on
 * tcgen05 with bfloat16 hi/lo operand splits (hi.hi + hi.lo + lo.hi, FP32
 * accumulation) and, by default, a per-line norm compensation: each output
 * line is rescaled so that |Z|^2 = n |X|^2 (Parseval), which removes the
 * uniform loss of the accumulation.  n = 256 or 512.
 *  msx_tc_dft:        z (lines, n) = sum_m x[m] e^{sign 2 pi i m k / n}, lines % 128 == 0
 *  msx_step_waves_tc: the msx_plan_step_waves slice with all four 1-D DFTs on the
 *                     tensor cores (square n x n grids)
 *  msx_tc_set_compensation: 1 (default) / 0 turns the norm compensation on / off
 *                     for the calling host thread
 *  msx_tc_check:      synchronises; MSX_ERR_TIMEOUT if a bounded wait gave up
 * Scratch is held per host thread and grows with the largest call.
 */
MSX_API int msx_tc_dft(const float* x_dev, int lines, int n, int sign, float* z_dev, void* stream);
MSX_API int msx_step_waves_tc(float* waves_dev, int num_waves, int n, const float* trans_dev, const float* ptab_dev,
                              void* stream);
MSX_API int msx_tc_set_compensation(int enable);
MSX_API int msx_tc_check(void);

/*
 * General BF16 tensor-core GEMM (no reference counterpart), the contraction
 * engine of the learned corrector: c (m x n) = a (m x k) . b (n x k)^T (+ bias[n])
 * with a and b rounded to bfloat16 and FP32 accumulation on tcgen05; with
 * accumulate = 1 the product is added to c.  a, b, c are FP32 row-major with
 * leading dimensions lda, ldb, ldc (elements); n <= 4096.  Operand images are
 * held per host thread and grow with the largest call.  msx_gemm_check
 * synchronises and reports MSX_ERR_TIMEOUT if a bounded wait gave up.
 */
MSX_API int msx_gemm_bf16(const float* a_dev, int lda, const float* b_dev, int ldb, int m, int n, int k, float* c_dev,
                          int ldc, const float* bias_dev, int accumulate, void* stream);
MSX_API int msx_gemm_check(void);

/*
 * Self-test of the bounded in-kernel wait (no reference counterpart).  One CTA
 * waits on an mbarrier with a limit of 2^limit_log2 cycles (10..31); with
 * arrive = 0 nothing arrives, so the wait runs out and the call returns
 * MSX_ERR_TIMEOUT, the status a pass reports through msx_plan_check when one
 * of its copies never lands.  With arrive = 1 it returns MSX_OK.  Synchronises
 * `stream`.
 */
MSX_API int msx_selftest_wait(int arrive, int limit_log2, void* stream);

/*
 * Learned coarse-slice corrector (no counterpart in the reference).  A
 * spectral-convolution network maps the potentials of the `ratio` fine slices
 * inside one coarse slice to two per-pixel complex maps A, B of the corrected
 * coarse step
 *     psi <- (1 + A) . ifft2( P_c . fft2( (1 + B) . t_c . psi ) )
 * (P_c the coarse propagator, t_c the coarse transmission).  The maps depend on
 * the crystal only: the network runs once per coarse slice and the corrected
 * multislice of every probe costs what the plain coarse one costs.
 *
 * Network: lift of `in_channels` inputs to C channels, L spectral layers
 * (per-mode C x C complex mixing on modes kx in [0, modes_x), ky in
 * [-modes_y/2, modes_y/2), plus a pointwise C x C layer, gelu), pointwise MLP
 * head C -> C -> 4.  Every contraction (lift, pointwise layers, head, their
 * weight gradients, the partial DFT stages) runs as a bfloat16 GEMM with FP32
 * accumulation on the tensor cores; activations are FP32, pixel-major
 * (samples, ny, nx, channels).  Parameters, gradients and Adam moments are
 * four consecutive float32 arrays of `count` values; msx_corrector_layout
 * gives the offsets of W0 (C x in), b0, then per layer R (modes_x * modes_y *
 * C * C complex, mode-major), W (C x C), b, then P1 (C x C), c1, P2 (4 x C), c2.
 * Parameters start at zero: the caller writes its initialisation.
 *  msx_corrector_forward:  features (S, ny, nx, in_channels) -> maps (S, ny, nx, 4) =
 *                          (Re A, Im A, Re B, Im B); keeps what the backward needs
 *  msx_corrector_backward: d loss / d maps (S, ny, nx, 4) -> parameter gradients
 *                          (overwritten), for the S samples of the last forward
 *  msx_corrector_adam:     one Adam step on the stored gradients
 *  msx_corrector_check:    synchronises; MSX_ERR_TIMEOUT if a GEMM wait gave up
 *  msx_corrector_features: inputs of S coarse slices from the fine potential
 *                          slices pot (S * ratio, ny, nx): sigma V of each fine
 *                          slice, their sum and the constant tval (in_channels =
 *                          ratio + 2)
 * Rollout helpers on complex64 waves (num, ny, nx) with one map set (ny, nx, 4).  A map M = A
 * (which 0) or B (which 1) acts as the factor 1 + M (form 0) or as the unit-modulus factor
 * exp(i Im M) (form 1, Re M unused: the corrected step then preserves the norm like the exact one):
 *  msx_corrector_apply_map:  waves *= factor (conj: its conjugate)
 *  msx_corrector_mul_plane:  waves *= plane (conj: its conjugate) for one complex (ny, nx) plane
 *  msx_corrector_map_trans:  out = trans * factor for one (ny, nx) plane
 *  msx_corrector_map_grad:   d loss / d (Re M, Im M) (+)= from G = sum_b conj(u_b) g_b, for a factor
 *                            that multiplied u with g the adjoint of the product: (2 Re G, 2 Im G)
 *                            for form 0, (0, 2 Re(conj(G) i factor)) for form 1 (maps_dev needed)
 *  msx_corrector_residual:   adjoint (+)= weight (psi - target); *loss_out = weight sum |psi - target|^2
 */
MSX_API int msx_corrector_create(int ny, int nx, int in_channels, int channels, int layers, int modes_x, int modes_y,
                                 int max_samples, msx_corrector** corrector);
MSX_API int msx_corrector_destroy(msx_corrector* corrector);
MSX_API int msx_corrector_params(msx_corrector* corrector, float** params_dev, float** grads_dev, size_t* count);
MSX_API int msx_corrector_layout(const msx_corrector* corrector, size_t* offsets, int n);
MSX_API int msx_corrector_forward(msx_corrector* corrector, const float* features_dev, int samples, float* maps_out_dev,
                                  void* stream);
MSX_API int msx_corrector_backward(msx_corrector* corrector, const float* dmaps_dev, void* stream);
MSX_API int msx_corrector_adam(msx_corrector* corrector, float lr, float beta1, float beta2, float eps, void* stream);
MSX_API int msx_corrector_check(msx_corrector* corrector);
MSX_API int msx_corrector_features(const float* pot_dev, int samples, int ratio, int ny, int nx, float sigma,
                                   float tval, float* features_out_dev, void* stream);
MSX_API int msx_corrector_apply_map(float* waves_dev, int num, int ny, int nx, const float* maps_dev, int which,
                                    int conj, int form, void* stream);
MSX_API int msx_corrector_mul_plane(float* waves_dev, int num, int ny, int nx, const float* plane_dev, int conj,
                                    void* stream);
MSX_API int msx_corrector_map_trans(const float* trans_dev, int ny, int nx, const float* maps_dev, int which,
                                    int form, float* out_dev, void* stream);
MSX_API int msx_corrector_map_grad(const float* u_dev, const float* g_dev, int num, int ny, int nx, int which,
                                   int accumulate, int form, const float* maps_dev, float* dmaps_dev, void* stream);
MSX_API int msx_corrector_residual(const float* psi_dev, const float* target_dev, int num, int ny, int nx, float weight,
                                   int accumulate, float* adjoint_dev, float* loss_out_dev, void* stream);

/*
 * Autotuner: times every (row schedule, column schedule, group size) of the
 * plan's grid on the given inputs -- `iters` slices of row + column passes
 * per candidate, CUDA events on `stream` -- and keeps the fastest.  Group
 * sizes range over resident sets of 8 MiB to 1 GiB of waves (capped by
 * num_probes and max_workspace_bytes, 0 = 1 GiB).  Writes the best time per
 * wave and slice (ns) to *best_ns_per_wave_slice when non-NULL.  Synchronises
 * `stream`.  No counterpart in the reference (its batch size comes from a
 * free-memory heuristic, namsa/msa.py:445-461).
 */
MSX_API int msx_plan_autotune(msx_plan* plan, const float* trans_dev, int num_slices, const float* psi_k_dev,
                              const double* normalization_dev, const float* positions_dev, int num_probes, float kmax,
                              double lambda, double slice_t, float k_band, int iters, size_t max_workspace_bytes,
                              float* best_ns_per_wave_slice, void* stream);

/*
 * Diagnostics: times one row pass and one column pass of the plan's first
 * group, `iters` times each, with CUDA events on `stream` (one slice of
 * msx_multislice per iteration).  ms_out[0] = mean row-pass ms, ms_out[1] =
 * mean column-pass ms, ms_out[2] = waves per launch.  Synchronises `stream`.
 * No counterpart in the reference (its launches are timed by host clocks,
 * namsa/msa.py:847-909).
 */
MSX_API int msx_plan_profile(msx_plan* plan, const float* trans_dev, int num_slices, const float* psi_k_dev,
                             const double* normalization_dev, const float* positions_dev, int num_probes, float kmax,
                             double lambda, double slice_t, float k_band, int iters, float* ms_out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MSX_H_ */
