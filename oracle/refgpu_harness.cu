// Reference-GPU harness -- TEST INFRASTRUCTURE ONLY.
//
// Drives the reference's own CUDA kernels (namsa/probe_kernels.cu and
// namsa/potential_kernels.cu, rendered by oracle/render_ref_kernels.py into
// oracle/_ref/) and cuFFT in the order MSAGPU uses them, so that the engine can
// be checked against, and timed beside, the reference GPU path on the same
// inputs.  The host logic below restates MSAGPU's calls (no pycuda here):
//
//   build_potential_slices  namsa/msa.py:580-647   (one BuildScatteringPotential launch)
//   build_probe             namsa/msa.py:669-735   (aperture, phase, product, IFFT, fftshift)
//   multislice              namsa/msa.py:767-924   (mask, propagator, product; one batch)
//   __propagate_beams       namsa/msa.py:926-992   (probe stack, IFFT, fftshift, S x
//                                                   [t/N, FFT, P, IFFT], /N, FFT, *sqrt N, |.|^2)
//
// Launch shapes follow MSAGPU._get_blockgrid (msa.py:738-758): 32x32 thread
// blocks, grid (ceil(Nx/32), ceil(Ny/32), z).  One deviation, for memory
// safety: the reference pads every slice's site list with -1 (msa.py:603-604),
// which makes BuildScatteringPotential read atom_pot_stack[-1]
// (potential_kernels.cu:27, 40).  Callers of refgpu_build_potential pad with
// the index of an extra all-zero window instead, which adds exactly +0.0f.
//
// Compiled once per rendered workload by oracle/build_ref.py with
// REF_NY, REF_NX, REF_S, REF_POT_Y, REF_POT_X, REF_SITES and the two rendered
// file names defined; the grid sizes are compile-time constants exactly as in
// the reference's run-time-compiled kernels.
#include <cuda_runtime.h>
#include <cufft.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>

#include REF_PROBE_SRC
#include REF_POT_SRC

#define REFGPU_API extern "C" __attribute__((visibility("default")))

namespace {

typedef pycuda::complex<float> cf;
constexpr int NY = REF_NY, NX = REF_NX;
char g_err[512] = "";

int fail(const char* what, int code) {
  snprintf(g_err, sizeof g_err, "%s failed (%d)", what, code);
  return -1;
}

#define CK(x)                                           \
  do {                                                  \
    cudaError_t e_ = (x);                               \
    if (e_ != cudaSuccess) return fail(#x, (int)e_);    \
  } while (0)
#define CF(x)                                           \
  do {                                                  \
    cufftResult r_ = (x);                               \
    if (r_ != CUFFT_SUCCESS) return fail(#x, (int)r_);  \
  } while (0)

const dim3 kBlock(32, 32, 1);
dim3 grid_xy(int z) { return dim3((NX + 31) / 32, (NY + 31) / 32, z); }

struct RefCtx {
  int P = 0;
  cufftHandle plan = 0;
  cf* propag = nullptr;  // NY x NX, propagator times the bandwidth mask
  float* mask = nullptr;
  cf* ones = nullptr;
  int* grid_steps = nullptr;  // passed to build_probes_stack, which does not read it
};

}  // namespace

REFGPU_API const char* refgpu_last_error() { return g_err; }

REFGPU_API void refgpu_shape(int* ny, int* nx, int* slices, int* pot_y, int* pot_x, int* sites_size) {
  *ny = NY;
  *nx = NX;
  *slices = REF_S;
  *pot_y = REF_POT_Y;
  *pot_x = REF_POT_X;
  *sites_size = REF_SITES;
}

// slices: REF_S x NY x NX complex64 (written); windows: (species + 1) x POT_Y x POT_X
// float32 with the last window all zero; sites: REF_S x REF_SITES float32 triplets
// (window index, y pixel, x pixel) padded with the zero window's index.
REFGPU_API int refgpu_build_potential(float2* slices, const float* windows, const float* sites, float sigma,
                                      cudaStream_t st) {
  CK(cudaMemsetAsync(slices, 0, sizeof(float2) * (size_t)REF_S * NY * NX, st));
  // grid z doubled as in msa.py:636
  BuildScatteringPotential<<<grid_xy(2 * REF_S), kBlock, 0, st>>>(
      reinterpret_cast<cf(*)[NY][NX]>(slices), reinterpret_cast<float(*)[REF_POT_Y][REF_POT_X]>(const_cast<float*>(windows)),
      reinterpret_cast<float(*)[REF_SITES]>(const_cast<float*>(sites)), sigma);
  CK(cudaGetLastError());
  return 0;
}

// psi_k, psi_x: NY x NX complex64; apert: NY x NX float32.  Synchronises the stream.
REFGPU_API int refgpu_build_probe(float kmax, float k_semi, float lambda, float c1, float c3, float c5, int smooth,
                                  float2* psi_k, float2* psi_x, float* apert, cudaStream_t st) {
  const dim3 g = grid_xy(1);
  if (smooth)
    soft_aperture<<<g, kBlock, 0, st>>>(apert, kmax, k_semi, NX, NY);
  else
    hard_aperture<<<g, kBlock, 0, st>>>(apert, kmax, k_semi, NX, NY);
  spherical_phase_error<<<g, kBlock, 0, st>>>(reinterpret_cast<cf*>(psi_k), kmax, lambda, c1, c3, c5, NX, NY);
  mult_wise_c2d_re2d<<<g, kBlock, 0, st>>>(reinterpret_cast<cf*>(psi_k), apert, NX, NY);
  CK(cudaGetLastError());
  cufftHandle plan;
  CF(cufftPlan2d(&plan, NY, NX, CUFFT_C2C));
  CF(cufftSetStream(plan, st));
  const cufftResult r = cufftExecC2C(plan, reinterpret_cast<cufftComplex*>(psi_k), reinterpret_cast<cufftComplex*>(psi_x),
                                     CUFFT_INVERSE);
  fftshift_2d<<<g, kBlock, 0, st>>>(reinterpret_cast<cf(*)[NX]>(psi_x), NY);
  const cudaError_t e = cudaStreamSynchronize(st);
  cufftDestroy(plan);
  if (r != CUFFT_SUCCESS) return fail("cufftExecC2C", (int)r);
  CK(e);
  CK(cudaGetLastError());
  return 0;
}

// Workspace and the batched cuFFT plan for P probes (msa.py:800-821, 862-869).
REFGPU_API int refgpu_ctx_create(int P, void** out) {
  *out = nullptr;
  if (P <= 0) return fail("refgpu_ctx_create: P must be positive", P);
  RefCtx* c = new RefCtx;
  c->P = P;
  int n[2] = {NY, NX};
  if (cufftPlanMany(&c->plan, 2, n, nullptr, 1, NY * NX, nullptr, 1, NY * NX, CUFFT_C2C, P) != CUFFT_SUCCESS) {
    delete c;
    return fail("cufftPlanMany", P);
  }
  if (cudaMalloc(&c->propag, sizeof(cf) * NY * NX) != cudaSuccess || cudaMalloc(&c->mask, sizeof(float) * NY * NX) ||
      cudaMalloc(&c->ones, sizeof(cf) * NY * NX) || cudaMalloc(&c->grid_steps, 2 * sizeof(int))) {
    cufftDestroy(c->plan);
    cudaFree(c->propag);
    cudaFree(c->mask);
    cudaFree(c->ones);
    cudaFree(c->grid_steps);
    delete c;
    return fail("cudaMalloc (reference workspace)", P);
  }
  float2* h = static_cast<float2*>(malloc(sizeof(float2) * NY * NX));
  for (int i = 0; i < NY * NX; ++i) h[i] = make_float2(1.f, 0.f);
  cudaMemcpy(c->ones, h, sizeof(float2) * NY * NX, cudaMemcpyHostToDevice);
  free(h);
  cudaMemset(c->grid_steps, 0, 2 * sizeof(int));
  *out = c;
  return 0;
}

REFGPU_API void refgpu_ctx_destroy(void* ctx) {
  RefCtx* c = static_cast<RefCtx*>(ctx);
  if (!c) return;
  cufftDestroy(c->plan);
  cudaFree(c->propag);
  cudaFree(c->mask);
  cudaFree(c->ones);
  cudaFree(c->grid_steps);
  delete c;
}

// Bandwidth mask and propagator (msa.py:829-839): k_band = float32(bandwidth * kmax).
REFGPU_API int refgpu_propagator(void* ctx, float kmax, float k_band, float slice_t, float lambda, cudaStream_t st) {
  RefCtx* c = static_cast<RefCtx*>(ctx);
  const dim3 g = grid_xy(1);
  hard_aperture<<<g, kBlock, 0, st>>>(c->mask, kmax, k_band, NX, NY);
  propagator<<<g, kBlock, 0, st>>>(c->propag, kmax, slice_t, lambda, NX, NY);
  mult_wise_c2d_re2d<<<g, kBlock, 0, st>>>(c->propag, c->mask, NX, NY);
  CK(cudaGetLastError());
  return 0;
}

// __propagate_beams for one batch of the context's P probes: psi (P x NY x NX
// complex64, written) ends with |psi|^2 in the real parts, before the host-side
// division by the probe normalisation (msa.py:910-918).
REFGPU_API int refgpu_propagate(void* ctx, const float2* slices, int S, const float2* psi_k, const float* pos_yx,
                                float kmax, float2* psi, cudaStream_t st) {
  RefCtx* c = static_cast<RefCtx*>(ctx);
  const int P = c->P;
  const dim3 g = grid_xy(P);
  auto stack = reinterpret_cast<cf(*)[NY][NX]>(psi);
  auto cslices = reinterpret_cast<cf(*)[NY][NX]>(const_cast<float2*>(slices));
  auto ck = reinterpret_cast<cufftComplex*>(psi);
  CF(cufftSetStream(c->plan, st));
  build_probes_stack<<<g, kBlock, 0, st>>>(stack, reinterpret_cast<cf(*)[NX]>(const_cast<float2*>(psi_k)), P, kmax,
                                           c->grid_steps, reinterpret_cast<float(*)[2]>(const_cast<float*>(pos_yx)));
  CF(cufftExecC2C(c->plan, ck, ck, CUFFT_INVERSE));
  fftshift_2d_stack<<<g, kBlock, 0, st>>>(stack, P);
  const float inv_n = (float)(1.0 / ((double)NY * NX));
  for (int i = 0; i < S; ++i) {
    mult_wise_c3d_c3d_ind<<<g, kBlock, 0, st>>>(stack, cslices, P, i, inv_n);
    CF(cufftExecC2C(c->plan, ck, ck, CUFFT_FORWARD));
    mult_wise_c3d_c2d<<<g, kBlock, 0, st>>>(stack, reinterpret_cast<cf(*)[NX]>(c->propag), P, 1.0f);
    CF(cufftExecC2C(c->plan, ck, ck, CUFFT_INVERSE));
  }
  auto ones = reinterpret_cast<cf(*)[NX]>(c->ones);
  mult_wise_c3d_c2d<<<g, kBlock, 0, st>>>(stack, ones, P, inv_n);
  CF(cufftExecC2C(c->plan, ck, ck, CUFFT_FORWARD));
  mult_wise_c3d_c2d<<<g, kBlock, 0, st>>>(stack, ones, P, (float)std::sqrt((double)NY * NX));
  mod_square_stack<<<g, kBlock, 0, st>>>(stack, P);
  CK(cudaGetLastError());
  return 0;
}
