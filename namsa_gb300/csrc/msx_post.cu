// Dataset post-processing and the integrated-potential slice source.
//
//  * process_cbed      -- per-pattern z-score to fp16
//                         (scripts/summit_scripts/utils.py:102-118, process_cbed)
//  * process_potential -- mean over slices of Im(t), Gaussian filter (sigma 1.2,
//                         radius 5, half-sample reflection), central crop,
//                         z-score, fp16 (scripts/summit_scripts/utils.py:74-100)
//  * integrate_potential -- slices from a sampled 3-D potential by the
//                         trapezoidal rule along z, t = exp(-i sigma V)
//                         (namsa/msa.py:373-424, 568-578)
#include "msx.h"
#include "msx_internal.h"

#include <cuda_fp16.h>

namespace msx {

// Block-wide sum of a double (blockDim.x a multiple of 32, at most 1024).
__device__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double s = 0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh[i];
  __syncthreads();
  if (threadIdx.x == 0) sh[0] = s;
  __syncthreads();
  return sh[0];
}

// One CTA per pattern: (x - mean) / std with the population std, as float16.
__global__ void process_cbed_kernel(const float* __restrict__ cbed, long long n, __half* __restrict__ out) {
  __shared__ double sh[32];
  const float* x = cbed + (size_t)blockIdx.x * n;
  double s = 0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) s += x[i];
  const double mean = block_sum(s, sh) / (double)n;
  double q = 0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) {
    const double d = x[i] - mean;
    q += d * d;
  }
  const double sd = sqrt(block_sum(q, sh) / (double)n);
  const float fm = (float)mean, fs = (float)sd;
  __half* o = out + (size_t)blockIdx.x * n;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) o[i] = __float2half_rn((x[i] - fm) / fs);
}

// proj[y][x] = mean over slices of Im t (float32 result).
__global__ void proj_imag_kernel(const float2* __restrict__ trans, int S, long long n, float* __restrict__ proj) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0;
  for (int k = 0; k < S; ++k) s += trans[(size_t)k * n + i].y;
  proj[i] = (float)(s / S);
}

// Separable Gaussian (11 taps) along one axis with half-sample reflection at
// the borders: index -k maps to k-1 and N-1+k to N-k.
__global__ void gauss_axis_kernel(const float* __restrict__ in, int ny, int nx, int axis, const double* __restrict__ w,
                                  float* __restrict__ out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= nx) return;
  const int n = axis == 0 ? ny : nx;
  const int c = axis == 0 ? y : x;
  double s = 0;
  for (int k = -5; k <= 5; ++k) {
    int j = c + k;
    if (j < 0) j = -j - 1;
    if (j >= n) j = 2 * n - j - 1;
    const float v = axis == 0 ? in[(size_t)j * nx + x] : in[(size_t)y * nx + j];
    s += w[k + 5] * (double)v;
  }
  out[(size_t)y * nx + x] = (float)s;
}

// Central crop rows/cols [n/4, 3n/4) (both axes use int(ny//4) : int(3*nx//4),
// as the reference applies one slice object to both), z-score with
// std floored at 1/sqrt(size), float16.
__global__ void crop_zscore_kernel(const float* __restrict__ img, int ny, int nx, int r0, int r1,
                                   __half* __restrict__ out) {
  __shared__ double sh[32];
  const int w = r1 - r0;
  const long long n = (long long)w * w;
  double s = 0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) s += img[(size_t)(r0 + i / w) * nx + r0 + i % w];
  const float mean = (float)(block_sum(s, sh) / (double)n);
  double q = 0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) {
    const double d = img[(size_t)(r0 + i / w) * nx + r0 + i % w] - mean;
    q += d * d;
  }
  float sd = (float)sqrt(block_sum(q, sh) / (double)n);
  const float floor_sd = (float)(1.0 / sqrt((double)n));
  if (sd < floor_sd) sd = floor_sd;
  for (long long i = threadIdx.x; i < n; i += blockDim.x)
    out[i] = __float2half_rn((img[(size_t)(r0 + i / w) * nx + r0 + i % w] - mean) / sd);
}

// V_s = sum_k (z_{k+1} - z_k) (p_k + p_{k+1}) / 2 over the d samples of slice s,
// then t = exp(-i sigma V_s) (the reference negates the integral, msa.py:406,
// and the GPU class takes exp(i sigma (-V)), msa.py:569-570).
__global__ void integrate_potential_kernel(const float* __restrict__ pot, const double* __restrict__ z, int d,
                                           int ny, int nx, int ld_y, int ld_x, float sigma, float2* __restrict__ trans) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, s = blockIdx.z;
  if (x >= nx) return;
  const size_t plane = (size_t)ld_y * ld_x;
  const float* p = pot + (size_t)s * d * plane + (size_t)y * ld_x + x;
  const double* zz = z + (size_t)s * d;
  double acc = 0;
  for (int k = 0; k + 1 < d; ++k) acc += (zz[k + 1] - zz[k]) * ((double)p[k * plane] + (double)p[(k + 1) * plane]) * 0.5;
  const float v = (float)(-acc);
  const float arg = sigma * v;
  trans[((size_t)s * ny + y) * nx + x] = make_float2(cosf(arg), sinf(arg));
}

// One CTA per (pattern p, detector d): out[p][d] = sum_k cbed[p][k] w_d[k] in double,
// strided partial sums then the block sum (a fixed order); w == null sums the pattern.
__global__ void integrate_cbed_kernel(const float* __restrict__ cbed, long long n, const float* __restrict__ w,
                                      int ndet, double* __restrict__ out) {
  __shared__ double sh[32];
  const long long p = blockIdx.x / ndet;
  const int d = (int)(blockIdx.x % ndet);
  const float* c = cbed + p * n;
  const float* wd = w ? w + (long long)d * n : nullptr;
  double acc = 0;
  for (long long k = threadIdx.x; k < n; k += blockDim.x) acc += wd ? (double)c[k] * (double)wd[k] : (double)c[k];
  const double s = block_sum(acc, sh);
  if (threadIdx.x == 0) out[blockIdx.x] = s;
}

}  // namespace msx

using namespace msx;

extern "C" {

int msx_integrate_cbed(const float* cbed_dev, int num_patterns, int height, int width, const float* weights_dev,
                       int num_detectors, double* out_dev, void* stream) {
  if (num_patterns < 0 || height <= 0 || width <= 0 || num_detectors < 1 || num_detectors > 65535) {
    set_last_error("integrate_cbed: bad sizes");
    return MSX_ERR_INVALID;
  }
  if (num_patterns == 0) return MSX_OK;
  if (!cbed_dev || !out_dev || (!weights_dev && num_detectors != 1)) {
    set_last_error("integrate_cbed: null pointer (weights may be null only for one plain sum)");
    return MSX_ERR_INVALID;
  }
  integrate_cbed_kernel<<<(unsigned)((long long)num_patterns * num_detectors), 256, 0, (cudaStream_t)stream>>>(
      cbed_dev, (long long)height * width, weights_dev, num_detectors, out_dev);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_last_error(cudaGetErrorString(e));
    return MSX_ERR_CUDA;
  }
  return MSX_OK;
}

int msx_process_cbed(const float* cbed_dev, int num_patterns, int height, int width, void* out_fp16_dev, void* stream) {
  if (num_patterns < 0 || height <= 0 || width <= 0) {
    set_last_error("process_cbed: bad sizes");
    return MSX_ERR_INVALID;
  }
  if (num_patterns == 0) return MSX_OK;
  if (!cbed_dev || !out_fp16_dev) {
    set_last_error("process_cbed: null pointer");
    return MSX_ERR_INVALID;
  }
  process_cbed_kernel<<<num_patterns, 256, 0, (cudaStream_t)stream>>>(cbed_dev, (long long)height * width,
                                                                     static_cast<__half*>(out_fp16_dev));
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_last_error(cudaGetErrorString(e));
    return MSX_ERR_CUDA;
  }
  return MSX_OK;
}

int msx_process_potential(const float* trans_dev, int num_slices, int ny, int nx, float* work_dev,
                          void* out_fp16_dev, void* stream) {
  if (num_slices <= 0 || ny < 4 || nx < 4 || !trans_dev || !work_dev || !out_fp16_dev) {
    set_last_error("process_potential: bad arguments");
    return MSX_ERR_INVALID;
  }
  const int r0 = ny / 4, r1 = 3 * nx / 4;
  if (r1 <= r0 || r1 > ny || r1 > nx) {
    set_last_error("process_potential: the crop [ny/4, 3nx/4) must lie inside the grid");
    return MSX_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const long long n = (long long)ny * nx;
  float* proj = work_dev;
  float* tmp = work_dev + n;
  double* w = reinterpret_cast<double*>(work_dev + 2 * n);  // 11 weights (needs 2*ny*nx + 22 floats)
  double hw[11], sum = 0;
  for (int k = -5; k <= 5; ++k) { hw[k + 5] = exp(-0.5 * (double)(k * k) / (1.2 * 1.2)); sum += hw[k + 5]; }
  for (double& v : hw) v /= sum;
  cudaError_t e = cudaMemcpyAsync(w, hw, sizeof(hw), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    proj_imag_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(reinterpret_cast<const float2*>(trans_dev), num_slices, n, proj);
    dim3 g((nx + 127) / 128, ny);
    gauss_axis_kernel<<<g, 128, 0, st>>>(proj, ny, nx, 0, w, tmp);
    gauss_axis_kernel<<<g, 128, 0, st>>>(tmp, ny, nx, 1, w, proj);
    crop_zscore_kernel<<<1, 1024, 0, st>>>(proj, ny, nx, r0, r1, static_cast<__half*>(out_fp16_dev));
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    set_last_error(cudaGetErrorString(e));
    return MSX_ERR_CUDA;
  }
  return MSX_OK;
}

int msx_integrate_potential(const float* pot_dev, const double* z_dev, int nz, int ld_y, int ld_x, int ny, int nx,
                            int num_slices, float sigma, float* trans_out_dev, void* stream) {
  if (num_slices <= 0 || nz < num_slices || ny <= 0 || nx <= 0 || ny > ld_y || nx > ld_x || !pot_dev || !z_dev ||
      !trans_out_dev) {
    set_last_error("integrate_potential: bad arguments");
    return MSX_ERR_INVALID;
  }
  const int d = nz / num_slices;  // samples per slice; trailing samples are dropped (msa.py:393-400)
  dim3 g((nx + 127) / 128, ny, num_slices);
  integrate_potential_kernel<<<g, 128, 0, (cudaStream_t)stream>>>(pot_dev, z_dev, d, ny, nx, ld_y, ld_x, sigma,
                                                                  reinterpret_cast<float2*>(trans_out_dev));
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_last_error(cudaGetErrorString(e));
    return MSX_ERR_CUDA;
  }
  return MSX_OK;
}

}  // extern "C"
