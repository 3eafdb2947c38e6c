// Learned coarse-slice corrector: a spectral-convolution network that maps the
// wave after one 4x-thick slice (and that slice's transmission) to the wave
// four fine slices would give.  Forward, backward and the Adam update are
// hand-written kernels; the host drives them from msx_corrector_* below.
//
// Network (C channels, L layers, K x K retained Fourier modes):
//   x0 = [Re psi_c, Im psi_c, Re t_c, Im t_c]                       (4 channels)
//   a0 = W0 x0 + b0
//   a_l = gelu( Spec_l(a_{l-1}) + W_l a_{l-1} + b_l ),  l = 1..L
//       Spec(u)[o] = Re( IDFT_K( sum_i R[k][o][i] DFT_K(u)[i][k] ) ) / (H W)
//       DFT_K keeps the K x K lowest modes (frequencies -K/2 .. K/2-1 per axis)
//   h  = gelu(P1 a_L + c1);  o = P2 h + c2                          (2 channels)
//   psi_pred = psi_c + (o_0 + i o_1)
// Waves are scaled by sqrt(H W) by the caller so that they are O(1).
// Loss: sum_b w_b sum |psi_pred - psi_f|^2 / denom (w_b = 1 without sample
// weights).  gelu is the tanh form.
// All arithmetic is FP32; reductions over pixels are two-stage and ordered.
#include "msx.h"
#include "msx_internal.h"

#include <cmath>
#include <cstring>
#include <vector>

namespace msx {
namespace nn {

constexpr int kMaxC = 32;
constexpr int kK = 8;  // retained modes per axis

__device__ __forceinline__ float gelu_f(float z) {
  const float k = 0.7978845608028654f;  // sqrt(2/pi)
  const float u = k * (z + 0.044715f * z * z * z);
  return 0.5f * z * (1.f + tanhf(u));
}
__device__ __forceinline__ float gelu_d(float z) {
  const float k = 0.7978845608028654f;
  const float u = k * (z + 0.044715f * z * z * z);
  const float th = tanhf(u);
  return 0.5f * (1.f + th) + 0.5f * z * (1.f - th * th) * k * (1.f + 3.f * 0.044715f * z * z);
}

// mode index m (0..K-1) -> frequency -K/2..K/2-1 mapped into [0, N)
__host__ __device__ __forceinline__ int mode_freq(int m, int n) { return m < kK / 2 ? m : n - (kK - m); }

// x0 from the interleaved complex inputs: x0[b][0..3][p]
__global__ void inputs_kernel(const float2* __restrict__ psi_c, const float2* __restrict__ tc, int HW, int B,
                              float* __restrict__ x0) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)B * HW) return;
  const int b = (int)(i / HW), p = (int)(i % HW);
  const float2 w = psi_c[i], t = tc[i];
  float* o = x0 + (size_t)b * 4 * HW + p;
  o[0] = w.x;
  o[HW] = w.y;
  o[2 * HW] = t.x;
  o[3 * HW] = t.y;
}

// z[b][o][p] = sum_i Wm[o][i] in[b][i][p] + bias[o] (+ add[b][o][p]); optional a = gelu(z)
__global__ void linear_fwd_kernel(const float* __restrict__ in, int Cin, const float* __restrict__ Wm,
                                  const float* __restrict__ bias, int Cout, int HW, int B, const float* __restrict__ add,
                                  float* __restrict__ z, float* __restrict__ a) {
  __shared__ float sw[kMaxC * kMaxC + kMaxC];
  for (int k = threadIdx.x; k < Cout * Cin; k += blockDim.x) sw[k] = Wm[k];
  for (int k = threadIdx.x; k < Cout; k += blockDim.x) sw[kMaxC * kMaxC + k] = bias[k];
  __syncthreads();
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)B * HW) return;
  const int b = (int)(i / HW), p = (int)(i % HW);
  float x[kMaxC];
  const float* ip = in + (size_t)b * Cin * HW + p;
#pragma unroll
  for (int c = 0; c < kMaxC; ++c)
    if (c < Cin) x[c] = ip[(size_t)c * HW];
  for (int o = 0; o < Cout; ++o) {
    float s = sw[kMaxC * kMaxC + o];
#pragma unroll
    for (int c = 0; c < kMaxC; ++c)
      if (c < Cin) s = fmaf(sw[o * Cin + c], x[c], s);
    const size_t oi = ((size_t)b * Cout + o) * HW + p;
    if (add) s += add[oi];
    z[oi] = s;
    if (a) a[oi] = gelu_f(s);
  }
}

// din[b][i][p] (+)= sum_o Wm[o][i] dz[b][o][p]
__global__ void linear_bwd_data_kernel(const float* __restrict__ dz, int Cout, const float* __restrict__ Wm, int Cin,
                                       int HW, int B, int accumulate, float* __restrict__ din) {
  __shared__ float sw[kMaxC * kMaxC];
  for (int k = threadIdx.x; k < Cout * Cin; k += blockDim.x) sw[k] = Wm[k];
  __syncthreads();
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)B * HW) return;
  const int b = (int)(i / HW), p = (int)(i % HW);
  float g[kMaxC];
#pragma unroll
  for (int o = 0; o < kMaxC; ++o)
    if (o < Cout) g[o] = dz[((size_t)b * Cout + o) * HW + p];
  for (int c = 0; c < Cin; ++c) {
    float s = 0.f;
#pragma unroll
    for (int o = 0; o < kMaxC; ++o)
      if (o < Cout) s = fmaf(sw[o * Cin + c], g[o], s);
    const size_t oi = ((size_t)b * Cin + c) * HW + p;
    din[oi] = accumulate ? din[oi] + s : s;
  }
}

// Partial weight/bias gradients of one chunk of (b, p): part[chunk][o*Cin+i], part[chunk][Cout*Cin+o].
// 256 threads; thread t owns the (o, i) pairs t, t+256, ...
__global__ void linear_bwd_weight_kernel(const float* __restrict__ dz, int Cout, const float* __restrict__ in, int Cin,
                                         int HW, int B, int chunk, float* __restrict__ part) {
  __shared__ float sg[32][kMaxC];
  __shared__ float sx[32][kMaxC];
  const long long total = (long long)B * HW;
  const long long start = (long long)blockIdx.x * chunk;
  const long long end = start + chunk < total ? start + chunk : total;
  const int npair = Cout * Cin + Cout;
  float acc[(kMaxC * kMaxC + kMaxC + 255) / 256];
#pragma unroll
  for (int k = 0; k < (kMaxC * kMaxC + kMaxC + 255) / 256; ++k) acc[k] = 0.f;
  for (long long q0 = start; q0 < end; q0 += 32) {
    // stage 32 pixels of dz and in
    for (int e = threadIdx.x; e < 32 * kMaxC; e += blockDim.x) {
      const int j = e / kMaxC, c = e % kMaxC;
      const long long q = q0 + j;
      float gv = 0.f, xv = 0.f;
      if (q < end) {
        const int b = (int)(q / HW), p = (int)(q % HW);
        if (c < Cout) gv = dz[((size_t)b * Cout + c) * HW + p];
        if (c < Cin) xv = in[((size_t)b * Cin + c) * HW + p];
      }
      sg[j][c] = gv;
      sx[j][c] = xv;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < (kMaxC * kMaxC + kMaxC + 255) / 256; ++k) {
      const int pr = threadIdx.x + 256 * k;
      if (pr < npair) {
        float s = acc[k];
        if (pr < Cout * Cin) {
          const int o = pr / Cin, c = pr % Cin;
          for (int j = 0; j < 32; ++j) s = fmaf(sg[j][o], sx[j][c], s);
        } else {
          const int o = pr - Cout * Cin;
          for (int j = 0; j < 32; ++j) s += sg[j][o];
        }
        acc[k] = s;
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int k = 0; k < (kMaxC * kMaxC + kMaxC + 255) / 256; ++k) {
    const int pr = threadIdx.x + 256 * k;
    if (pr < npair) part[(size_t)blockIdx.x * npair + pr] = acc[k];
  }
}

// grad[j] (+)= sum over chunks of part[chunk][j], chunks in order
__global__ void reduce_parts_kernel(const float* __restrict__ part, int nchunks, int n, float* __restrict__ grad) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  float s = 0.f;
  for (int k = 0; k < nchunks; ++k) s += part[(size_t)k * n + j];
  grad[j] = s;
}

__global__ void gelu_bwd_kernel(const float* __restrict__ da, const float* __restrict__ z, long long n,
                                float* __restrict__ dz) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dz[i] = da[i] * gelu_d(z[i]);
}

// out[r][m] = scale * sum_x in[r][x] e^{-2 pi i f_m x / W}, rows r of real input.  One warp per row.
__global__ void dft_x_kernel(const float* __restrict__ in, long long rows, int W, float scale, float2* __restrict__ out) {
  const long long r = (long long)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= rows) return;
  const float* row = in + (size_t)r * W;
  float re[kK], im[kK];
#pragma unroll
  for (int m = 0; m < kK; ++m) re[m] = im[m] = 0.f;
  for (int x = lane; x < W; x += 32) {
    const float v = row[x];
#pragma unroll
    for (int m = 0; m < kK; ++m) {
      float s, c;
      sincospif(-2.f * (float)((long long)mode_freq(m, W) * x % W) / (float)W, &s, &c);
      re[m] = fmaf(v, c, re[m]);
      im[m] = fmaf(v, s, im[m]);
    }
  }
#pragma unroll
  for (int m = 0; m < kK; ++m) {
    for (int o = 16; o > 0; o >>= 1) {
      re[m] += __shfl_down_sync(0xffffffffu, re[m], o);
      im[m] += __shfl_down_sync(0xffffffffu, im[m], o);
    }
  }
  if (lane == 0)
#pragma unroll
    for (int m = 0; m < kK; ++m) out[(size_t)r * kK + m] = make_float2(re[m] * scale, im[m] * scale);
}

// out[q][a][m] = sum_y in[q][y][m] e^{sgn 2 pi i f_a y / H} for the planes q; one warp per (q, m).
__global__ void dft_y_kernel(const float2* __restrict__ in, long long planes, int H, float sgn, float2* __restrict__ out) {
  const long long w = (long long)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= planes * kK) return;
  const long long q = w / kK;
  const int m = (int)(w % kK);
  float re[kK], im[kK];
#pragma unroll
  for (int a = 0; a < kK; ++a) re[a] = im[a] = 0.f;
  for (int y = lane; y < H; y += 32) {
    const float2 v = in[((size_t)q * H + y) * kK + m];
#pragma unroll
    for (int a = 0; a < kK; ++a) {
      float s, c;
      sincospif(sgn * 2.f * (float)((long long)mode_freq(a, H) * y % H) / (float)H, &s, &c);
      re[a] += v.x * c - v.y * s;
      im[a] += v.x * s + v.y * c;
    }
  }
#pragma unroll
  for (int a = 0; a < kK; ++a) {
    for (int o = 16; o > 0; o >>= 1) {
      re[a] += __shfl_down_sync(0xffffffffu, re[a], o);
      im[a] += __shfl_down_sync(0xffffffffu, im[a], o);
    }
  }
  if (lane == 0)
#pragma unroll
    for (int a = 0; a < kK; ++a) out[((size_t)q * kK + a) * kK + m] = make_float2(re[a], im[a]);
}

// out[q][y][m] = sum_a in[q][a][m] e^{+2 pi i f_a y / H}; one thread per (q, y, m)
__global__ void idft_y_kernel(const float2* __restrict__ in, long long planes, int H, float2* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= planes * H * kK) return;
  const int m = (int)(i % kK);
  const int y = (int)((i / kK) % H);
  const long long q = i / ((long long)kK * H);
  float re = 0.f, im = 0.f;
#pragma unroll
  for (int a = 0; a < kK; ++a) {
    const float2 v = in[((size_t)q * kK + a) * kK + m];
    float s, c;
    sincospif(2.f * (float)((long long)mode_freq(a, H) * y % H) / (float)H, &s, &c);
    re += v.x * c - v.y * s;
    im += v.x * s + v.y * c;
  }
  out[i] = make_float2(re, im);
}

// v[r][x] (+)= scale * Re( sum_m in[r][m] e^{+2 pi i f_m x / W} ); one thread per (r, x)
__global__ void idft_x_real_kernel(const float2* __restrict__ in, long long rows, int W, float scale, int accumulate,
                                   float* __restrict__ v) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows * W) return;
  const int x = (int)(i % W);
  const long long r = i / W;
  float s = 0.f;
#pragma unroll
  for (int m = 0; m < kK; ++m) {
    const float2 c = in[(size_t)r * kK + m];
    float sn, cs;
    sincospif(2.f * (float)((long long)mode_freq(m, W) * x % W) / (float)W, &sn, &cs);
    s += c.x * cs - c.y * sn;
  }
  s *= scale;
  v[i] = accumulate ? v[i] + s : s;
}

// Y[b][o][a][m] = sum_i R[a][m][o][i] X[b][i][a][m]; R as (re, im) planes
__global__ void mix_fwd_kernel(const float* __restrict__ Rr, const float* __restrict__ Ri, const float2* __restrict__ X,
                               int C, int B, float2* __restrict__ Y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B * C * kK * kK) return;
  const int am = i % (kK * kK), o = (i / (kK * kK)) % C, b = i / (kK * kK * C);
  float re = 0.f, im = 0.f;
  for (int c = 0; c < C; ++c) {
    const size_t ri = ((size_t)am * C + o) * C + c;
    const float2 x = X[((size_t)b * C + c) * kK * kK + am];
    re += Rr[ri] * x.x - Ri[ri] * x.y;
    im += Rr[ri] * x.y + Ri[ri] * x.x;
  }
  Y[i] = make_float2(re, im);
}

// dR[a][m][o][i] = sum_b dY[b][o][a][m] conj(X[b][i][a][m])
__global__ void mix_bwd_weight_kernel(const float2* __restrict__ dY, const float2* __restrict__ X, int C, int B,
                                      float* __restrict__ dRr, float* __restrict__ dRi) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kK * kK * C * C) return;
  const int c = i % C, o = (i / C) % C, am = i / (C * C);
  float re = 0.f, im = 0.f;
  for (int b = 0; b < B; ++b) {
    const float2 g = dY[((size_t)b * C + o) * kK * kK + am];
    const float2 x = X[((size_t)b * C + c) * kK * kK + am];
    re += g.x * x.x + g.y * x.y;
    im += g.y * x.x - g.x * x.y;
  }
  dRr[i] = re;
  dRi[i] = im;
}

// dX[b][i][a][m] = sum_o conj(R[a][m][o][i]) dY[b][o][a][m]
__global__ void mix_bwd_data_kernel(const float* __restrict__ Rr, const float* __restrict__ Ri, const float2* __restrict__ dY,
                                    int C, int B, float2* __restrict__ dX) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B * C * kK * kK) return;
  const int am = i % (kK * kK), c = (i / (kK * kK)) % C, b = i / (kK * kK * C);
  float re = 0.f, im = 0.f;
  for (int o = 0; o < C; ++o) {
    const size_t ri = ((size_t)am * C + o) * C + c;
    const float2 g = dY[((size_t)b * C + o) * kK * kK + am];
    re += Rr[ri] * g.x + Ri[ri] * g.y;
    im += Rr[ri] * g.y - Ri[ri] * g.x;
  }
  dX[i] = make_float2(re, im);
}

// psi_pred = psi_c + (o0 + i o1); with a target: dO = 2 (psi_pred - psi_f) / denom and per-block sums of |r|^2
__global__ void output_kernel(const float* __restrict__ o, const float2* __restrict__ psi_c, const float2* __restrict__ psi_f,
                              int HW, int B, float inv_denom, const float* __restrict__ sample_w, float2* __restrict__ pred,
                              float* __restrict__ dO, double* __restrict__ block_sums) {
  __shared__ double red[256];
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double sq = 0;
  if (i < (long long)B * HW) {
    const int b = (int)(i / HW), p = (int)(i % HW);
    const float o0 = o[((size_t)b * 2) * HW + p], o1 = o[((size_t)b * 2 + 1) * HW + p];
    const float2 c = psi_c[i];
    const float2 w = make_float2(c.x + o0, c.y + o1);
    if (pred) pred[i] = w;
    if (psi_f) {
      const float2 f = psi_f[i];
      const float rx = w.x - f.x, ry = w.y - f.y;
      const float wt = sample_w ? sample_w[b] * inv_denom : inv_denom;
      sq = ((double)rx * rx + (double)ry * ry) * (double)wt;
      dO[((size_t)b * 2) * HW + p] = 2.f * rx * wt;
      dO[((size_t)b * 2 + 1) * HW + p] = 2.f * ry * wt;
    }
  }
  if (!block_sums) return;
  red[threadIdx.x] = sq;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) block_sums[blockIdx.x] = red[0];
}

__global__ void sum_blocks_kernel(const double* __restrict__ s, int n, double scale, float* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double acc = 0;
  for (int i = 0; i < n; ++i) acc += s[i];
  out[0] = (float)(acc * scale);
}

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                            long long n, float lr, float b1, float b2, float eps, float c1, float c2) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

}  // namespace nn
}  // namespace msx

using namespace msx;
using namespace msx::nn;

// ------------------------------------------------------------------ host object
struct msx_corrector {
  int H = 0, W = 0, C = 0, L = 0, maxB = 0;
  size_t nparams = 0;
  // parameter offsets (floats)
  size_t oW0, ob0, oP1, oc1, oP2, oc2;
  std::vector<size_t> oRr, oRi, oWl, obl;
  float *params = nullptr, *grads = nullptr, *m = nullptr, *v = nullptr;
  // activations
  float *x0 = nullptr, *a = nullptr, *z = nullptr, *h = nullptr, *zh = nullptr, *o = nullptr;
  float *da = nullptr, *dz = nullptr, *dh = nullptr, *dO = nullptr;
  float2 *X1 = nullptr, *X2 = nullptr, *Y = nullptr, *Z1 = nullptr;  // spectral scratch
  float2 *dX2 = nullptr;
  float* part = nullptr;
  size_t part_words = 0;
  double* sums = nullptr;
  float* loss = nullptr;
  int step = 0;
};

namespace {

int cfail(int code, const char* msg) {
  set_last_error(msg);
  return code;
}

#define NN_CUDA(call)                                               \
  do {                                                              \
    cudaError_t e_ = (call);                                        \
    if (e_ != cudaSuccess) return cfail(MSX_ERR_CUDA, cudaGetErrorString(e_)); \
  } while (0)

inline unsigned blocks_for(long long n, int t) { return (unsigned)((n + t - 1) / t); }

size_t act(const msx_corrector* k, int B) { return (size_t)B * k->C * k->H * k->W; }

// forward; keeps what the backward needs.  x0 from psi_c / tc.
int forward(msx_corrector* k, const float2* psi_c, const float2* tc, int B, cudaStream_t st) {
  const int HW = k->H * k->W, C = k->C;
  const long long nb = (long long)B * HW;
  float* P = k->params;
  inputs_kernel<<<blocks_for(nb, 256), 256, 0, st>>>(psi_c, tc, HW, B, k->x0);
  // a_0 = W0 x0 + b0 (stored at layer slot 0)
  linear_fwd_kernel<<<blocks_for(nb, 128), 128, 0, st>>>(k->x0, 4, P + k->oW0, P + k->ob0, C, HW, B, nullptr,
                                                         k->a, nullptr);
  for (int l = 0; l < k->L; ++l) {
    float* ain = k->a + (size_t)l * act(k, B);
    float* aout = k->a + (size_t)(l + 1) * act(k, B);
    float* zl = k->z + (size_t)l * act(k, B);
    float2* X2l = k->X2 + (size_t)l * B * C * kK * kK;
    const long long rows = (long long)B * C * k->H;
    dft_x_kernel<<<blocks_for(rows * 32, 256), 256, 0, st>>>(ain, rows, k->W, 1.f, k->X1);
    dft_y_kernel<<<blocks_for((long long)B * C * kK * 32, 256), 256, 0, st>>>(k->X1, (long long)B * C, k->H, -1.f, X2l);
    mix_fwd_kernel<<<blocks_for((long long)B * C * kK * kK, 256), 256, 0, st>>>(P + k->oRr[l], P + k->oRi[l], X2l, C, B, k->Y);
    idft_y_kernel<<<blocks_for((long long)B * C * k->H * kK, 256), 256, 0, st>>>(k->Y, (long long)B * C, k->H, k->Z1);
    idft_x_real_kernel<<<blocks_for(rows * k->W, 256), 256, 0, st>>>(k->Z1, rows, k->W, 1.f / (float)HW, 0, zl);
    linear_fwd_kernel<<<blocks_for(nb, 128), 128, 0, st>>>(ain, C, P + k->oWl[l], P + k->obl[l], C, HW, B, zl, zl, aout);
  }
  linear_fwd_kernel<<<blocks_for(nb, 128), 128, 0, st>>>(k->a + (size_t)k->L * act(k, B), C, P + k->oP1, P + k->oc1, C,
                                                         HW, B, nullptr, k->zh, k->h);
  linear_fwd_kernel<<<blocks_for(nb, 128), 128, 0, st>>>(k->h, C, P + k->oP2, P + k->oc2, 2, HW, B, nullptr, k->o,
                                                         nullptr);
  NN_CUDA(cudaGetLastError());
  return MSX_OK;
}

int weight_grad(msx_corrector* k, const float* dzp, int Cout, const float* in, int Cin, int B, float* gW, float* gb,
                cudaStream_t st) {
  const long long total = (long long)B * k->H * k->W;
  const int chunk = 8192;
  const int nchunks = (int)((total + chunk - 1) / chunk);
  const int npair = Cout * Cin + Cout;
  if ((size_t)nchunks * npair > k->part_words) return cfail(MSX_ERR_INVALID, "corrector partial buffer too small");
  linear_bwd_weight_kernel<<<nchunks, 256, 0, st>>>(dzp, Cout, in, Cin, k->H * k->W, B, chunk, k->part);
  // gW and gb are contiguous in the parameter layout (W then bias)
  (void)gb;
  reduce_parts_kernel<<<blocks_for(npair, 256), 256, 0, st>>>(k->part, nchunks, npair, gW);
  NN_CUDA(cudaGetLastError());
  return MSX_OK;
}

int backward(msx_corrector* k, int B, cudaStream_t st) {
  const int HW = k->H * k->W, C = k->C;
  const long long nb = (long long)B * HW;
  float* P = k->params;
  float* G = k->grads;
  const size_t A = act(k, B);
  // output layer: o = P2 h + c2
  int rc = weight_grad(k, k->dO, 2, k->h, C, B, G + k->oP2, G + k->oc2, st);
  if (rc) return rc;
  linear_bwd_data_kernel<<<blocks_for(nb, 128), 128, 0, st>>>(k->dO, 2, P + k->oP2, C, HW, B, 0, k->dh);
  gelu_bwd_kernel<<<blocks_for((long long)A, 256), 256, 0, st>>>(k->dh, k->zh, (long long)A, k->dz);
  rc = weight_grad(k, k->dz, C, k->a + (size_t)k->L * A, C, B, G + k->oP1, G + k->oc1, st);
  if (rc) return rc;
  float* da = k->da;  // gradient w.r.t. a_L
  linear_bwd_data_kernel<<<blocks_for(nb, 128), 128, 0, st>>>(k->dz, C, P + k->oP1, C, HW, B, 0, da);
  for (int l = k->L - 1; l >= 0; --l) {
    float* ain = k->a + (size_t)l * A;
    float* zl = k->z + (size_t)l * A;
    float2* X2l = k->X2 + (size_t)l * B * C * kK * kK;
    gelu_bwd_kernel<<<blocks_for((long long)A, 256), 256, 0, st>>>(da, zl, (long long)A, k->dz);
    rc = weight_grad(k, k->dz, C, ain, C, B, G + k->oWl[l], G + k->obl[l], st);
    if (rc) return rc;
    // da_{l} = W_l^T dz + spectral adjoint (written into da, which held da_{l+1})
    linear_bwd_data_kernel<<<blocks_for(nb, 128), 128, 0, st>>>(k->dz, C, P + k->oWl[l], C, HW, B, 0, da);
    const long long rows = (long long)B * C * k->H;
    dft_x_kernel<<<blocks_for(rows * 32, 256), 256, 0, st>>>(k->dz, rows, k->W, 1.f / (float)HW, k->X1);
    dft_y_kernel<<<blocks_for((long long)B * C * kK * 32, 256), 256, 0, st>>>(k->X1, (long long)B * C, k->H, -1.f, k->Y);
    mix_bwd_weight_kernel<<<blocks_for((long long)kK * kK * C * C, 256), 256, 0, st>>>(k->Y, X2l, C, B, G + k->oRr[l],
                                                                                      G + k->oRi[l]);
    mix_bwd_data_kernel<<<blocks_for((long long)B * C * kK * kK, 256), 256, 0, st>>>(P + k->oRr[l], P + k->oRi[l], k->Y,
                                                                                    C, B, k->dX2);
    idft_y_kernel<<<blocks_for((long long)B * C * k->H * kK, 256), 256, 0, st>>>(k->dX2, (long long)B * C, k->H, k->Z1);
    idft_x_real_kernel<<<blocks_for(rows * k->W, 256), 256, 0, st>>>(k->Z1, rows, k->W, 1.f, 1, da);
  }
  // lift: a0 = W0 x0 + b0
  rc = weight_grad(k, da, C, k->x0, 4, B, G + k->oW0, G + k->ob0, st);
  if (rc) return rc;
  NN_CUDA(cudaGetLastError());
  return MSX_OK;
}

}  // namespace

extern "C" {

int msx_corrector_create(int ny, int nx, int channels, int layers, int max_batch, msx_corrector** out) {
  if (!out) return cfail(MSX_ERR_INVALID, "null corrector pointer");
  *out = nullptr;
  if (ny < kK || nx < kK || channels < 1 || channels > kMaxC || layers < 1 || layers > 16 || max_batch < 1)
    return cfail(MSX_ERR_INVALID, "corrector: grid >= 8, 1..32 channels, 1..16 layers, batch >= 1");
  msx_corrector* k = new msx_corrector();
  k->H = ny; k->W = nx; k->C = channels; k->L = layers; k->maxB = max_batch;
  const int C = channels;
  size_t off = 0;
  // each weight matrix is immediately followed by its bias (the gradient reduction writes both)
  k->oW0 = off; off += (size_t)C * 4; k->ob0 = off; off += C;
  for (int l = 0; l < layers; ++l) {
    k->oRr.push_back(off); off += (size_t)kK * kK * C * C;
    k->oRi.push_back(off); off += (size_t)kK * kK * C * C;
    k->oWl.push_back(off); off += (size_t)C * C;
    k->obl.push_back(off); off += C;
  }
  k->oP1 = off; off += (size_t)C * C; k->oc1 = off; off += C;
  k->oP2 = off; off += (size_t)2 * C; k->oc2 = off; off += 2;
  k->nparams = off;
  const size_t HW = (size_t)ny * nx, B = max_batch;
  const size_t A = B * C * HW;
  const size_t chunks = (B * HW + 8191) / 8192;
  k->part_words = chunks * (size_t)(kMaxC * kMaxC + kMaxC);
  cudaError_t e = cudaSuccess;
  auto alloc = [&](void** p, size_t bytes) { if (e == cudaSuccess) e = cudaMalloc(p, bytes); };
  alloc((void**)&k->params, 4 * off * sizeof(float));
  if (e == cudaSuccess) { k->grads = k->params + off; k->m = k->grads + off; k->v = k->m + off; }
  alloc((void**)&k->x0, B * 4 * HW * sizeof(float));
  alloc((void**)&k->a, (layers + 1) * A * sizeof(float));
  alloc((void**)&k->z, layers * A * sizeof(float));
  alloc((void**)&k->h, A * sizeof(float));
  alloc((void**)&k->zh, A * sizeof(float));
  alloc((void**)&k->o, B * 2 * HW * sizeof(float));
  alloc((void**)&k->da, A * sizeof(float));
  alloc((void**)&k->dz, A * sizeof(float));
  alloc((void**)&k->dh, A * sizeof(float));
  alloc((void**)&k->dO, B * 2 * HW * sizeof(float));
  alloc((void**)&k->X1, B * C * ny * kK * sizeof(float2));
  alloc((void**)&k->Z1, B * C * ny * kK * sizeof(float2));
  alloc((void**)&k->X2, layers * B * C * kK * kK * sizeof(float2));
  alloc((void**)&k->Y, B * C * kK * kK * sizeof(float2));
  alloc((void**)&k->dX2, B * C * kK * kK * sizeof(float2));
  alloc((void**)&k->part, k->part_words * sizeof(float));
  alloc((void**)&k->sums, ((B * HW + 255) / 256) * sizeof(double));
  alloc((void**)&k->loss, sizeof(float));
  if (e == cudaSuccess) e = cudaMemset(k->params, 0, 4 * off * sizeof(float));
  if (e != cudaSuccess) {
    msx_corrector_destroy(k);
    return cfail(MSX_ERR_ALLOC, "corrector allocation failed");
  }
  *out = k;
  return MSX_OK;
}

int msx_corrector_destroy(msx_corrector* k) {
  if (!k) return MSX_OK;
  for (void* p : {(void*)k->params, (void*)k->x0, (void*)k->a, (void*)k->z, (void*)k->h, (void*)k->zh, (void*)k->o,
                  (void*)k->da, (void*)k->dz, (void*)k->dh, (void*)k->dO, (void*)k->X1, (void*)k->Z1, (void*)k->X2,
                  (void*)k->Y, (void*)k->dX2, (void*)k->part, (void*)k->sums, (void*)k->loss})
    if (p) cudaFree(p);
  delete k;
  return MSX_OK;
}

int msx_corrector_params(msx_corrector* k, float** params_dev, float** grads_dev, size_t* count) {
  if (!k) return cfail(MSX_ERR_INVALID, "null corrector");
  if (params_dev) *params_dev = k->params;
  if (grads_dev) *grads_dev = k->grads;
  if (count) *count = k->nparams;
  return MSX_OK;
}

int msx_corrector_forward(msx_corrector* k, const float* psi_c_dev, const float* tc_dev, int batch, float* pred_out_dev,
                          void* stream) {
  if (!k || !psi_c_dev || !tc_dev || !pred_out_dev || batch < 1 || batch > k->maxB)
    return cfail(MSX_ERR_INVALID, "corrector forward: bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  int rc = forward(k, reinterpret_cast<const float2*>(psi_c_dev), reinterpret_cast<const float2*>(tc_dev), batch, st);
  if (rc) return rc;
  const long long nb = (long long)batch * k->H * k->W;
  output_kernel<<<blocks_for(nb, 256), 256, 0, st>>>(k->o, reinterpret_cast<const float2*>(psi_c_dev), nullptr, k->H * k->W,
                                                     batch, 0.f, nullptr, reinterpret_cast<float2*>(pred_out_dev), nullptr,
                                                     nullptr);
  NN_CUDA(cudaGetLastError());
  return MSX_OK;
}

int msx_corrector_loss_grad(msx_corrector* k, const float* psi_c_dev, const float* tc_dev, const float* psi_f_dev,
                            int batch, double denom, const float* sample_weights_dev, float* loss_out_dev, void* stream) {
  if (!k || !psi_c_dev || !tc_dev || !psi_f_dev || batch < 1 || batch > k->maxB || !(denom > 0))
    return cfail(MSX_ERR_INVALID, "corrector loss: bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  int rc = forward(k, reinterpret_cast<const float2*>(psi_c_dev), reinterpret_cast<const float2*>(tc_dev), batch, st);
  if (rc) return rc;
  const long long nb = (long long)batch * k->H * k->W;
  const unsigned nblk = blocks_for(nb, 256);
  output_kernel<<<nblk, 256, 0, st>>>(k->o, reinterpret_cast<const float2*>(psi_c_dev),
                                       reinterpret_cast<const float2*>(psi_f_dev), k->H * k->W, batch,
                                       (float)(1.0 / denom), sample_weights_dev, nullptr, k->dO, k->sums);
  sum_blocks_kernel<<<1, 32, 0, st>>>(k->sums, (int)nblk, 1.0, loss_out_dev ? loss_out_dev : k->loss);
  rc = backward(k, batch, st);
  return rc;
}

int msx_corrector_adam(msx_corrector* k, float lr, float beta1, float beta2, float eps, void* stream) {
  if (!k) return cfail(MSX_ERR_INVALID, "null corrector");
  k->step += 1;
  const float c1 = 1.f - powf(beta1, (float)k->step), c2 = 1.f - powf(beta2, (float)k->step);
  adam_kernel<<<blocks_for((long long)k->nparams, 256), 256, 0, (cudaStream_t)stream>>>(
      k->params, k->grads, k->m, k->v, (long long)k->nparams, lr, beta1, beta2, eps, c1, c2);
  NN_CUDA(cudaGetLastError());
  return MSX_OK;
}

}  // extern "C"
