// Learned coarse-slice corrector: a spectral-convolution network that turns
// the potentials of the fine slices inside one thick (coarse) slice into two
// per-pixel complex correction maps A, B of the coarse multislice step
//
//   psi <- (1 + A) . IFFT[ P_c . FFT[ (1 + B) . t_c . psi ] ]
//
// so that one corrected coarse step follows `ratio` fine steps more closely
// than the plain coarse step does.  The maps depend on the crystal only, so
// the network runs once per coarse slice; the corrected multislice of every
// probe then costs what a plain coarse-slice multislice costs (the maps fold
// into the transmission slices).
//
// Network (C channels, L spectral layers, MX x MY retained modes), all
// activations pixel-major (S, H, W, channels) float32:
//   a_0 = x W0^T + b0                                   (lift of Cin input channels)
//   a_l = gelu( Spec_l(a_{l-1}) + a_{l-1} W_l^T + b_l ), l = 1..L
//         Spec(u) = IDFT( R[mode] . DFT(u) ) on the modes kx in [0, MX),
//         ky in [-MY/2, MY/2) (real fields: kx >= 1 counted twice)
//   h   = gelu(a_L P1^T + c1);  o = h P2^T + c2            (4 outputs: Re A, Im A, Re B, Im B)
// Every contraction -- the lift, the pointwise layers, the head, their weight
// gradients, the four partial-DFT stages of each spectral layer and the per-mode
// channel mixing (four batched real GEMMs per complex C x C product, one batch
// per mode) -- is a bfloat16 GEMM with FP32 accumulation on the tensor cores
// (TcGemm, msx_tcgemm.cu); the activations, reductions and Adam are FP32
// kernels here.  gelu is the tanh form.
#include "msx.h"
#include "msx_internal.h"

#include <cmath>
#include <cstring>
#include <vector>

namespace msx {
namespace nn {

__device__ __forceinline__ float gelu_d(float z) {
  const float k = 0.7978845608028654f;
  const float u = k * (z + 0.044715f * z * z * z);
  const float th = tanhf(u);
  return 0.5f * (1.f + th) + 0.5f * z * (1.f - th * th) * k * (1.f + 3.f * 0.044715f * z * z);
}

__global__ void gelu_bwd_kernel(const float* __restrict__ da, const float* __restrict__ z, long long n,
                                float* __restrict__ dz) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dz[i] = da[i] * gelu_d(z[i]);
}

// Column sums of a (rows x n) row-major matrix, first stage: part[chunk][c] over
// the chunk's rows.  n divides 256; thread t sums column t % n over rows t / n,
// t / n + 256 / n, ...; the 256 / n partial sums of a column are then added in order.
__global__ void colsum_part_kernel(const float* __restrict__ x, long long rows, int n, long long chunk,
                                   float* __restrict__ part) {
  __shared__ float red[256];
  const int t = threadIdx.x, c = t % n, step = 256 / n;
  const long long r0 = (long long)blockIdx.x * chunk;
  const long long r1 = r0 + chunk < rows ? r0 + chunk : rows;
  float s = 0.f;
  for (long long r = r0 + t / n; r < r1; r += step) s += x[r * n + c];
  red[t] = s;
  __syncthreads();
  if (t < n) {
    float a = 0.f;
    for (int j = 0; j < step; ++j) a += red[j * n + t];
    part[(size_t)blockIdx.x * n + t] = a;
  }
}

// out[j] = sum over chunks k (in order) of part[k][j]
__global__ void reduce_parts_kernel(const float* __restrict__ part, int nchunks, int n, float* __restrict__ out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  float s = 0.f;
  for (int k = 0; k < nchunks; ++k) s += part[(size_t)k * n + j];
  out[j] = s;
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

// Network inputs of S coarse slices: out[s][p][c] for c < ratio: sigma * V of fine slice
// ratio * s + c; c = ratio: their sum; c = ratio + 1: the constant `tval`.
__global__ void features_kernel(const float* __restrict__ pot, int S, int ratio, long long P, float sigma, float tval,
                                float* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)S * P) return;
  const long long s = i / P, p = i % P;
  const int cin = ratio + 2;
  float* o = out + i * cin;
  float sum = 0.f;
  for (int j = 0; j < ratio; ++j) {
    const float ph = sigma * pot[((size_t)s * ratio + j) * P + p];
    o[j] = ph;
    sum += ph;
  }
  o[ratio] = sum;
  o[ratio + 1] = tval;
}

// Correction maps: maps (S, P, 4) = (Re A, Im A, Re B, Im B); `which` 0 = A, 1 = B.
// form 0: the factor is 1 + M; form 1: the unit-modulus factor exp(i Im M) (Re M unused),
// which keeps the corrected step as norm-preserving as the exact one.
__device__ __forceinline__ float2 one_plus(const float* maps, long long sp, int which, int form) {
  const float* m = maps + sp * 4 + 2 * which;
  if (form) {
    float sn, cs;
    sincosf(m[1], &sn, &cs);
    return make_float2(cs, sn);
  }
  return make_float2(1.f + m[0], m[1]);
}

// w[b][p] *= (1 + M_s[p]) (or its conjugate) for nb waves that all use sample s
__global__ void map_mul_kernel(float2* __restrict__ w, int nb, long long P, const float* __restrict__ maps, int which,
                               int conj, int form) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)nb * P) return;
  float2 f = one_plus(maps, i % P, which, form);
  if (conj) f.y = -f.y;
  w[i] = cmul(w[i], f);
}

// w[b][p] *= plane[p] (or its conjugate)
__global__ void plane_mul_kernel(float2* __restrict__ w, long long n, long long P, const float2* __restrict__ plane,
                                 int conj) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float2 f = plane[i % P];
  if (conj) f.y = -f.y;
  w[i] = cmul(w[i], f);
}

// out[p] = t[p] (1 + M[p]) for one plane
__global__ void map_trans_kernel(const float2* __restrict__ t, long long P, const float* __restrict__ maps, int which,
                                 int form, float2* __restrict__ out) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  out[p] = cmul(t[p], one_plus(maps, p, which, form));
}

// G = sum_b conj(u[b][p]) g[b][p] (b in order) is d loss / d conj(factor) for a factor
// that multiplied u.  form 0: dmaps[p][2 which], [2 which + 1] (+)= 2 Re G, 2 Im G;
// form 1 (factor exp(i theta), theta = Im M): d/d theta = 2 Re(conj(G) i factor)
// = 2 (Im G cos theta - Re G sin theta), and 0 for Re M.
__global__ void map_grad_kernel(const float2* __restrict__ u, const float2* __restrict__ g, int nb, long long P,
                                int which, int accumulate, int form, const float* __restrict__ maps,
                                float* __restrict__ dmaps) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  float re = 0.f, im = 0.f;
  for (int b = 0; b < nb; ++b) {
    const float2 a = u[(size_t)b * P + p], c = g[(size_t)b * P + p];
    re = fmaf(a.x, c.x, fmaf(a.y, c.y, re));
    im = fmaf(a.x, c.y, fmaf(-a.y, c.x, im));
  }
  if (form) {
    const float2 f = one_plus(maps, p, which, 1);
    const float dth = im * f.x - re * f.y;
    re = 0.f;
    im = dth;
  }
  float* d = dmaps + p * 4 + 2 * which;
  if (accumulate) {
    d[0] += 2.f * re;
    d[1] += 2.f * im;
  } else {
    d[0] = 2.f * re;
    d[1] = 2.f * im;
  }
}

// g[i] (+)= wt (psi[i] - f[i]); per-block sums of wt |psi - f|^2 (double)
__global__ void resid_kernel(const float2* __restrict__ psi, const float2* __restrict__ f, long long n, float wt,
                             int accumulate, float2* __restrict__ g, double* __restrict__ sums) {
  __shared__ double red[256];
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double sq = 0;
  if (i < n) {
    const float2 a = psi[i], b = f[i];
    const float rx = a.x - b.x, ry = a.y - b.y;
    sq = ((double)rx * rx + (double)ry * ry) * wt;
    const float2 v = make_float2(wt * rx, wt * ry);
    g[i] = accumulate ? make_float2(g[i].x + v.x, g[i].y + v.y) : v;
  }
  red[threadIdx.x] = sq;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) sums[blockIdx.x] = red[0];
}

// out[0] = sum of s[0..n): one block of 256 threads, strided partial sums then a
// fixed-order tree, so the result does not depend on timing.
__global__ void sum_blocks_kernel(const double* __restrict__ s, int n, float* __restrict__ out) {
  __shared__ double red[256];
  double acc = 0;
  for (int i = threadIdx.x; i < n; i += 256) acc += s[i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = (float)red[0];
}

}  // namespace nn
}  // namespace msx

using namespace msx;
using namespace msx::nn;

struct msx_corrector {
  int H = 0, W = 0, Cin = 0, C = 0, L = 0, MX = 0, MY = 0, maxS = 0;
  long long P = 0;
  size_t nparams = 0;
  size_t oW0 = 0, ob0 = 0, oP1 = 0, oc1 = 0, oP2 = 0, oc2 = 0;
  std::vector<size_t> oR, oW, ob;
  float *params = nullptr, *grads = nullptr, *m = nullptr, *v = nullptr;
  float *Bdx = nullptr, *Bdy = nullptr, *Biy = nullptr, *Bix = nullptr;  // partial DFT matrices
  float *xin = nullptr, *a = nullptr, *z = nullptr, *zh = nullptr, *h = nullptr, *o = nullptr;
  float *U1 = nullptr, *Xh = nullptr, *Yh = nullptr, *U2 = nullptr;
  float *da = nullptr, *da2 = nullptr, *dz = nullptr;
  float* part = nullptr;
  size_t part_words = 0;
  double* sums = nullptr;
  size_t sums_words = 0;
  TcGemm gemm;
  int S_last = 0, step = 0;
};

namespace {

int cfail(int code, const char* msg) {
  set_last_error(msg);
  return code;
}

#define NN_CUDA(call)                                                            \
  do {                                                                           \
    cudaError_t e_ = (call);                                                     \
    if (e_ != cudaSuccess) return cfail(MSX_ERR_CUDA, cudaGetErrorString(e_));   \
  } while (0)
#define NN_GEMM(call)                                                                              \
  do {                                                                                             \
    int r_ = (call);                                                                               \
    if (r_ != MSX_OK) return cfail(r_, "corrector: tensor-core GEMM failed (sizes or allocation)"); \
  } while (0)

inline unsigned blocks_for(long long n, int t) { return (unsigned)((n + t - 1) / t); }

size_t act_words(const msx_corrector* k, int S) { return (size_t)S * k->P * k->C; }
size_t u_words(const msx_corrector* k, int S) { return (size_t)S * k->H * k->C * k->MX * 2; }
size_t x_words(const msx_corrector* k, int S) { return (size_t)S * k->C * k->MX * k->MY * 2; }

Epi epi(float* y, Addr out) {
  Epi e{};
  e.y = y;
  e.out = out;
  e.scale = 1.f;
  return e;
}

// Pixel-major activation (S, H, W, C) as rows (s, y, c) x columns x.
Addr rows_syc(const msx_corrector* k) { return Addr{(long long)k->W * k->C, 1, k->C, k->C, 0, 1}; }
// Complex (S, H, C, MX) as rows (s, c, m) x columns (2 y + re/im).
Addr rows_scm(const msx_corrector* k) {
  const long long cm = (long long)k->C * k->MX;
  return Addr{(long long)k->H * cm * 2, 2, cm, cm * 2, 1, 2};
}

// out[j] = column sums of x (rows x n), n in {4, 32, 64, ...} dividing 256
int colsum(msx_corrector* k, const float* x, long long rows, int n, float* out, cudaStream_t st) {
  const long long chunk = 4096;
  const int nchunks = (int)((rows + chunk - 1) / chunk);
  if ((size_t)nchunks * n > k->part_words) return cfail(MSX_ERR_INVALID, "corrector: reduction buffer too small");
  colsum_part_kernel<<<nchunks, 256, 0, st>>>(x, rows, n, chunk, k->part);
  reduce_parts_kernel<<<blocks_for(n, 128), 128, 0, st>>>(k->part, nchunks, n, out);
  NN_CUDA(cudaGetLastError());
  return MSX_OK;
}

// weight gradient dW (n_out x n_in) = dY^T X over the S * P pixels (split K on the tensor cores)
int wgrad(msx_corrector* k, const float* dY, int n_out, const float* X, int n_in, int S, float* dW, cudaStream_t st) {
  const long long K = (long long)S * k->P;
  const int ksplit = (int)std::min<long long>(128, std::max<long long>(1, K / 8192));
  NN_GEMM(k->gemm.run(dY, colmajor(n_out), X, colmajor(n_in), n_out, n_in, K, epi(dW, rowmajor(n_in)), st, ksplit));
  return MSX_OK;
}

// Per-mode channel mixing as batched tensor-core GEMMs, one batch per mode m, each
// complex product as one real GEMM over [real, imaginary] planes (TcGemm::run_cplx).
//   X, Y: (S, C, NM) complex (float index ((s C + c) NM + m) 2 + e); R: (NM, C, C) complex.
// Rows s, columns (part, channel) of an (S, C, NM) complex array, for one mode.
Addr modes_rows_s_parts(const msx_corrector* k) {
  const long long nm2 = 2LL * k->MX * k->MY;
  return Addr{(long long)k->C * nm2, 0, 1, 1, nm2, k->C};
}

// Y = R X per mode: [Yr, Yi] = [Xr, Xi] against rows [Rr, -Ri] and [Ri, Rr]
int mix_forward(msx_corrector* k, const float* R, const float* X, int S, float* Y, cudaStream_t st) {
  const int C = k->C, NM = k->MX * k->MY;
  const Addr xa = modes_rows_s_parts(k);
  NN_GEMM(k->gemm.run_cplx(X, xa, 2, R, 2LL * C, 2, 2LL * C * C, C, C, 1, S, epi(Y, xa), 2, NM, st));
  return MSX_OK;
}

// dX = conj(R)^T dY per mode: dXr = dYr Rr + dYi Ri, dXi = dYi Rr - dYr Ri
// dR = dY X^H over the samples: dRr = dYr^T Xr + dYi^T Xi, dRi = dYi^T Xr - dYr^T Xi
int mix_backward(msx_corrector* k, const float* R, const float* X, const float* dY, int S, float* dX, float* dR,
                 cudaStream_t st) {
  const int C = k->C, NM = k->MX * k->MY;
  const long long nm2 = 2LL * NM;
  const Addr xa = modes_rows_s_parts(k);
  // dX: rows s, K = (part, o) of dY; B row (part, c), column (part', o) = R[o][c] (xor), - for (1, 0)
  NN_GEMM(k->gemm.run_cplx(dY, xa, 2, R, 2, 2LL * C, 2LL * C * C, C, C, 2, S, epi(dX, xa), 2, NM, st));
  // dR: rows o, K = (part, s) of dY; B row (part, c), column (part', s) = X[s][c] (xor), - for (1, 0);
  // out (o, part, c) in R's layout
  const Addr ya = Addr{nm2, 0, 1, 1, (long long)C * nm2, S};
  const Addr ro = Addr{2LL * C, 0, 1, 1, 2, C};
  NN_GEMM(k->gemm.run_cplx(dY, ya, 2, X, nm2, (long long)C * nm2, 2, C, S, 2, C, epi(dR, ro), 2LL * C * C, NM, st));
  return MSX_OK;
}

int forward(msx_corrector* k, int S, cudaStream_t st) {
  const long long SP = (long long)S * k->P;
  const int C = k->C, H = k->H, W = k->W, MX = k->MX, MY = k->MY;
  float* Pm = k->params;
  const size_t A = act_words(k, S);
  // lift
  {
    Epi e = epi(k->a, rowmajor(C));
    e.bias = Pm + k->ob0;
    NN_GEMM(k->gemm.run(k->xin, rowmajor(k->Cin), Pm + k->oW0, rowmajor(k->Cin), SP, C, k->Cin, e, st));
  }
  for (int l = 0; l < k->L; ++l) {
    float* ain = k->a + (size_t)l * A;
    float* aout = k->a + (size_t)(l + 1) * A;
    float* zl = k->z + (size_t)l * A;
    float* Xl = k->Xh + (size_t)l * x_words(k, S);
    // DFT along x: rows (s, y, c), K = W -> U1 (S, H, C, MX) complex
    NN_GEMM(k->gemm.run(ain, rows_syc(k), k->Bdx, rowmajor(W), (long long)S * H * C, 2 * MX, W,
                        epi(k->U1, rowmajor(2 * MX)), st));
    // DFT along y: rows (s, c, m), K = 2H -> X (S, C, MX, MY) complex
    NN_GEMM(k->gemm.run(k->U1, rows_scm(k), k->Bdy, rowmajor(2 * H), (long long)S * C * MX, 2 * MY, 2 * H,
                        epi(Xl, rowmajor(2 * MY)), st));
    {
      const int rc = mix_forward(k, Pm + k->oR[l], Xl, S, k->Yh, st);
      if (rc) return rc;
    }
    // inverse DFT along y: rows (s, o, m), K = 2 MY -> U2 (S, H, C, MX) complex
    NN_GEMM(k->gemm.run(k->Yh, rowmajor(2 * MY), k->Biy, rowmajor(2 * MY), (long long)S * C * MX, 2 * H, 2 * MY,
                        epi(k->U2, rows_scm(k)), st));
    // inverse DFT along x (real part, 1/(H W) folded in): rows (s, y, o), K = 2 MX -> z_l pixel-major
    NN_GEMM(k->gemm.run(k->U2, rowmajor(2 * MX), k->Bix, rowmajor(2 * MX), (long long)S * H * C, W, 2 * MX,
                        epi(zl, rows_syc(k)), st));
    // pointwise layer: z_l += a W_l^T + b_l; a_l = gelu(z_l)
    Epi e = epi(zl, rowmajor(C));
    e.bias = Pm + k->ob[l];
    e.accumulate = 1;
    e.act = aout;
    NN_GEMM(k->gemm.run(ain, rowmajor(C), Pm + k->oW[l], rowmajor(C), SP, C, C, e, st));
  }
  {
    Epi e = epi(k->zh, rowmajor(C));
    e.bias = Pm + k->oc1;
    e.act = k->h;
    NN_GEMM(k->gemm.run(k->a + (size_t)k->L * A, rowmajor(C), Pm + k->oP1, rowmajor(C), SP, C, C, e, st));
    Epi e2 = epi(k->o, rowmajor(4));
    e2.bias = Pm + k->oc2;
    NN_GEMM(k->gemm.run(k->h, rowmajor(C), Pm + k->oP2, rowmajor(C), SP, 4, C, e2, st));
  }
  return MSX_OK;
}

int backward(msx_corrector* k, const float* dmaps, cudaStream_t st) {
  const int S = k->S_last;
  const long long SP = (long long)S * k->P;
  const int C = k->C, H = k->H, W = k->W, MX = k->MX, MY = k->MY;
  float* Pm = k->params;
  float* G = k->grads;
  const size_t A = act_words(k, S);
  int rc;
  // head: o = h P2^T + c2
  if ((rc = wgrad(k, dmaps, 4, k->h, C, S, G + k->oP2, st))) return rc;
  if ((rc = colsum(k, dmaps, SP, 4, G + k->oc2, st))) return rc;
  NN_GEMM(k->gemm.run(dmaps, rowmajor(4), Pm + k->oP2, colmajor(C), SP, C, 4, epi(k->dz, rowmajor(C)), st));
  gelu_bwd_kernel<<<blocks_for((long long)A, 256), 256, 0, st>>>(k->dz, k->zh, (long long)A, k->dz);
  if ((rc = wgrad(k, k->dz, C, k->a + (size_t)k->L * A, C, S, G + k->oP1, st))) return rc;
  if ((rc = colsum(k, k->dz, SP, C, G + k->oc1, st))) return rc;
  NN_GEMM(k->gemm.run(k->dz, rowmajor(C), Pm + k->oP1, colmajor(C), SP, C, C, epi(k->da, rowmajor(C)), st));
  for (int l = k->L - 1; l >= 0; --l) {
    const float* ain = k->a + (size_t)l * A;
    const float* zl = k->z + (size_t)l * A;
    const float* Xl = k->Xh + (size_t)l * x_words(k, S);
    gelu_bwd_kernel<<<blocks_for((long long)A, 256), 256, 0, st>>>(k->da, zl, (long long)A, k->dz);
    NN_CUDA(cudaGetLastError());
    if ((rc = wgrad(k, k->dz, C, ain, C, S, G + k->oW[l], st))) return rc;
    if ((rc = colsum(k, k->dz, SP, C, G + k->ob[l], st))) return rc;
    // pointwise part: da2 = dz W_l
    NN_GEMM(k->gemm.run(k->dz, rowmajor(C), Pm + k->oW[l], colmajor(C), SP, C, C, epi(k->da2, rowmajor(C)), st));
    // spectral part, in reverse: IDFT_x^T, IDFT_y^T, mixing, DFT_y^T, DFT_x^T
    NN_GEMM(k->gemm.run(k->dz, rows_syc(k), k->Bix, colmajor(2 * MX), (long long)S * H * C, 2 * MX, W,
                        epi(k->U2, rowmajor(2 * MX)), st));
    NN_GEMM(k->gemm.run(k->U2, rows_scm(k), k->Biy, colmajor(2 * MY), (long long)S * C * MX, 2 * MY, 2 * H,
                        epi(k->Yh, rowmajor(2 * MY)), st));
    // dX (S, C, MX, MY) complex into U1's space; dR into the gradients
    if ((rc = mix_backward(k, Pm + k->oR[l], Xl, k->Yh, S, k->U1, G + k->oR[l], st))) return rc;
    // dX -> dU1 (S, H, C, MX): write into U2 (free now)
    NN_GEMM(k->gemm.run(k->U1, rowmajor(2 * MY), k->Bdy, colmajor(2 * H), (long long)S * C * MX, 2 * H, 2 * MY,
                        epi(k->U2, rows_scm(k)), st));
    Epi e = epi(k->da2, rows_syc(k));
    e.accumulate = 1;
    NN_GEMM(k->gemm.run(k->U2, rowmajor(2 * MX), k->Bdx, colmajor(W), (long long)S * H * C, W, 2 * MX, e, st));
    std::swap(k->da, k->da2);
  }
  // lift: a_0 = x W0^T + b0 (no activation)
  if ((rc = wgrad(k, k->da, C, k->xin, k->Cin, S, G + k->oW0, st))) return rc;
  if ((rc = colsum(k, k->da, SP, C, G + k->ob0, st))) return rc;
  return MSX_OK;
}

// Partial DFT matrices (FP32, row-major) of an H x W grid with MX x MY modes.
void build_dft(int H, int W, int MX, int MY, std::vector<float>& dx, std::vector<float>& dy, std::vector<float>& iy,
               std::vector<float>& ix) {
  const double two_pi = 6.283185307179586476925286766559;
  dx.assign((size_t)2 * MX * W, 0.f);
  for (int m = 0; m < MX; ++m)
    for (int x = 0; x < W; ++x) {
      const double th = two_pi * (double)(((long long)m * x) % W) / W;
      dx[(size_t)(2 * m) * W + x] = (float)std::cos(th);
      dx[(size_t)(2 * m + 1) * W + x] = (float)-std::sin(th);
    }
  dy.assign((size_t)2 * MY * 2 * H, 0.f);
  iy.assign((size_t)2 * H * 2 * MY, 0.f);
  for (int q = 0; q < MY; ++q) {
    const long long f = q < MY / 2 ? q : q - MY;
    for (int y = 0; y < H; ++y) {
      const long long r = ((f * y) % H + H) % H;
      const double th = two_pi * (double)r / H;
      const float c = (float)std::cos(th), s = (float)std::sin(th);
      dy[(size_t)(2 * q) * 2 * H + 2 * y] = c;
      dy[(size_t)(2 * q) * 2 * H + 2 * y + 1] = s;
      dy[(size_t)(2 * q + 1) * 2 * H + 2 * y] = -s;
      dy[(size_t)(2 * q + 1) * 2 * H + 2 * y + 1] = c;
      iy[(size_t)(2 * y) * 2 * MY + 2 * q] = c;
      iy[(size_t)(2 * y) * 2 * MY + 2 * q + 1] = -s;
      iy[(size_t)(2 * y + 1) * 2 * MY + 2 * q] = s;
      iy[(size_t)(2 * y + 1) * 2 * MY + 2 * q + 1] = c;
    }
  }
  ix.assign((size_t)W * 2 * MX, 0.f);
  const double inv = 1.0 / ((double)H * W);
  for (int x = 0; x < W; ++x)
    for (int m = 0; m < MX; ++m) {
      const double th = two_pi * (double)(((long long)m * x) % W) / W;
      const double wm = (m == 0 ? 1.0 : 2.0) * inv;
      ix[(size_t)x * 2 * MX + 2 * m] = (float)(wm * std::cos(th));
      ix[(size_t)x * 2 * MX + 2 * m + 1] = (float)(-wm * std::sin(th));
    }
}

}  // namespace

extern "C" {

int msx_corrector_create(int ny, int nx, int in_channels, int channels, int layers, int modes_x, int modes_y,
                         int max_samples, msx_corrector** out) {
  if (!out) return cfail(MSX_ERR_INVALID, "null corrector pointer");
  *out = nullptr;
  if (ny < 8 || nx < 8 || ny > 4096 || nx > 4096 || in_channels < 1 || in_channels > 64 || channels < 1 ||
      channels > 64 || 256 % channels || layers < 1 || layers > 16 || modes_x < 1 || modes_x > nx / 2 ||
      modes_y < 2 || modes_y % 2 || modes_y > ny || max_samples < 1)
    return cfail(MSX_ERR_INVALID, "corrector: grid 8..4096, 1..64 input channels, channels dividing 256 (<= 64), "
                                  "1..16 layers, modes_x <= nx/2, even modes_y <= ny, samples >= 1");
  msx_corrector* k = new msx_corrector();
  k->H = ny; k->W = nx; k->P = (long long)ny * nx; k->Cin = in_channels; k->C = channels; k->L = layers;
  k->MX = modes_x; k->MY = modes_y; k->maxS = max_samples;
  const int C = channels;
  size_t off = 0;
  k->oW0 = off; off += (size_t)C * in_channels; k->ob0 = off; off += C;
  for (int l = 0; l < layers; ++l) {
    k->oR.push_back(off); off += (size_t)modes_x * modes_y * C * C * 2;
    k->oW.push_back(off); off += (size_t)C * C;
    k->ob.push_back(off); off += C;
  }
  k->oP1 = off; off += (size_t)C * C; k->oc1 = off; off += C;
  k->oP2 = off; off += (size_t)4 * C; k->oc2 = off; off += 4;
  k->nparams = off;
  const size_t S = max_samples, A = act_words(k, max_samples);
  k->part_words = ((S * k->P + 4095) / 4096) * 64;
  cudaError_t e = cudaSuccess;
  auto alloc = [&](float** p, size_t words) { if (e == cudaSuccess) e = cudaMalloc((void**)p, words * sizeof(float)); };
  alloc(&k->params, 4 * off);
  if (e == cudaSuccess) { k->grads = k->params + off; k->m = k->grads + off; k->v = k->m + off; }
  alloc(&k->Bdx, (size_t)2 * modes_x * nx);
  alloc(&k->Bdy, (size_t)4 * modes_y * ny);
  alloc(&k->Biy, (size_t)4 * modes_y * ny);
  alloc(&k->Bix, (size_t)2 * modes_x * nx);
  alloc(&k->xin, S * k->P * in_channels);
  alloc(&k->a, (layers + 1) * A);
  alloc(&k->z, layers * A);
  alloc(&k->zh, A);
  alloc(&k->h, A);
  alloc(&k->o, S * k->P * 4);
  alloc(&k->U1, std::max(u_words(k, max_samples), x_words(k, max_samples)));
  alloc(&k->U2, u_words(k, max_samples));
  alloc(&k->Xh, layers * x_words(k, max_samples));
  alloc(&k->Yh, x_words(k, max_samples));
  alloc(&k->da, A);
  alloc(&k->da2, A);
  alloc(&k->dz, A);
  alloc(&k->part, k->part_words);
  k->sums_words = (S * k->P * 64 + 255) / 256;
  if (e == cudaSuccess) e = cudaMalloc((void**)&k->sums, k->sums_words * sizeof(double));
  if (e == cudaSuccess) e = cudaMemset(k->params, 0, 4 * off * sizeof(float));
  if (e == cudaSuccess) {
    std::vector<float> dx, dy, iy, ix;
    build_dft(ny, nx, modes_x, modes_y, dx, dy, iy, ix);
    e = cudaMemcpy(k->Bdx, dx.data(), dx.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(k->Bdy, dy.data(), dy.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(k->Biy, iy.data(), iy.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(k->Bix, ix.data(), ix.size() * sizeof(float), cudaMemcpyHostToDevice);
  }
  if (e != cudaSuccess) {
    msx_corrector_destroy(k);
    return cfail(MSX_ERR_ALLOC, "corrector allocation failed");
  }
  *out = k;
  return MSX_OK;
}

int msx_corrector_destroy(msx_corrector* k) {
  if (!k) return MSX_OK;
  for (void* p : {(void*)k->params, (void*)k->Bdx, (void*)k->Bdy, (void*)k->Biy, (void*)k->Bix, (void*)k->xin,
                  (void*)k->a, (void*)k->z, (void*)k->zh, (void*)k->h, (void*)k->o, (void*)k->U1, (void*)k->U2,
                  (void*)k->Xh, (void*)k->Yh, (void*)k->da, (void*)k->da2, (void*)k->dz, (void*)k->part,
                  (void*)k->sums})
    if (p) cudaFree(p);
  k->gemm.release();
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

int msx_corrector_layout(const msx_corrector* k, size_t* offsets, int n) {
  // W0, b0, then per layer R, W, b, then P1, c1, P2, c2
  if (!k || !offsets || n < 6 + 3 * k->L) return cfail(MSX_ERR_INVALID, "corrector layout: need 6 + 3 L offsets");
  int i = 0;
  offsets[i++] = k->oW0;
  offsets[i++] = k->ob0;
  for (int l = 0; l < k->L; ++l) {
    offsets[i++] = k->oR[l];
    offsets[i++] = k->oW[l];
    offsets[i++] = k->ob[l];
  }
  offsets[i++] = k->oP1;
  offsets[i++] = k->oc1;
  offsets[i++] = k->oP2;
  offsets[i++] = k->oc2;
  return MSX_OK;
}

int msx_corrector_forward(msx_corrector* k, const float* features_dev, int samples, float* maps_out_dev, void* stream) {
  if (!k || !features_dev || !maps_out_dev || samples < 1 || samples > k->maxS)
    return cfail(MSX_ERR_INVALID, "corrector forward: bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  NN_CUDA(cudaMemcpyAsync(k->xin, features_dev, sizeof(float) * samples * k->P * k->Cin, cudaMemcpyDeviceToDevice, st));
  int rc = forward(k, samples, st);
  if (rc) return rc;
  k->S_last = samples;
  NN_CUDA(cudaMemcpyAsync(maps_out_dev, k->o, sizeof(float) * samples * k->P * 4, cudaMemcpyDeviceToDevice, st));
  return MSX_OK;
}

int msx_corrector_backward(msx_corrector* k, const float* dmaps_dev, void* stream) {
  if (!k || !dmaps_dev || k->S_last < 1) return cfail(MSX_ERR_INVALID, "corrector backward: run forward first");
  return backward(k, dmaps_dev, (cudaStream_t)stream);
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

int msx_corrector_check(msx_corrector* k) {
  if (!k) return cfail(MSX_ERR_INVALID, "null corrector");
  NN_CUDA(cudaDeviceSynchronize());
  const int rc = k->gemm.check();
  if (rc == MSX_ERR_TIMEOUT) return cfail(rc, "a tensor-core GEMM wait of the corrector gave up");
  return rc;
}

int msx_corrector_features(const float* pot_dev, int samples, int ratio, int ny, int nx, float sigma, float tval,
                           float* features_out_dev, void* stream) {
  if (!pot_dev || !features_out_dev || samples < 1 || ratio < 1 || ratio > 62 || ny < 1 || nx < 1)
    return cfail(MSX_ERR_INVALID, "corrector features: bad arguments");
  const long long P = (long long)ny * nx;
  features_kernel<<<blocks_for((long long)samples * P, 256), 256, 0, (cudaStream_t)stream>>>(pot_dev, samples, ratio, P,
                                                                                             sigma, tval,
                                                                                             features_out_dev);
  NN_CUDA(cudaGetLastError());
  return MSX_OK;
}

int msx_corrector_apply_map(float* waves_dev, int num, int ny, int nx, const float* maps_dev, int which, int conj,
                            int form, void* stream) {
  if (!waves_dev || !maps_dev || num < 0 || ny < 1 || nx < 1 || (which != 0 && which != 1))
    return cfail(MSX_ERR_INVALID, "corrector apply map: bad arguments");
  const long long P = (long long)ny * nx;
  if (num == 0) return MSX_OK;
  map_mul_kernel<<<blocks_for((long long)num * P, 256), 256, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<float2*>(waves_dev), num, P, maps_dev, which, conj ? 1 : 0, form ? 1 : 0);
  NN_CUDA(cudaGetLastError());
  return MSX_OK;
}

int msx_corrector_mul_plane(float* waves_dev, int num, int ny, int nx, const float* plane_dev, int conj,
                            void* stream) {
  if (!waves_dev || !plane_dev || num < 0 || ny < 1 || nx < 1)
    return cfail(MSX_ERR_INVALID, "corrector plane product: bad arguments");
  const long long P = (long long)ny * nx;
  if (num == 0) return MSX_OK;
  plane_mul_kernel<<<blocks_for((long long)num * P, 256), 256, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<float2*>(waves_dev), (long long)num * P, P, reinterpret_cast<const float2*>(plane_dev),
      conj ? 1 : 0);
  NN_CUDA(cudaGetLastError());
  return MSX_OK;
}

int msx_corrector_map_trans(const float* trans_dev, int ny, int nx, const float* maps_dev, int which, int form,
                            float* out_dev, void* stream) {
  if (!trans_dev || !maps_dev || !out_dev || ny < 1 || nx < 1 || (which != 0 && which != 1))
    return cfail(MSX_ERR_INVALID, "corrector map transmission: bad arguments");
  const long long P = (long long)ny * nx;
  map_trans_kernel<<<blocks_for(P, 256), 256, 0, (cudaStream_t)stream>>>(reinterpret_cast<const float2*>(trans_dev), P,
                                                                         maps_dev, which, form ? 1 : 0,
                                                                         reinterpret_cast<float2*>(out_dev));
  NN_CUDA(cudaGetLastError());
  return MSX_OK;
}

int msx_corrector_map_grad(const float* u_dev, const float* g_dev, int num, int ny, int nx, int which, int accumulate,
                           int form, const float* maps_dev, float* dmaps_dev, void* stream) {
  if (!u_dev || !g_dev || !dmaps_dev || num < 1 || ny < 1 || nx < 1 || (which != 0 && which != 1) ||
      (form && !maps_dev))
    return cfail(MSX_ERR_INVALID, "corrector map gradient: bad arguments");
  const long long P = (long long)ny * nx;
  map_grad_kernel<<<blocks_for(P, 256), 256, 0, (cudaStream_t)stream>>>(reinterpret_cast<const float2*>(u_dev),
                                                                        reinterpret_cast<const float2*>(g_dev), num, P,
                                                                        which, accumulate ? 1 : 0, form ? 1 : 0,
                                                                        maps_dev, dmaps_dev);
  NN_CUDA(cudaGetLastError());
  return MSX_OK;
}

int msx_corrector_residual(const float* psi_dev, const float* target_dev, int num, int ny, int nx, float weight,
                           int accumulate, float* adjoint_dev, float* loss_out_dev, void* stream) {
  if (!psi_dev || !target_dev || !adjoint_dev || !loss_out_dev || num < 1 || ny < 1 || nx < 1)
    return cfail(MSX_ERR_INVALID, "corrector residual: bad arguments");
  const long long n = (long long)num * ny * nx;
  const unsigned nb = blocks_for(n, 256);
  thread_local double* sums = nullptr;
  thread_local size_t cap = 0;
  if (nb > cap) {
    if (sums) cudaFree(sums);
    sums = nullptr;
    cap = 0;
    if (cudaMalloc(&sums, nb * sizeof(double)) != cudaSuccess) return cfail(MSX_ERR_ALLOC, "loss partials");
    cap = nb;
  }
  cudaStream_t st = (cudaStream_t)stream;
  resid_kernel<<<nb, 256, 0, st>>>(reinterpret_cast<const float2*>(psi_dev), reinterpret_cast<const float2*>(target_dev),
                                   n, weight, accumulate ? 1 : 0, reinterpret_cast<float2*>(adjoint_dev), sums);
  sum_blocks_kernel<<<1, 256, 0, st>>>(sums, (int)nb, loss_out_dev);
  NN_CUDA(cudaGetLastError());
  return MSX_OK;
}

}  // extern "C"
