// Device kernels that prepare the multislice inputs: Kirkland atom windows,
// the transmission slices exp(i sigma V), the k-space probe and its
// normalisation, and the propagator table.
#include "msx_internal.h"

#include <cmath>

namespace msx {

// ------------------------------------------------------------------ Bessel K0
// K0(x) = int_0^inf exp(-x cosh u) du (x > 0).  The integrand is analytic and
// decays double-exponentially in the strip |Im u| < pi/2, so the trapezoidal
// rule with step h converges like exp(-pi^2 / h); h = 1/8 leaves an error far
// below double rounding for the arguments used here (x >= 0.1).  The sum stops
// once a term falls below 1e-18 of the running sum.
__device__ double bessel_k0(double x) {
  const double h = 0.125;
  double sum = 0.5 * exp(-x);
  for (int k = 1; k < 400; ++k) {
    const double term = exp(-x * cosh(k * h));
    sum += term;
    if (term < 1e-18 * sum) break;
  }
  return h * sum;
}

// ------------------------------------------------------------------ atom windows
// Follows _get_potential (namsa/msa.py:180-196) and bin_2d_array
// (namsa/utils.py:101-108): oversampled inclusive grid
// x_i = -range/2 + i*range/(n-1), Kirkland sum
//   v = 4 pi^2 a0 e sum_i a_i K0(2 pi r sqrt(b_i) + 0.1) + 2 pi^2 a0 e sum_i c_i/d_i exp(-pi^2 r^2/d_i)
// with a0 = 0.529, e = 14.4, the oversample x oversample mean, minus the window
// minimum, rounded to float32.  All arithmetic is double.
//
// Every Kirkland coefficient is positive, so v decreases with r and the
// window minimum is the corner bin (each of its samples lies farther out than
// the matching sample of any other bin); every CTA evaluates the corner bins
// itself, which needs no grid-wide reduction.  Grid: (species, bin blocks).
__device__ double window_bin(const double* c, int i, int j, int os, double sx, double sy, double start) {
  const double pi = 3.14159265358979323846;
  const double pre = 4.0 * pi * pi * 0.529 * 14.4;
  double acc0 = 0;  // numpy's order: mean over the last axis, then over the second-to-last
  for (int a = 0; a < os; ++a) {
    double accr = 0;
    for (int b = 0; b < os; ++b) {
      const double gx = (double)(i * os + a) * sx + start;
      const double gy = (double)(j * os + b) * sy + start;
      const double r = sqrt(gx * gx + gy * gy);
      double v = 0;
      for (int k = 0; k < 3; ++k) {
        const double ak = c[k], bk = c[3 + k], ck = c[6 + k], dk = c[9 + k];
        const double term = pre * ak * bessel_k0(2 * pi * r * sqrt(bk) + 0.1) + pre / 2. * ck / dk * exp(-pi * pi * r * r / dk);
        v = (k == 0) ? term : v + term;
      }
      accr = (b == 0) ? v : accr + v;
    }
    accr /= os;
    acc0 = (a == 0) ? accr : acc0 + accr;
  }
  return acc0 / os;
}

__global__ void atom_window_kernel(const double* __restrict__ coeff, int n0, int n1, int os, double range,
                                   float* __restrict__ out) {
  __shared__ double corner[4];
  const int h0 = n0 / os, h1 = n1 / os;
  const double* c = coeff + 12 * blockIdx.x;
  const double start = -range / 2, sx = range / (double)(n0 - 1), sy = range / (double)(n1 - 1);
  if (threadIdx.x < 4) {
    const int ci = (threadIdx.x & 1) ? h0 - 1 : 0, cj = (threadIdx.x & 2) ? h1 - 1 : 0;
    corner[threadIdx.x] = window_bin(c, ci, cj, os, sx, sy, start);
  }
  __syncthreads();
  const double vmin = fmin(fmin(corner[0], corner[1]), fmin(corner[2], corner[3]));
  const int o = blockIdx.y * blockDim.x + threadIdx.x;
  if (o < h0 * h1) {
    const double v = window_bin(c, o / h1, o % h1, os, sx, sy, start);
    out[(size_t)blockIdx.x * h0 * h1 + o] = (float)(v - vmin);
  }
}

// ------------------------------------------------------------------ transmission slices
// One CTA per 32x32 pixel tile of one slice.  Follows BuildScatteringPotential
// (namsa/potential_kernels.cu:5-60): a site (zidx, yc, xc) covers rows
// [rintf(yc - H/2), rintf(yc + H/2)) and the matching columns, clipped to the
// grid (no wrap) and to the window extent.  Each pixel sums the windows of its
// slice's sites in site order in float32 (the order of the reference's
// per-pixel atomicAdds, which come from one thread per pixel), then
// t = (cos(sigma V), sin(sigma V)) with NaN -> 1.
//
// Sites are binned per tile in shared memory: each chunk of 256 sites is
// tested against the tile and the overlapping ones are compacted in order.
constexpr int kPotTile = 32;
constexpr int kPotThreads = 256;

__global__ void __launch_bounds__(kPotThreads)
potential_kernel(const int4* __restrict__ sites, const int* __restrict__ slice_off, const float* __restrict__ windows,
                 int H, int W, int Ny, int Nx, float sigma, float2* __restrict__ trans, float* __restrict__ pot) {
  __shared__ int4 list[kPotThreads];
  __shared__ int warp_count[kPotThreads / 32];
  const int s = blockIdx.z;
  const int ty0 = blockIdx.y * kPotTile, tx0 = blockIdx.x * kPotTile;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int px = tx0 + lane;
  const int py0 = ty0 + warp;  // rows py0 + 8*k, k = 0..3
  float acc[kPotTile / 8] = {0.f, 0.f, 0.f, 0.f};
  const int begin = slice_off[s], end = slice_off[s + 1];
  const float hh = H * 0.5f, hw = W * 0.5f;
  for (int base = begin; base < end; base += kPotThreads) {
    const int idx = base + threadIdx.x;
    int4 st = make_int4(0, 0, 0, 0);
    bool hit = false;
    if (idx < end) {
      st = sites[idx];
      const int ys = (int)rintf((float)st.y - hh), ye = (int)rintf((float)st.y + hh);
      const int xs = (int)rintf((float)st.z - hw), xe = (int)rintf((float)st.z + hw);
      const int r0 = max(max(ys, 0), ty0), r1 = min(min(min(ye, Ny), ys + H), ty0 + kPotTile);
      const int c0 = max(max(xs, 0), tx0), c1 = min(min(min(xe, Nx), xs + W), tx0 + kPotTile);
      hit = (r1 > r0) && (c1 > c0);
      st.w = ys;  // keep the start row; the start column is recomputed below
    }
    const unsigned ballot = __ballot_sync(0xffffffffu, hit);
    if (lane == 0) warp_count[warp] = __popc(ballot);
    __syncthreads();
    int offset = 0, total = 0;
    for (int w = 0; w < kPotThreads / 32; ++w) {
      if (w < warp) offset += warp_count[w];
      total += warp_count[w];
    }
    if (hit) list[offset + __popc(ballot & ((1u << lane) - 1u))] = st;
    __syncthreads();
    for (int i = 0; i < total; ++i) {
      const int4 e = list[i];
      const int ys = e.w;
      const int ye = (int)rintf((float)e.y + hh);
      const int xs = (int)rintf((float)e.z - hw), xe = (int)rintf((float)e.z + hw);
      const float* win = windows + (size_t)e.x * H * W;
      const bool colok = px >= 0 && px < xe && px < Nx && px >= xs && (px - xs) < W;
#pragma unroll
      for (int k = 0; k < kPotTile / 8; ++k) {
        const int py = py0 + 8 * k;
        if (colok && py < ye && py < Ny && py >= ys && (py - ys) < H) acc[k] += __ldg(win + (py - ys) * W + (px - xs));
      }
    }
    __syncthreads();
  }
  if (px < Nx) {
#pragma unroll
    for (int k = 0; k < kPotTile / 8; ++k) {
      const int py = py0 + 8 * k;
      if (py < Ny) {
        const size_t o = ((size_t)s * Ny + py) * Nx + px;
        const float arg = acc[k] * sigma;
        float2 tv = make_float2(cosf(arg), sinf(arg));
        if (isnan(tv.x)) tv.x = 1.f;
        if (isnan(tv.y)) tv.y = 1.f;
        trans[o] = tv;
        if (pot) pot[o] = acc[k];
      }
    }
  }
}

// ------------------------------------------------------------------ probe
// |k| on the centred grid, evaluated with the reference's operation order
// (calc_krad, probe_kernels.cu:11-16) and without FMA contraction, so that the
// float32 aperture and bandwidth decisions are reproducible on the host.
__device__ __forceinline__ double krad_exact(int x, int y, int Nx, int Ny, float kmax) {
  const double km = (double)kmax;
  const double kx = __dsub_rn(__ddiv_rn(__dmul_rn((double)x, km), (double)(Nx - 1)), __ddiv_rn(km, 2.0));
  const double ky = __dsub_rn(__ddiv_rn(__dmul_rn((double)y, km), (double)(Ny - 1)), __ddiv_rn(km, 2.0));
  return __dsqrt_rn(__dadd_rn(__dmul_rn(kx, kx), __dmul_rn(ky, ky)));
}

// k-space probe psi_k = A(k) exp(-i chi(k)) on the centred grid
// k = j*kmax/(N-1) - kmax/2 (probe_kernels.cu:11-16).  A is the smooth
// aperture 1/(1 + exp(-160 (k_semi - k))) (probe_kernels.cu:196-206, smoothing
// fixed at 80) or the hard one k < k_semi compared in float32
// (probe_kernels.cu:180-194); chi = 2 pi/lambda (-C1/2 (k lambda)^2 +
// C3/4 (k lambda)^4 + C5/6 (k lambda)^6) (probe_kernels.cu:208-222).  Evaluated
// in double, stored as complex64 like the reference's psi_k (msa.py:710-717).
__global__ void probe_kernel(int Ny, int Nx, float kmax, double lambda, float k_semi, double C1, double C3, double C5,
                             int smooth, float2* __restrict__ psik, float* __restrict__ aperture) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  if (x >= Nx) return;
  const double k = krad_exact(x, y, Nx, Ny, kmax);
  double a;
  if (smooth) a = 1.0 / (1.0 + exp(-160.0 * ((double)k_semi - k)));
  else a = ((float)k < k_semi) ? 1.0 : 0.0;
  const double kl = k * lambda, kl2 = kl * kl;
  const double chi = 2.0 * 3.14159265358979323846 / lambda * (-0.5 * C1 * kl2 + 0.25 * C3 * kl2 * kl2 + C5 / 6.0 * kl2 * kl2 * kl2);
  double sn, cs;
  sincos(chi, &sn, &cs);
  const size_t o = (size_t)y * Nx + x;
  psik[o] = make_float2((float)(a * cs), (float)(-a * sn));
  if (aperture) aperture[o] = (float)a;
}

// normalisation = sum |fftshift(ifft2_u(psi_k))|^2 = N * sum |psi_k|^2 (Parseval),
// accumulated in double by one CTA in a fixed order (msa.py:721-727).
__global__ void probe_norm_kernel(const float2* __restrict__ psik, long long n, double* __restrict__ out) {
  __shared__ double red[1024];
  double acc = 0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) {
    const float2 v = psik[i];
    acc += (double)v.x * v.x + (double)v.y * v.y;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = red[0] * (double)n;
}

// ------------------------------------------------------------------ propagator table
// P(k) * mask(k) / N with P = exp(-i pi lambda t k^2) (probe_kernels.cu:167-178)
// and mask = float(k) < float(bandwidth*kmax) (hard_aperture, msa.py:833-839).
// The phase is reduced in double (pi lambda t k^2 = 2 pi * f, f taken modulo 1).
__global__ void ptab_kernel(int Ny, int Nx, float kmax, double lambda, double slice_t, float k_band, float2* __restrict__ ptab) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  if (x >= Nx) return;
  const double k = krad_exact(x, y, Nx, Ny, kmax);
  const double k2 = k * k;
  const float kf = (float)k;
  float2 v = make_float2(0.f, 0.f);
  if (kf < k_band) {
    double f = 0.5 * lambda * slice_t * k2;  // phase / (2 pi)
    f -= rint(f);
    float sn, cs;
    sincospif(2.0f * (float)f, &sn, &cs);
    const float inv_n = (float)(1.0 / ((double)Ny * (double)Nx));
    v = make_float2(cs * inv_n, -sn * inv_n);
  }
  ptab[(size_t)y * Nx + x] = v;
}

// Separable propagator factors for the persistent column pass:
// py[y] = exp(-i pi lambda t ky^2), px[x] = exp(-i pi lambda t kx^2) / N, and per
// column x the band [lo, hi] of rows whose float32 |k| passes the mask test
// (the same comparison as ptab_kernel).  |k| is monotone in |ky|, so the rows
// that pass form one interval.
__global__ void pfac_kernel(int Ny, int Nx, float kmax, double lambda, double slice_t, float k_band,
                            float2* __restrict__ pyx, int2* __restrict__ band) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const double km = (double)kmax;
  if (i < Ny) {
    const double ky = __dsub_rn(__ddiv_rn(__dmul_rn((double)i, km), (double)(Ny - 1)), __ddiv_rn(km, 2.0));
    double f = 0.5 * lambda * slice_t * ky * ky;
    f -= rint(f);
    float sn, cs;
    sincospif(2.0f * (float)f, &sn, &cs);
    pyx[i] = make_float2(cs, -sn);
  }
  if (i < Nx) {
    const double kx = __dsub_rn(__ddiv_rn(__dmul_rn((double)i, km), (double)(Nx - 1)), __ddiv_rn(km, 2.0));
    double f = 0.5 * lambda * slice_t * kx * kx;
    f -= rint(f);
    float sn, cs;
    sincospif(2.0f * (float)f, &sn, &cs);
    const float inv_n = (float)(1.0 / ((double)Ny * (double)Nx));
    pyx[Ny + i] = make_float2(cs * inv_n, -sn * inv_n);
  }
  // band of column x: one warp per column, the lanes stride over the rows; the
  // first and last passing rows are the minimum and maximum over the lanes
  const int warp = i >> 5, lane = i & 31;
  if (warp < Nx) {
    int lo = Ny, hi = -1;
    for (int y = lane; y < Ny; y += 32) {
      if ((float)krad_exact(warp, y, Nx, Ny, kmax) < k_band) {
        lo = min(lo, y);
        hi = max(hi, y);
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
      hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if (lane == 0) band[warp] = hi < 0 ? make_int2(1, 0) : make_int2(lo, hi);
  }
}

__global__ void store_double_kernel(double* dst, double value) { *dst = value; }

cudaError_t launch_store_double(double* dst, double value, cudaStream_t st) {
  store_double_kernel<<<1, 1, 0, st>>>(dst, value);
  return cudaGetLastError();
}

cudaError_t launch_pfac(int Ny, int Nx, float kmax, double lambda, double slice_t, float k_band, float2* pyx,
                        int2* band, cudaStream_t st) {
  // 32 threads per column for the bands; that also covers the Ny + Nx factors
  const long long threads = 32LL * Nx > (long long)(Ny > Nx ? Ny : Nx) ? 32LL * Nx : (long long)(Ny > Nx ? Ny : Nx);
  pfac_kernel<<<(unsigned)((threads + 127) / 128), 128, 0, st>>>(Ny, Nx, kmax, lambda, slice_t, k_band, pyx, band);
  return cudaGetLastError();
}

// Detector signals: out[p][d] = sum over column tiles of partial[p][tile][d],
// in tile order (deterministic).
__global__ void detect_reduce_kernel(const float* __restrict__ partial, int G, int tiles, int ndet,
                                     float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= G * ndet) return;
  const int p = i / ndet, d = i % ndet;
  float s = 0.f;
  for (int k = 0; k < tiles; ++k) s += partial[((size_t)p * tiles + k) * ndet + d];
  out[i] = s;
}

cudaError_t launch_detect_reduce(const float* partial, int G, int tiles, int ndet, float* out, cudaStream_t st) {
  const int n = G * ndet;
  detect_reduce_kernel<<<(n + 127) / 128, 128, 0, st>>>(partial, G, tiles, ndet, out);
  return cudaGetLastError();
}

cudaError_t launch_atom_windows(const double* coeff, int nspecies, int n0, int n1, int os, double range, float* out,
                                cudaStream_t st) {
  const int h0 = n0 / os, h1 = n1 / os;
  const int threads = 128;
  const dim3 grid(nspecies, (h0 * h1 + threads - 1) / threads);
  atom_window_kernel<<<grid, threads, 0, st>>>(coeff, n0, n1, os, range, out);
  return cudaGetLastError();
}

cudaError_t launch_potential(const int4* sites, const int* slice_off, int num_slices, const float* windows, int H, int W,
                             int Ny, int Nx, float sigma, float2* trans, float* pot, cudaStream_t st) {
  dim3 grid((Nx + kPotTile - 1) / kPotTile, (Ny + kPotTile - 1) / kPotTile, num_slices);
  potential_kernel<<<grid, kPotThreads, 0, st>>>(sites, slice_off, windows, H, W, Ny, Nx, sigma, trans, pot);
  return cudaGetLastError();
}

cudaError_t launch_probe(int Ny, int Nx, float kmax, double lambda, float k_semi, double C1, double C3, double C5,
                         int smooth, float2* psik, float* aperture, double* norm, cudaStream_t st) {
  dim3 grid((Nx + 127) / 128, Ny);
  probe_kernel<<<grid, 128, 0, st>>>(Ny, Nx, kmax, lambda, k_semi, C1, C3, C5, smooth, psik, aperture);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || norm == nullptr) return e;
  probe_norm_kernel<<<1, 1024, 0, st>>>(psik, (long long)Ny * Nx, norm);
  return cudaGetLastError();
}

cudaError_t launch_probe_norm(const float2* psik, int Ny, int Nx, double* norm, cudaStream_t st) {
  probe_norm_kernel<<<1, 1024, 0, st>>>(psik, (long long)Ny * Nx, norm);
  return cudaGetLastError();
}

cudaError_t launch_ptab(int Ny, int Nx, float kmax, double lambda, double slice_t, float k_band, float2* ptab,
                        cudaStream_t st) {
  dim3 grid((Nx + 127) / 128, Ny);
  ptab_kernel<<<grid, 128, 0, st>>>(Ny, Nx, kmax, lambda, slice_t, k_band, ptab);
  return cudaGetLastError();
}

}  // namespace msx
