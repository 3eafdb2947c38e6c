// Multislice passes over a group of G waves resident in the plan workspace.
//
// Between passes a wave is stored "mixed": y in real space, x in reciprocal
// space, both in natural order, complex64, (G, Ny, Nx) row-major.  One slice of
// the reference's loop (namsa/msa.py:971-981:  psi <- ifft2(P * fft2(psi * t_i / N)))
// becomes two passes:
//
//   row pass  (per row):    inverse FFT_x -> * t_i -> forward FFT_x
//   col pass  (per column): forward FFT_y -> * P/N -> inverse FFT_y
//
// The probe formation (msa.py:959-964: ramp, inverse FFT, fftshift) is one
// column pass that builds psi_k * ramp * (-1)^(kx+ky) (the sign realises the
// fftshift of an even grid) and applies the inverse FFT_y; the first row pass
// then finishes the inverse transform.  The final column pass applies P/N
// after the forward FFT_y and writes |psi|^2 * N / normalisation for the
// crop window: the reference's closing ifft2 -> /N -> fft2 -> *sqrt(N)
// (msa.py:981-989) is the identity times N, so it is folded into that scale.
#pragma once
#include "msx_fft.cuh"
#include <cuda_runtime.h>
#include <type_traits>

namespace msx {

// A schedule fixes the line transform (threads per line T, radices) and the
// launch shape for one line length N.  Several schedules exist per N; the
// autotuner in the host library picks one per grid size.  COL_C columns share
// a column-pass CTA, whose COL_C * T threads (256 or 512) are also the CTA size
// of the row pass; MINB is the minimum number of resident CTAs requested from
// the register allocator.
template <int N_, int T_, int COL_C_, int MINB_, int... Rs>
struct Sched {
  static constexpr int N = N_;
  static constexpr int T = T_;
  static constexpr int C = COL_C_;
  static constexpr int MINB = MINB_;
  static constexpr int THREADS = COL_C_ * T_;        // CTA size of every pass of the schedule
  static constexpr int WARPS = THREADS / 32;
  using FFT = LineFFT<N_, T_, Radices<Rs...>>;
  static constexpr int E = FFT::E;
  static constexpr int TW = FFT::tw_words();
  static constexpr int TW_PAD = (TW + 31) / 32 * 32;
  static constexpr int LPW = 32 / T;                 // row lines per warp
  static constexpr int ROW_LINES = LPW * WARPS;      // row lines per CTA
  static constexpr int ROW_LINE_WORDS = PaddedLine::words(N);
  static constexpr size_t row_smem() { return sizeof(float2) * (TW_PAD + (size_t)ROW_LINES * ROW_LINE_WORDS); }
  // plain column pass: twiddles, the exchange buffer and (probe formation) one complex factor per row
  static constexpr size_t col_smem() { return sizeof(float2) * (TW_PAD + (size_t)C * N + N); }
  static_assert(THREADS == 256 || THREADS == 512, "CTA of 256 or 512 threads");
  static_assert(T <= 32 && 32 % T == 0, "a row line must live inside one warp");
  static constexpr bool PAIRED = false;  // persistent row pass uses PairedFFT512
};

// The same schedule with the persistent row pass transforming through
// PairedFFT512 (radix-2 stage across lane pairs); every other pass unchanged.
template <class S>
struct PairedRow : S {
  static_assert(std::is_same_v<typename S::FFT, LineFFT<512, 32, Radices<16, 2, 16>>>,
                "paired row transform: lines of 512, 32 threads, radices 16 x 2 x 16");
  static constexpr bool PAIRED = true;
};

template <int TW>
__device__ __forceinline__ void load_twiddles(float2* dst, const float2* __restrict__ src) {
  for (int i = threadIdx.x; i < TW; i += blockDim.x) dst[i] = src[i];
  __syncthreads();
}

// ---------------------------------------------------------------- row pass
// Lines are ordered (y, p) with the wave index fastest so the waves of one CTA
// share the transmission row.  RMODE selects the work on each row:
//   ROW_FULL  inverse FFT_x -> * t -> forward FFT_x  (one slice, mixed domain)
//   ROW_TF    * t -> forward FFT_x                    (real-space wave in)
//   ROW_I     inverse FFT_x                           (real-space wave out)
//   ROW_F     forward FFT_x
enum RowMode { ROW_FULL = 0, ROW_TF = 1, ROW_I = 2, ROW_F = 3 };

template <class S, int RMODE = ROW_FULL>
__global__ void __launch_bounds__(S::THREADS, S::MINB)
row_pass_kernel(float2* __restrict__ psi, const float2* __restrict__ trans, const float2* __restrict__ tw_g,
                int G, int Ny) {
  constexpr int NX = S::N;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  load_twiddles<S::TW>(tw, tw_g);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int lw = lane / S::T, t = lane % S::T;
  const int total = G * Ny;
  const int line = blockIdx.x * S::ROW_LINES + warp * S::LPW + lw;
  const bool valid = line < total;
  const int ln = valid ? line : total - 1;
  const int y = ln / G, p = ln - y * G;
  float2* row = psi + ((size_t)p * Ny + y) * NX;
  float2 v[S::E];
#pragma unroll
  for (int m = 0; m < S::E; ++m) v[m] = row[t + S::T * m];
  PaddedLine buf{smem + S::TW_PAD + (warp * S::LPW + lw) * S::ROW_LINE_WORDS};
  if constexpr (RMODE == ROW_FULL || RMODE == ROW_I) S::FFT::template run<true, false>(v, buf, tw, t);
  if constexpr (RMODE == ROW_FULL || RMODE == ROW_TF) {
    const float2* trow = trans + (size_t)y * NX;
#pragma unroll
    for (int m = 0; m < S::E; ++m) v[m] = cmul(v[m], __ldg(trow + t + S::T * m));
  }
  if constexpr (RMODE == ROW_FULL || RMODE == ROW_TF || RMODE == ROW_F) S::FFT::template run<false, false>(v, buf, tw, t);
  if (valid) {
#pragma unroll
    for (int m = 0; m < S::E; ++m) row[t + S::T * m] = v[m];
  }
}

// ---------------------------------------------------------------- column passes
enum ColMode { COL_INIT = 0, COL_MID = 1, COL_FINAL = 2, COL_INIT_FINAL = 3, COL_DETECT = 4 };
constexpr int kMaxDetectors = 8;

struct ColArgs {
  float2* psi;             // (G, Ny, Nx) group workspace
  const float2* ptab;      // (Ny, Nx) propagator * mask / (Ny*Nx)
  const float2* psik;      // (Ny, Nx) k-space probe (init)
  const float* pos_yx;     // (G, 2) probe positions of the group, [y, x] Angstrom (init)
  const float2* tw;        // twiddle table for the y lines
  const double* norm;      // device normalisation sum |ifft2_u(psi_k)|^2 (final)
  float* cbed;             // (G, crop_y, crop_x) output of the group (final)
  int G, Nx;
  int x_begin, ncols;      // columns handled: x_begin .. x_begin + ncols - 1
  int y0, crop_y;          // output rows y0 .. y0 + crop_y - 1 (final)
  float kmax;              // k-grid extent (float32 like the reference)
  const float* det;        // (ndet, Ny, Nx) detector weights over the CBED grid (detect)
  int ndet;
  float* partial;          // (G, Nx / C, ndet) per-tile detector sums (detect)
  const double* init_norm; // init: when set, the probe is scaled by 1/sqrt(*init_norm)
};

template <class S, int MODE>
__global__ void __launch_bounds__(S::THREADS, S::MINB) col_pass_kernel(ColArgs a) {
  constexpr int NY = S::N;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  load_twiddles<S::TW>(tw, a.tw);
  const int p = blockIdx.x % a.G;
  const int tile = blockIdx.x / a.G;
  const int c = threadIdx.x % S::C, t = threadIdx.x / S::C;
  const int xl = tile * S::C + c;
  const bool valid = xl < a.ncols;
  const int x = a.x_begin + (valid ? xl : a.ncols - 1);
  const int Nx = a.Nx;
  float2* __restrict__ col = a.psi + (size_t)p * NY * Nx + x;
  const float2* __restrict__ pcol = a.ptab + x;
  InterleavedLine<S::C> buf{smem + S::TW_PAD + c};
  float2 v[S::E];

  if constexpr (MODE == COL_INIT || MODE == COL_INIT_FINAL) {
    // psi_k * exp(2 pi i (-kx x_p - ky y_p)) * (-1)^(kx_idx + ky_idx); k on the centred
    // grid j*kmax/(N-1) - kmax/2 (probe_kernels.cu:11-16, 37-57, 239-253).  The ramp
    // factors into exp(-2 pi i ky y_p) exp(-2 pi i kx x_p): each phase (in turns) is
    // formed in double and reduced modulo one turn, then evaluated in float -- the
    // row factors once per CTA into shared memory, the column factor per thread --
    // and the element takes their product.
    float2* ey = smem + S::TW_PAD + S::C * NY;
    const double km = (double)a.kmax;
    const double py = (double)a.pos_yx[2 * p], px = (double)a.pos_yx[2 * p + 1];
    for (int i = threadIdx.x; i < NY; i += blockDim.x) {
      const double ky = (double)i * km / (double)(NY - 1) - km * 0.5;
      const double ph = -ky * py;
      float sn, cs;
      sincospif(2.0f * (float)(ph - rint(ph)), &sn, &cs);
      ey[i] = make_float2(cs, sn);
    }
    __syncthreads();
    const double kx = (double)x * km / (double)(a.Nx - 1) - km * 0.5;
    const double phx = -kx * px;
    float2 ex;
    sincospif(2.0f * (float)(phx - rint(phx)), &ex.y, &ex.x);
    if (a.init_norm) {  // unit-norm probe stack (msa.py:915): the scale folds into the column factor
      const float sc = (float)(1.0 / sqrt(*a.init_norm));
      ex = make_float2(ex.x * sc, ex.y * sc);
    }
#pragma unroll
    for (int m = 0; m < S::E; ++m) {
      const int ky_i = t + S::T * m;
      float2 val = cmul(__ldg(a.psik + ky_i * Nx + x), cmul(ey[ky_i], ex));
      if ((x + ky_i) & 1) val = make_float2(-val.x, -val.y);
      v[m] = val;
    }
  } else {
#pragma unroll
    for (int m = 0; m < S::E; ++m) v[m] = col[(t + S::T * m) * Nx];
  }

  if constexpr (MODE == COL_INIT) {
    S::FFT::template run<true, true>(v, buf, tw, t);
  } else if constexpr (MODE == COL_MID) {
    S::FFT::template run<false, true>(v, buf, tw, t);
#pragma unroll
    for (int m = 0; m < S::E; ++m) v[m] = cmul(v[m], __ldg(pcol + (t + S::T * m) * Nx));
    S::FFT::template run<true, true>(v, buf, tw, t);
  } else if constexpr (MODE == COL_FINAL || MODE == COL_DETECT) {
    S::FFT::template run<false, true>(v, buf, tw, t);
#pragma unroll
    for (int m = 0; m < S::E; ++m) v[m] = cmul(v[m], __ldg(pcol + (t + S::T * m) * Nx));
  }
  // COL_INIT_FINAL (no slices): fft2(ifft2_u(Y)) = N*Y, so v already holds Y.

  if constexpr (MODE == COL_DETECT) {
    // Integrated detector signals (MSA.integrate_cbed, namsa/msa.py:426-439) of
    // this CTA's columns: sum_k I(k) w_d(k), reduced in a fixed order.
    const double ntot = (double)NY * (double)a.Nx;
    const float scale = (float)(ntot / *a.norm);
    float acc[kMaxDetectors];
#pragma unroll
    for (int d = 0; d < kMaxDetectors; ++d) acc[d] = 0.f;
#pragma unroll
    for (int m = 0; m < S::E; ++m) {
      const float inten = fmaf(v[m].x, v[m].x, v[m].y * v[m].y) * scale;
      const int ky = t + S::T * m;
#pragma unroll
      for (int d = 0; d < kMaxDetectors; ++d)
        if (d < a.ndet && valid) acc[d] = fmaf(inten, __ldg(a.det + ((size_t)d * NY + ky) * Nx + x), acc[d]);
    }
    __syncthreads();  // the exchange buffer is reused for the reduction
    float* red = reinterpret_cast<float*>(smem + S::TW_PAD);
#pragma unroll
    for (int d = 0; d < kMaxDetectors; ++d) {
      if (d >= a.ndet) break;
      red[threadIdx.x] = acc[d];
      __syncthreads();
      for (int sh = S::THREADS / 2; sh > 0; sh >>= 1) {
        if ((int)threadIdx.x < sh) red[threadIdx.x] += red[threadIdx.x + sh];
        __syncthreads();
      }
      if (threadIdx.x == 0) a.partial[((size_t)p * (a.ncols / S::C) + tile) * a.ndet + d] = red[0];
      __syncthreads();
    }
  } else if constexpr (MODE == COL_FINAL || MODE == COL_INIT_FINAL) {
    const double ntot = (double)NY * (double)a.Nx;
    // COL_FINAL: I = N |P/N * fft2_u(psi t)|^2 / norm ; COL_INIT_FINAL: I = N |Y|^2 / norm
    const float scale = (float)(ntot / *a.norm);
    if (valid) {
      float* out = a.cbed + (size_t)p * a.crop_y * a.ncols + xl;
#pragma unroll
      for (int m = 0; m < S::E; ++m) {
        const int ky = t + S::T * m - a.y0;
        if (ky >= 0 && ky < a.crop_y) out[(size_t)ky * a.ncols] = fmaf(v[m].x, v[m].x, v[m].y * v[m].y) * scale;
      }
    }
  } else {
    if (valid) {
#pragma unroll
      for (int m = 0; m < S::E; ++m) col[(t + S::T * m) * Nx] = v[m];
    }
  }
}

}  // namespace msx
