// Split-BF16 DFT stages on the 5th-generation tensor cores (tcgen05).
//
// A length-N complex DFT of L lines is the real GEMM
//   [Zr | Zi] (L x 2N) = [Xr | Xi] (L x 2N) . B^T,  B (2N x 2N) built from cos/sin,
// run with both operands split into bfloat16 pairs x = hi + lo and the three
// products hi.hi + hi.lo + lo.hi accumulated in FP32 in tensor memory (the
// lo.lo term, below FP32 rounding of the sum, is dropped).  This is the
// precision-study form of the multislice step for grids up to 512^2; the FP32
// FFT passes remain the production path.
//
// GEMM kernel: one CTA computes a 128 x 256 tile of Z.  Operand tiles are
// stored in global memory already in the tensor-core shared-memory layout
// (K-major, 128-byte swizzle: 8-row atoms of 128 B, 16-byte chunk c of row r
// at chunk c ^ (r mod 8)), so each K block (64 bf16) of A_hi, A_lo, B_hi, B_lo
// arrives with four 1-D bulk copies.  Warp 0 lane 0 produces (double-buffered,
// mbarrier full/empty), warp 1 lane 0 issues tcgen05.mma (M=128, N=256, K=16)
// and commits to the stage's empty barrier; all four warps then read the
// accumulator with tcgen05.ld and write FP32 results.  Every mbarrier wait is
// bounded (~1 s); on a timeout the kernel sets *err, still commits and waits
// (bounded) for its MMAs, frees its tensor memory and returns.
#include "msx.h"
#include "msx_internal.h"

#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <vector>

namespace msx {
namespace tc {

constexpr int BM = 128, BN = 256, BK = 64, STAGES = 2;
constexpr int A_BYTES = BM * BK * 2;                     // 16 KB
constexpr int B_BYTES = BN * BK * 2;                     // 32 KB
constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;   // 96 KB
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024;  // 192 KB + alignment slack (dynamic)

// byte offset of element (row, k) (k in [0, 64)) inside a 128B-swizzled K-major block
__host__ __device__ __forceinline__ uint32_t sw128_offset(int row, int k) {
  return (uint32_t)row * 128u + ((uint32_t)((k >> 3) ^ (row & 7)) << 4) + (uint32_t)(k & 7) * 2u;
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  // start address >> 4 (bits 0-13), leading byte offset 16 B (unused for swizzled
  // K-major; bits 16-29), stride byte offset 1024 B between 8-row atoms (bits 32-45),
  // descriptor version 1 (bits 46-47), base offset 0, swizzle mode 128B (= 2, bits 61-63)
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// kind::f16 instruction descriptor: D f32, A/B bf16, both K-major, N = BN, M = BM
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n\t .reg .pred p;\n\t setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__global__ void __launch_bounds__(128, 1)
tc_gemm_kernel(const uint8_t* __restrict__ a_hi, const uint8_t* __restrict__ a_lo, const uint8_t* __restrict__ b_hi,
               const uint8_t* __restrict__ b_lo, int kblocks, int ntiles_n, int N, float* __restrict__ Z,
               float* __restrict__ out_norm, int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  // the 128-byte swizzle is anchored to 1024-byte boundaries: align the stages explicitly
  uint8_t* smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  __shared__ uint64_t full[STAGES], empty[STAGES], done;
  __shared__ uint32_t tmem_base;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int mt = blockIdx.x / ntiles_n, nt = blockIdx.x % ntiles_n;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (threadIdx.x == 32) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(&done, 1);
    fence_mbar_init();
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;

  if (threadIdx.x == 0) {  // producer
    const size_t a_tile = (size_t)mt * kblocks * A_BYTES;
    const size_t b_tile = (size_t)nt * kblocks * B_BYTES;
    for (int kb = 0; kb < kblocks; ++kb) {
      const int s = kb % STAGES;
      if (kb >= STAGES && !mbar_wait_bounded(&empty[s], ((kb / STAGES) - 1) & 1)) {
        atomicOr(err, 2);
        break;
      }
      uint8_t* st = smem + s * STAGE_BYTES;
      mbar_expect_tx(&full[s], STAGE_BYTES);
      bulk_g2s(st, a_hi + a_tile + (size_t)kb * A_BYTES, A_BYTES, &full[s]);
      bulk_g2s(st + A_BYTES, a_lo + a_tile + (size_t)kb * A_BYTES, A_BYTES, &full[s]);
      bulk_g2s(st + 2 * A_BYTES, b_hi + b_tile + (size_t)kb * B_BYTES, B_BYTES, &full[s]);
      bulk_g2s(st + 2 * A_BYTES + B_BYTES, b_lo + b_tile + (size_t)kb * B_BYTES, B_BYTES, &full[s]);
    }
  } else if (threadIdx.x == 32) {  // MMA issuer
    for (int kb = 0; kb < kblocks; ++kb) {
      const int s = kb % STAGES;
      if (!mbar_wait_bounded(&full[s], (kb / STAGES) & 1)) {
        atomicOr(err, 4);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t st = smem_u32(smem + s * STAGE_BYTES);
      const uint32_t ahi = st, alo = st + A_BYTES, bhi = st + 2 * A_BYTES, blo = st + 2 * A_BYTES + B_BYTES;
#pragma unroll
      for (int j = 0; j < BK / 16; ++j) {  // K = 16 per MMA: 32 bytes along the swizzled row
        const uint32_t off = (uint32_t)j * 32u;
        const uint32_t acc0 = (kb > 0 || j > 0) ? 1u : 0u;
        mma_bf16(tmem, smem_desc(ahi + off), smem_desc(bhi + off), acc0);
        mma_bf16(tmem, smem_desc(ahi + off), smem_desc(blo + off), 1u);
        mma_bf16(tmem, smem_desc(alo + off), smem_desc(bhi + off), 1u);
      }
      mma_commit(&empty[s]);  // the stage is free once these MMAs have read it
    }
    mma_commit(&done);
  }
  __syncwarp();
  const bool ok = mbar_wait_bounded(&done, 0);
  if (!ok && lane == 0) atomicOr(err, 8);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok) {
    // lane quarter of this warp: TMEM lanes 32*warp .. 32*warp+31 = tile rows
    const int row = mt * BM + warp * 32 + lane;
    float sq = 0.f;  // this row's sum of squares over the tile's columns
    for (int c0 = 0; c0 < BN; c0 += 32) {
      uint32_t r[32];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
          "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
            "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
            "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
          : "r"(taddr)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
      for (int i = 0; i < 32; ++i) {
        const int j = nt * BN + c0 + i;  // output column: real parts then imaginary parts
        const int e = j < N ? j : j - N;
        const float z = __uint_as_float(r[i]);
        Z[((size_t)row * N + e) * 2 + (j < N ? 0 : 1)] = z;
        sq = fmaf(z, z, sq);
      }
    }
    if (out_norm) out_norm[(size_t)row * ntiles_n + nt] = sq;  // one partial per (line, N tile)
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN) : "memory");
}

// A tiles from complex lines: A[l][n] = X[l][n] * mult[l % lm][n] (mult optional),
// real parts at k = n, imaginary parts at k = N + n, split into bf16 hi + lo.
// One CTA per line; with in_norm it also stores the line's sum |A|^2.
__global__ void __launch_bounds__(256) tc_split_kernel(const float2* __restrict__ X, int N,
                                                       const float2* __restrict__ mult, int lm,
                                                       __nv_bfloat16* __restrict__ a_hi, __nv_bfloat16* __restrict__ a_lo,
                                                       float* __restrict__ in_norm) {
  __shared__ float red[8];
  const long long l = blockIdx.x;
  const int kblocks = 2 * N / BK;
  const long long mt = l / BM;
  const int m = (int)(l % BM);
  float q = 0.f;
  for (int n = threadIdx.x; n < N; n += blockDim.x) {
    float2 v = X[l * N + n];
    if (mult) v = cmul(v, mult[(size_t)(l % lm) * N + n]);
    q = fmaf(v.x, v.x, fmaf(v.y, v.y, q));
#pragma unroll
    for (int part = 0; part < 2; ++part) {
      const float x = part ? v.y : v.x;
      const int kk = part ? N + n : n;
      const __nv_bfloat16 hi = __float2bfloat16_rn(x);
      const __nv_bfloat16 lo = __float2bfloat16_rn(x - __bfloat162float(hi));
      const size_t byte = ((size_t)mt * kblocks + kk / BK) * A_BYTES + sw128_offset(m, kk % BK);
      a_hi[byte / 2] = hi;
      a_lo[byte / 2] = lo;
    }
  }
  if (in_norm) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) q += __shfl_xor_sync(0xffffffffu, q, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = q;
    __syncthreads();
    if (threadIdx.x == 0) {
      float t = 0.f;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
      in_norm[l] = t;
    }
  }
}

// Norm compensation: a length-N DFT multiplies each line's norm by N exactly
// (Parseval), so Z[l] *= sqrt(N * |A_l|^2 / |Z_l|^2) removes the uniform scale
// error of the split-bf16 products and their FP32 accumulation (the tensor
// core's accumulation loses magnitude systematically), leaving the random part
// of the rounding.  One CTA per line; |Z_l|^2 is the sum of the GEMM's
// per-tile partials.
__global__ void __launch_bounds__(256) tc_rescale_kernel(float2* __restrict__ Z, int N, const float* __restrict__ in_norm,
                                                         const float* __restrict__ out_part, int parts) {
  const long long l = blockIdx.x;
  float zo = 0.f;
  for (int j = 0; j < parts; ++j) zo += out_part[l * parts + j];
  if (!(zo > 0.f)) return;
  const float f = sqrtf((float)N * in_norm[l] / zo);
  for (int n = threadIdx.x; n < N; n += blockDim.x) {
    const float2 z = Z[l * N + n];
    Z[l * N + n] = make_float2(z.x * f, z.y * f);
  }
}

// out[p][c][r] = in[p][r][c] for n x n complex planes
__global__ void transpose_kernel(const float2* __restrict__ in, int n, float2* __restrict__ out) {
  __shared__ float2 tile[32][33];
  const size_t plane = (size_t)blockIdx.z * n * n;
  const int x = blockIdx.x * 32 + threadIdx.x, y0 = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += 8) tile[j][threadIdx.x] = in[plane + (size_t)(y0 + j) * n + x];
  __syncthreads();
  const int ox = y0 + threadIdx.x, oy0 = blockIdx.x * 32;
  for (int j = threadIdx.y; j < 32; j += 8) out[plane + (size_t)(oy0 + j) * n + ox] = tile[threadIdx.x][j];
}

}  // namespace tc
}  // namespace msx

using namespace msx;
using namespace msx::tc;

namespace {

int tfail(int code, const char* msg) {
  set_last_error(msg);
  return code;
}

// B (2N x 2N) of a DFT of sign s (e^{s 2 pi i n k / N}) in 128B-swizzled K-major
// tiles of 256 rows x 64 columns, split into bf16 hi and lo.
void build_dft_tiles(int N, int sign, std::vector<__nv_bfloat16>& hi, std::vector<__nv_bfloat16>& lo) {
  const int K = 2 * N, NO = 2 * N, kblocks = K / BK, ntiles = NO / BN;
  hi.assign((size_t)NO * K, __float2bfloat16(0.f));
  lo.assign((size_t)NO * K, __float2bfloat16(0.f));
  const double two_pi = 6.283185307179586476925286766559;
  for (int j = 0; j < NO; ++j)
    for (int kk = 0; kk < K; ++kk) {
      const int k = j % N, n = kk % N;
      const double th = two_pi * (double)(((long long)n * k) % N) / (double)N;
      const double c = std::cos(th), s = std::sin(th);
      double v;
      if (j < N) v = kk < N ? c : -sign * s;   // Zr = Xr cos - s Xi sin
      else v = kk < N ? sign * s : c;           // Zi = s Xr sin + Xi cos
      const float f = (float)v;
      const __nv_bfloat16 h = __float2bfloat16_rn(f);
      const __nv_bfloat16 l = __float2bfloat16_rn(f - __bfloat162float(h));
      const int nt = j / BN, r = j % BN, kb = kk / BK;
      const size_t byte = ((size_t)nt * kblocks + kb) * B_BYTES + sw128_offset(r, kk % BK);
      hi[byte / 2] = h;
      lo[byte / 2] = l;
    }
  (void)ntiles;
}

struct TcState {
  int N = 0;
  __nv_bfloat16 *fwd_hi = nullptr, *fwd_lo = nullptr, *inv_hi = nullptr, *inv_lo = nullptr;
  __nv_bfloat16 *a_hi = nullptr, *a_lo = nullptr;
  float2 *z0 = nullptr, *z1 = nullptr, *ptab_t = nullptr;
  float *nin = nullptr, *nout = nullptr;  // per-line input norms and per-(line, N tile) output partials
  int* err = nullptr;
  size_t lines_cap = 0;
  bool configured = false;
};
thread_local TcState g_tc;  // one per host thread; sized by the largest call
thread_local bool g_tc_compensate = true;

int tc_prepare(int N, size_t lines) {
  TcState& s = g_tc;
  if (s.N != N) {
    for (void* p : {(void*)s.fwd_hi, (void*)s.fwd_lo, (void*)s.inv_hi, (void*)s.inv_lo})
      if (p) cudaFree(p);
    std::vector<__nv_bfloat16> h, l;
    const size_t bytes = sizeof(__nv_bfloat16) * 4 * (size_t)N * N;
    if (cudaMalloc(&s.fwd_hi, bytes) || cudaMalloc(&s.fwd_lo, bytes) || cudaMalloc(&s.inv_hi, bytes) ||
        cudaMalloc(&s.inv_lo, bytes))
      return tfail(MSX_ERR_ALLOC, "tensor-core DFT matrices: allocation failed");
    build_dft_tiles(N, -1, h, l);
    cudaMemcpy(s.fwd_hi, h.data(), bytes, cudaMemcpyHostToDevice);
    cudaMemcpy(s.fwd_lo, l.data(), bytes, cudaMemcpyHostToDevice);
    build_dft_tiles(N, +1, h, l);
    cudaMemcpy(s.inv_hi, h.data(), bytes, cudaMemcpyHostToDevice);
    cudaMemcpy(s.inv_lo, l.data(), bytes, cudaMemcpyHostToDevice);
    s.N = N;
    s.lines_cap = 0;
  }
  if (!s.err) {
    if (cudaMalloc(&s.err, sizeof(int)) || cudaMemset(s.err, 0, sizeof(int))) return tfail(MSX_ERR_ALLOC, "tc error word");
  }
  if (lines > s.lines_cap) {
    for (void* p : {(void*)s.a_hi, (void*)s.a_lo, (void*)s.z0, (void*)s.z1, (void*)s.ptab_t, (void*)s.nin,
                    (void*)s.nout})
      if (p) cudaFree(p);
    const size_t abytes = sizeof(__nv_bfloat16) * lines * 2 * N;
    if (cudaMalloc(&s.a_hi, abytes) || cudaMalloc(&s.a_lo, abytes) || cudaMalloc(&s.z0, sizeof(float2) * lines * N) ||
        cudaMalloc(&s.z1, sizeof(float2) * lines * N) || cudaMalloc(&s.ptab_t, sizeof(float2) * (size_t)N * N) ||
        cudaMalloc(&s.nin, sizeof(float) * lines) || cudaMalloc(&s.nout, sizeof(float) * lines * (2 * N / BN)))
      return tfail(MSX_ERR_ALLOC, "tensor-core DFT scratch: allocation failed");
    s.lines_cap = lines;
  }
  if (!s.configured) {
    if (cudaFuncSetAttribute(tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES) != cudaSuccess)
      return tfail(MSX_ERR_CUDA, "tensor-core GEMM: shared memory attribute");
    s.configured = true;
  }
  return MSX_OK;
}

// Z (lines x N complex) = DFT of sign `sign` of X (lines x N) (X * mult when mult != null)
int tc_dft(const float2* X, size_t lines, int N, const float2* mult, int lm, int sign, float2* Z, cudaStream_t st) {
  TcState& s = g_tc;
  const bool comp = g_tc_compensate;
  tc_split_kernel<<<(unsigned)lines, 256, 0, st>>>(X, N, mult, lm, s.a_hi, s.a_lo, comp ? s.nin : nullptr);
  const int kblocks = 2 * N / BK, ntn = 2 * N / BN;
  const unsigned grid = (unsigned)((lines / BM) * ntn);
  tc_gemm_kernel<<<grid, 128, SMEM_BYTES, st>>>(reinterpret_cast<const uint8_t*>(s.a_hi),
                                                 reinterpret_cast<const uint8_t*>(s.a_lo),
                                                 reinterpret_cast<const uint8_t*>(sign < 0 ? s.fwd_hi : s.inv_hi),
                                                 reinterpret_cast<const uint8_t*>(sign < 0 ? s.fwd_lo : s.inv_lo),
                                                 kblocks, ntn, N, reinterpret_cast<float*>(Z),
                                                 comp ? s.nout : nullptr, s.err);
  if (comp) tc_rescale_kernel<<<(unsigned)lines, 256, 0, st>>>(Z, N, s.nin, s.nout, ntn);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MSX_OK : tfail(MSX_ERR_CUDA, cudaGetErrorString(e));
}

}  // namespace

extern "C" {

int msx_tc_dft(const float* x_dev, int lines, int n, int sign, float* z_dev, void* stream) {
  if (!x_dev || !z_dev || (n != 256 && n != 512) || lines <= 0 || lines % BM || (sign != 1 && sign != -1))
    return tfail(MSX_ERR_INVALID, "tc_dft: n must be 256 or 512, lines a positive multiple of 128, sign +-1");
  int rc = tc_prepare(n, (size_t)lines);
  if (rc) return rc;
  return tc_dft(reinterpret_cast<const float2*>(x_dev), (size_t)lines, n, nullptr, 1, sign,
                reinterpret_cast<float2*>(z_dev), (cudaStream_t)stream);
}

int msx_step_waves_tc(float* waves_dev, int num_waves, int n, const float* trans_dev, const float* ptab_dev,
                      void* stream) {
  if (!waves_dev || !trans_dev || !ptab_dev || num_waves <= 0 || (n != 256 && n != 512))
    return tfail(MSX_ERR_INVALID, "step_waves_tc: square grids of 256 or 512 only");
  const size_t lines = (size_t)num_waves * n;
  int rc = tc_prepare(n, lines);
  if (rc) return rc;
  TcState& s = g_tc;
  cudaStream_t st = (cudaStream_t)stream;
  float2* w = reinterpret_cast<float2*>(waves_dev);
  const dim3 tb(32, 8), tg(n / 32, n / 32, num_waves), tg1(n / 32, n / 32, 1);
  // P^T once per call: rows kx, columns ky
  transpose_kernel<<<tg1, tb, 0, st>>>(reinterpret_cast<const float2*>(ptab_dev), n, s.ptab_t);
  // psi (rows y, cols x) -> t psi -> DFT_x
  if ((rc = tc_dft(w, lines, n, reinterpret_cast<const float2*>(trans_dev), n, -1, s.z0, st))) return rc;
  transpose_kernel<<<tg, tb, 0, st>>>(s.z0, n, s.z1);                      // rows kx, cols y
  if ((rc = tc_dft(s.z1, lines, n, nullptr, 1, -1, s.z0, st))) return rc;  // DFT_y: rows kx, cols ky
  if ((rc = tc_dft(s.z0, lines, n, s.ptab_t, n, +1, s.z1, st))) return rc; // * P/N, inverse DFT_y
  transpose_kernel<<<tg, tb, 0, st>>>(s.z1, n, s.z0);                      // rows y, cols kx
  if ((rc = tc_dft(s.z0, lines, n, nullptr, 1, +1, w, st))) return rc;     // inverse DFT_x
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MSX_OK : tfail(MSX_ERR_CUDA, cudaGetErrorString(e));
}

int msx_tc_set_compensation(int enable) {
  g_tc_compensate = enable != 0;
  return MSX_OK;
}

int msx_tc_check(void) {
  if (!g_tc.err) return MSX_OK;
  int h = 0;
  if (cudaMemcpy(&h, g_tc.err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    return tfail(MSX_ERR_CUDA, "reading the tensor-core error word");
  if (h) {
    cudaMemset(g_tc.err, 0, sizeof(int));
    return tfail(MSX_ERR_TIMEOUT, "a tensor-core DFT wait gave up");
  }
  return MSX_OK;
}

}  // extern "C"
