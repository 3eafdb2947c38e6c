// General BF16 GEMM on the 5th-generation tensor cores (tcgen05) with FP32
// accumulation, for the contractions of the learned corrector (pointwise
// channel mixing, its weight gradients and the partial DFT stages of its
// spectral layers).
//
//   D (M x N) = A (M x K) . B (N x K)^T,   A and B rounded to bfloat16.
//
// Operands are read from FP32 arrays of any 2-level strided layout: element
// (r, k) of an operand sits at (r / rc) * s1 + (r % rc) * s2 + (k / kc) * t1 +
// (k % kc) * t2.  A pack
// kernel rounds them to bfloat16 into the tensor-core shared-memory image
// (K-major, 128-byte swizzle, 8-row atoms of 128 B, 16-byte chunk c of row r
// at chunk c ^ (r mod 8)), tile by tile and K block (64) by K block, zero
// padded to whole tiles; the GEMM kernel then moves each (tile, K block) with
// one 1-D bulk copy.  Output element (r, c) is written at the same kind of
// strided address, so results land directly in pixel-major or transposed
// layouts.  Epilogue: z = acc (+ bias[c]) (+ add[r, c]); out = z or out += z;
// optionally act = gelu(z) (tanh form) into a second array.
//
// Kernel: one CTA of 128 threads per 128 x BN tile of D.  Thread 0 produces
// (bulk copies into STAGES stages, full/empty mbarriers), thread 32 issues
// tcgen05.mma (M = 128, N = BN, K = 16) and commits each stage to its empty
// barrier; all four warps read the accumulator with tcgen05.ld (warp w owns
// TMEM lanes 32w..32w+31 = tile rows).  Every wait is bounded; on a timeout
// the kernel sets *err, waits (bounded) for its MMAs, frees its tensor memory
// and returns.
#include "msx.h"
#include "msx_internal.h"

#include <cuda_bf16.h>

#include <atomic>
#include <cstring>

namespace msx {
namespace tg {

constexpr int BM = 128, BK = 64, STAGES = 3;
constexpr int A_BYTES = BM * BK * 2;  // 16 KB per (tile, K block)

__host__ __device__ __forceinline__ uint32_t sw128(int row, int k) {
  return (uint32_t)row * 128u + ((uint32_t)((k >> 3) ^ (row & 7)) << 4) + (uint32_t)(k & 7) * 2u;
}

__device__ __forceinline__ uint64_t sdesc(uint32_t addr) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

template <int BN>
struct Cfg {
  static_assert(BN == 32 || BN == 64 || BN == 128 || BN == 256, "BN must be 32, 64, 128 or 256");
  static constexpr int B_BYTES = BN * BK * 2;
  static constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
  static constexpr int SMEM = STAGES * STAGE_BYTES + 1024;
  // kind::f16: D f32 (bit 4), A bf16 (bits 7-9 = 1), B bf16 (bits 10-12 = 1), K-major both, N >> 3, M >> 4
  static constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                                    ((uint32_t)(BM >> 4) << 24);
};

__device__ __forceinline__ float gelu_t(float z) {
  const float u = 0.7978845608028654f * (z + 0.044715f * z * z * z);
  return 0.5f * z * (1.f + tanhf(u));
}

__host__ __device__ __forceinline__ long long addr_of(const Addr& a, long long r, long long k) {
  return (r / a.rc) * a.s1 + (r % a.rc) * a.s2 + (k / a.kc) * a.t1 + (k % a.kc) * a.t2;
}

// img[(tile * kblocks + kb)][row][k] (swizzled) = bf16(src(r, k)); zero outside rows x K.
// One thread per (padded row, 8 consecutive k): 16 bytes out.  The row part of the
// address and the split of k0 are computed once per thread; the 8 elements step
// through k incrementally, with two 16-byte loads when they are contiguous.
__global__ void pack_kernel(const float* __restrict__ src, Addr a, long long rows, long long K, int tile_rows,
                            long long rows_pad, int kblocks, uint4* __restrict__ img, int batch = 1,
                            long long src_bs = 0) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long chunks = (long long)kblocks * (BK / 8);
  const long long per = rows_pad * chunks;
  if (i >= per * batch) return;
  const long long bt = i / per;  // batch of this element; its image and source are offset by it
  i -= bt * per;
  src += bt * src_bs;
  img += bt * (per * 8 * 2 / 16);
  const long long r = i / chunks;
  const int ch = (int)(i - r * chunks);
  const long long k0 = (long long)ch * 8;
  __align__(16) __nv_bfloat16 v[8];
  if (r < rows && k0 < K) {
    const float* base = src + (r / a.rc) * a.s1 + (r % a.rc) * a.s2;
    if (a.kc == 1 && a.t1 == 1 && k0 + 8 <= K && ((reinterpret_cast<uintptr_t>(base + k0) & 15u) == 0)) {
      const float4 lo = __ldg(reinterpret_cast<const float4*>(base + k0));
      const float4 hi = __ldg(reinterpret_cast<const float4*>(base + k0) + 1);
      v[0] = __float2bfloat16_rn(lo.x); v[1] = __float2bfloat16_rn(lo.y);
      v[2] = __float2bfloat16_rn(lo.z); v[3] = __float2bfloat16_rn(lo.w);
      v[4] = __float2bfloat16_rn(hi.x); v[5] = __float2bfloat16_rn(hi.y);
      v[6] = __float2bfloat16_rn(hi.z); v[7] = __float2bfloat16_rn(hi.w);
    } else {
      long long q = k0 / a.kc, rem = k0 - q * a.kc;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const float x = (k0 + j < K) ? __ldg(base + q * a.t1 + rem * a.t2) : 0.f;
        v[j] = __float2bfloat16_rn(x);
        if (++rem == a.kc) { rem = 0; ++q; }
      }
    }
  } else {
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = __float2bfloat16_rn(0.f);
  }
  const long long tile = r / tile_rows;
  const int row = (int)(r - tile * tile_rows), kb = (int)(k0 / BK);
  const size_t byte = ((size_t)tile * kblocks + kb) * ((size_t)tile_rows * BK * 2) + sw128(row, (int)(k0 % BK));
  img[byte / 16] = *reinterpret_cast<const uint4*>(v);
}

// With part != null the CTA (tile, split) sums K blocks [split * kper, ...) and
// writes its raw 128 x BN partial to part[(split * tiles + tile) * 128 * BN].
template <int BN>
__global__ void __launch_bounds__(128) gemm_kernel(const uint8_t* __restrict__ A, const uint8_t* __restrict__ B,
                                                   int kblocks, int ntiles_n, int ntiles_total, int kper,
                                                   float* __restrict__ part, Epi e, int* __restrict__ err) {
  using C = Cfg<BN>;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  __shared__ uint64_t full[STAGES], empty[STAGES], done;
  __shared__ uint32_t tmem_base;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int splits = (kblocks + kper - 1) / kper;
  const int tiles = ntiles_total;
  const int bt = (int)blockIdx.x / (tiles * splits);  // batch
  const int inb = (int)blockIdx.x - bt * tiles * splits;
  const int split = inb / tiles, tile = inb % tiles;
  A += (size_t)bt * (size_t)(tiles / ntiles_n) * kblocks * A_BYTES;
  B += (size_t)bt * (size_t)ntiles_n * kblocks * C::B_BYTES;
  e.y += bt * e.ybs;
  if (e.add) e.add += bt * e.ybs;
  if (e.act) e.act += bt * e.ybs;
  const int mt = tile / ntiles_n, nt = tile % ntiles_n;
  const int kb0 = split * kper, kb1 = kb0 + kper < kblocks ? kb0 + kper : kblocks;
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
    const uint8_t* a_tile = A + (size_t)mt * kblocks * A_BYTES;
    const uint8_t* b_tile = B + (size_t)nt * kblocks * C::B_BYTES;
    for (int i = 0; i < kb1 - kb0; ++i) {
      const int kb = kb0 + i, s = i % STAGES;
      if (i >= STAGES && !mbar_wait_bounded(&empty[s], ((i / STAGES) - 1) & 1)) {
        atomicOr(err, 2);
        break;
      }
      uint8_t* st = smem + s * C::STAGE_BYTES;
      mbar_expect_tx(&full[s], C::STAGE_BYTES);
      bulk_g2s(st, a_tile + (size_t)kb * A_BYTES, A_BYTES, &full[s]);
      bulk_g2s(st + A_BYTES, b_tile + (size_t)kb * C::B_BYTES, C::B_BYTES, &full[s]);
    }
  } else if (threadIdx.x == 32) {  // MMA issuer
    for (int i = 0; i < kb1 - kb0; ++i) {
      const int s = i % STAGES;
      if (!mbar_wait_bounded(&full[s], (i / STAGES) & 1)) {
        atomicOr(err, 4);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t st = smem_u32(smem + s * C::STAGE_BYTES);
#pragma unroll
      for (int j = 0; j < BK / 16; ++j) {
        const uint32_t off = (uint32_t)j * 32u;
        const uint32_t acc = (i > 0 || j > 0) ? 1u : 0u;
        asm volatile(
            "{\n\t .reg .pred p;\n\t setp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
            "l"(sdesc(st + off)), "l"(sdesc(st + A_BYTES + off)), "r"(C::IDESC), "r"(acc)
            : "memory");
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(&empty[s]))
                   : "memory");
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(&done))
                 : "memory");
  }
  __syncwarp();
  const bool ok = mbar_wait_bounded(&done, 0);
  if (!ok && lane == 0) atomicOr(err, 8);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok) {
    const long long r = (long long)mt * BM + warp * 32 + lane;
    const bool row_ok = r < e.M;
    const long long rbase = row_ok ? (r / e.out.rc) * e.out.s1 + (r % e.out.rc) * e.out.s2 : 0;
    const bool split_cols = e.out.kc != 1;
    const bool stage_cols = !split_cols && e.out.t1 == 1;
    for (int c0 = 0; c0 < BN; c0 += 32) {
      uint32_t v[32];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
          "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
            "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
            "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
          : "r"(taddr)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (!part && stage_cols) {
        // columns contiguous in the output: pass the warp's 32 x 32 block through shared
        // memory (the pipeline stages are idle now) and store each row with the lanes
        // along its columns
        float* blk = reinterpret_cast<float*>(smem) + warp * (32 * 33);
#pragma unroll
        for (int i = 0; i < 32; ++i) blk[lane * 33 + i] = __uint_as_float(v[i]);
        __syncwarp();
        const int c = nt * BN + c0 + lane;
        const float bias_c = (e.bias && c < e.N) ? __ldg(e.bias + c) : 0.f;
        for (int rr = 0; rr < 32; ++rr) {
          const long long rw = (long long)mt * BM + warp * 32 + rr;
          if (rw < e.M && c < e.N) {
            const long long o = (rw / e.out.rc) * e.out.s1 + (rw % e.out.rc) * e.out.s2 + c;
            float z = blk[rr * 33 + lane] * e.scale + bias_c;
            if (e.add) z += e.add[o];
            if (e.accumulate) z += e.y[o];
            e.y[o] = z;
            if (e.act) e.act[o] = gelu_t(z);
          }
        }
        __syncwarp();
      } else if (part) {
        float* pp = part + ((size_t)split * tiles + tile) * (size_t)(BM * BN) + (size_t)(warp * 32 + lane) * BN + c0;
#pragma unroll
        for (int i = 0; i < 32; ++i) pp[i] = __uint_as_float(v[i]);
      } else if (row_ok) {
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          const int c = nt * BN + c0 + i;
          if (c < e.N) {
            const long long o =
                rbase + (split_cols ? (long long)(c / e.out.kc) * e.out.t1 + (long long)(c % e.out.kc) * e.out.t2
                                    : (long long)c * e.out.t1);
            float z = __uint_as_float(v[i]) * e.scale;
            if (e.bias) z += __ldg(e.bias + c);
            if (e.add) z += e.add[o];
            if (e.accumulate) z += e.y[o];
            e.y[o] = z;
            if (e.act) e.act[o] = gelu_t(z);
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN) : "memory");
}

// Sums the split-K partials in split order and applies the epilogue; one thread per (row, column).
__global__ void splitk_reduce_kernel(const float* __restrict__ part, int splits, int tiles, int ntiles_n, int bn, Epi e) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= e.M * (long long)e.N) return;
  const long long r = i / e.N;
  const int c = (int)(i % e.N);
  const int mt = (int)(r / BM), nt = c / bn;
  const int tile = mt * ntiles_n + nt;
  const size_t off = (size_t)tile * (BM * bn) + (size_t)(r % BM) * bn + (c % bn);
  float z = 0.f;
  for (int s = 0; s < splits; ++s) z += part[(size_t)s * tiles * (BM * bn) + off];
  z *= e.scale;
  const long long o = addr_of(e.out, r, c);
  if (e.bias) z += e.bias[c];
  if (e.add) z += e.add[o];
  if (e.accumulate) z += e.y[o];
  e.y[o] = z;
  if (e.act) e.act[o] = gelu_t(z);
}

template <int BN>
cudaError_t launch_gemm_bn(const uint8_t* a, const uint8_t* b, long long mtiles, int ntiles, int kblocks, int kper,
                           float* part, const Epi& e, int* err, cudaStream_t st, int batch = 1) {
  // the shared-memory attribute is set once per device (it belongs to the device's context)
  static std::atomic<unsigned long long> configured{0};
  int dev = 0;
  cudaError_t c0 = cudaGetDevice(&dev);
  if (c0 != cudaSuccess) return c0;
  const unsigned long long bit = 1ull << (dev & 63);
  if (!(configured.load(std::memory_order_acquire) & bit)) {
    cudaError_t c = cudaFuncSetAttribute(gemm_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg<BN>::SMEM);
    if (c != cudaSuccess) return c;
    configured.fetch_or(bit, std::memory_order_release);
  }
  const int splits = (kblocks + kper - 1) / kper;
  gemm_kernel<BN><<<(unsigned)(mtiles * ntiles * splits * batch), 128, Cfg<BN>::SMEM, st>>>(
      a, b, kblocks, ntiles, (int)(mtiles * ntiles), kper, part, e, err);
  if (part) {
    const long long n = e.M * (long long)e.N;
    splitk_reduce_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(part, splits, (int)(mtiles * ntiles), ntiles, BN,
                                                                      e);
  }
  return cudaGetLastError();
}

}  // namespace tg

// ------------------------------------------------------------------ host side
namespace {
int bn_for(int n) { return n <= 32 ? 32 : n <= 64 ? 64 : n <= 128 ? 128 : 256; }
}  // namespace

int TcGemm::reserve(size_t a_bytes, size_t b_bytes) {
  if (!err) {
    if (cudaMalloc(&err, sizeof(int)) != cudaSuccess || cudaMemset(err, 0, sizeof(int)) != cudaSuccess)
      return MSX_ERR_ALLOC;
  }
  if (a_bytes > a_cap) {
    if (a_img) cudaFree(a_img);
    a_img = nullptr;
    a_cap = 0;
    if (cudaMalloc(&a_img, a_bytes) != cudaSuccess) return MSX_ERR_ALLOC;
    a_cap = a_bytes;
  }
  if (b_bytes > b_cap) {
    if (b_img) cudaFree(b_img);
    b_img = nullptr;
    b_cap = 0;
    if (cudaMalloc(&b_img, b_bytes) != cudaSuccess) return MSX_ERR_ALLOC;
    b_cap = b_bytes;
  }
  return MSX_OK;
}

void TcGemm::release() {
  for (void* p : {(void*)a_img, (void*)b_img, (void*)err, (void*)part})
    if (p) cudaFree(p);
  a_img = b_img = nullptr;
  err = nullptr;
  part = nullptr;
  a_cap = b_cap = part_cap = 0;
}

int TcGemm::run(const float* a, Addr aa, const float* b, Addr ba, long long M, int N, long long K, const Epi& epi,
                cudaStream_t st, int ksplit) {
  if (M <= 0 || N <= 0 || K <= 0 || N > 4096 || ksplit < 1) return MSX_ERR_INVALID;
  const int bn = bn_for(N);
  const long long mtiles = (M + tg::BM - 1) / tg::BM;
  const int ntiles = (N + bn - 1) / bn;
  const long long kbl = (K + tg::BK - 1) / tg::BK;
  if (kbl > (1LL << 30) || mtiles * ntiles > (1LL << 30)) return MSX_ERR_INVALID;
  const int kblocks = (int)kbl;
  int kper = kblocks;
  if (ksplit > 1) kper = (kblocks + ksplit - 1) / ksplit;
  const int splits = (kblocks + kper - 1) / kper;
  const size_t a_bytes = (size_t)mtiles * kblocks * tg::A_BYTES;
  const size_t b_bytes = (size_t)ntiles * kblocks * bn * tg::BK * 2;
  int rc = reserve(a_bytes, b_bytes);
  if (rc != MSX_OK) return rc;
  float* pbuf = nullptr;
  if (splits > 1) {
    const size_t need = (size_t)splits * mtiles * ntiles * tg::BM * bn;
    if (need > part_cap) {
      if (part) cudaFree(part);
      part = nullptr;
      part_cap = 0;
      if (cudaMalloc(&part, need * sizeof(float)) != cudaSuccess) return MSX_ERR_ALLOC;
      part_cap = need;
    }
    pbuf = part;
  }
  const long long a_rows = mtiles * tg::BM, b_rows = (long long)ntiles * bn;
  const long long a_thr = a_rows * kblocks * (tg::BK / 8), b_thr = b_rows * kblocks * (tg::BK / 8);
  tg::pack_kernel<<<(unsigned)((a_thr + 255) / 256), 256, 0, st>>>(a, aa, M, K, tg::BM, a_rows, kblocks,
                                                                   reinterpret_cast<uint4*>(a_img));
  tg::pack_kernel<<<(unsigned)((b_thr + 255) / 256), 256, 0, st>>>(b, ba, N, K, bn, b_rows, kblocks,
                                                                   reinterpret_cast<uint4*>(b_img));
  Epi e = epi;
  e.M = M;
  e.N = N;
  const uint8_t* ai = reinterpret_cast<const uint8_t*>(a_img);
  const uint8_t* bi = reinterpret_cast<const uint8_t*>(b_img);
  cudaError_t c;
  switch (bn) {
    case 32: c = tg::launch_gemm_bn<32>(ai, bi, mtiles, ntiles, kblocks, kper, pbuf, e, err, st); break;
    case 64: c = tg::launch_gemm_bn<64>(ai, bi, mtiles, ntiles, kblocks, kper, pbuf, e, err, st); break;
    case 128: c = tg::launch_gemm_bn<128>(ai, bi, mtiles, ntiles, kblocks, kper, pbuf, e, err, st); break;
    default: c = tg::launch_gemm_bn<256>(ai, bi, mtiles, ntiles, kblocks, kper, pbuf, e, err, st); break;
  }
  return c == cudaSuccess ? MSX_OK : MSX_ERR_CUDA;
}

int TcGemm::run_batched(const float* a, Addr aa, long long a_bs, const float* b, Addr ba, long long b_bs, long long M,
                        int N, long long K, const Epi& epi, long long y_bs, int batch, cudaStream_t st) {
  if (batch < 1 || M <= 0 || N <= 0 || K <= 0 || N > 4096) return MSX_ERR_INVALID;
  const int bn = bn_for(N);
  const long long mtiles = (M + tg::BM - 1) / tg::BM;
  const int ntiles = (N + bn - 1) / bn;
  const long long kbl = (K + tg::BK - 1) / tg::BK;
  if (kbl > (1LL << 30) || mtiles * ntiles * batch > (1LL << 30)) return MSX_ERR_INVALID;
  const int kblocks = (int)kbl;
  const size_t a_bytes = (size_t)batch * mtiles * kblocks * tg::A_BYTES;
  const size_t b_bytes = (size_t)batch * ntiles * kblocks * bn * tg::BK * 2;
  int rc = reserve(a_bytes, b_bytes);
  if (rc != MSX_OK) return rc;
  const long long a_rows = mtiles * tg::BM, b_rows = (long long)ntiles * bn;
  const long long a_thr = a_rows * kblocks * (tg::BK / 8) * batch, b_thr = b_rows * kblocks * (tg::BK / 8) * batch;
  tg::pack_kernel<<<(unsigned)((a_thr + 255) / 256), 256, 0, st>>>(a, aa, M, K, tg::BM, a_rows, kblocks,
                                                                   reinterpret_cast<uint4*>(a_img), batch, a_bs);
  tg::pack_kernel<<<(unsigned)((b_thr + 255) / 256), 256, 0, st>>>(b, ba, N, K, bn, b_rows, kblocks,
                                                                   reinterpret_cast<uint4*>(b_img), batch, b_bs);
  Epi e = epi;
  e.M = M;
  e.N = N;
  e.ybs = y_bs;
  const uint8_t* ai = reinterpret_cast<const uint8_t*>(a_img);
  const uint8_t* bi = reinterpret_cast<const uint8_t*>(b_img);
  cudaError_t c;
  switch (bn) {
    case 32: c = tg::launch_gemm_bn<32>(ai, bi, mtiles, ntiles, kblocks, kblocks, nullptr, e, err, st, batch); break;
    case 64: c = tg::launch_gemm_bn<64>(ai, bi, mtiles, ntiles, kblocks, kblocks, nullptr, e, err, st, batch); break;
    case 128: c = tg::launch_gemm_bn<128>(ai, bi, mtiles, ntiles, kblocks, kblocks, nullptr, e, err, st, batch); break;
    default: c = tg::launch_gemm_bn<256>(ai, bi, mtiles, ntiles, kblocks, kblocks, nullptr, e, err, st, batch); break;
  }
  return c == cudaSuccess ? MSX_OK : MSX_ERR_CUDA;
}

int TcGemm::check() {
  if (!err) return MSX_OK;
  int h = 0;
  if (cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return MSX_ERR_CUDA;
  if (h) {
    cudaMemset(err, 0, sizeof(int));
    return MSX_ERR_TIMEOUT;
  }
  return MSX_OK;
}

}  // namespace msx

namespace {
thread_local msx::TcGemm g_gemm;  // scratch of msx_gemm_bf16, one per host thread
}

extern "C" int msx_gemm_bf16(const float* a_dev, int lda, const float* b_dev, int ldb, int m, int n, int k,
                             float* c_dev, int ldc, const float* bias_dev, int accumulate, void* stream) {
  if (!a_dev || !b_dev || !c_dev || m <= 0 || n <= 0 || k <= 0 || lda < k || ldb < k || ldc < n || n > 4096) {
    msx::set_last_error("gemm_bf16: bad arguments (need m, n, k > 0, n <= 4096, leading dimensions >= row lengths)");
    return MSX_ERR_INVALID;
  }
  msx::Epi e{};
  e.y = c_dev;
  e.out = msx::rowmajor(ldc);
  e.bias = bias_dev;
  e.accumulate = accumulate ? 1 : 0;
  e.scale = 1.f;
  // long K with few output tiles: split K over CTAs
  const long long tiles = ((m + 127) / 128) * (long long)((n + 255) / 256);
  const int ksplit = (k >= 4096 && tiles < 64) ? (int)((k / 2048) < 64 ? (k / 2048) : 64) : 1;
  const int rc = g_gemm.run(a_dev, msx::rowmajor(lda), b_dev, msx::rowmajor(ldb), m, n, k, e, (cudaStream_t)stream,
                            ksplit);
  if (rc == MSX_ERR_ALLOC) msx::set_last_error("gemm_bf16: operand image allocation failed");
  else if (rc == MSX_ERR_CUDA) msx::set_last_error("gemm_bf16: launch failed");
  else if (rc != MSX_OK) msx::set_last_error("gemm_bf16: bad sizes");
  return rc;
}

extern "C" int msx_gemm_check(void) {
  const int rc = g_gemm.check();
  if (rc == MSX_ERR_TIMEOUT) msx::set_last_error("a tensor-core GEMM wait gave up");
  return rc;
}
