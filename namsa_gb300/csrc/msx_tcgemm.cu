// General BF16 GEMM on the 5th-generation tensor cores (tcgen05) with FP32
// accumulation, for the contractions of the learned corrector (pointwise
// channel mixing, its weight gradients, the per-mode complex channel mixing and
// the partial DFT stages of its spectral layers).
//
//   D (M x N) = A (M x K) . B (N x K)^T,   A and B rounded to bfloat16.
//
// Operands are read from FP32 arrays of any 2-level strided layout: element
// (r, k) of an operand sits at (r / rc) * s1 + (r % rc) * s2 + (k / kc) * t1 +
// (k % kc) * t2.  The tensor cores read both from shared memory in the K-major,
// 128-byte-swizzled layout (8-row atoms of 128 B, 16-byte chunk c of row r at
// chunk c ^ (r mod 8)).  Output element (r, c) is written at the same kind of
// strided address, so results land directly in pixel-major or transposed
// layouts.  Epilogue: z = acc (+ bias[c]) (+ add[r, c]); out = z or out += z;
// optionally act = gelu(z) (tanh form) into a second array.
//
// Main path (gemm_ws_kernel): a persistent, warp-specialised kernel; A is
// staged in FP32 by bulk or asynchronous copies and rounded to bfloat16 in
// shared memory, B comes from a small packed image (pack_kernel, or
// pack_cplx_kernel for the real embedding of a complex product) or, for the
// long-K weight gradients (N <= 32), is staged and rounded like A while K is
// split over the CTAs.  The per-tile kernel (gemm_kernel, both operands packed)
// remains for split-K products with N > 32.
#include "msx.h"
#include "msx_internal.h"

#include <cuda_bf16.h>

#include <algorithm>
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

// Real embedding of a complex product, packed like pack_kernel: B is N x K with
// N = 2 hn, K = 2 hk; row n = (bn, i) = (n / hn, n % hn), column k = (bk, j); the
// element is src[i si + j sj + (bn xor bk)] (a complex array, parts interleaved),
// negated where (bn, bk) = (0, 1) (neg = 1) or (1, 0) (neg = 2).  With the
// right orientation of src, D = A B^T then gives real and imaginary parts of a
// complex product in one GEMM: [Re, Im] of x z^T is [xr, xi] against rows
// [zr, -zi] and [zi, zr].
__global__ void pack_cplx_kernel(const float* __restrict__ src, long long si, long long sj, long long src_bs, int hn,
                                 int hk, int neg, int tile_rows, int rows_pad, int kblocks, uint4* __restrict__ img,
                                 int batch) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long chunks = (long long)kblocks * (BK / 8);
  const long long per = (long long)rows_pad * chunks;
  if (i >= per * batch) return;
  const long long bt = i / per;
  i -= bt * per;
  src += bt * src_bs;
  img += bt * (per * 8 * 2 / 16);
  const int r = (int)(i / chunks);
  const int ch = (int)(i - (long long)r * chunks);
  const int k0 = ch * 8;
  __align__(16) __nv_bfloat16 v[8];
  const int N = 2 * hn, K = 2 * hk;
  const int bn = r / hn, ii = r - (r / hn) * hn;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int k = k0 + j;
    float x = 0.f;
    if (r < N && k < K) {
      const int bk = k / hk, jj = k - bk * hk;
      x = __ldg(src + ii * si + jj * sj + (bn ^ bk));
      if ((neg == 1 && bn == 0 && bk == 1) || (neg == 2 && bn == 1 && bk == 0)) x = -x;
    }
    v[j] = __float2bfloat16_rn(x);
  }
  const int tile = r / tile_rows, row = r - tile * tile_rows, kb = k0 / BK;
  const size_t byte = ((size_t)tile * kblocks + kb) * ((size_t)tile_rows * BK * 2) + sw128(row, k0 % BK);
  img[byte / 16] = *reinterpret_cast<const uint4*>(v);
}

// Per-tile kernel: one CTA of 128 threads per 128 x BN tile of D and K split.
// Thread 0 moves each (tile, K block) of the packed images with one bulk copy into
// STAGES stages (full/empty mbarriers), thread 32 issues tcgen05.mma (M = 128,
// N = BN, K = 16) and commits each stage to its empty barrier; all four warps read
// the accumulator with tcgen05.ld (warp w owns TMEM lanes 32w..32w+31 = tile rows).
// Every wait is bounded; on a timeout the kernel sets *err, waits (bounded) for its
// MMAs, frees its tensor memory and returns.
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

// Sums the split-K partials and applies the epilogue; one warp per (row, column): lane l
// adds splits l, l + 32, ... in order, then the lanes combine by a fixed butterfly, so
// the result does not depend on scheduling.
constexpr int REDUCE_WARPS = 8;  // outputs per block of the reduction
__global__ void splitk_reduce_kernel(const float* __restrict__ part, int splits, int tiles, int ntiles_n, int bn, Epi e) {
  const long long i = (long long)blockIdx.x * REDUCE_WARPS + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= e.M * (long long)e.N) return;  // warp-uniform
  const long long r = i / e.N;
  const int c = (int)(i % e.N);
  const int mt = (int)(r / BM), nt = c / bn;
  const int tile = mt * ntiles_n + nt;
  const size_t off = (size_t)tile * (BM * bn) + (size_t)(r % BM) * bn + (c % bn);
  float z = 0.f;
  for (int s = lane; s < splits; s += 32) z += part[(size_t)s * tiles * (BM * bn) + off];
#pragma unroll
  for (int m = 16; m > 0; m >>= 1) z += __shfl_xor_sync(0xffffffffu, z, m);
  if (lane != 0) return;
  z *= e.scale;
  const long long o = addr_of(e.out, r, c);
  if (e.bias) z += e.bias[c];
  if (e.add) z += e.add[o];
  if (e.accumulate) z += e.y[o];
  e.y[o] = z;
  if (e.act) e.act[o] = gelu_t(z);
}

// ------------------------------------------------------------ persistent, warp-specialised GEMM
// One CTA of 416 threads per SM loops over the output tiles (batch, mt, nt) =
// blockIdx.x, blockIdx.x + gridDim.x, ... (nt fastest):
//   warps 0-3   operand loaders: bring the FP32 rows of A for a K block into an FP32
//               staging slot (bulk copies where A's rows or row groups are contiguous,
//               else 4-byte asynchronous copies), then round them to bfloat16 into the
//               swizzled stage (no packing pass over A); thread 0 also moves the stage's
//               packed B block with one bulk copy;
//   warps 4-11  epilogue, two groups of four taking alternate tiles; warp w reads
//               TMEM lanes 32 (w mod 4) .. + 31 (tile rows);
//   warp 12     holds two BN-column accumulators in TMEM; lane 0 issues the MMAs.
// The accumulators alternate between tiles, so a tile's epilogue overlaps the next
// tile's loads and MMAs.  Barriers: afull[slot] (staging slot filled: 128 loader
// arrivals with the bulk bytes), full[s] (128 loader arrivals: bfloat16 A written),
// bfull[s] (the B bytes), empty[s] (MMA commit), accf[b] (MMA commit of accumulator
// b), acce[b] (one arrival per warp of the epilogue group).  Rows of A at or past M
// are not converted (an MMA row depends on its own A row only, and those rows are not
// stored); K steps of 16 past K are not issued, and the rest of the last K step is
// zero.  Every wait is bounded; the loaders take each decision together (a barrier
// reduction), on a timeout a role sets *err and stops, the MMA issuer waits (bounded)
// for its MMAs and the loaders for their copies before the tensor memory is freed.
namespace ws {
constexpr int LOADERS = 128;  // warps 0-3
constexpr int EPI_WARPS = 8;  // warps 4-11
constexpr int MMA_WARP = 12;
constexpr int THREADS = 13 * 32;
constexpr int SLOT_FLOATS = BM * BK;  // one FP32 staging slot (32 KB)
template <int BN>
struct Cfg {
  static constexpr int STAGES = BN == 256 ? 2 : 3;  // bfloat16 operand stages
  static constexpr int DEPTH = BN <= 64 ? 3 : 2;    // FP32 staging slots: A stages in flight
  static constexpr int B_BYTES = BN * BK * 2;
  static constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
  static constexpr int BROWS = BN;                          // rows of a B tile
  static constexpr int BSLOT_FLOATS = BN == 32 ? 32 * BK : 0;  // FP32 B staging slot (B from FP32: BN = 32)
  static constexpr int EPI_FLOATS = EPI_WARPS * 32 * 33;
  static constexpr int SMEM =
      STAGES * STAGE_BYTES + DEPTH * (SLOT_FLOATS + BSLOT_FLOATS) * 4 + EPI_FLOATS * 4 + 1024;
  static constexpr uint32_t TMEM_COLS = 2 * BN;
};

__device__ __forceinline__ void cp4(float* dst, const float* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
// the barrier's phase completes (for this thread's arrival) once this thread's copies have landed
__device__ __forceinline__ void cp_arrive(uint64_t* bar) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// barrier 1 over the 128 loader threads: true on all of them iff `ok` on all of them
__device__ __forceinline__ bool loaders_all(bool ok) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.and.pred q, 1, 128, p;\n selp.u32 %0, 1, 0, q;\n}\n"
      : "=r"(r)
      : "r"((uint32_t)ok)
      : "memory");
  return r != 0;
}
__device__ __forceinline__ void loaders_sync() { asm volatile("bar.sync 1, 128;" ::: "memory"); }

__device__ __forceinline__ void store_chunk(uint8_t* sa, int row, int ch, const float (&x)[8]) {
  __align__(16) __nv_bfloat162 h[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) h[j] = __floats2bfloat162_rn(x[2 * j], x[2 * j + 1]);
  *reinterpret_cast<uint4*>(sa + sw128(row, ch * 8)) = *reinterpret_cast<const uint4*>(h);
}

// How the rows r0 .. r0 + R - 1 of an operand (R = 128 for A, BN for B), K block kb
// (nk = min(64, K - 64 kb) values), reach a staging slot:
//   ROWRUN   k contiguous: thread i copies row r0 + i to slot[i][0 .. nk) with one bulk
//            copy (16-byte aligned runs), else with plain loads;
//   GROUPRUN rows contiguous in groups of rc with k stride rc (a group's K block is one
//            run of nk * rc values; rc may be all the operand's rows): thread i < R / rc
//            copies group i to slot[i * 64 rc ..], element (k, r mod rc) at k rc + r mod rc;
//   GENERIC  thread i copies row r0 + i value by value (4-byte asynchronous copies),
//            element (r, k) at ((k / 8) R + i) 8 + k mod 8;
//   TILERUN  rows of K <= 64 values stored back to back: thread 0 copies the tile's rows
//            as one run (or the loaders load it, when the run is not 16-byte aligned),
//            element (r, k) at r K + k.
// Bulk bytes are announced on the slot's barrier without arriving; each loader thread
// arrives once per slot after its copies of A and B are issued (through the async-copy
// unit when it issued 4-byte copies, so the arrival waits for them).
enum { ROWRUN = 0, GROUPRUN = 1, GENERIC = 2, TILERUN = 3 };

__device__ __forceinline__ void expect_tx_only(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

struct Op {
  const float* p;  // FP32 operand (batch 0)
  Addr a;
  long long bs;    // batch stride (floats)
  long long rows;  // M or N
  int mode, rc;
};

__host__ __device__ inline void op_mode(Op& o, int tile_rows, long long k_total) {
  const Addr& a = o.a;
  o.rc = (int)a.rc;
  o.mode = GENERIC;
  if (a.kc == 1 && a.t1 == 1) {
    o.mode = ROWRUN;
    if (a.rc == 1 && k_total <= BK && a.s1 == k_total) o.mode = TILERUN;
    return;
  }
  long long g = -1;
  if (a.s2 == 1 && a.rc > 1) g = a.rc;
  else if (a.rc == 1 && a.s1 == 1) g = o.rows;  // all rows contiguous
  if (g > 0 && g <= tile_rows && a.kc == 1 && a.t1 == g && g % 4 == 0 && tile_rows % g == 0 && o.rows % g == 0 &&
      (g == o.rows || a.s1 % 4 == 0) && o.bs % 4 == 0 && (reinterpret_cast<uintptr_t>(o.p) & 15u) == 0) {
    o.mode = GROUPRUN;
    o.rc = (int)g;
  }
}

// Thread i's copies of rows r0 .. r0 + R - 1 of operand o (batch bt) into slot stg;
// returns true when it issued 4-byte asynchronous copies.
template <int R>
__device__ __forceinline__ bool issue_op(float* stg, uint64_t* bar, const Op& o, long long bt, long long K,
                                         long long r0, int kb, int i) {
  const long long kb0 = (long long)kb * BK;
  const int nk = (int)(K - kb0 < BK ? K - kb0 : BK);
  const float* const P = o.p + bt * o.bs;
  const Addr& a = o.a;
  if (o.mode == TILERUN) {
    const long long nrow = o.rows - r0 < R ? o.rows - r0 : R;
    const float* src = P + r0 * a.s1;
    const int n = (int)(nrow * nk);
    if (nrow > 0 && (n & 3) == 0 && (reinterpret_cast<uintptr_t>(src) & 15u) == 0) {
      if (i == 0) {
        expect_tx_only(bar, (uint32_t)n * 4u);
        bulk_g2s(stg, src, (uint32_t)n * 4u, bar);
      }
    } else {
      for (int j = i; j < n; j += LOADERS) stg[j] = __ldg(src + j);
    }
    return false;
  }
  if (i >= R && o.mode != GROUPRUN) return false;
  if (o.mode == ROWRUN) {
    const long long r = r0 + i;
    if (r < o.rows) {
      const float* src = P + (r / a.rc) * a.s1 + (r % a.rc) * a.s2 + kb0;
      if ((nk & 3) == 0 && (reinterpret_cast<uintptr_t>(src) & 15u) == 0) {
        expect_tx_only(bar, (uint32_t)nk * 4u);
        bulk_g2s(stg + i * BK, src, (uint32_t)nk * 4u, bar);
      } else {
        for (int k = 0; k < nk; ++k) stg[i * BK + k] = __ldg(src + k);
      }
    }
    return false;
  }
  if (o.mode == GROUPRUN) {
    const int rc = o.rc;
    const long long r = r0 + (long long)i * rc;
    if (i < R / rc && r < o.rows) {
      const uint32_t bytes = (uint32_t)nk * (uint32_t)rc * 4u;
      expect_tx_only(bar, bytes);
      bulk_g2s(stg + i * BK * rc, P + (r / a.rc) * a.s1 + kb0 * a.t1, bytes, bar);
    }
    return false;
  }
  const long long r = r0 + i;
  if (r >= o.rows) return false;
  const float* row = P + (r / a.rc) * a.s1 + (r % a.rc) * a.s2;
  long long q = kb0 / a.kc, rem = kb0 - q * a.kc;
  for (int k = 0; k < nk; ++k) {
    cp4(stg + ((k >> 3) * R + i) * 8 + (k & 7), row + q * a.t1 + rem * a.t2);
    if (++rem == a.kc) { rem = 0; ++q; }
  }
  return nk > 0;
}

// Converts the rows r0 .. r0 + R - 1 of a filled slot into the bfloat16 operand image at
// sa (R rows of 128 bytes, swizzled); any loader thread may convert any value.
template <int R>
__device__ __forceinline__ void convert_op(uint8_t* sa, const float* stg, const Op& o, long long K, long long r0,
                                           int kb, int i) {
  const long long kb0 = (long long)kb * BK;
  const int nk = (int)(K - kb0 < BK ? K - kb0 : BK);
  const int nch = nk >= BK ? 8 : 2 * ((nk + 15) / 16);  // chunks the MMAs read
  const int nrow = (int)(o.rows - r0 < R ? o.rows - r0 : R);  // rows to convert
  if (nrow <= 0) return;
  if (o.mode == ROWRUN || o.mode == TILERUN) {
    const int ld = o.mode == ROWRUN ? BK : nk;
    for (int t = i; t < nrow * nch; t += LOADERS) {  // (row, chunk), chunk fastest
      const int row = t / nch, ch = t - (t / nch) * nch;
      const float* src = stg + row * ld + ch * 8;
      float x[8];
      if (ch * 8 + 8 <= nk && (ld & 3) == 0) {
        const float4 lo = *reinterpret_cast<const float4*>(src), hi = *reinterpret_cast<const float4*>(src + 4);
        x[0] = lo.x; x[1] = lo.y; x[2] = lo.z; x[3] = lo.w; x[4] = hi.x; x[5] = hi.y; x[6] = hi.z; x[7] = hi.w;
      } else {
#pragma unroll
        for (int e = 0; e < 8; ++e) x[e] = ch * 8 + e < nk ? src[e] : 0.f;
      }
      store_chunk(sa, row, ch, x);
    }
  } else if (o.mode == GROUPRUN) {
    const int rc = o.rc;
    for (int t = i; t < nrow * nch; t += LOADERS) {  // (row, chunk), row fastest
      const int ch = t / nrow, row = t - ch * nrow;
      const float* src = stg + (row / rc) * (BK * rc) + (ch * 8) * rc + (row % rc);
      float x[8];
#pragma unroll
      for (int e = 0; e < 8; ++e) x[e] = ch * 8 + e < nk ? src[e * rc] : 0.f;
      store_chunk(sa, row, ch, x);
    }
  } else {
    for (int t = i; t < nrow * nch; t += LOADERS) {  // (row, chunk), row fastest
      const int ch = t / nrow, row = t - ch * nrow;
      const float* src = stg + (ch * R + row) * 8;
      float x[8];
#pragma unroll
      for (int e = 0; e < 8; ++e) x[e] = ch * 8 + e < nk ? src[e] : 0.f;
      store_chunk(sa, row, ch, x);
    }
  }
}
}  // namespace ws

// 16 consecutive accumulator columns of this warp's 32 TMEM lanes (one per lane).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
        "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// The work of one launch.  Items (batch, split, mt, nt), nt fastest; item `split` sums K
// blocks [split * kper, min(kblocks, (split + 1) * kper)).  B comes either packed
// (b_img, one image per batch) or, for BN = 32, as an FP32 operand (b.p) staged and
// rounded like A.  With part set the epilogue writes raw partial tiles
// part[((batch * splits + split) * tiles + tile) * 128 * BN + row * BN + col] instead.
struct WsArgs {
  ws::Op a, b;
  const uint8_t* b_img;
  long long K;
  int kblocks, kper, splits, ntiles;
  long long mtiles, items;
  float* part;
};

template <int BN>
__global__ void __launch_bounds__(ws::THREADS, 1) gemm_ws_kernel(WsArgs w, Epi e, int* __restrict__ err) {
  using C = ws::Cfg<BN>;
  constexpr int ST = C::STAGES, D = C::DEPTH;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  float* const stg0 = reinterpret_cast<float*>(smem + ST * C::STAGE_BYTES);
  float* const stgb = stg0 + D * ws::SLOT_FLOATS;  // B staging (BN = 32 only)
  float* const epi_buf = stgb + D * C::BSLOT_FLOATS;
  __shared__ uint64_t full[ST], bfull[ST], empty[ST], afull[D], accf[2], acce[2], drain;
  __shared__ uint32_t tmem_base;
  __shared__ long long off_s[ws::EPI_WARPS][32];  // epilogue: per warp, 32 row (or column) offsets
  __shared__ float bias_s[ws::EPI_WARPS][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool fuse_b = w.b_img == nullptr;
  if (fuse_b && C::BSLOT_FLOATS == 0) {  // host error: FP32 B needs BN = 32
    if (threadIdx.x == 0) atomicOr(err, 64);
    return;
  }
  if (warp == ws::MMA_WARP) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(C::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (threadIdx.x == 0) {
    for (int s = 0; s < ST; ++s) {
      mbar_init(&full[s], ws::LOADERS);
      mbar_init(&bfull[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int d = 0; d < D; ++d) mbar_init(&afull[d], ws::LOADERS);
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], 4);
    }
    mbar_init(&drain, 1);
    fence_mbar_init();
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;
  const long long tiles = w.mtiles * w.ntiles;
  // item -> (batch, split, mt, nt) and its K blocks
  auto decode = [&](long long it, long long& bt, int& split, long long& mt, int& nt, int& kb0, int& kb1) {
    nt = (int)(it % w.ntiles);
    const long long t2 = it / w.ntiles;
    mt = t2 % w.mtiles;
    const long long t3 = t2 / w.mtiles;
    split = (int)(t3 % w.splits);
    bt = t3 / w.splits;
    kb0 = split * w.kper;
    kb1 = kb0 + w.kper < w.kblocks ? kb0 + w.kper : w.kblocks;
  };

  if (warp < 4) {  // operand loaders
    const int i = threadIdx.x;
    // stages of this CTA in order: a cursor over (item, K block)
    struct Cur {
      long long it, bt, mt;
      int nt, split, kb, kb1;
    };
    auto start = [&](Cur& c, long long it) {
      c.it = it;
      if (it < w.items) decode(it, c.bt, c.split, c.mt, c.nt, c.kb, c.kb1);
    };
    auto advance = [&](Cur& c) {
      if (++c.kb >= c.kb1) start(c, c.it + gridDim.x);
    };
    auto issue = [&](const Cur& c, long long g) {
      const int d = (int)(g % D);
      bool cp = ws::issue_op<BM>(stg0 + d * ws::SLOT_FLOATS, &afull[d], w.a, c.bt, w.K, c.mt * BM, c.kb, i);
      if (fuse_b)
        cp |= ws::issue_op<C::BROWS>(stgb + d * C::BSLOT_FLOATS, &afull[d], w.b, c.bt, w.K, (long long)c.nt * BN,
                                     c.kb, i);
      if (cp) ws::cp_arrive(&afull[d]);
      else mbar_arrive(&afull[d]);
    };
    Cur cur, ahead;
    start(cur, blockIdx.x);
    start(ahead, blockIdx.x);
    long long issued = 0;
    for (; issued < D && ahead.it < w.items; ++issued, advance(ahead)) issue(ahead, issued);
    long long g = 0;
    for (; cur.it < w.items; ++g, advance(cur)) {
      const int s = (int)(g % ST), d = (int)(g % D);
      bool ok = mbar_wait_bounded(&afull[d], (uint32_t)((g / D) & 1));
      if (ok && g >= ST) ok = mbar_wait_bounded(&empty[s], (uint32_t)(((g / ST) - 1) & 1));
      if (!ws::loaders_all(ok)) {
        if (i == 0) atomicOr(err, 2);
        break;
      }
      uint8_t* st = smem + s * C::STAGE_BYTES;
      if (fuse_b) {
        ws::convert_op<C::BROWS>(st + A_BYTES, stgb + d * C::BSLOT_FLOATS, w.b, w.K, (long long)cur.nt * BN, cur.kb,
                                 i);
      } else if (i == 0) {
        mbar_expect_tx(&bfull[s], C::B_BYTES);
        bulk_g2s(st + A_BYTES, w.b_img + (((size_t)cur.bt * w.ntiles + cur.nt) * w.kblocks + cur.kb) * C::B_BYTES,
                 C::B_BYTES, &bfull[s]);
      }
      ws::convert_op<BM>(st, stg0 + d * ws::SLOT_FLOATS, w.a, w.K, cur.mt * BM, cur.kb, i);
      fence_proxy_async();  // the tensor cores read the stage through the async proxy
      mbar_arrive(&full[s]);
      if (fuse_b && i == 0) mbar_arrive(&bfull[s]);
      ws::loaders_sync();  // every loader is done with slot d
      if (ahead.it < w.items) {
        issue(ahead, issued++);
        advance(ahead);
      }
    }
    // copies in flight land before the CTA's shared memory is released
    for (long long j = g; j < issued; ++j) mbar_wait_bounded(&afull[j % D], (uint32_t)((j / D) & 1));
    if (i == 0 && !fuse_b)
      for (long long j = g > ST ? g - ST : 0; j < g; ++j) mbar_wait_bounded(&bfull[j % ST], (uint32_t)((j / ST) & 1));
  } else if (warp == ws::MMA_WARP) {  // MMA issuer
    if (lane == 0) {
      long long g = 0, n = 0;
      bool ok = true;
      for (long long it = blockIdx.x; it < w.items && ok; it += gridDim.x, ++n) {
        long long bt, mt;
        int split, nt, kb0, kb1;
        decode(it, bt, split, mt, nt, kb0, kb1);
        const int buf = (int)(n & 1);
        if (n >= 2 && !mbar_wait_bounded(&acce[buf], (uint32_t)(((n >> 1) - 1) & 1))) {
          atomicOr(err, 16);
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t dacc = tmem + (uint32_t)(buf * BN);
        for (int kb = kb0; kb < kb1; ++kb, ++g) {
          const int s = (int)(g % ST);
          const uint32_t par = (uint32_t)((g / ST) & 1);
          if (!mbar_wait_bounded(&full[s], par) || !mbar_wait_bounded(&bfull[s], par)) {
            atomicOr(err, 4);
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t sa = smem_u32(smem + s * C::STAGE_BYTES);
          const long long krem = w.K - (long long)kb * BK;
          const int nk = krem >= BK ? BK / 16 : (int)((krem + 15) / 16);
          for (int j = 0; j < nk; ++j) {
            const uint32_t off = (uint32_t)j * 32u;
            const uint32_t acc = (kb > kb0 || j > 0) ? 1u : 0u;
            asm volatile(
                "{\n\t .reg .pred p;\n\t setp.ne.b32 p, %4, 0;\n\t"
                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dacc),
                "l"(sdesc(sa + off)), "l"(sdesc(sa + A_BYTES + off)), "r"(tg::Cfg<BN>::IDESC), "r"(acc)
                : "memory");
          }
          asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                           smem_u32(&empty[s]))
                       : "memory");
        }
        if (!ok) break;
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         smem_u32(&accf[buf]))
                     : "memory");
      }
      // every MMA issued has completed before the tensor memory and the stages are released
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(&drain))
                   : "memory");
      if (!mbar_wait_bounded(&drain, 0)) atomicOr(err, 32);
    }
    __syncwarp();
  } else {  // epilogue, warps 4-11: group eg takes this CTA's tiles n = eg, eg + 2, ... (accumulator eg)
    const int wi = warp - 4, eg = wi >> 2, q = warp & 3;
    float* const blk = epi_buf + wi * (32 * 33);
    const bool split_cols = e.out.kc != 1;
    const bool stage_cols = !split_cols && e.out.t1 == 1;
    const uint32_t lanes = (uint32_t)(q * 32) << 16;
    for (long long it = blockIdx.x + (long long)eg * gridDim.x, n = eg; it < w.items;
         it += 2LL * gridDim.x, n += 2) {
      const int buf = (int)(n & 1);
      if (!mbar_wait_bounded(&accf[buf], (uint32_t)((n >> 1) & 1))) {
        if (lane == 0) atomicOr(err, 8);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      long long bt, mt;
      int split, nt, kb0, kb1;
      decode(it, bt, split, mt, nt, kb0, kb1);
      const long long r = mt * BM + q * 32 + lane;
      const bool row_ok = r < e.M;
      if (w.part) {  // raw partial tile: each lane stores its row's BN values
        float* pp = w.part + ((bt * w.splits + split) * tiles + mt * w.ntiles + nt) * (long long)(BM * BN) +
                    (long long)(q * 32 + lane) * BN;
        for (int c0 = 0; c0 < BN; c0 += 16) {
          uint32_t v[16];
          tmem_ld16(tmem + lanes + (uint32_t)(buf * BN + c0), v);
          if (row_ok) {
#pragma unroll
            for (int j = 0; j < 16; j += 4)
              *reinterpret_cast<float4*>(pp + c0 + j) = make_float4(__uint_as_float(v[j]), __uint_as_float(v[j + 1]),
                                                                    __uint_as_float(v[j + 2]),
                                                                    __uint_as_float(v[j + 3]));
          }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(&acce[buf]);
        continue;
      }
      float* const ey = e.y + bt * e.ybs;
      const float* const eadd = e.add ? e.add + bt * e.ybs : nullptr;
      float* const eact = e.act ? e.act + bt * e.ybs : nullptr;
      const float* const p1 = eadd ? eadd : ey;  // first addend (add, else the accumulated output)
      const bool have_prev = eadd || e.accumulate, both = eadd && e.accumulate;
      const long long rbase = row_ok ? (r / e.out.rc) * e.out.s1 + (r % e.out.rc) * e.out.s2 : -1;
      // Offsets and biases of the warp's 32 rows or columns go through shared memory, and
      // the loads of add / accumulate are unconditional (an invalid element reads word 0
      // of its array), so 16 of them are in flight before the first is used.
      for (int c0 = 0; c0 < BN && nt * BN + c0 < e.N; c0 += 32) {
        const int c = nt * BN + c0 + lane;  // this lane's column
        const bool col_ok = c < e.N;
        const uint32_t taddr = tmem + lanes + (uint32_t)(buf * BN + c0);
        if (stage_cols) {
          // columns contiguous in the output: the warp's 32 x 32 block goes through shared
          // memory and each row is stored with the lanes along its columns
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            uint32_t v[16];
            tmem_ld16(taddr + (uint32_t)(h * 16), v);
#pragma unroll
            for (int j = 0; j < 16; ++j) blk[lane * 33 + h * 16 + j] = __uint_as_float(v[j]);
          }
          off_s[wi][lane] = rbase;
          __syncwarp();
          const float bias_c = (e.bias && col_ok) ? __ldg(e.bias + c) : 0.f;
#pragma unroll
          for (int h = 0; h < 32; h += 16) {
            float prev[16];
            if (have_prev) {
#pragma unroll
              for (int j = 0; j < 16; ++j) {
                const long long ro = off_s[wi][h + j];
                prev[j] = p1[(ro >= 0 && col_ok) ? ro + c : 0];
              }
              if (both) {
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                  const long long ro = off_s[wi][h + j];
                  prev[j] += ey[(ro >= 0 && col_ok) ? ro + c : 0];
                }
              }
            }
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              const long long ro = off_s[wi][h + j];
              if (ro >= 0 && col_ok) {
                float z = fmaf(blk[(h + j) * 33 + lane], e.scale, bias_c);
                if (have_prev) z += prev[j];
                ey[ro + c] = z;
                if (eact) eact[ro + c] = gelu_t(z);
              }
            }
          }
          __syncwarp();
        } else {
          // lanes along rows; the column offsets (this lane's for column c0 + lane) in shared memory
          off_s[wi][lane] = col_ok ? (split_cols ? (long long)(c / e.out.kc) * e.out.t1 +
                                                       (long long)(c % e.out.kc) * e.out.t2
                                                 : (long long)c * e.out.t1)
                                   : -1;
          bias_s[wi][lane] = (e.bias && col_ok) ? __ldg(e.bias + c) : 0.f;
          __syncwarp();
#pragma unroll
          for (int h = 0; h < 32; h += 16) {
            uint32_t v[16];
            tmem_ld16(taddr + (uint32_t)h, v);
            float prev[16];
            if (have_prev) {
#pragma unroll
              for (int j = 0; j < 16; ++j) {
                const long long cj = off_s[wi][h + j];
                prev[j] = p1[(row_ok && cj >= 0) ? rbase + cj : 0];
              }
              if (both) {
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                  const long long cj = off_s[wi][h + j];
                  prev[j] += ey[(row_ok && cj >= 0) ? rbase + cj : 0];
                }
              }
            }
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              const long long cj = off_s[wi][h + j];
              if (row_ok && cj >= 0) {
                float z = fmaf(__uint_as_float(v[j]), e.scale, bias_s[wi][h + j]);
                if (have_prev) z += prev[j];
                ey[rbase + cj] = z;
                if (eact) eact[rbase + cj] = gelu_t(z);
              }
            }
          }
          __syncwarp();
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(&acce[buf]);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == ws::MMA_WARP)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(C::TMEM_COLS) : "memory");
}

// Resident CTAs per SM of gemm_ws_kernel<BN> (shared memory, registers and the two
// accumulators' tensor-memory columns), per device.
template <int BN>
cudaError_t ws_slots(int& slots) {
  static std::atomic<int> cache[64];
  int dev = 0;
  cudaError_t c = cudaGetDevice(&dev);
  if (c != cudaSuccess) return c;
  const int d = dev & 63;
  int v = cache[d].load(std::memory_order_acquire);
  if (v <= 0) {
    c = cudaFuncSetAttribute(gemm_ws_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, ws::Cfg<BN>::SMEM);
    if (c != cudaSuccess) return c;
    // all of the unified L1 as shared memory
    c = cudaFuncSetAttribute(gemm_ws_kernel<BN>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
    if (c != cudaSuccess) return c;
    int occ = 0, sms = 0;
    c = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, gemm_ws_kernel<BN>, ws::THREADS, ws::Cfg<BN>::SMEM);
    if (c != cudaSuccess) return c;
    c = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (c != cudaSuccess) return c;
    occ = std::min(occ, (int)(512 / ws::Cfg<BN>::TMEM_COLS));
    if (occ < 1) return cudaErrorInvalidConfiguration;
    v = occ * sms;
    cache[d].store(v, std::memory_order_release);
  }
  slots = v;
  return cudaSuccess;
}

template <int BN>
cudaError_t launch_ws_bn(WsArgs w, const Epi& e, int* err, cudaStream_t st, long long batch) {
  int slots = 0;
  cudaError_t c = ws_slots<BN>(slots);
  if (c != cudaSuccess) return c;
  ws::op_mode(w.a, BM, w.K);
  if (!w.b_img) ws::op_mode(w.b, BN, w.K);
  w.items = batch * w.splits * w.mtiles * w.ntiles;
  const unsigned grid = (unsigned)std::min<long long>(w.items, slots);
  gemm_ws_kernel<BN><<<grid, ws::THREADS, ws::Cfg<BN>::SMEM, st>>>(w, e, err);
  return cudaGetLastError();
}

cudaError_t launch_ws(int bn, const WsArgs& w, const Epi& e, int* err, cudaStream_t st, long long batch) {
  switch (bn) {
    case 32: return launch_ws_bn<32>(w, e, err, st, batch);
    case 64: return launch_ws_bn<64>(w, e, err, st, batch);
    case 128: return launch_ws_bn<128>(w, e, err, st, batch);
    default: return launch_ws_bn<256>(w, e, err, st, batch);
  }
}

// Split-K with B from FP32 (BN = 32): one split per resident CTA.
int ws_split_count(int kblocks, int ksplit) {
  int slots = 0;
  if (ws_slots<32>(slots) != cudaSuccess) slots = 1;
  return std::max(1, std::min(kblocks, std::max(ksplit, slots)));
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
    splitk_reduce_kernel<<<(unsigned)((n + REDUCE_WARPS - 1) / REDUCE_WARPS), 32 * REDUCE_WARPS, 0, st>>>(
        part, splits, (int)(mtiles * ntiles), ntiles, BN, e);
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
  Epi e = epi;
  e.M = M;
  e.N = N;
  e.ybs = 0;
  tg::WsArgs w{};
  w.a = tg::ws::Op{a, aa, 0, M, 0, 0};
  w.b = tg::ws::Op{b, ba, 0, N, 0, 0};
  w.K = K;
  w.kblocks = kblocks;
  w.ntiles = ntiles;
  w.mtiles = mtiles;
  auto ensure_part = [&](size_t need) -> int {
    if (need > part_cap) {
      if (part) cudaFree(part);
      part = nullptr;
      part_cap = 0;
      if (cudaMalloc(&part, need * sizeof(float)) != cudaSuccess) return MSX_ERR_ALLOC;
      part_cap = need;
    }
    return MSX_OK;
  };
  if (ksplit > 1 && bn == 32) {
    // long K, narrow output (weight gradients): split K over the persistent CTAs, both
    // operands rounded to bfloat16 as they are loaded, partial tiles summed in split order
    const int splits = tg::ws_split_count(kblocks, ksplit);
    w.kper = (kblocks + splits - 1) / splits;
    w.splits = (kblocks + w.kper - 1) / w.kper;
    int rc = reserve(0, 0);
    if (rc != MSX_OK) return rc;
    rc = ensure_part((size_t)w.splits * mtiles * ntiles * tg::BM * bn);
    if (rc != MSX_OK) return rc;
    w.part = part;
    w.b_img = nullptr;
    cudaError_t c = tg::launch_ws(bn, w, e, err, st, 1);
    if (c != cudaSuccess) return MSX_ERR_CUDA;
    const long long n = M * (long long)N;
    tg::splitk_reduce_kernel<<<(unsigned)((n + tg::REDUCE_WARPS - 1) / tg::REDUCE_WARPS), 32 * tg::REDUCE_WARPS, 0,
                               st>>>(part, w.splits, (int)(mtiles * ntiles), ntiles, bn, e);
    return cudaGetLastError() == cudaSuccess ? MSX_OK : MSX_ERR_CUDA;
  }
  int kper = kblocks;
  if (ksplit > 1) kper = (kblocks + ksplit - 1) / ksplit;
  const int splits = (kblocks + kper - 1) / kper;
  const size_t a_bytes = splits > 1 ? (size_t)mtiles * kblocks * tg::A_BYTES : 0;
  const size_t b_bytes = (size_t)ntiles * kblocks * bn * tg::BK * 2;
  int rc = reserve(a_bytes, b_bytes);
  if (rc != MSX_OK) return rc;
  const long long a_rows = mtiles * tg::BM, b_rows = (long long)ntiles * bn;
  const long long a_thr = a_rows * kblocks * (tg::BK / 8), b_thr = b_rows * kblocks * (tg::BK / 8);
  tg::pack_kernel<<<(unsigned)((b_thr + 255) / 256), 256, 0, st>>>(b, ba, N, K, bn, b_rows, kblocks,
                                                                   reinterpret_cast<uint4*>(b_img));
  const uint8_t* bi = reinterpret_cast<const uint8_t*>(b_img);
  cudaError_t c;
  if (splits == 1) {  // persistent kernel, A rounded to bfloat16 as it is loaded
    w.kper = kblocks;
    w.splits = 1;
    w.b_img = bi;
    c = tg::launch_ws(bn, w, e, err, st, 1);
    return c == cudaSuccess ? MSX_OK : MSX_ERR_CUDA;
  }
  // split K with a wide output: both operands packed, one CTA per (tile, split)
  rc = ensure_part((size_t)splits * mtiles * ntiles * tg::BM * bn);
  if (rc != MSX_OK) return rc;
  tg::pack_kernel<<<(unsigned)((a_thr + 255) / 256), 256, 0, st>>>(a, aa, M, K, tg::BM, a_rows, kblocks,
                                                                   reinterpret_cast<uint4*>(a_img));
  const uint8_t* ai = reinterpret_cast<const uint8_t*>(a_img);
  switch (bn) {
    case 32: c = tg::launch_gemm_bn<32>(ai, bi, mtiles, ntiles, kblocks, kper, part, e, err, st); break;
    case 64: c = tg::launch_gemm_bn<64>(ai, bi, mtiles, ntiles, kblocks, kper, part, e, err, st); break;
    case 128: c = tg::launch_gemm_bn<128>(ai, bi, mtiles, ntiles, kblocks, kper, part, e, err, st); break;
    default: c = tg::launch_gemm_bn<256>(ai, bi, mtiles, ntiles, kblocks, kper, part, e, err, st); break;
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
  const size_t b_bytes = (size_t)batch * ntiles * kblocks * bn * tg::BK * 2;
  int rc = reserve(0, b_bytes);
  if (rc != MSX_OK) return rc;
  const long long b_rows = (long long)ntiles * bn;
  const long long b_thr = b_rows * kblocks * (tg::BK / 8) * batch;
  tg::pack_kernel<<<(unsigned)((b_thr + 255) / 256), 256, 0, st>>>(b, ba, N, K, bn, b_rows, kblocks,
                                                                   reinterpret_cast<uint4*>(b_img), batch, b_bs);
  Epi e = epi;
  e.M = M;
  e.N = N;
  e.ybs = y_bs;
  const uint8_t* bi = reinterpret_cast<const uint8_t*>(b_img);
  cudaError_t c;
  tg::WsArgs w{};
  w.a = tg::ws::Op{a, aa, a_bs, M, 0, 0};
  w.b_img = bi;
  w.K = K;
  w.kblocks = kblocks;
  w.kper = kblocks;
  w.splits = 1;
  w.ntiles = ntiles;
  w.mtiles = mtiles;
  c = tg::launch_ws(bn, w, e, err, st, batch);
  return c == cudaSuccess ? MSX_OK : MSX_ERR_CUDA;
}

int TcGemm::run_cplx(const float* a, Addr aa, long long a_bs, const float* src, long long si, long long sj,
                     long long src_bs, int hn, int hk, int neg, long long M, const Epi& epi, long long y_bs, int batch,
                     cudaStream_t st) {
  if (batch < 1 || M <= 0 || hn <= 0 || hk <= 0 || 2 * hn > 4096 || neg < 0 || neg > 2) return MSX_ERR_INVALID;
  const int N = 2 * hn;
  const long long K = 2LL * hk;
  const int bn = bn_for(N);
  const long long mtiles = (M + tg::BM - 1) / tg::BM;
  const int ntiles = (N + bn - 1) / bn;
  const int kblocks = (int)((K + tg::BK - 1) / tg::BK);
  if (mtiles * ntiles * batch > (1LL << 30)) return MSX_ERR_INVALID;
  const size_t b_bytes = (size_t)batch * ntiles * kblocks * bn * tg::BK * 2;
  int rc = reserve(0, b_bytes);
  if (rc != MSX_OK) return rc;
  const int b_rows = ntiles * bn;
  const long long b_thr = (long long)b_rows * kblocks * (tg::BK / 8) * batch;
  tg::pack_cplx_kernel<<<(unsigned)((b_thr + 255) / 256), 256, 0, st>>>(src, si, sj, src_bs, hn, hk, neg, bn, b_rows,
                                                                        kblocks, reinterpret_cast<uint4*>(b_img),
                                                                        batch);
  Epi e = epi;
  e.M = M;
  e.N = N;
  e.ybs = y_bs;
  const uint8_t* bi = reinterpret_cast<const uint8_t*>(b_img);
  cudaError_t c;
  tg::WsArgs w{};
  w.a = tg::ws::Op{a, aa, a_bs, M, 0, 0};
  w.b_img = bi;
  w.K = K;
  w.kblocks = kblocks;
  w.kper = kblocks;
  w.splits = 1;
  w.ntiles = ntiles;
  w.mtiles = mtiles;
  c = tg::launch_ws(bn, w, e, err, st, batch);
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
